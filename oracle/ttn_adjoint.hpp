// ttn_adjoint.hpp -- reverse-mode (adjoint) form of the oracle's sweep.  TEST
// INFRASTRUCTURE ONLY, like the rest of oracle/: included by ttn_oracle.cpp inside
// namespace orc after Engine.
//
// Objective: J = sum_t w_t Re <psi(t)| O |psi(t)> over the ends of the integrator's steps
// (the first step sub-stepped as in projector_splitting_integrator.hpp:136-169), O a
// one-mode operator evaluated by the leaf-to-root contraction of
// observables/matrix_element.hpp:264-314.  Gradients: dJ/dc_r for every term coefficient
// (real perturbations) and the cotangent of every primitive operator matrix, from which a
// caller forms the derivative with respect to any parameter its operators depend on
// (bath couplings, frequencies, bias, tunnelling).
//
// Method (discrete adjoint of the sweep as it is computed):
//   * the state is checkpointed every K steps; a segment is recomputed from its
//     checkpoint, and every sweep is re-run once more with its operations recorded
//     (inputs and the environments they read), then reversed operation by operation;
//   * single-particle environments are consistent with the state at every sweep boundary
//     (each is last written from the node's final tensor), so a re-run from a stored state
//     recomputes them bottom-up and reproduces the original sweep bit for bit;
//   * y = exp(z H) x (z = coeff * tau): x_bar = exp(conj(z) H) y_bar, and the cotangents of
//     the environments and coefficients inside H come from
//     Re <y_bar, dy> = Re int_0^1 <conj(z) a(s), dH b(s)> ds,
//     a(s) = exp((1-s) conj(z) H) y_bar, b(s) = exp(s z H) x (H Hermitian), evaluated by
//     Gauss-Legendre quadrature with the node count set from a Lanczos estimate of the
//     spectral width (the integrand oscillates at most at |z| (l_max - l_min));
//   * QR (A = Q R, R with a real diagonal, the LAPACK zgeqrf gauge):
//     M1 = R R_bar^H, M2 = Q_bar^H Q, N = M2 - M1, K = upper part of N - N^H with
//     K_ii = i Im N_ii, W = M1 + K, A_bar = (Q_bar + Q (W^H - M2^H)) R^-H;
//   * contractions reverse into contractions of the same kinds (mode products with S^H,
//     mode_contract for the operator cotangents).
// Requires full-rank gauge factors (R invertible): from a product state the tensors
// of rank-deficient bonds are not differentiable functions of the inputs.

static double gl_leg(int n, double x, double& dp) {
  double p0 = 1.0, p1 = x;
  for (int k = 2; k <= n; ++k) {
    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1; p1 = p2;
  }
  dp = n * (x * p1 - p0) / (x * x - 1.0);
  return p1;
}
// Gauss-Legendre nodes and weights on [0, 1], nodes ascending.
static void gauss_legendre01(int n, std::vector<double>& s, std::vector<double>& w) {
  s.assign(n, 0.0); w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double x = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      const double p = gl_leg(n, x, dp);
      const double dx = p / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    gl_leg(n, x, dp);
    s[n - 1 - i] = 0.5 * (x + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - x * x) * dp * dp);
  }
}

static cd dotc(const cd* x, const cd* y, size_t n) {  // sum conj(x) y
  cd s = 0.0;
  for (size_t i = 0; i < n; ++i) s += cmulc(x[i], y[i]);
  return s;
}
static std::vector<cd> herm(const cd* S, int d) {  // S^H
  std::vector<cd> o((size_t)d * d);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) o[(size_t)i * d + j] = std::conj(S[(size_t)j * d + i]);
  return o;
}
// dst(i,j) += alpha * M(j,i)
static void add_transposed(const cd* M, int d, cd* dst, cd alpha = 1.0) {
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) dst[(size_t)i * d + j] += alpha * M[(size_t)j * d + i];
}

// Reverse of A = Q R (m x n, m >= n, Householder gauge: real diagonal of R).
static std::vector<cd> qr_vjp(const cd* Q, const cd* R, const cd* Qb, const cd* Rb, size_t m, int n) {
  const size_t nn = (size_t)n * n;
  std::vector<cd> M1(nn, 0.0), M2(nn, 0.0), W(nn);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      cd s = 0.0;
      for (int k = 0; k < n; ++k) s += R[(size_t)i * n + k] * std::conj(Rb[(size_t)j * n + k]);
      M1[(size_t)i * n + j] = s;
    }
  for (size_t x = 0; x < m; ++x)
    for (int i = 0; i < n; ++i) {
      const cd qb = std::conj(Qb[x * n + i]);
      for (int j = 0; j < n; ++j) M2[(size_t)i * n + j] += qb * Q[x * n + j];
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const cd Nij = M2[(size_t)i * n + j] - M1[(size_t)i * n + j];
      const cd Nji = M2[(size_t)j * n + i] - M1[(size_t)j * n + i];
      cd K = 0.0;
      if (i < j) K = Nij - std::conj(Nji);
      else if (i == j) K = cd(0.0, Nij.imag());
      W[(size_t)i * n + j] = M1[(size_t)i * n + j] + K;
    }
  // C = W^H - M2^H;  B = Q_bar + Q C;  A_bar = B R^-H (row by row: y R^H = b)
  std::vector<cd> C(nn);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      C[(size_t)i * n + j] = std::conj(W[(size_t)j * n + i]) - std::conj(M2[(size_t)j * n + i]);
  std::vector<cd> Ab(m * n);
  std::vector<cd> b(n);
  for (size_t x = 0; x < m; ++x) {
    for (int j = 0; j < n; ++j) {
      cd s = Qb[x * n + j];
      for (int k = 0; k < n; ++k) s += Q[x * n + k] * C[(size_t)k * n + j];
      b[j] = s;
    }
    cd* y = &Ab[x * n];
    for (int j = n - 1; j >= 0; --j) {
      cd s = b[j];
      for (int k = j + 1; k < n; ++k) s -= y[k] * std::conj(R[(size_t)j * n + k]);
      const double d = R[(size_t)j * n + j].real();
      if (d == 0.0) throw Error(ENUM, "adjoint: singular gauge factor R (rank-deficient bond)");
      y[j] = s / d;
    }
  }
  return Ab;
}

struct EnvSnap { int which, nd, g; std::vector<cd> v; };  // which: 0 spf, 1 mf
struct TapeRec {
  int kind = 0, nd = 0, aux = 0;
  double tau = 0.0;
  cd cf = 0.0;
  std::vector<cd> x0, x1;
  std::vector<EnvSnap> env;
};

// One link of a chain of mode products: out = S x_mode in, S of size d x d; Sb collects
// the cotangent of S (null for operators without one).
struct Link { const cd* S; int d; size_t na, nb; cd* Sb; };

struct Adjoint {
  Engine& E;
  const Tree& T;
  const Plan& P;
  std::vector<std::vector<cd>> Ab, rb;                  // cotangents of A, rmat
  std::vector<std::vector<std::vector<cd>>> sb, mb;     // of spf, mf  [node][group]
  std::vector<std::vector<std::vector<cd>>> gop;        // of the operators [mode][k]
  std::vector<double> gc;                               // dJ/dc_r
  std::vector<TapeRec> tape;
  bool recording = false;
  int quad_min = 8, quad_max = 96;

  explicit Adjoint(Engine& e) : E(e), T(e.T), P(e.P) {
    Ab.assign(T.n, {}); rb.assign(T.n, {}); sb.assign(T.n, {}); mb.assign(T.n, {});
    for (int i = 0; i < T.n; ++i) {
      Ab[i].assign(T.size(i), 0.0);
      rb[i].assign(E.rmat[i].size(), 0.0);
      sb[i].assign(P.groups[i].size(), {});
      mb[i].assign(P.groups[i].size(), {});
      const size_t rr = (size_t)T.hrank[i] * T.hrank[i];
      for (size_t g = 0; g < P.groups[i].size(); ++g) { sb[i][g].assign(rr, 0.0); mb[i][g].assign(rr, 0.0); }
    }
    gop.assign(E.H.nmodes, {});
    for (int m = 0; m < E.H.nmodes; ++m)
      for (auto& M : E.H.ops[m]) gop[m].push_back(std::vector<cd>(M.size(), 0.0));
    gc.assign(E.H.nterms, 0.0);
    if (const char* q = std::getenv("ORC_ADJ_QUAD_MIN")) quad_min = std::max(2, std::atoi(q));
  }

  // ---- environment snapshots of what each operation reads
  void snap(TapeRec& rc, int which, int nd, int g) {
    const auto& v = which == 0 ? E.spf[nd][g] : E.mf[nd][g];
    rc.env.push_back({which, nd, g, v});
  }
  void snap_items(TapeRec& rc, int nd, const std::vector<Item>& items) {
    for (const Item& it : items)
      if (it.slot >= 0) snap(rc, 0, T.children[nd][it.slot], it.grp);
  }
  void restore(const TapeRec& rc) {
    for (const EnvSnap& s : rc.env) (s.which == 0 ? E.spf[s.nd][s.g] : E.mf[s.nd][s.g]) = s.v;
  }

  void record(int kind, int nd, int aux) {
    if (!recording) return;
    TapeRec rc;
    rc.kind = kind; rc.nd = nd; rc.aux = aux;
    const int r = T.hrank[nd];
    switch (kind) {
      case OP_AFP: {
        const int p = T.parent[nd];
        rc.x0 = E.A[nd];
        rc.x1.assign(E.rmat[p].begin(), E.rmat[p].begin() + (size_t)r * r);
        break;
      }
      case OP_R2L: case OP_L2R: rc.x0 = E.A[nd]; break;
      case OP_MF: {
        const int p = T.parent[nd];
        rc.x0 = E.A[p];
        for (size_t g = 0; g < P.groups[nd].size(); ++g) {
          const Group& G = P.groups[nd][g];
          if (G.id_mf) continue;
          for (const MfKey& k : G.mf) {
            if (!P.groups[p][k.pg].id_mf) snap(rc, 1, p, k.pg);
            snap_items(rc, p, k.sib);
          }
        }
        break;
      }
      case OP_NODE: {
        rc.x0 = E.A[nd];
        rc.tau = E.dt / 2.0; rc.cf = E.coeff;
        for (size_t g = 0; g < P.groups[nd].size(); ++g) {
          const Group& G = P.groups[nd][g];
          if (!G.id_mf) snap(rc, 1, nd, (int)g);
          if (!G.id_spf) for (const SpfTuple& t : G.spf) snap_items(rc, nd, t.items);
        }
        break;
      }
      case OP_SPF: {
        rc.x0 = E.A[nd];
        for (size_t g = 0; g < P.groups[nd].size(); ++g) {
          const Group& G = P.groups[nd][g];
          if (!G.id_spf) for (const SpfTuple& t : G.spf) snap_items(rc, nd, t.items);
        }
        break;
      }
      case OP_BOND: {
        rc.x0.assign(E.rmat[aux].begin(), E.rmat[aux].begin() + (size_t)r * r);
        rc.tau = -E.dt / 2.0; rc.cf = E.coeff;
        for (size_t g = 0; g < P.groups[nd].size(); ++g) {
          const Group& G = P.groups[nd][g];
          if (!G.id_spf) snap(rc, 0, nd, (int)g);
          if (!G.id_mf) snap(rc, 1, nd, (int)g);
        }
        break;
      }
      case OP_ATP: {
        rc.x0 = E.A[T.parent[nd]];
        rc.x1.assign(E.rmat[nd].begin(), E.rmat[nd].begin() + (size_t)r * r);
        break;
      }
      default: throw Error(EINVAL_, "adjoint: unknown operation");
    }
    tape.push_back(std::move(rc));
  }

  // ---- chains of mode products
  std::vector<Link> links_items(int nd, const std::vector<Item>& items) {
    std::vector<Link> L;
    for (const Item& it : items) {
      size_t na, nb; int d;
      if (it.slot < 0) {
        const int mode = T.leaf_mode[nd];
        L.push_back({E.H.ops[mode][it.grp].data(), T.dims[nd][0], 1, (size_t)T.hrank[nd], gop[mode][it.grp].data()});
      } else {
        E.r3(nd, it.slot, na, d, nb);
        const int c = T.children[nd][it.slot];
        L.push_back({E.spf[c][it.grp].data(), d, na, nb, sb[c][it.grp].data()});
      }
    }
    return L;
  }
  std::vector<Link> links_sibs(int p, const std::vector<Item>& items) {
    std::vector<Link> L;
    for (const Item& it : items) {
      size_t na, nb; int d;
      E.r3(p, it.slot, na, d, nb);
      const int c = T.children[p][it.slot];
      L.push_back({E.spf[c][it.grp].data(), d, na, nb, sb[c][it.grp].data()});
    }
    return L;
  }
  // forward: ins[k] is the input of link k; returns the output
  std::vector<cd> chain_fwd(const std::vector<Link>& L, const cd* v, size_t n, std::vector<std::vector<cd>>& ins) {
    ins.clear();
    std::vector<cd> cur(v, v + n);
    for (const Link& l : L) {
      ins.push_back(cur);
      std::vector<cd> nxt(n);
      mode_apply(l.S, l.d, cur.data(), nxt.data(), l.na, l.nb);
      cur.swap(nxt);
    }
    return cur;
  }
  // reverse: g holds the output cotangent and, on return, the input cotangent
  void chain_rev(const std::vector<Link>& L, const std::vector<std::vector<cd>>& ins, std::vector<cd>& g) {
    const size_t n = g.size();
    for (int k = (int)L.size() - 1; k >= 0; --k) {
      const Link& l = L[k];
      if (l.Sb) {
        std::vector<cd> t((size_t)l.d * l.d);
        mode_contract(ins[k].data(), g.data(), l.na, l.d, l.nb, t.data(), 1.0, false);
        add_transposed(t.data(), l.d, l.Sb);
      }
      std::vector<cd> SH = herm(l.S, l.d), nxt(n);
      mode_apply(SH.data(), l.d, g.data(), nxt.data(), l.na, l.nb);
      g.swap(nxt);
    }
  }

  // ---- spectral width of a Hermitian operator (Lanczos Ritz values from v)
  template <typename Op>
  double spectral_width(Op&& hop, const cd* v, size_t n) {
    const int k = (int)std::min<size_t>(n, 30);
    std::vector<cd> q(v, v + n), qp(n, 0.0), w(n);
    double nv = std::sqrt(dotc(q.data(), q.data(), n).real());
    if (nv == 0.0) return 0.0;
    for (auto& z : q) z /= nv;
    std::vector<double> al, be;
    double bprev = 0.0;
    for (int j = 0; j < k; ++j) {
      hop(q.data(), w.data());
      const double a = dotc(q.data(), w.data(), n).real();
      for (size_t i = 0; i < n; ++i) w[i] -= a * q[i] + bprev * qp[i];
      const double b = std::sqrt(dotc(w.data(), w.data(), n).real());
      al.push_back(a);
      if (b <= 1e-12 * (std::fabs(a) + bprev) || j == k - 1) break;
      be.push_back(b);
      qp = q;
      for (size_t i = 0; i < n; ++i) q[i] = w[i] / b;
      bprev = b;
    }
    const int m = (int)al.size();
    std::vector<double> d(al), e(std::max(m - 1, 1), 0.0), z((size_t)m * m);
    for (int i = 0; i + 1 < m; ++i) e[i] = be[i];
    tql2(m, d.data(), e.data(), z.data());
    return *std::max_element(d.begin(), d.end()) - *std::min_element(d.begin(), d.end());
  }

  // ---- reverse of y = exp(cf tau H) x: returns x_bar; vjp(b, g) adds the cotangents of
  // H's environments and coefficients for Re <g, dH b>
  template <typename Op, typename Vjp>
  std::vector<cd> expm_vjp(Op&& hop, Vjp&& vjp, size_t n, const std::vector<cd>& x, const std::vector<cd>& yb,
                           double tau, cd cf) {
    const cd z = cf * tau;
    bool zero = true;
    for (const cd& v : yb) if (v != cd(0.0)) { zero = false; break; }
    if (zero) return std::vector<cd>(n, 0.0);
    const double width = std::max(spectral_width(hop, x.data(), n), spectral_width(hop, yb.data(), n));
    const double omega = std::abs(z) * width * 1.1;
    const int nq = std::min(quad_max, std::max(quad_min, (int)std::ceil(0.5 * omega) + 10));
    std::vector<double> s, w;
    gauss_legendre01(nq, s, w);
    std::vector<std::vector<cd>> B(nq);
    std::vector<cd> b = x;
    double sp = 0.0;
    for (int j = 0; j < nq; ++j) {
      E.expm(hop, b.data(), n, (s[j] - sp) * tau, cf);
      B[j] = b;
      sp = s[j];
    }
    std::vector<cd> a = yb, g(n);
    sp = 1.0;
    for (int j = nq - 1; j >= 0; --j) {
      E.expm(hop, a.data(), n, (sp - s[j]) * tau, std::conj(cf));
      const cd f = w[j] * std::conj(z);
      for (size_t i = 0; i < n; ++i) g[i] = f * a[i];
      vjp(B[j], g);
      sp = s[j];
    }
    E.expm(hop, a.data(), n, sp * tau, std::conj(cf));
    return a;
  }

  // cotangents of the scalar s and of mf for out = s * mf_apply(X, M) (or s * X when the
  // mean field is the identity); returns the cotangent of X
  std::vector<cd> mf_stage_vjp(const Group& G, int nd, int gi, const std::vector<cd>& X, const std::vector<cd>& g) {
    const int r = T.hrank[nd];
    const size_t n = X.size(), nx = n / r;
    std::vector<cd> Xb(n);
    cd sig;
    if (G.id_mf) {
      sig = dotc(X.data(), g.data(), n);
      for (size_t i = 0; i < n; ++i) Xb[i] = std::conj(G.s) * g[i];
    } else {
      const cd* M = E.mf[nd][gi].data();
      std::vector<cd> F(n);
      mf_apply(X.data(), M, r, nx, F.data(), 1.0, false);
      sig = dotc(F.data(), g.data(), n);
      std::vector<cd> t((size_t)r * r);
      adj_mul(X.data(), g.data(), nx, r, t.data(), 1.0, false);
      add_transposed(t.data(), r, mb[nd][gi].data(), std::conj(G.s));
      std::vector<cd> MH = herm(M, r);
      mf_apply(g.data(), MH.data(), r, nx, Xb.data(), std::conj(G.s), false);
    }
    if (G.type == G_1) gc[G.members[0]] += sig.real();
    return Xb;
  }

  // cotangents of everything H_eff(nd) depends on, for Re <g, dH_eff v>
  void heff_vjp(int nd, const std::vector<cd>& v, const std::vector<cd>& g) {
    const size_t n = v.size();
    for (size_t gi = 0; gi < P.groups[nd].size(); ++gi) {
      const Group& G = P.groups[nd][gi];
      std::vector<std::vector<std::vector<cd>>> ins(G.spf.size());
      std::vector<std::vector<cd>> Y(G.spf.size());
      std::vector<std::vector<Link>> L(G.spf.size());
      std::vector<cd> X;
      if (G.id_spf) X = v;
      else {
        X.assign(n, 0.0);
        for (size_t q = 0; q < G.spf.size(); ++q) {
          L[q] = links_items(nd, G.spf[q].items);
          Y[q] = chain_fwd(L[q], v.data(), n, ins[q]);
          for (size_t i = 0; i < n; ++i) X[i] += G.spf[q].a * Y[q][i];
        }
      }
      std::vector<cd> Xb = mf_stage_vjp(G, nd, (int)gi, X, g);
      if (G.id_spf) continue;
      for (size_t q = 0; q < G.spf.size(); ++q) {
        const SpfTuple& t = G.spf[q];
        if (!t.a_mem.empty()) {
          const double ab = dotc(Y[q].data(), Xb.data(), n).real();
          for (int rr : t.a_mem) gc[rr] += ab;
        }
        std::vector<cd> gt(n);
        for (size_t i = 0; i < n; ++i) gt[i] = std::conj(t.a) * Xb[i];
        chain_rev(L[q], ins[q], gt);
      }
    }
  }

  // the same for the bond Hamiltonian K(nd) acting on an r x r matrix R
  void kbond_vjp(int nd, const std::vector<cd>& R, const std::vector<cd>& g) {
    const int r = T.hrank[nd];
    const size_t rr = (size_t)r * r;
    for (size_t gi = 0; gi < P.groups[nd].size(); ++gi) {
      const Group& G = P.groups[nd][gi];
      std::vector<cd> X = R;
      if (!G.id_spf) matmul(E.spf[nd][gi].data(), R.data(), r, r, r, X.data());
      std::vector<cd> Xb = mf_stage_vjp(G, nd, (int)gi, X, g);
      if (G.id_spf) continue;
      cd* Sb = sb[nd][gi].data();  // S_bar += X_bar R^H
      for (int i = 0; i < r; ++i)
        for (int k = 0; k < r; ++k) {
          cd s = 0.0;
          for (int j = 0; j < r; ++j) s += Xb[(size_t)i * r + j] * std::conj(R[(size_t)k * r + j]);
          Sb[(size_t)i * r + k] += s;
        }
      (void)rr;
    }
  }

  // ---- permutation of r2l: M[(y*pre + x)*dm + i] = a[(x*dm + i)*post + y]
  void r2l_shape(int nd, int mu, size_t& pre, int& dm, size_t& post) const {
    pre = 1; post = (size_t)T.hrank[nd];
    for (int i = 0; i < mu; ++i) pre *= T.dims[nd][i];
    dm = T.dims[nd][mu];
    for (int i = mu + 1; i < T.nmodes[nd]; ++i) post *= T.dims[nd][i];
  }
  static void permute(const cd* a, cd* M, size_t pre, int dm, size_t post, bool inverse) {
    for (size_t x = 0; x < pre; ++x)
      for (int i = 0; i < dm; ++i)
        for (size_t y = 0; y < post; ++y) {
          if (!inverse) M[(y * pre + x) * dm + i] = a[(x * dm + i) * post + y];
          else M[(x * dm + i) * post + y] = a[(y * pre + x) * dm + i];
        }
  }

  // ---- reverse of one recorded operation
  void reverse(const TapeRec& rc) {
    const int nd = rc.nd, r = T.hrank[nd];
    const size_t rr = (size_t)r * r;
    switch (rc.kind) {
      case OP_AFP: {  // A <- A Rp
        const int p = T.parent[nd];
        const size_t m = T.dimen[nd];
        std::vector<cd> Ain(m * r, 0.0), RH = herm(rc.x1.data(), r), t(rr);
        matmul(Ab[nd].data(), RH.data(), (int)m, r, r, Ain.data());
        adj_mul(rc.x0.data(), Ab[nd].data(), m, r, t.data(), 1.0, false);
        for (size_t i = 0; i < rr; ++i) rb[p][i] += t[i];
        Ab[nd] = Ain;
        break;
      }
      case OP_ATP: {  // A_p <- R x_mu A_p
        const int p = T.parent[nd], mu = T.slot[nd];
        size_t na, nb; int d;
        E.r3(p, mu, na, d, nb);
        std::vector<cd> RH = herm(rc.x1.data(), d), Ain(T.size(p)), t((size_t)d * d);
        mode_apply(RH.data(), d, Ab[p].data(), Ain.data(), na, nb);
        mode_contract(rc.x0.data(), Ab[p].data(), na, d, nb, t.data(), 1.0, false);
        add_transposed(t.data(), d, rb[nd].data());
        Ab[p] = Ain;
        break;
      }
      case OP_L2R: {  // A = Q R; A <- Q, rmat <- R
        const size_t m = T.dimen[nd];
        std::vector<cd> Q = rc.x0, R(rr), tau;
        householder_qr(Q.data(), m, r, R.data(), tau);
        std::vector<cd> Rb(rb[nd].begin(), rb[nd].begin() + rr);
        Ab[nd] = qr_vjp(Q.data(), R.data(), Ab[nd].data(), Rb.data(), m, r);
        std::fill(rb[nd].begin(), rb[nd].end(), cd(0.0));
        break;
      }
      case OP_R2L: {  // permuted M = Q R; A <- unpermute(Q), rmat <- R^T
        size_t pre, post; int dm;
        r2l_shape(nd, rc.aux, pre, dm, post);
        const size_t d1 = pre * post, sz = T.size(nd);
        std::vector<cd> Q(sz), R((size_t)dm * dm), tau, Qb(sz), Rb((size_t)dm * dm);
        permute(rc.x0.data(), Q.data(), pre, dm, post, false);
        householder_qr(Q.data(), d1, dm, R.data(), tau);
        permute(Ab[nd].data(), Qb.data(), pre, dm, post, false);
        for (int i = 0; i < dm; ++i)
          for (int j = 0; j < dm; ++j) Rb[(size_t)j * dm + i] = rb[nd][(size_t)i * dm + j];
        std::vector<cd> Mb = qr_vjp(Q.data(), R.data(), Qb.data(), Rb.data(), d1, dm);
        permute(Mb.data(), Ab[nd].data(), pre, dm, post, true);
        std::fill(rb[nd].begin(), rb[nd].end(), cd(0.0));
        break;
      }
      case OP_NODE: {
        restore(rc);
        const size_t n = T.size(nd);
        Ab[nd] = expm_vjp([&](const cd* v, cd* o) { E.heff(nd, v, o); },
                          [&](const std::vector<cd>& b, const std::vector<cd>& g) { heff_vjp(nd, b, g); },
                          n, rc.x0, Ab[nd], rc.tau, rc.cf);
        break;
      }
      case OP_BOND: {
        restore(rc);
        std::vector<cd> yb(rb[rc.aux].begin(), rb[rc.aux].begin() + rr);
        std::vector<cd> xb = expm_vjp([&](const cd* v, cd* o) { E.kbond(nd, v, o); },
                                      [&](const std::vector<cd>& b, const std::vector<cd>& g) { kbond_vjp(nd, b, g); },
                                      rr, rc.x0, yb, rc.tau, rc.cf);
        std::copy(xb.begin(), xb.end(), rb[rc.aux].begin());
        break;
      }
      case OP_SPF: {
        restore(rc);
        const size_t n = T.size(nd), nx = n / r;
        const cd* A = rc.x0.data();
        for (size_t gi = 0; gi < P.groups[nd].size(); ++gi) {
          const Group& G = P.groups[nd][gi];
          if (G.id_spf) continue;
          const cd* Sb = sb[nd][gi].data();
          std::vector<cd> SbC(rr), SbT(rr);
          for (int i = 0; i < r; ++i)
            for (int j = 0; j < r; ++j) {
              SbC[(size_t)i * r + j] = std::conj(Sb[(size_t)i * r + j]);
              SbT[(size_t)i * r + j] = Sb[(size_t)j * r + i];
            }
          for (const SpfTuple& t : G.spf) {
            std::vector<std::vector<cd>> ins;
            std::vector<Link> L = links_items(nd, t.items);
            std::vector<cd> X = chain_fwd(L, A, n, ins);
            mf_apply(X.data(), SbC.data(), r, nx, Ab[nd].data(), t.a, true);  // bra side
            if (!t.a_mem.empty()) {
              std::vector<cd> z(rr);
              adj_mul(A, X.data(), nx, r, z.data(), 1.0, false);
              const double ab = dotc(z.data(), Sb, rr).real();
              for (int q : t.a_mem) gc[q] += ab;
            }
            std::vector<cd> Xb(n);
            mf_apply(A, SbT.data(), r, nx, Xb.data(), std::conj(t.a), false);
            chain_rev(L, ins, Xb);
            for (size_t i = 0; i < n; ++i) Ab[nd][i] += Xb[i];  // ket side
          }
          std::fill(sb[nd][gi].begin(), sb[nd][gi].end(), cd(0.0));
        }
        break;
      }
      case OP_MF: {
        restore(rc);
        const int p = T.parent[nd], mu = T.slot[nd], rp = T.hrank[p];
        size_t na, nb; int d;
        E.r3(p, mu, na, d, nb);
        const size_t szp = T.size(p), dd = (size_t)d * d;
        const cd* Ap = rc.x0.data();
        for (size_t gi = 0; gi < P.groups[nd].size(); ++gi) {
          const Group& G = P.groups[nd][gi];
          if (G.id_mf) continue;
          const cd* Mb = mb[nd][gi].data();
          for (const MfKey& k : G.mf) {
            std::vector<std::vector<cd>> ins;
            std::vector<Link> L = links_sibs(p, k.sib);
            std::vector<cd> Y0 = chain_fwd(L, Ap, szp, ins), Tm;
            const bool pm = !P.groups[p][k.pg].id_mf;
            if (pm) {
              Tm.assign(szp, 0.0);
              mf_apply(Y0.data(), E.mf[p][k.pg].data(), rp, szp / rp, Tm.data(), 1.0, false);
            } else Tm = Y0;
            std::vector<cd> S1(dd), S2(dd);
            for (int i = 0; i < d; ++i)
              for (int j = 0; j < d; ++j) {
                S1[(size_t)i * d + j] = k.b * std::conj(Mb[(size_t)i * d + j]);
                S2[(size_t)j * d + i] = std::conj(k.b) * Mb[(size_t)i * d + j];
              }
            std::vector<cd> tmp(szp);
            mode_apply(S1.data(), d, Tm.data(), tmp.data(), na, nb);  // bra side
            for (size_t i = 0; i < szp; ++i) Ab[p][i] += tmp[i];
            if (!k.b_mem.empty()) {
              std::vector<cd> z(dd);
              mode_contract(Ap, Tm.data(), na, d, nb, z.data(), 1.0, false);
              const double bb = dotc(z.data(), Mb, dd).real();
              for (int q : k.b_mem) gc[q] += bb;
            }
            std::vector<cd> Tb(szp);
            mode_apply(S2.data(), d, Ap, Tb.data(), na, nb);
            std::vector<cd> Yb;
            if (pm) {
              const cd* Mp = E.mf[p][k.pg].data();
              std::vector<cd> t((size_t)rp * rp), MH = herm(Mp, rp);
              adj_mul(Y0.data(), Tb.data(), szp / rp, rp, t.data(), 1.0, false);
              add_transposed(t.data(), rp, mb[p][k.pg].data());
              Yb.assign(szp, 0.0);
              mf_apply(Tb.data(), MH.data(), rp, szp / rp, Yb.data(), 1.0, false);
            } else Yb = Tb;
            chain_rev(L, ins, Yb);
            for (size_t i = 0; i < szp; ++i) Ab[p][i] += Yb[i];  // ket side
          }
          std::fill(mb[nd][gi].begin(), mb[nd][gi].end(), cd(0.0));
        }
        break;
      }
      default: throw Error(EINVAL_, "adjoint: unknown operation");
    }
  }

  // ---- reverse of J += w Re <psi| O_mode |psi> (the leaf-to-root contraction of expect)
  void expect_vjp(int mode, const cd* op, double w) {
    std::vector<std::vector<cd>> mel(T.n), melb(T.n), X(T.n);
    std::vector<std::vector<std::vector<cd>>> ins(T.n);
    std::vector<std::vector<Link>> L(T.n);
    for (int id = T.n - 1; id >= 0; --id) {
      const int r = T.hrank[id];
      const size_t sz = T.size(id);
      mel[id].assign((size_t)r * r, 0.0);
      melb[id].assign((size_t)r * r, 0.0);
      if (T.leaf(id)) {
        X[id] = E.A[id];
        if (op && T.leaf_mode[id] == mode) mode_apply(op, T.dims[id][0], E.A[id].data(), X[id].data(), 1, r);
      } else {
        for (int s = 0; s < T.nmodes[id]; ++s) {
          size_t na, nb; int d;
          E.r3(id, s, na, d, nb);
          const int c = T.children[id][s];
          L[id].push_back({mel[c].data(), d, na, nb, melb[c].data()});
        }
        X[id] = chain_fwd(L[id], E.A[id].data(), sz, ins[id]);
      }
      adj_mul(E.A[id].data(), X[id].data(), sz / r, r, mel[id].data(), 1.0, false);
    }
    const int r0 = T.hrank[0];
    for (int k = 0; k < r0; ++k) melb[0][(size_t)k * r0 + k] = w;
    for (int id = 0; id < T.n; ++id) {
      const int r = T.hrank[id];
      const size_t sz = T.size(id), nx = sz / r, rr = (size_t)r * r;
      std::vector<cd> MC(rr), MT(rr), Xb(sz);
      for (int i = 0; i < r; ++i)
        for (int j = 0; j < r; ++j) {
          MC[(size_t)i * r + j] = std::conj(melb[id][(size_t)i * r + j]);
          MT[(size_t)i * r + j] = melb[id][(size_t)j * r + i];
        }
      mf_apply(X[id].data(), MC.data(), r, nx, Ab[id].data(), 1.0, true);  // bra side
      mf_apply(E.A[id].data(), MT.data(), r, nx, Xb.data(), 1.0, false);
      if (T.leaf(id)) {
        if (op && T.leaf_mode[id] == mode) {
          const int d = T.dims[id][0];
          std::vector<cd> OH = herm(op, d), t(sz);
          mode_apply(OH.data(), d, Xb.data(), t.data(), 1, r);
          Xb.swap(t);
        }
      } else chain_rev(L[id], ins[id], Xb);
      for (size_t i = 0; i < sz; ++i) Ab[id][i] += Xb[i];  // ket side
    }
  }

  void recompute_spf() { for (int id = T.n - 1; id >= 1; --id) E.update_spf(id); }
  void plain_sweep(double dt) { E.dt = dt; E.forward(true); E.backward(true); }

  // one sweep from A0 re-run with its operations recorded, then reversed
  void sweep_rev(const std::vector<std::vector<cd>>& A0, double dt, cd cf) {
    E.A = A0; E.dt = dt; E.coeff = cf;
    tape.clear();
    recording = true;
    E.on_op = [this](int k, int nd, int aux) { record(k, nd, aux); };
    try {
      recompute_spf();
      E.forward(true);
      E.backward(true);
    } catch (...) { E.on_op = nullptr; recording = false; throw; }
    E.on_op = nullptr;
    recording = false;
    for (auto it = tape.rbegin(); it != tape.rend(); ++it) reverse(*it);
    tape.clear();
  }

  static std::vector<double> step_schedule(double dt, bool first) {
    std::vector<double> s;
    if (!first) { s.push_back(dt); return s; }
    double tevolve = 0.0, sdt = dt / 1e5;
    while (tevolve < dt) {
      s.push_back((sdt + tevolve <= dt) ? sdt : dt - tevolve);
      tevolve += sdt;
      sdt *= 10.0;
    }
    return s;
  }

  // J and its gradients over nsteps integrator steps from the engine's current state.
  double run(double dt, cd cf, int nsteps, const double* w, int mode, const cd* op, int K, bool skip_prepare) {
    if (E.nsteps != 0) throw Error(EINVAL_, "adjoint: the integrator must be at step 0");
    if (nsteps < 1) throw Error(EINVAL_, "adjoint: nsteps must be >= 1");
    K = std::max(1, K);
    std::vector<std::vector<double>> sched(nsteps);
    for (int k = 0; k < nsteps; ++k) sched[k] = step_schedule(dt, k == 0);
    E.coeff = cf;
    if (skip_prepare) recompute_spf(); else E.prepare();
    std::vector<std::vector<std::vector<cd>>> ckpt((nsteps + K - 1) / K);
    double J = 0.0;
    for (int k = 0; k < nsteps; ++k) {
      if (k % K == 0) ckpt[k / K] = E.A;
      for (double d : sched[k]) plain_sweep(d);
      J += w[k] * E.expect(mode, op).real();
    }
    const auto final_state = E.A;
    for (int sg = (int)ckpt.size() - 1; sg >= 0; --sg) {
      const int k0 = sg * K, k1 = std::min(nsteps, k0 + K);
      std::vector<std::vector<std::vector<cd>>> st;  // starts of steps k0..k1-1, then the end
      E.A = ckpt[sg];
      recompute_spf();
      st.push_back(E.A);
      for (int k = k0; k < k1; ++k) {
        for (double d : sched[k]) plain_sweep(d);
        st.push_back(E.A);
      }
      for (int k = k1 - 1; k >= k0; --k) {
        E.A = st[k - k0 + 1];
        expect_vjp(mode, op, w[k]);
        std::vector<std::vector<std::vector<cd>>> sw;
        E.A = st[k - k0];
        recompute_spf();
        for (size_t q = 0; q < sched[k].size(); ++q) {
          sw.push_back(E.A);
          if (q + 1 < sched[k].size()) plain_sweep(sched[k][q]);
        }
        for (int q = (int)sched[k].size() - 1; q >= 0; --q) sweep_rev(sw[q], sched[k][q], cf);
      }
    }
    // the root's S-group mean fields are (sum of the members' coefficients) * identity
    const int r0 = T.hrank[0];
    for (size_t g = 0; g < P.groups[0].size(); ++g) {
      const Group& G = P.groups[0][g];
      if (G.id_mf) continue;
      cd tr = 0.0;
      for (int k = 0; k < r0; ++k) tr += mb[0][g][(size_t)k * r0 + k];
      for (int q : G.members) gc[q] += tr.real();
    }
    E.A = final_state;
    recompute_spf();
    E.nsteps = nsteps;
    return J;
  }
};
