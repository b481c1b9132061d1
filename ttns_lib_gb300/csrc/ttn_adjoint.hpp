// ttn_adjoint.hpp -- the adjoint (reverse-mode) sweep on the device.  Included by
// ttn_host.cpp inside namespace ttn, after Integrator.  No counterpart in the reference:
// it differentiates the one-site sweep of projector_splitting_engine.hpp:117-165 /
// tdvp_algorithm_engine.hpp:208-501 as this library computes it.
//
// Objective J = sum_k w_k Re <psi(t_k)| O |psi(t_k)> at the ends of the integrator's
// steps (the first step sub-stepped as in projector_splitting_integrator.hpp:136-169), O
// a one-mode operator.  Gradients: dJ/dc_r (real perturbations of every term
// coefficient), the cotangent of every operator matrix (hence of every physical parameter
// an operator is linear in), and of the starting state.
//
// Method: the state is checkpointed every K steps; a segment is recomputed from its
// checkpoint; each sweep is re-run with its operations recorded (inputs and the
// environment matrices each one reads, copied into a device tape) and reversed operation
// by operation:
//   * A <- A R, A_p <- R x_mu A_p:  A_bar R^H, R^H x_mu A_bar; R_bar from one reduction;
//   * QR (real diagonal of R): M1 = R R_bar^H, M2 = Q_bar^H Q, N = M2 - M1, K = upper part
//     of N - N^H with K_ii = i Im N_ii, W = M1 + K, A_bar = (Q_bar + Q (W^H - M2^H)) R^-H;
//   * y = exp(z H) x: x_bar = exp(conj(z) H) y_bar; H's environments and coefficients get
//     Re int_0^1 <conj(z) a(s), dH b(s)> ds with a(s) = exp((1-s) conj(z) H) y_bar,
//     b(s) = exp(s z H) x, by Gauss-Legendre quadrature (node count from the Gershgorin
//     width of the Lanczos matrix of the exponential: the integrand oscillates at most at
//     |z| (l_max - l_min)), every exponential on the persistent Krylov kernel;
//   * environment updates and H_eff reverse into mode products with S^H and reductions
//     of the same shapes as the forward ones.
// Node tensors and their cotangents live on the device; the r x r cotangents of the
// environments and gauge factors and the small matrix algebra (Hermitian conjugates,
// the QR's n x n terms, R^-1) are kept on the host.  Contractions run in FP64.

static double gl_leg(int n, double x, double& dp) {
  double p0 = 1.0, p1 = x;
  for (int k = 2; k <= n; ++k) {
    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  dp = n * (x * p1 - p0) / (x * x - 1.0);
  return p1;
}
// Gauss-Legendre nodes (ascending) and weights on [0, 1]
static void gauss_legendre01(int n, std::vector<double>& s, std::vector<double>& w) {
  s.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double x = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      const double pv = gl_leg(n, x, dp);
      const double dx = pv / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    gl_leg(n, x, dp);
    s[n - 1 - i] = 0.5 * (x + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - x * x) * dp * dp);
  }
}
static std::vector<cd> hmat(const std::vector<cd>& S, int d) {  // S^H
  std::vector<cd> o((size_t)d * d);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) o[(size_t)i * d + j] = std::conj(S[(size_t)j * d + i]);
  return o;
}
static void add_transposed(const std::vector<cd>& M, int d, cd* dst, cd alpha = 1.0) {  // dst(i,j) += a M(j,i)
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) dst[(size_t)i * d + j] += alpha * M[(size_t)j * d + i];
}
static cd hdot(const std::vector<cd>& x, const cd* y) {  // sum conj(x) y
  cd s = 0.0;
  for (size_t i = 0; i < x.size(); ++i) s += std::conj(x[i]) * y[i];
  return s;
}

struct DevAdjoint {
  Integrator& I;
  const Tree& T;
  ttn_state* S;
  cudaStream_t st;
  long long mx;                                      // largest node size (elements)
  // cotangents
  DevBuf ab_buf;
  std::vector<double2*> ab;                          // device, one per node (state layout)
  std::vector<std::vector<cd>> rb;                   // host, gauge factors (stride = their dimension)
  std::vector<std::vector<std::vector<cd>>> sb, mb;  // host, environments [node][group]
  std::vector<std::vector<std::vector<cd>>> gop;     // host, operators [mode][k]
  std::vector<double> gc;                            // dJ/dc_r
  // device scratch
  DevBuf vec_buf, chain_buf, quad_buf, small_buf, tape_buf, exp_buf;
  enum { V_Q, V_QB, V_M, V_B, V_W, V_BV, V_AV, V_G, V_X, V_XB, V_F, V_GT, V_Y0, V_TM, V_TB, V_YB, V_T1, V_T2, V_NV };
  double2* v[V_NV] = {};
  int max_items = 1;
  size_t small_cap = 0, small_used = 0;
  std::vector<std::vector<double2>> keep;            // host sources of uploads in flight
  int quad_min = 8, quad_max = 96, quad_alloc = 0;
  // the tape of one sweep
  struct Snap { int which, nd, g; size_t off; };     // which: 0 spf, 1 mf
  struct Rec {
    int kind = 0, nd = 0, aux = 0;
    double tau = 0.0;
    cd cf = 0.0;
    size_t x0 = 0, x1 = 0;
    std::vector<Snap> env;
  };
  std::vector<Rec> tape;
  size_t tape_used = 0, tape_need = 0;
  bool recording = false;
  // expectation-value reverse
  DevBuf mel_buf, melx_buf, melins_buf;
  std::vector<double2*> melv, melx, melins;

  DevAdjoint(Integrator& in, ttn_state* s) : I(in), T(in.T), S(s), st(in.stream) {
    mx = I.maxsize;
    ab.assign(T.n, nullptr);
    ab_buf.alloc((size_t)S->arena.bytes);
    for (int i = 0; i < T.n; ++i) ab[i] = ab_buf.as<double2>() + S->off[i];
    rb.assign(T.n, {});
    sb.assign(T.n, {});
    mb.assign(T.n, {});
    for (int i = 0; i < T.n; ++i) {
      long long rmx = T.hrank[i];
      for (int d : T.dims[i]) rmx = std::max<long long>(rmx, d);
      rb[i].assign((size_t)(rmx * rmx), 0.0);
      const size_t rr = (size_t)T.hrank[i] * T.hrank[i];
      sb[i].assign(I.G[i].size(), std::vector<cd>(rr, 0.0));
      mb[i].assign(I.G[i].size(), std::vector<cd>(rr, 0.0));
      max_items = std::max(max_items, T.nmodes[i]);
    }
    gop.assign(I.H.nmodes, {});
    for (int m = 0; m < I.H.nmodes; ++m)
      for (auto& M : I.H.ops[m]) gop[m].push_back(std::vector<cd>(M.size(), 0.0));
    gc.assign(I.H.nterms, 0.0);
    const size_t vb = align256((size_t)mx * sizeof(double2));
    vec_buf.alloc(vb * V_NV);
    for (int k = 0; k < V_NV; ++k) v[k] = reinterpret_cast<double2*>(static_cast<char*>(vec_buf.p) + vb * k);
    chain_buf.alloc(vb * (max_items + 1));
    small_cap = (size_t)64 * 64 * 1024;
    small_buf.alloc(small_cap * sizeof(double2));
    exp_buf.alloc(vb);
    // expectation values: per-node matrices, contracted tensors and chain inputs
    size_t nm = 0, ni = 0;
    for (int i = 0; i < T.n; ++i) {
      nm += align256((size_t)T.hrank[i] * T.hrank[i] * sizeof(double2));
      ni += align256((size_t)T.size(i) * sizeof(double2)) * (size_t)std::max(1, T.nmodes[i]);
    }
    mel_buf.alloc(nm);
    melx_buf.alloc((size_t)S->arena.bytes);
    melins_buf.alloc(ni);
    melv.assign(T.n, nullptr); melx.assign(T.n, nullptr); melins.assign(T.n, nullptr);
    size_t om = 0, oi = 0;
    for (int i = 0; i < T.n; ++i) {
      melv[i] = reinterpret_cast<double2*>(static_cast<char*>(mel_buf.p) + om);
      om += align256((size_t)T.hrank[i] * T.hrank[i] * sizeof(double2));
      melx[i] = melx_buf.as<double2>() + S->off[i];
      melins[i] = reinterpret_cast<double2*>(static_cast<char*>(melins_buf.p) + oi);
      oi += align256((size_t)T.size(i) * sizeof(double2)) * (size_t)std::max(1, T.nmodes[i]);
    }
    if (const char* q = std::getenv("TTN_ADJ_QUAD_MIN")) quad_min = std::max(2, std::atoi(q));
    CK(cudaMemsetAsync(ab_buf.p, 0, ab_buf.bytes, st));
  }

  // ---- host <-> device small matrices.  Staging slots are handed out until the next
  // reset(), which waits for the stream: device work of one reverse operation (or one
  // quadrature node) may use any slot handed out since the last reset.
  double2* chain_slot(int k) const {
    return reinterpret_cast<double2*>(static_cast<char*>(chain_buf.p) + align256((size_t)mx * sizeof(double2)) * k);
  }
  void reset() {
    CK(cudaStreamSynchronize(st));
    keep.clear();
    small_used = 0;
    herm_cache.clear();
  }
  // S^H of a device matrix that stays unchanged until the next reset() (environments
  // restored for one reverse operation, operators), uploaded once per reset
  std::map<const double2*, double2*> herm_cache;
  double2* herm_of(const double2* S, int d) {
    auto it = herm_cache.find(S);
    if (it != herm_cache.end()) return it->second;
    double2* h = up(hmat(down(S, (size_t)d * d), d));
    herm_cache[S] = h;
    return h;
  }
  double2* small_out(size_t n) {
    const size_t need = (n + 15) / 16 * 16;
    TTN_REQUIRE(small_used + need <= small_cap, TTN_ECAPACITY, "adjoint: small-matrix staging buffer exhausted");
    double2* dst = small_buf.as<double2>() + small_used;
    small_used += need;
    return dst;
  }
  double2* up(const std::vector<cd>& M) {
    const size_t n = M.size();
    double2* dst = small_out(n);
    keep.emplace_back(n);
    for (size_t i = 0; i < n; ++i) keep.back()[i] = d2(M[i]);
    CK(cudaMemcpyAsync(dst, keep.back().data(), n * sizeof(double2), cudaMemcpyHostToDevice, st));
    return dst;
  }
  std::vector<cd> down(const double2* p, size_t n) {
    std::vector<double2> h(n);
    CK(cudaMemcpyAsync(h.data(), p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<cd> o(n);
    for (size_t i = 0; i < n; ++i) o[i] = cd(h[i].x, h[i].y);
    return o;
  }
  cd dotc(const double2* x, const double2* y, long long n) {  // sum conj(x) y on the device
    double2* o = small_out(1);
    I.adj_mul(x, y, n, 1, o, 1.0, false);
    return down(o, 1)[0];
  }
  void copy(double2* dst, const double2* src, long long n) { zcopy(dst, src, n, st); }
  void axpy(double2* out, const double2* x, cd s, long long n, bool acc) { zaxpy(out, x, d2(s), n, acc, st); }

  // ---- recording (device-to-device copies into the tape arena)
  size_t tape_put(const double2* src, long long n) {
    const size_t off = tape_used;
    const size_t bytes = align256((size_t)n * sizeof(double2));
    tape_need += bytes;
    if (tape_used + bytes <= tape_buf.bytes)
      CK(cudaMemcpyAsync(reinterpret_cast<char*>(tape_buf.p) + off, src, (size_t)n * sizeof(double2),
                         cudaMemcpyDeviceToDevice, st));
    tape_used += bytes;
    return off;
  }
  double2* tape_at(size_t off) const { return reinterpret_cast<double2*>(reinterpret_cast<char*>(tape_buf.p) + off); }
  void snap(Rec& rc, int which, int nd, int g) {
    const Group& G = I.G[nd][g];
    const long long rr = (long long)T.hrank[nd] * T.hrank[nd];
    rc.env.push_back({which, nd, g, tape_put(which == 0 ? G.spf_dev : G.mf_dev, rr)});
  }
  void snap_items(Rec& rc, int nd, const std::vector<Item>& items) {
    for (const Item& it : items)
      if (it.slot >= 0) snap(rc, 0, T.children[nd][it.slot], it.grp);
  }
  void restore(const Rec& rc) {
    for (const Snap& s : rc.env) {
      const Group& G = I.G[s.nd][s.g];
      const long long rr = (long long)T.hrank[s.nd] * T.hrank[s.nd];
      copy(s.which == 0 ? G.spf_dev : G.mf_dev, tape_at(s.off), rr);
    }
  }
  void record(int kind, int nd, int aux) {
    if (!recording) return;
    Rec rc;
    rc.kind = kind; rc.nd = nd; rc.aux = aux;
    const long long r = T.hrank[nd];
    switch (kind) {
      case OP_AFP:
        rc.x0 = tape_put(S->node(nd), T.size(nd));
        rc.x1 = tape_put(I.rmat[T.parent[nd]], r * r);
        break;
      case OP_R2L: case OP_L2R:
        rc.x0 = tape_put(S->node(nd), T.size(nd));
        break;
      case OP_MF: {
        const int p = T.parent[nd];
        rc.x0 = tape_put(S->node(p), T.size(p));
        for (const Group& G : I.G[nd]) {
          if (G.id_mf) continue;
          for (const MfKey& k : G.mf) {
            if (!I.G[p][k.pg].id_mf) snap(rc, 1, p, k.pg);
            snap_items(rc, p, k.sib);
          }
        }
        break;
      }
      case OP_NODE:
        rc.x0 = tape_put(S->node(nd), T.size(nd));
        rc.tau = I.dt / 2.0; rc.cf = I.coeff;
        for (size_t g = 0; g < I.G[nd].size(); ++g) {
          const Group& G = I.G[nd][g];
          if (!G.id_mf) snap(rc, 1, nd, (int)g);
          if (!G.id_spf) for (const SpfTuple& t : G.spf) snap_items(rc, nd, t.items);
        }
        break;
      case OP_SPF:
        rc.x0 = tape_put(S->node(nd), T.size(nd));
        for (const Group& G : I.G[nd])
          if (!G.id_spf) for (const SpfTuple& t : G.spf) snap_items(rc, nd, t.items);
        break;
      case OP_BOND:
        rc.x0 = tape_put(I.rmat[aux], r * r);
        rc.tau = -I.dt / 2.0; rc.cf = I.coeff;
        for (size_t g = 0; g < I.G[nd].size(); ++g) {
          const Group& G = I.G[nd][g];
          if (!G.id_spf) snap(rc, 0, nd, (int)g);
          if (!G.id_mf) snap(rc, 1, nd, (int)g);
        }
        break;
      case OP_ATP:
        rc.x0 = tape_put(S->node(T.parent[nd]), T.size(T.parent[nd]));
        rc.x1 = tape_put(I.rmat[nd], r * r);
        break;
      default: throw Err(TTN_EINVAL, "adjoint: unknown operation");
    }
    tape.push_back(std::move(rc));
  }

  // ---- chains of mode products (device intermediates in chain slots)
  struct Link { const double2* S; int d; long long na, nb; cd* Sb; };
  std::vector<Link> links_items(int nd, const std::vector<Item>& items) {
    std::vector<Link> L;
    for (const Item& it : items) {
      if (it.slot < 0) {
        const int mode = T.leaf_mode[nd];
        L.push_back({I.leaf_ops[mode][it.grp], T.dims[nd][0], 1, (long long)T.hrank[nd], gop[mode][it.grp].data()});
      } else {
        long long na, nb; int d;
        I.r3(nd, it.slot, na, d, nb);
        const int c = T.children[nd][it.slot];
        L.push_back({I.G[c][it.grp].spf_dev, d, na, nb, sb[c][it.grp].data()});
      }
    }
    return L;
  }
  std::vector<Link> links_sibs(int p, const std::vector<Item>& items) {
    std::vector<Link> L;
    for (const Item& it : items) {
      long long na, nb; int d;
      I.r3(p, it.slot, na, d, nb);
      const int c = T.children[p][it.slot];
      L.push_back({I.G[c][it.grp].spf_dev, d, na, nb, sb[c][it.grp].data()});
    }
    return L;
  }
  // chain slot k holds the input of link k (slot 0 a copy of v); returns the output slot
  double2* chain_fwd(const std::vector<Link>& L, const double2* v, long long n) {
    TTN_REQUIRE((int)L.size() <= max_items, TTN_ECAPACITY, "adjoint: chain longer than the node's mode count");
    copy(chain_slot(0), v, n);
    for (size_t k = 0; k < L.size(); ++k)
      I.mode_apply(L[k].S, L[k].d, chain_slot((int)k), chain_slot((int)k + 1), L[k].na, L[k].nb, 1.0, false, false);
    return chain_slot((int)L.size());
  }
  // g (device, n) holds the output cotangent and on return the input cotangent; uses
  // the chain slots of the matching chain_fwd and the scratch vector V_T1
  void chain_rev(const std::vector<Link>& L, double2* g, long long n) {
    for (int k = (int)L.size() - 1; k >= 0; --k) {
      const Link& l = L[k];
      const size_t dd = (size_t)l.d * l.d;
      double2* t = small_out(dd);
      I.mode_contract(chain_slot(k), g, l.na, l.d, l.nb, t, 1.0, false);
      add_transposed(down(t, dd), l.d, l.Sb);
      double2* SH = herm_of(l.S, l.d);
      I.mode_apply(SH, l.d, g, v[V_T1], l.na, l.nb, 1.0, false, false);
      copy(g, v[V_T1], n);
    }
  }

  // ---- exponentials
  void check_status() {
    int h = 0;
    CK(cudaMemcpyAsync(&h, I.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    TTN_REQUIRE(!(h & kErrBarrierTimeout), TTN_ETIMEOUT, "adjoint: a device-side grid barrier gave up waiting");
    TTN_REQUIRE(h == 0, TTN_ENUMERIC, "adjoint: Krylov exponential failed (status " + std::to_string(h) + ")");
  }
  void expm(int kind, int nd, double2* y, long long n, double tau, cd cf) {
    I.expm_dev(nd, kind, y, n, tau, cf, false, false);
  }
  // Gershgorin width of the Lanczos matrix of the exponential last run
  double lanczos_width() {
    KrylovCtl c;
    CK(cudaMemcpyAsync(&c, I.ctl, sizeof(KrylovCtl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const int mb = std::max(1, std::min(c.mb, kKrylovMax));
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < mb; ++i) {
      const double off = (i > 0 ? std::fabs(c.bet[i]) : 0.0) + (i + 1 < mb ? std::fabs(c.bet[i + 1]) : 0.0);
      lo = std::min(lo, c.alpha[i] - off);
      hi = std::max(hi, c.alpha[i] + off);
    }
    return hi > lo ? hi - lo : 0.0;
  }
  double2* quad_slot(int j) const {
    return reinterpret_cast<double2*>(static_cast<char*>(quad_buf.p) + align256((size_t)mx * sizeof(double2)) * j);
  }
  // reverse of y = exp(cf tau H) x (H = H_eff(nd) for kind 0, K_bond(nd) for kind 1):
  // yb (device) becomes x_bar; vjp(b, g) adds H's cotangents for Re <g, dH b>
  template <typename Vjp>
  void expm_vjp(int kind, int nd, long long n, const double2* x, double2* yb, double tau, cd cf, Vjp&& vjp) {
    const cd z = cf * tau;
    if (dotc(yb, yb, n).real() == 0.0) return;
    copy(v[V_W], x, n);
    expm(kind, nd, v[V_W], n, tau, cf);
    double width = lanczos_width();
    copy(v[V_W], yb, n);
    expm(kind, nd, v[V_W], n, tau, cf);
    width = std::max(width, lanczos_width());
    const double omega = std::abs(z) * width * 1.1;
    const int nq = std::min(quad_max, std::max(quad_min, (int)std::ceil(0.5 * omega) + 10));
    if (nq > quad_alloc) {
      quad_buf.alloc(align256((size_t)mx * sizeof(double2)) * nq);
      quad_alloc = nq;
    }
    std::vector<double> s, w;
    gauss_legendre01(nq, s, w);
    copy(v[V_BV], x, n);
    double sp = 0.0;
    for (int j = 0; j < nq; ++j) {
      expm(kind, nd, v[V_BV], n, (s[j] - sp) * tau, cf);
      copy(quad_slot(j), v[V_BV], n);
      sp = s[j];
    }
    copy(v[V_AV], yb, n);
    sp = 1.0;
    for (int j = nq - 1; j >= 0; --j) {
      expm(kind, nd, v[V_AV], n, (sp - s[j]) * tau, std::conj(cf));
      axpy(v[V_G], v[V_AV], w[j] * std::conj(z), n, false);
      vjp(quad_slot(j), v[V_G]);
      reset();
      sp = s[j];
    }
    expm(kind, nd, v[V_AV], n, sp * tau, std::conj(cf));
    copy(yb, v[V_AV], n);
    check_status();
  }

  // out = s * mf_apply(X, M) (or s * X when the mean field is the identity): cotangents of
  // s and M; the cotangent of X into V_XB
  void mf_stage_vjp(const Group& G, int nd, int gi, const double2* X, const double2* g, long long n) {
    const int r = T.hrank[nd];
    const long long nx = n / r;
    cd sig;
    if (G.id_mf) {
      sig = dotc(X, g, n);
      axpy(v[V_XB], g, std::conj(G.s), n, false);
    } else {
      const double2* M = G.mf_dev;
      I.mf_apply(X, M, r, nx, v[V_F], 1.0, false, false);
      sig = dotc(v[V_F], g, n);
      double2* t = small_out((size_t)r * r);
      I.adj_mul(X, g, nx, r, t, 1.0, false);
      add_transposed(down(t, (size_t)r * r), r, mb[nd][gi].data(), std::conj(G.s));
      double2* MH = herm_of(M, r);
      I.mf_apply(g, MH, r, nx, v[V_XB], std::conj(G.s), false, false);
    }
    if (G.type == G_1) gc[G.members[0]] += sig.real();
  }

  // cotangents of everything H_eff(nd) depends on, for Re <g, dH_eff v>
  void heff_vjp(int nd, const double2* vin, const double2* g) {
    const long long n = T.size(nd);
    for (size_t gi = 0; gi < I.G[nd].size(); ++gi) {
      const Group& G = I.G[nd][gi];
      const double2* X = vin;
      if (!G.id_spf) {
        for (size_t q = 0; q < G.spf.size(); ++q) {
          const double2* Y = chain_fwd(links_items(nd, G.spf[q].items), vin, n);
          axpy(v[V_X], Y, G.spf[q].a, n, q > 0);
        }
        X = v[V_X];
      }
      mf_stage_vjp(G, nd, (int)gi, X, g, n);
      if (G.id_spf) continue;
      for (const SpfTuple& t : G.spf) {
        std::vector<Link> L = links_items(nd, t.items);
        const double2* Y = chain_fwd(L, vin, n);
        if (!t.a_mem.empty()) {
          const double a = dotc(Y, v[V_XB], n).real();
          for (int q : t.a_mem) gc[q] += a;
        }
        axpy(v[V_GT], v[V_XB], std::conj(t.a), n, false);
        chain_rev(L, v[V_GT], n);
      }
    }
  }

  // the same for the bond Hamiltonian K(nd) on an r x r matrix R
  void kbond_vjp(int nd, const double2* R, const double2* g) {
    const int r = T.hrank[nd];
    const long long rr = (long long)r * r;
    for (size_t gi = 0; gi < I.G[nd].size(); ++gi) {
      const Group& G = I.G[nd][gi];
      const double2* X = R;
      if (!G.id_spf) {
        I.right_mul(G.spf_dev, R, r, r, v[V_X]);
        X = v[V_X];
      }
      mf_stage_vjp(G, nd, (int)gi, X, g, rr);
      if (G.id_spf) continue;
      const std::vector<cd> Xb = down(v[V_XB], (size_t)rr), Rh = down(R, (size_t)rr);
      cd* Sb = sb[nd][gi].data();  // S_bar += X_bar R^H
      for (int i = 0; i < r; ++i)
        for (int k = 0; k < r; ++k) {
          cd s = 0.0;
          for (int j = 0; j < r; ++j) s += Xb[(size_t)i * r + j] * std::conj(Rh[(size_t)k * r + j]);
          Sb[(size_t)i * r + k] += s;
        }
    }
  }

  // ---- reverse of A = Q R (m x n, real diagonal of R): out = A_bar (may alias Qb)
  void qr_vjp(const double2* Q, const std::vector<cd>& R, const double2* Qb, const std::vector<cd>& Rb, long long m,
              int n, double2* out) {
    const size_t nn = (size_t)n * n;
    std::vector<cd> M1(nn, 0.0), W(nn), C(nn), Ri(nn, 0.0);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        cd s = 0.0;
        for (int k = 0; k < n; ++k) s += R[(size_t)i * n + k] * std::conj(Rb[(size_t)j * n + k]);
        M1[(size_t)i * n + j] = s;
      }
    double2* t = small_out(nn);
    I.adj_mul(Qb, Q, m, n, t, 1.0, false);  // M2 = Q_bar^H Q
    const std::vector<cd> M2 = down(t, nn);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const cd Nij = M2[(size_t)i * n + j] - M1[(size_t)i * n + j];
        const cd Nji = M2[(size_t)j * n + i] - M1[(size_t)j * n + i];
        cd K = 0.0;
        if (i < j) K = Nij - std::conj(Nji);
        else if (i == j) K = cd(0.0, Nij.imag());
        W[(size_t)i * n + j] = M1[(size_t)i * n + j] + K;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        C[(size_t)i * n + j] = std::conj(W[(size_t)j * n + i]) - std::conj(M2[(size_t)j * n + i]);
    // R^-1 (upper triangular), then (R^-1)^H
    for (int j = 0; j < n; ++j) {
      const double djj = R[(size_t)j * n + j].real();
      TTN_REQUIRE(djj != 0.0, TTN_ENUMERIC, "adjoint: singular gauge factor R (rank-deficient bond)");
      Ri[(size_t)j * n + j] = 1.0 / djj;
      for (int i = j - 1; i >= 0; --i) {
        cd s = 0.0;
        for (int k = i + 1; k <= j; ++k) s += R[(size_t)i * n + k] * Ri[(size_t)k * n + j];
        Ri[(size_t)i * n + j] = -s / R[(size_t)i * n + i].real();
      }
    }
    double2* Cd = up(C);
    double2* RiH = up(hmat(Ri, n));
    I.right_mul(Q, Cd, m, n, v[V_B]);              // Q C
    axpy(v[V_B], Qb, 1.0, m * n, true);             // + Q_bar
    I.right_mul(v[V_B], RiH, m, n, out);            // R^-H
  }

  void r2l_shape(int nd, int mu, long long& pre, int& dm, long long& post) const {
    pre = 1;
    post = T.hrank[nd];
    for (int i = 0; i < mu; ++i) pre *= T.dims[nd][i];
    dm = T.dims[nd][mu];
    for (int i = mu + 1; i < T.nmodes[nd]; ++i) post *= T.dims[nd][i];
  }

  // ---- reverse of one recorded operation
  void reverse(const Rec& rc) {
    reset();
    const int nd = rc.nd, r = T.hrank[nd];
    const long long rr = (long long)r * r;
    switch (rc.kind) {
      case OP_AFP: {  // A <- A Rp
        const int p = T.parent[nd];
        const long long m = T.dimen[nd];
        double2* RH = up(hmat(down(tape_at(rc.x1), (size_t)rr), r));
        I.right_mul(ab[nd], RH, m, r, v[V_T2]);
        double2* t = small_out((size_t)rr);
        I.adj_mul(tape_at(rc.x0), ab[nd], m, r, t, 1.0, false);
        const std::vector<cd> th = down(t, (size_t)rr);
        for (long long i = 0; i < rr; ++i) rb[p][(size_t)i] += th[(size_t)i];
        copy(ab[nd], v[V_T2], T.size(nd));
        break;
      }
      case OP_ATP: {  // A_p <- R x_mu A_p
        const int p = T.parent[nd];
        long long na, nb; int d;
        I.r3(p, T.slot[nd], na, d, nb);
        const size_t dd = (size_t)d * d;
        double2* RH = up(hmat(down(tape_at(rc.x1), dd), d));
        I.mode_apply(RH, d, ab[p], v[V_T2], na, nb, 1.0, false, false);
        double2* t = small_out(dd);
        I.mode_contract(tape_at(rc.x0), ab[p], na, d, nb, t, 1.0, false);
        add_transposed(down(t, dd), d, rb[nd].data());
        copy(ab[p], v[V_T2], T.size(p));
        break;
      }
      case OP_L2R: {  // A = Q R; A <- Q, rmat <- R
        const long long m = T.dimen[nd];
        copy(v[V_Q], tape_at(rc.x0), T.size(nd));
        double2* Rd = small_out((size_t)rr);
        I.qr(v[V_Q], m, r, Rd, 0);
        const std::vector<cd> R = down(Rd, (size_t)rr);
        const std::vector<cd> Rb(rb[nd].begin(), rb[nd].begin() + rr);
        qr_vjp(v[V_Q], R, ab[nd], Rb, m, r, ab[nd]);
        std::fill(rb[nd].begin(), rb[nd].end(), cd(0.0));
        break;
      }
      case OP_R2L: {  // permuted M = Q R; A <- unpermute(Q), rmat <- R^T
        long long pre, post; int dm;
        r2l_shape(nd, rc.aux, pre, dm, post);
        const size_t dd = (size_t)dm * dm;
        permute_mode_last(tape_at(rc.x0), v[V_Q], pre, dm, post, st);
        double2* Rd = small_out(dd);
        I.qr(v[V_Q], pre * post, dm, Rd, 0);
        const std::vector<cd> R = down(Rd, dd);
        permute_mode_last(ab[nd], v[V_QB], pre, dm, post, st);
        std::vector<cd> Rb(dd);
        for (int i = 0; i < dm; ++i)
          for (int j = 0; j < dm; ++j) Rb[(size_t)j * dm + i] = rb[nd][(size_t)i * dm + j];
        qr_vjp(v[V_Q], R, v[V_QB], Rb, pre * post, dm, v[V_M]);
        unpermute_mode_last(v[V_M], ab[nd], pre, dm, post, st);
        std::fill(rb[nd].begin(), rb[nd].end(), cd(0.0));
        break;
      }
      case OP_NODE: {
        restore(rc);
        expm_vjp(0, nd, T.size(nd), tape_at(rc.x0), ab[nd], rc.tau, rc.cf,
                 [&](const double2* b, const double2* g) { heff_vjp(nd, b, g); });
        break;
      }
      case OP_BOND: {
        restore(rc);
        const int owner = rc.aux;
        copy(v[V_T2], up(std::vector<cd>(rb[owner].begin(), rb[owner].begin() + rr)), rr);
        expm_vjp(1, nd, rr, tape_at(rc.x0), v[V_T2], rc.tau, rc.cf,
                 [&](const double2* b, const double2* g) { kbond_vjp(nd, b, g); });
        const std::vector<cd> xb = down(v[V_T2], (size_t)rr);
        std::copy(xb.begin(), xb.end(), rb[owner].begin());
        break;
      }
      case OP_SPF: {
        restore(rc);
        const long long n = T.size(nd), nx = n / r;
        const double2* A = tape_at(rc.x0);
        for (size_t gi = 0; gi < I.G[nd].size(); ++gi) {
          const Group& G = I.G[nd][gi];
          if (G.id_spf) continue;
          const std::vector<cd>& Sb = sb[nd][gi];
          std::vector<cd> SbC((size_t)rr), SbT((size_t)rr);
          for (int i = 0; i < r; ++i)
            for (int j = 0; j < r; ++j) {
              SbC[(size_t)i * r + j] = std::conj(Sb[(size_t)i * r + j]);
              SbT[(size_t)i * r + j] = Sb[(size_t)j * r + i];
            }
          double2* SbCd = up(SbC);
          double2* SbTd = up(SbT);
          for (const SpfTuple& t : G.spf) {
            std::vector<Link> L = links_items(nd, t.items);
            const double2* X = chain_fwd(L, A, n);
            I.mf_apply(X, SbCd, r, nx, ab[nd], t.a, true, false);  // bra side
            if (!t.a_mem.empty()) {
              double2* z = small_out((size_t)rr);
              I.adj_mul(A, X, nx, r, z, 1.0, false);
              const double a = hdot(down(z, (size_t)rr), Sb.data()).real();
              for (int q : t.a_mem) gc[q] += a;
            }
            I.mf_apply(A, SbTd, r, nx, v[V_XB], std::conj(t.a), false, false);
            chain_rev(L, v[V_XB], n);
            axpy(ab[nd], v[V_XB], 1.0, n, true);  // ket side
          }
          std::fill(sb[nd][gi].begin(), sb[nd][gi].end(), cd(0.0));
        }
        break;
      }
      case OP_MF: {
        restore(rc);
        const int p = T.parent[nd], rp = T.hrank[p];
        long long na, nb; int d;
        I.r3(p, T.slot[nd], na, d, nb);
        const long long szp = T.size(p);
        const size_t dd = (size_t)d * d, rpp = (size_t)rp * rp;
        const double2* Ap = tape_at(rc.x0);
        for (size_t gi = 0; gi < I.G[nd].size(); ++gi) {
          const Group& G = I.G[nd][gi];
          if (G.id_mf) continue;
          const std::vector<cd>& Mb = mb[nd][gi];
          for (const MfKey& k : G.mf) {
            std::vector<Link> L = links_sibs(p, k.sib);
            const double2* Y0 = chain_fwd(L, Ap, szp);
            const bool pm = !I.G[p][k.pg].id_mf;
            const double2* Tm = Y0;
            if (pm) {
              I.mf_apply(Y0, I.G[p][k.pg].mf_dev, rp, szp / rp, v[V_TM], 1.0, false, false);
              Tm = v[V_TM];
            }
            std::vector<cd> S1(dd), S2(dd);
            for (int i = 0; i < d; ++i)
              for (int j = 0; j < d; ++j) {
                S1[(size_t)i * d + j] = k.b * std::conj(Mb[(size_t)i * d + j]);
                S2[(size_t)j * d + i] = std::conj(k.b) * Mb[(size_t)i * d + j];
              }
            I.mode_apply(up(S1), d, Tm, ab[p], na, nb, 1.0, true, false);  // bra side
            if (!k.b_mem.empty()) {
              double2* z = small_out(dd);
              I.mode_contract(Ap, Tm, na, d, nb, z, 1.0, false);
              const double b = hdot(down(z, dd), Mb.data()).real();
              for (int q : k.b_mem) gc[q] += b;
            }
            I.mode_apply(up(S2), d, Ap, v[V_TB], na, nb, 1.0, false, false);
            if (pm) {
              double2* t = small_out(rpp);
              I.adj_mul(Y0, v[V_TB], szp / rp, rp, t, 1.0, false);
              add_transposed(down(t, rpp), rp, mb[p][k.pg].data());
              double2* MH = up(hmat(down(I.G[p][k.pg].mf_dev, rpp), rp));
              I.mf_apply(v[V_TB], MH, rp, szp / rp, v[V_YB], 1.0, false, false);
            } else {
              copy(v[V_YB], v[V_TB], szp);
            }
            chain_rev(L, v[V_YB], szp);
            axpy(ab[p], v[V_YB], 1.0, szp, true);  // ket side
          }
          std::fill(mb[nd][gi].begin(), mb[nd][gi].end(), cd(0.0));
        }
        break;
      }
      default: throw Err(TTN_EINVAL, "adjoint: unknown operation");
    }
    reset();
  }

  // ---- reverse of J += w Re <psi| O_mode |psi> (the leaf-to-root contraction of expect)
  double2* mel_in(int id, int k) const {
    return reinterpret_cast<double2*>(reinterpret_cast<char*>(melins[id]) +
                                      align256((size_t)T.size(id) * sizeof(double2)) * k);
  }
  void expect_vjp(int mode, const double2* op, double w) {
    for (int id = T.n - 1; id >= 0; --id) {
      const int r = T.hrank[id];
      const long long sz = T.size(id);
      const double2* A = S->node(id);
      if (T.leaf(id)) {
        if (op && T.leaf_mode[id] == mode) I.mode_apply(op, T.dims[id][0], A, melx[id], 1, r, 1.0, false, false);
        else copy(melx[id], A, sz);
      } else {
        copy(mel_in(id, 0), A, sz);
        for (int s = 0; s < T.nmodes[id]; ++s) {
          long long na, nb; int d;
          I.r3(id, s, na, d, nb);
          double2* out = (s + 1 < T.nmodes[id]) ? mel_in(id, s + 1) : melx[id];
          I.mode_apply(melv[T.children[id][s]], d, mel_in(id, s), out, na, nb, 1.0, false, false);
        }
      }
      I.adj_mul(A, melx[id], sz / r, r, melv[id], 1.0, false);
    }
    std::vector<std::vector<cd>> melb(T.n);
    for (int id = 0; id < T.n; ++id) melb[id].assign((size_t)T.hrank[id] * T.hrank[id], 0.0);
    for (int k = 0; k < T.hrank[0]; ++k) melb[0][(size_t)k * T.hrank[0] + k] = w;
    for (int id = 0; id < T.n; ++id) {
      reset();
      const int r = T.hrank[id];
      const long long sz = T.size(id), nx = sz / r, rr = (long long)r * r;
      const double2* A = S->node(id);
      std::vector<cd> MC((size_t)rr), MT((size_t)rr);
      for (int i = 0; i < r; ++i)
        for (int j = 0; j < r; ++j) {
          MC[(size_t)i * r + j] = std::conj(melb[id][(size_t)i * r + j]);
          MT[(size_t)i * r + j] = melb[id][(size_t)j * r + i];
        }
      I.mf_apply(melx[id], up(MC), r, nx, ab[id], 1.0, true, false);  // bra side
      I.mf_apply(A, up(MT), r, nx, v[V_XB], 1.0, false, false);
      if (T.leaf(id)) {
        if (op && T.leaf_mode[id] == mode) {
          const int d = T.dims[id][0];
          I.mode_apply(up(hmat(down(op, (size_t)d * d), d)), d, v[V_XB], v[V_T2], 1, r, 1.0, false, false);
          copy(v[V_XB], v[V_T2], sz);
        }
      } else {
        for (int s = T.nmodes[id] - 1; s >= 0; --s) {
          long long na, nb; int d;
          I.r3(id, s, na, d, nb);
          const int c = T.children[id][s];
          const size_t dd = (size_t)d * d;
          double2* t = small_out(dd);
          I.mode_contract(mel_in(id, s), v[V_XB], na, d, nb, t, 1.0, false);
          add_transposed(down(t, dd), d, melb[c].data());
          I.mode_apply(up(hmat(down(melv[c], dd), d)), d, v[V_XB], v[V_T1], na, nb, 1.0, false, false);
          copy(v[V_XB], v[V_T1], sz);
        }
      }
      axpy(ab[id], v[V_XB], 1.0, sz, true);  // ket side
    }
    reset();
  }

  // ---- driver
  void recompute_spf() { for (int id = T.n - 1; id >= 1; --id) I.update_spf(id, S->node(id)); }
  void plain_sweep(double d) {
    I.dt = d;
    I.forward(S, true);
    I.backward(S, true);
  }
  void load_state(const void* src) {
    CK(cudaMemcpyAsync(S->arena.p, src, S->arena.bytes, cudaMemcpyDeviceToDevice, st));
  }
  void save_state(void* dst) {
    CK(cudaMemcpyAsync(dst, S->arena.p, S->arena.bytes, cudaMemcpyDeviceToDevice, st));
  }
  char* slot(DevBuf& b, size_t k) const { return static_cast<char*>(b.p) + align256(S->arena.bytes) * k; }

  struct HookGuard {
    Integrator& I;
    bool& rec;
    ~HookGuard() { I.on_op = nullptr; rec = false; }
  };
  // one sweep from the state at A0 re-run with its operations recorded, then reversed
  void sweep_rev(const void* A0, double d, cd cf) {
    for (int attempt = 0; attempt < 2; ++attempt) {
      load_state(A0);
      I.dt = d;
      I.coeff = cf;
      tape.clear();
      tape_used = 0;
      tape_need = 0;
      {
        HookGuard g{I, recording};
        recording = true;
        I.on_op = [this](int k, int nd, int aux) { record(k, nd, aux); };
        recompute_spf();
        I.forward(S, true);
        I.backward(S, true);
      }
      if (tape_need <= tape_buf.bytes) break;
      TTN_REQUIRE(attempt == 0, TTN_ECAPACITY, "adjoint: tape sizing failed");
      CK(cudaStreamSynchronize(st));
      tape_buf.alloc(tape_need + tape_need / 8 + 4096);
    }
    check_status();
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

  double run(double dt, cd cf, int nsteps, const double* w, int mode, const double2* op, int K, bool skip_prepare) {
    K = std::max(1, std::min(K, nsteps));
    std::vector<std::vector<double>> sched(nsteps);
    for (int k = 0; k < nsteps; ++k) sched[k] = step_schedule(dt, k == 0);
    const int nck = (nsteps + K - 1) / K;
    const size_t sb_bytes = align256(S->arena.bytes);
    DevBuf ck_buf, seg_buf, sw_buf;
    ck_buf.alloc(sb_bytes * nck);
    seg_buf.alloc(sb_bytes * (K + 1));
    sw_buf.alloc(sb_bytes * sched[0].size());
    I.coeff = cf;
    if (skip_prepare) recompute_spf(); else I.prepare(S);
    double J = 0.0;
    for (int k = 0; k < nsteps; ++k) {
      if (k % K == 0) save_state(slot(ck_buf, k / K));
      for (double d : sched[k]) plain_sweep(d);
      J += w[k] * I.expect(S, mode, op).real();
    }
    check_status();
    DevBuf fin;
    fin.alloc(sb_bytes);
    save_state(fin.p);
    for (int sg = nck - 1; sg >= 0; --sg) {
      const int k0 = sg * K, k1 = std::min(nsteps, k0 + K);
      load_state(slot(ck_buf, sg));
      recompute_spf();
      save_state(slot(seg_buf, 0));
      for (int k = k0; k < k1; ++k) {
        for (double d : sched[k]) plain_sweep(d);
        save_state(slot(seg_buf, k - k0 + 1));
      }
      for (int k = k1 - 1; k >= k0; --k) {
        load_state(slot(seg_buf, k - k0 + 1));
        expect_vjp(mode, op, w[k]);
        load_state(slot(seg_buf, k - k0));
        recompute_spf();
        for (size_t q = 0; q < sched[k].size(); ++q) {
          save_state(slot(sw_buf, q));
          if (q + 1 < sched[k].size()) plain_sweep(sched[k][q]);
        }
        for (int q = (int)sched[k].size() - 1; q >= 0; --q) sweep_rev(slot(sw_buf, q), sched[k][q], cf);
      }
    }
    // the root's S-group mean fields are (sum of the members' coefficients) * identity
    const int r0 = T.hrank[0];
    for (size_t g = 0; g < I.G[0].size(); ++g) {
      const Group& G = I.G[0][g];
      if (G.id_mf) continue;
      cd tr = 0.0;
      for (int k = 0; k < r0; ++k) tr += mb[0][g][(size_t)k * r0 + k];
      for (int q : G.members) gc[q] += tr.real();
    }
    load_state(fin.p);
    recompute_spf();
    CK(cudaStreamSynchronize(st));
    I.nsteps = nsteps;
    I.dt = dt;
    return J;
  }
};
