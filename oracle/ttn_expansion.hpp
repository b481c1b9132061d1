// ttn_expansion.hpp -- subspace expansion (adaptive bond dimension) of the oracle's
// sweep.  TEST INFRASTRUCTURE ONLY, like the rest of oracle/: included by
// ttn_oracle.cpp inside namespace orc after Engine.
//
// Restates include/ttns_lib/tdvp_core/subspace_expansion_projector_splitting_engine.hpp
// (subspace_expansion_down :207-358, _up :361-510, get_nunoccupied :577-585) and
// two_site_energy_variations.hpp (terms :78-222, M^H M / M M^H :264-338, trial vector
// :341-372, expand_tensor / expand_matrix :375-444), driven as in
// tdvp_algorithm_engine.hpp:257-321 (prepare_evolution) and :331-501 (the expansion calls
// inside the half-sweeps) and projector_splitting_integrator.hpp:281-326.
//
// At the gauge move between a node C and its parent P (forward: after P's root-to-leaf
// decomposition towards C; backward: after C's leaf-to-root decomposition) the two-site
// wavefunction is C r P.  For every term group of C whose operator is neither the identity
// below C nor above it:
//   L_g = (1 - C C^H) [sum_t a_t (spf product of tuple t) C] r          (dimen_C x d)
//   U_g = s_g sum_k b_k (sibling spf products, parent mean field) P, with the part in the
//         span of P's slices removed                                   (pre x d x post)
// and M = sum_g L_g . U_g (over the bond index) maps P's outer space to C's row space:
// the component of H (C r P) outside both one-site tangent spaces.  Going down, the
// dominant right singular vectors of M (at most `neigenvalues`, those with
// sqrt(lambda) dt/2 > spawning threshold, within C's capacity) become new slices of P
// and C, r gain zero columns/rows; going up, the dominant left singular vectors become
// new columns of C and P, r gain zeros.  The state itself is unchanged by an expansion.
// Where the neighbour is square (or C has rank 1) and fewer than `minimum_unoccupied`
// singular values of r are unoccupied, random orthonormal directions are added instead.
//
// Ours, because the reference's versions live in the absent utils submodule or are
// library-specific: the dominant eigenpairs of M^H M (M M^H) come from a dense Hermitian
// Jacobi solve of the smaller Gram matrix instead of the reference's Krylov `eigs`; the
// random trial vectors use std::mt19937 with std::normal_distribution components like the
// reference but are orthogonalised with the Hermitian inner product; the singular values
// of r ("pops") are those of the QR gauge factor, equal to the reference's SVD values;
// and a bond grows by at most as much as keeps both of its tensors' matricisations tall
// (the child's dimen x hrank, the parent's outer x mode), which the QR gauge moves need
// (the reference bounds the two directions by one side each).

// Hermitian eigen-decomposition (cyclic Jacobi): on exit w holds the eigenvalues in
// descending order and the columns of Z (n x n row-major) the eigenvectors.
static void herm_eig(std::vector<cd> a, int n, std::vector<double>& w, std::vector<cd>& Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double v = std::norm(a[(size_t)i * n + j]);
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-30 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const cd apq = a[(size_t)p * n + q];
        const double ab = std::abs(apq);
        if (ab < 1e-300) continue;
        const double app = a[(size_t)p * n + p].real(), aqq = a[(size_t)q * n + q].real();
        const double th = 0.5 * std::atan2(2.0 * ab, aqq - app);
        const double c = std::cos(th), s = std::sin(th);
        const cd ph = apq / ab;
        // J with J_pp = J_qq = c, J_pq = s ph, J_qp = -s conj(ph); a <- J^H a J, Z <- Z J
        for (int k = 0; k < n; ++k) {
          const cd akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * std::conj(ph) * akq;
          a[(size_t)k * n + q] = s * ph * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const cd apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * ph * aqk;
          a[(size_t)q * n + k] = s * std::conj(ph) * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const cd zkp = Z[(size_t)k * n + p], zkq = Z[(size_t)k * n + q];
          Z[(size_t)k * n + p] = c * zkp - s * std::conj(ph) * zkq;
          Z[(size_t)k * n + q] = s * ph * zkp + c * zkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int x, int y) { return a[(size_t)x * n + x].real() > a[(size_t)y * n + y].real(); });
  std::vector<cd> Zs((size_t)n * n);
  w.assign(n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = a[(size_t)ord[j] * n + ord[j]].real();
    for (int i = 0; i < n; ++i) Zs[(size_t)i * n + j] = Z[(size_t)i * n + ord[j]];
  }
  Z.swap(Zs);
}

struct Expander {
  Engine& E;
  std::vector<int> cap;                     // bond capacity above each node
  double spawning_threshold = -1.0, unoccupied_threshold = -1.0;
  int minimum_unoccupied = 0, neigenvalues = 2;
  bool only_when_no_unoccupied = false;
  std::mt19937 rng;
  std::normal_distribution<double> nd{0.0, 1.0};
  long long n_twosite = 0, n_onesite = 0;

  explicit Expander(Engine& e) : E(e) {}

  // singular values (descending) of a d x d gauge factor held with row stride d
  static std::vector<double> svals(const cd* R, int d) {
    std::vector<cd> G((size_t)d * d, 0.0);
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        cd s = 0.0;
        for (int k = 0; k < d; ++k) s += std::conj(R[(size_t)k * d + i]) * R[(size_t)k * d + j];
        G[(size_t)i * d + j] = s;
      }
    std::vector<double> w;
    std::vector<cd> Z;
    herm_eig(G, d, w, Z);
    for (auto& x : w) x = std::sqrt(std::max(0.0, x));
    return w;
  }
  int n_unoccupied(const std::vector<double>& pops) const {
    int n = 0;
    for (double p : pops)
      if (pops[0] > 0.0 ? p / pops[0] < unoccupied_threshold : true) ++n;
    return n;
  }

  // M (dimen_C x pre*post, row-major) of the two-site variation at the bond above C with
  // gauge factor r (d x d, the state being C r P)
  std::vector<cd> two_site_matrix(int C, const std::vector<cd>& r) {
    const Tree& T = E.T;
    const int P = T.parent[C], mu = T.slot[C], d = T.hrank[C], rp = T.hrank[P];
    size_t pre, post; int dd;
    E.r3(P, mu, pre, dd, post);
    const size_t mC = T.dimen[C], szC = T.size(C), szP = T.size(P), outer = pre * post;
    const cd* A = E.A[C].data();
    const cd* Ap = E.A[P].data();
    std::vector<cd> M(mC * outer, 0.0), L(szC), Lr(szC), U(szP), X(szP), HA((size_t)d * d);
    std::vector<cd> b1(std::max(szC, szP)), b2(std::max(szC, szP));
    for (size_t gi = 0; gi < E.P.groups[C].size(); ++gi) {
      const Group& G = E.P.groups[C][gi];
      if (G.id_spf || G.id_mf) continue;
      // lower: sum_t a_t chain_t(C), times r, projected off C's columns
      std::fill(L.begin(), L.end(), cd(0.0));
      for (const SpfTuple& t : G.spf) {
        const cd* Y = E.apply_items(C, t.items, A, b1.data(), b2.data());
        for (size_t i = 0; i < szC; ++i) L[i] += t.a * Y[i];
      }
      matmul(L.data(), r.data(), (int)mC, d, d, Lr.data());
      adj_mul(A, Lr.data(), mC, d, HA.data(), 1.0, false);      // C^H L r
      for (size_t x = 0; x < mC; ++x)
        for (int k = 0; k < d; ++k) {
          cd s = 0.0;
          for (int j = 0; j < d; ++j) s += A[x * d + j] * HA[(size_t)j * d + k];
          Lr[x * d + k] -= s;
        }
      // upper: s_g sum_k b_k (sibling products, parent mean field) P, projected off P's slices
      std::fill(U.begin(), U.end(), cd(0.0));
      for (const MfKey& k : G.mf) {
        const cd* Y = E.apply_sibs(P, k.sib, Ap, b1.data(), b2.data());
        if (!E.P.groups[P][k.pg].id_mf) {
          mf_apply(Y, E.mf[P][k.pg].data(), rp, szP / rp, X.data(), 1.0, false);
          Y = X.data();
        }
        for (size_t i = 0; i < szP; ++i) U[i] += G.s * k.b * Y[i];
      }
      mode_contract(Ap, U.data(), pre, d, post, HA.data(), 1.0, false);  // HA(j,i) = sum conj(P(a,j,b)) U(a,i,b)
      for (size_t a = 0; a < pre; ++a)
        for (int i = 0; i < d; ++i)
          for (size_t b = 0; b < post; ++b) {
            cd s = 0.0;
            for (int j = 0; j < d; ++j) s += HA[(size_t)j * d + i] * Ap[(a * d + j) * post + b];
            U[(a * d + i) * post + b] -= s;
          }
      // M(x, a*post + b) += sum_i Lr(x, i) U(a, i, b)
      for (size_t x = 0; x < mC; ++x)
        for (int i = 0; i < d; ++i) {
          const cd l = Lr[x * d + i];
          if (l == cd(0.0)) continue;
          for (size_t a = 0; a < pre; ++a)
            for (size_t b = 0; b < post; ++b) M[x * outer + a * post + b] += l * U[(a * d + i) * post + b];
        }
    }
    return M;
  }

  // dominant singular values and vectors of M (m x n): the right ones (length n) when
  // the k largest eigenpairs of a Hermitian g x g matrix G: a dense Jacobi solve up to
  // g = 96, above that Lanczos (at most 48 steps, full re-orthogonalisation, twice) from a
  // fixed start vector with the Ritz pairs of the tridiagonal
  static void top_eig(const std::vector<cd>& G, size_t g, int k, std::vector<double>& vals,
                      std::vector<std::vector<cd>>& vecs) {
    vals.clear();
    vecs.clear();
    if (g <= 96) {
      std::vector<double> w;
      std::vector<cd> Z;
      herm_eig(G, (int)g, w, Z);
      for (int j = 0; j < std::min<int>(k, (int)g); ++j) {
        vals.push_back(w[j]);
        std::vector<cd> z(g);
        for (size_t i = 0; i < g; ++i) z[i] = Z[i * g + j];
        vecs.push_back(z);
      }
      return;
    }
    const int m = (int)std::min<size_t>(g, 48);
    std::vector<std::vector<cd>> Q;
    std::vector<double> al, be;
    std::vector<cd> q(g), w(g);
    double nq = 0.0;
    for (size_t i = 0; i < g; ++i) { q[i] = 1.0 + 0.5 * std::sin((double)(i + 1)); nq += std::norm(q[i]); }
    for (auto& z : q) z /= std::sqrt(nq);
    for (int j = 0; j < m; ++j) {
      Q.push_back(q);
      for (size_t i = 0; i < g; ++i) { cd t = 0.0; for (size_t c = 0; c < g; ++c) t += G[i * g + c] * q[c]; w[i] = t; }
      double a = 0.0;
      for (size_t i = 0; i < g; ++i) a += (std::conj(q[i]) * w[i]).real();
      al.push_back(a);
      for (int pass = 0; pass < 2; ++pass)
        for (const auto& u : Q) {
          cd h = 0.0;
          for (size_t i = 0; i < g; ++i) h += std::conj(u[i]) * w[i];
          for (size_t i = 0; i < g; ++i) w[i] -= h * u[i];
        }
      double b = 0.0;
      for (auto& z : w) b += std::norm(z);
      b = std::sqrt(b);
      if (j + 1 == m || b <= 1e-14 * (std::fabs(a) + (be.empty() ? 0.0 : be.back()) + 1e-300)) break;
      be.push_back(b);
      for (size_t i = 0; i < g; ++i) q[i] = w[i] / b;
    }
    const int mm = (int)al.size();
    std::vector<cd> Tm((size_t)mm * mm, 0.0);
    for (int i = 0; i < mm; ++i) {
      Tm[(size_t)i * mm + i] = al[i];
      if (i + 1 < mm) { Tm[(size_t)i * mm + i + 1] = be[i]; Tm[(size_t)(i + 1) * mm + i] = be[i]; }
    }
    std::vector<double> tw;
    std::vector<cd> Y;
    herm_eig(Tm, mm, tw, Y);
    for (int j = 0; j < std::min(k, mm); ++j) {
      vals.push_back(tw[j]);
      std::vector<cd> z(g, 0.0);
      for (int i = 0; i < mm; ++i)
        for (size_t r = 0; r < g; ++r) z[r] += Y[(size_t)i * mm + j] * Q[i][r];
      vecs.push_back(z);
    }
  }

  // right, else the left ones (length m); sv descending, at most k of them
  static void dominant(const std::vector<cd>& M, size_t m, size_t n, int k, bool right, std::vector<double>& sv,
                       std::vector<std::vector<cd>>& vecs) {
    const bool small_left = m <= n;  // Gram of the smaller side
    const size_t g = small_left ? m : n;
    std::vector<cd> G(g * g, 0.0);
    for (size_t i = 0; i < g; ++i)
      for (size_t j = 0; j < g; ++j) {
        cd s = 0.0;
        if (small_left) for (size_t c = 0; c < n; ++c) s += M[i * n + c] * std::conj(M[j * n + c]);      // M M^H
        else for (size_t rr = 0; rr < m; ++rr) s += std::conj(M[rr * n + i]) * M[rr * n + j];           // M^H M
        G[i * g + j] = s;
      }
    std::vector<double> w;
    std::vector<std::vector<cd>> Zv;
    top_eig(G, g, k, w, Zv);
    sv.clear();
    vecs.clear();
    for (int j = 0; j < (int)w.size(); ++j) {
      const double s2 = w[j];
      sv.push_back(s2 > 0.0 ? std::sqrt(s2) : 0.0);
      const std::vector<cd>& z = Zv[j];
      if (right == !small_left) { vecs.push_back(z); continue; }
      // the other side: v = M^H u / sigma (right from left) or u = M v / sigma
      const double s = sv.back();
      std::vector<cd> o(right ? n : m, 0.0);
      if (s > 0.0) {
        if (right) for (size_t c = 0; c < n; ++c) { cd t = 0.0; for (size_t rr = 0; rr < m; ++rr) t += std::conj(M[rr * n + c]) * z[rr]; o[c] = t / s; }
        else for (size_t rr = 0; rr < m; ++rr) { cd t = 0.0; for (size_t c = 0; c < n; ++c) t += M[rr * n + c] * z[c]; o[rr] = t / s; }
      }
      vecs.push_back(o);
    }
  }

  // a random unit vector of length len orthogonal to the given unit vectors (Hermitian
  // Gram-Schmidt, twice); components complex normal from the generator
  std::vector<cd> random_orthogonal(size_t len, const std::vector<std::vector<cd>>& basis) {
    for (;;) {
      std::vector<cd> x(len);
      for (auto& z : x) { const double re = nd(rng); const double im = nd(rng); z = cd(re, im); }
      double n0 = 0.0;
      for (auto& z : x) n0 += std::norm(z);
      n0 = std::sqrt(n0);
      for (auto& z : x) z /= n0;
      for (int pass = 0; pass < 2; ++pass)
        for (const auto& u : basis) {
          cd h = 0.0;
          for (size_t i = 0; i < len; ++i) h += std::conj(u[i]) * x[i];
          for (size_t i = 0; i < len; ++i) x[i] -= h * u[i];
        }
      double nx = 0.0;
      for (auto& z : x) nx += std::norm(z);
      nx = std::sqrt(nx);
      if (nx > 1e-12) {
        for (auto& z : x) z /= nx;
        return x;
      }
    }
  }
  // the slices P(:, i, :) (length pre*post) and the columns C(:, k)
  std::vector<std::vector<cd>> parent_slices(int C) {
    const Tree& T = E.T;
    const int P = T.parent[C], mu = T.slot[C];
    size_t pre, post; int d;
    E.r3(P, mu, pre, d, post);
    std::vector<std::vector<cd>> s(d, std::vector<cd>(pre * post));
    for (size_t a = 0; a < pre; ++a)
      for (int i = 0; i < d; ++i)
        for (size_t b = 0; b < post; ++b) s[i][a * post + b] = E.A[P][(a * d + i) * post + b];
    return s;
  }
  std::vector<std::vector<cd>> child_columns(int C) {
    const Tree& T = E.T;
    const int r = T.hrank[C];
    const size_t m = T.dimen[C];
    std::vector<std::vector<cd>> s(r, std::vector<cd>(m));
    for (size_t x = 0; x < m; ++x)
      for (int k = 0; k < r; ++k) s[k][x] = E.A[C][x * r + k];
    return s;
  }

  // grow the bond above C by the given parent slices (down) or child columns (up); the
  // other side and the gauge factor (rmat of P going down, of C going up) gain zeros
  void grow(int C, const std::vector<std::vector<cd>>& pslices, const std::vector<std::vector<cd>>& ccols, bool down) {
    Tree& T = E.T;
    const int P = T.parent[C], mu = T.slot[C];
    const int nadd = (int)(down ? pslices.size() : ccols.size());
    const int r0 = T.hrank[C], r1 = r0 + nadd;
    size_t pre, post; int d;
    E.r3(P, mu, pre, d, post);
    const size_t mC = T.dimen[C];
    // child
    std::vector<cd> Ac(mC * r1, 0.0);
    for (size_t x = 0; x < mC; ++x) {
      for (int k = 0; k < r0; ++k) Ac[x * r1 + k] = E.A[C][x * r0 + k];
      if (!down) for (int k = 0; k < nadd; ++k) Ac[x * r1 + r0 + k] = ccols[k][x];
    }
    // parent
    std::vector<cd> Ap(pre * r1 * post, 0.0);
    for (size_t a = 0; a < pre; ++a)
      for (size_t b = 0; b < post; ++b) {
        for (int i = 0; i < r0; ++i) Ap[(a * r1 + i) * post + b] = E.A[P][(a * r0 + i) * post + b];
        if (down) for (int j = 0; j < nadd; ++j) Ap[(a * r1 + r0 + j) * post + b] = pslices[j][a * post + b];
      }
    // gauge factor
    std::vector<cd>& R = E.rmat[down ? P : C];
    std::vector<cd> Rn((size_t)r1 * r1, 0.0);
    for (int i = 0; i < r0; ++i)
      for (int j = 0; j < r0; ++j) Rn[(size_t)i * r1 + j] = R[(size_t)i * r0 + j];
    // topology and buffers
    T.hrank[C] = r1;
    T.dims[P][mu] = r1;
    T.dimen[P] = 1;
    for (int dm : T.dims[P]) T.dimen[P] *= (size_t)dm;
    E.A[C].swap(Ac);
    E.A[P].swap(Ap);
    for (int nd : {C, P}) {
      size_t rmx = (size_t)T.hrank[nd];
      for (int dm : T.dims[nd]) rmx = std::max(rmx, (size_t)dm);
      if (E.rmat[nd].size() < rmx * rmx) E.rmat[nd].resize(rmx * rmx, 0.0);
    }
    std::copy(Rn.begin(), Rn.end(), E.rmat[down ? P : C].begin());
    for (size_t g = 0; g < E.P.groups[C].size(); ++g) {
      if (!E.P.groups[C][g].id_spf) E.spf[C][g].assign((size_t)r1 * r1, 0.0);
      if (!E.P.groups[C][g].id_mf) E.mf[C][g].assign((size_t)r1 * r1, 0.0);
    }
    const size_t need = std::max(T.size(C), T.size(P));
    for (auto* w : {&E.w1, &E.w2, &E.w3, &E.w4})
      if (w->size() < need) w->resize(need, 0.0);
  }

  // subspace_expansion_down: C below P, after P's decomposition towards C (r = rmat[P])
  bool down(int C) {
    const Tree& T = E.T;
    const int P = T.parent[C], mu = T.slot[C], d = T.hrank[C];
    if (d >= cap[C]) return false;
    size_t pre, post; int dd;
    E.r3(P, mu, pre, dd, post);
    const size_t outer = pre * post;
    if ((size_t)d >= outer) return false;
    const std::vector<double> pops = svals(E.rmat[P].data(), d);
    const int nunocc = n_unoccupied(pops);
    if (only_when_no_unoccupied && nunocc >= minimum_unoccupied) return false;
    const int max_add = (int)std::min<size_t>(std::min<size_t>((size_t)(cap[C] - d), outer - d),
                                              T.dimen[C] > (size_t)d ? T.dimen[C] - d : 0);
    const int required = nunocc < minimum_unoccupied ? std::min(minimum_unoccupied - nunocc, max_add) : 0;
    int nadd = 0;
    if ((size_t)d < T.dimen[C] && d != 1) {
      std::vector<cd> r(E.rmat[P].begin(), E.rmat[P].begin() + (size_t)d * d);
      const std::vector<cd> M = two_site_matrix(C, r);
      std::vector<double> sv;
      std::vector<std::vector<cd>> V;
      dominant(M, T.dimen[C], outer, neigenvalues, true, sv, V);
      for (double s : sv)
        if (s > 0.0 && std::isfinite(s) && s * E.dt / 2.0 > spawning_threshold) ++nadd;
      nadd = std::min(nadd, max_add);
      if (nadd) {
        // the parent-side functions of M = sum sigma u v^H are conj(v)
        std::vector<std::vector<cd>> f(nadd);
        for (int j = 0; j < nadd; ++j) {
          f[j] = V[j];
          for (auto& z : f[j]) z = std::conj(z);
        }
        grow(C, f, {}, true);
      }
      ++n_twosite;  // down counts every two-site attempt
    } else {
      while (nadd < required) {
        const std::vector<cd> x = random_orthogonal(outer, parent_slices(C));
        grow(C, {x}, {}, true);
        ++nadd;
      }
      ++n_onesite;
    }
    return nadd > 0;
  }

  // subspace_expansion_up: C below P, after C's leaf-to-root decomposition (r = rmat[C])
  bool up(int C) {
    const Tree& T = E.T;
    const int P = T.parent[C], mu = T.slot[C], d = T.hrank[C];
    if (d >= cap[C]) return false;
    const size_t mC = T.dimen[C];
    if ((size_t)d >= mC) return false;
    const std::vector<double> pops = svals(E.rmat[C].data(), d);
    const int nunocc = n_unoccupied(pops);
    if (only_when_no_unoccupied && nunocc >= minimum_unoccupied) return false;
    size_t pre, post; int dd;
    E.r3(P, mu, pre, dd, post);
    const int max_add = (int)std::min<size_t>(std::min<size_t>((size_t)(cap[C] - d), mC - d),
                                              pre * post > (size_t)d ? pre * post - d : 0);
    const int required = nunocc < minimum_unoccupied ? std::min(minimum_unoccupied - nunocc, max_add) : 0;
    int nadd = 0;
    if ((size_t)d < pre * post && d != 1) {
      std::vector<cd> r(E.rmat[C].begin(), E.rmat[C].begin() + (size_t)d * d);
      const std::vector<cd> M = two_site_matrix(C, r);
      std::vector<double> sv;
      std::vector<std::vector<cd>> U;
      dominant(M, mC, pre * post, neigenvalues, false, sv, U);
      for (double s : sv)
        if (s > 0.0 && std::isfinite(s) && s * E.dt / 2.0 > spawning_threshold) ++nadd;
      nadd = std::min(nadd, max_add);
      if (nadd) {
        U.resize(nadd);
        grow(C, {}, U, false);
        ++n_twosite;  // up counts only the attempts that grew the bond
      }
    } else {
      while (nadd < required) {
        const std::vector<cd> x = random_orthogonal(mC, child_columns(C));
        grow(C, {}, {x}, false);
        ++nadd;
      }
      ++n_onesite;
    }
    return nadd > 0;
  }

  void attach() {
    E.expand_down = [this](int c) { return down(c); };
    E.expand_up = [this](int c) { return up(c); };
  }
  void detach() { E.expand_down = nullptr; E.expand_up = nullptr; }

  // prepare_evolution: environments, then expansion half-sweeps without evolution until
  // nothing grows (tdvp_algorithm_engine.hpp:257-321)
  bool prepare() {
    for (int id = E.T.n - 1; id >= 1; --id) E.update_spf(id);
    bool any = false;
    for (int it = 0; it < 1000; ++it) {
      E.expanded = false;
      attach();
      E.expand_up = nullptr;
      E.forward(false);
      const bool f = E.expanded;
      E.expanded = false;
      attach();
      E.expand_down = nullptr;
      E.backward(false);
      const bool b = E.expanded;
      detach();
      any = any || f || b;
      if (!f && !b) break;
    }
    return any;
  }
  // one sweep with expansion: down in the forward half, up in the backward half
  void sweep() {
    attach();
    E.expand_up = nullptr;
    E.forward(true);
    E.t_engine += E.dt / 2.0;
    attach();
    E.expand_down = nullptr;
    E.backward(true);
    E.t_engine += E.dt / 2.0;
    detach();
  }
  // subspace_expansion_projector_splitting_integrator::operator()
  void step(double step_dt, cd cf) {
    E.coeff = cf;
    if (E.nsteps == 0) {
      E.dt = step_dt;
      prepare();
      double tevolve = 0.0, sdt = step_dt / 1e5;
      while (tevolve < step_dt) {
        E.dt = (sdt + tevolve <= step_dt) ? sdt : step_dt - tevolve;
        E.t_engine = tevolve;
        sweep();
        tevolve += sdt;
        sdt *= 10.0;
      }
    } else {
      E.dt = step_dt;
      E.t_engine = E.nsteps * step_dt;
      sweep();
    }
    E.dt = step_dt;
    ++E.nsteps;
  }
};
