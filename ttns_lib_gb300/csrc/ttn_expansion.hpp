// ttn_expansion.hpp -- subspace expansion (adaptive bond dimension) on the device.
// Included by ttn_host.cpp inside namespace ttn, after Integrator.
//
// Follows include/ttns_lib/tdvp_core/subspace_expansion_projector_splitting_engine.hpp
// (subspace_expansion_down :207-358, _up :361-510, get_nunoccupied :577-585) with the
// two-site terms of two_site_energy_variations.hpp:78-222 and the growth of
// :375-444, driven like tdvp_algorithm_engine.hpp:257-321 (repeated expansion before the
// first step) and projector_splitting_integrator.hpp:281-326.
//
// At the gauge move between node C and its parent P the two-site wavefunction is C r P.
// For every term group of C that is neither the identity below C nor above it,
//   L_g = (1 - C C^H) [sum_t a_t (spf product of tuple t) C] r          (dimen_C x d)
//   U_g = s_g sum_k b_k (sibling spf products, parent mean field) P, minus its part in the
//         span of P's slices                                          (pre x d x post)
// and M = sum_g L_g . U_g (over the bond index).  L_g, U_g and M are built on the device
// with the sweep's own contractions (mode and mean-field products, reductions, right
// products, one batched GEMM for M); the dominant singular directions of M come from a
// Hermitian eigensolve of the smaller Gram matrix on the host.  Going down, the dominant
// right directions (conjugated) become new slices of P, C and r gain zeros; going up, the
// dominant left directions become new columns of C, P and r gain zeros; at most
// `neigenvalues` of them, those with sigma dt/2 above the spawning threshold, within the
// bond's capacity and keeping both tensors' matricisations tall.  Where the neighbour is
// square or the bond has rank 1, random orthonormal directions (std::mt19937, normal
// components) are added while fewer than `minimum_unoccupied` singular values of r are
// unoccupied.  Tensors live in slabs sized for the capacities; a growth re-lays the two
// tensors and the gauge factor through the host and recompiles the term programs.

static void herm_eig_host(std::vector<cd> a, int n, std::vector<double>& w, std::vector<cd>& Z) {
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

struct DevExpander {
  Integrator& I;
  double spawning_threshold = -1.0, unoccupied_threshold = -1.0;
  int minimum_unoccupied = 0, neigenvalues = 2;
  bool only_when_no_unoccupied = false;
  std::mt19937 rng;
  std::normal_distribution<double> nd{0.0, 1.0};
  long long n_twosite = 0, n_onesite = 0;
  const ttn_state* state = nullptr;  // the state re-laid at capacity for this integrator
  DevBuf m_buf, s_buf;  // M; scratch vectors and a small matrix

  explicit DevExpander(Integrator& in) : I(in) {
    const size_t vb = align256((size_t)I.maxsize * sizeof(double2));
    s_buf.alloc(vb * 6 + align256((size_t)kMaxBond * kMaxBond * sizeof(double2)));
  }
  double2* scratch(int k) const { return reinterpret_cast<double2*>(static_cast<char*>(s_buf.p) + align256((size_t)I.maxsize * sizeof(double2)) * k); }

  std::vector<cd> down(const double2* p, size_t n) {
    std::vector<double2> h(n);
    CK(cudaMemcpyAsync(h.data(), p, n * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
    CK(cudaStreamSynchronize(I.stream));
    std::vector<cd> o(n);
    for (size_t i = 0; i < n; ++i) o[i] = cd(h[i].x, h[i].y);
    return o;
  }
  void up(double2* p, const std::vector<cd>& v) {
    std::vector<double2> h(v.size());
    for (size_t i = 0; i < v.size(); ++i) h[i] = d2(v[i]);
    CK(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
    CK(cudaStreamSynchronize(I.stream));  // h is pageable and goes out of scope
  }

  static std::vector<double> svals(const std::vector<cd>& R, int d) {
    std::vector<cd> G((size_t)d * d, 0.0);
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        cd s = 0.0;
        for (int k = 0; k < d; ++k) s += std::conj(R[(size_t)k * d + i]) * R[(size_t)k * d + j];
        G[(size_t)i * d + j] = s;
      }
    std::vector<double> w;
    std::vector<cd> Z;
    herm_eig_host(G, d, w, Z);
    for (auto& x : w) x = std::sqrt(std::max(0.0, x));
    return w;
  }
  int n_unoccupied(const std::vector<double>& pops) const {
    int n = 0;
    for (double p : pops)
      if (pops[0] > 0.0 ? p / pops[0] < unoccupied_threshold : true) ++n;
    return n;
  }

  // M (dimen_C x pre*post, row-major, on the host) at the bond above C; r: gauge factor (d x d)
  std::vector<cd> two_site_matrix(ttn_state* S, int C, const double2* r, bool download = true) {
    const Tree& T = I.T;
    const int P = T.parent[C], mu = T.slot[C], d = T.hrank[C], rp = T.hrank[P];
    long long pre, post;
    int dd;
    I.r3(P, mu, pre, dd, post);
    const long long mC = T.dimen[C], szC = T.size(C), szP = T.size(P), outer = pre * post;
    const double2* A = S->node(C);
    const double2* Ap = S->node(P);
    const size_t mbytes = (size_t)(mC * outer) * sizeof(double2);
    if (m_buf.bytes < mbytes) m_buf.alloc(mbytes);
    double2* M = m_buf.as<double2>();
    zfill(M, make_double2(0.0, 0.0), mC * outer, I.stream);
    double2 *L = scratch(0), *Lr = scratch(1), *U = scratch(2), *X = scratch(3), *tmp = scratch(4), *HA = scratch(6);
    for (size_t gi = 0; gi < I.G[C].size(); ++gi) {
      const Group& G = I.G[C][gi];
      if (G.id_spf || G.id_mf) continue;
      // lower: sum_t a_t chain_t(C), times r, projected off C's columns
      bool first = true;
      for (const SpfTuple& t : G.spf) {
        const double2* Y = I.apply_items(C, t.items, A, I.w1, I.w2);
        zaxpy(L, Y, d2(t.a), szC, !first, I.stream);
        first = false;
      }
      I.right_mul(L, r, mC, d, Lr);
      I.adj_mul(A, Lr, mC, d, HA, 1.0, false);
      I.right_mul(A, HA, mC, d, tmp);
      zaxpy(Lr, tmp, make_double2(-1.0, 0.0), szC, true, I.stream);
      // upper: s_g sum_k b_k (sibling products, parent mean field) P, projected off P's slices
      first = true;
      for (const MfKey& k : G.mf) {
        const double2* Y = I.apply_sibs(P, k.sib, Ap, I.w1, I.w2);
        if (!I.G[P][k.pg].id_mf) {
          I.mf_apply(Y, I.G[P][k.pg].mf_dev, rp, szP / rp, X, 1.0, false, false);
          Y = X;
        }
        zaxpy(U, Y, d2(G.s * k.b), szP, !first, I.stream);
        first = false;
      }
      I.mode_contract(Ap, U, pre, d, post, HA, 1.0, false);  // HA(j,i) = sum conj(P(a,j,b)) U(a,i,b)
      const std::vector<cd> h = down(HA, (size_t)d * d);
      std::vector<cd> St((size_t)d * d);
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) St[(size_t)i * d + j] = h[(size_t)j * d + i];
      up(tmp, St);
      I.mode_apply(tmp, d, Ap, U, pre, post, -1.0, true, false);
      // M(x, a post + b) += sum_i Lr(x, i) U(a, i, b): one GEMM per a
      ZGemm g{};
      g.M = (int)mC; g.N = (int)post; g.K = d;
      g.A = op_rowmajor(Lr, d);
      g.B = op_colk(U, post, 1);  // B(i, b) = U[i post + b] within slice a
      g.C = M; g.ci = outer; g.cj = 1;
      g.bsA = 0; g.bsB = (long long)d * post; g.bsC = post;
      g.batch = (int)pre;
      g.alpha = make_double2(1.0, 0.0);
      g.beta = make_double2(1.0, 0.0);
      zgemm(g, I.gws, I.gws_bytes, I.stream);
    }
    if (!download) return {};
    return down(M, (size_t)(mC * outer));
  }

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
      herm_eig_host(G, (int)g, w, Z);
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
    herm_eig_host(Tm, mm, tw, Y);
    for (int j = 0; j < std::min(k, mm); ++j) {
      vals.push_back(tw[j]);
      std::vector<cd> z(g, 0.0);
      for (int i = 0; i < mm; ++i)
        for (size_t r = 0; r < g; ++r) z[r] += Y[(size_t)i * mm + j] * Q[i][r];
      vecs.push_back(z);
    }
  }

  // dominant_dev: the same result as dominant() for the M left in m_buf by
  // two_site_matrix(..., false), without bringing M or its Gram matrix to the host: the
  // Gram matrix of the smaller side by one GEMM, the Lanczos process of top_eig on the
  // device (w = G q by GEMM, two passes of classical Gram-Schmidt against all earlier
  // vectors by GEMM, only alpha and beta copied back per step), the tridiagonal solved
  // and the Ritz vectors formed on the host from the Lanczos vectors (48 x g), and the
  // other side's vectors M^H z / s or M z / s by GEMM.
  void dominant_dev(size_t m, size_t n, int k, bool right, std::vector<double>& sv, std::vector<std::vector<cd>>& vecs) {
    const bool small_left = m <= n;
    const size_t g = small_left ? m : n;
    const int mmax = (int)std::min<size_t>(g, 48);
    DevBuf gb, qb, wb;
    gb.alloc(g * g * sizeof(double2));
    qb.alloc((size_t)mmax * g * sizeof(double2));
    wb.alloc((g + 64 + 4) * sizeof(double2));
    double2* Gd = gb.as<double2>();
    double2* Qd = qb.as<double2>();
    double2* w = wb.as<double2>();
    double2* h = w + g;         // projections on the Lanczos vectors (<= 48)
    double2* sc = h + 64;       // alpha, beta^2
    const double2* M = m_buf.as<double2>();
    auto gemm = [&](int Mr, int Nc, int K, ZOperand A, ZOperand B, double2* C, long long ci, long long cj, double2 al,
                    double2 be) {
      ZGemm z{};
      z.M = Mr; z.N = Nc; z.K = K; z.A = A; z.B = B; z.C = C; z.ci = ci; z.cj = cj;
      z.batch = 1; z.alpha = al; z.beta = be;
      zgemm(z, I.gws, I.gws_bytes, I.stream);
    };
    const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0), mone = make_double2(-1.0, 0.0);
    // Gram matrix of the smaller side
    {
      ZOperand A, B;
      if (small_left) {
        A = op_rowmajor(M, (long long)n);
        B = op_rowmajor(M, (long long)n);
        B.cj = 1;
        gemm((int)g, (int)g, (int)n, A, B, Gd, (long long)g, 1, one, zero);
      } else {
        A = op_colk(M, (long long)n, 1);
        A.cj = 1;
        B = op_colk(M, (long long)n, 1);
        gemm((int)g, (int)g, (int)m, A, B, Gd, (long long)g, 1, one, zero);
      }
    }
    // the start vector of top_eig
    {
      std::vector<cd> q(g);
      double nq = 0.0;
      for (size_t i = 0; i < g; ++i) { q[i] = 1.0 + 0.5 * std::sin((double)(i + 1)); nq += std::norm(q[i]); }
      for (auto& z : q) z /= std::sqrt(nq);
      up(Qd, q);
    }
    std::vector<double> al, be;
    for (int j = 0; j < mmax; ++j) {
      const double2* q = Qd + (size_t)j * g;
      const ZOperand vec_q = op_colk(q, 1, 0);
      gemm((int)g, 1, (int)g, op_rowmajor(Gd, (long long)g), vec_q, w, 1, 0, one, zero);  // w = G q
      ZOperand qc = op_colk(q, 1, 0);
      qc.cj = 1;
      gemm(1, 1, (int)g, qc, op_colk(w, 1, 0), sc, 1, 0, one, zero);  // alpha = q^H w
      for (int pass = 0; pass < 2; ++pass) {
        ZOperand Qc = op_rowmajor(Qd, (long long)g);
        Qc.cj = 1;
        gemm(j + 1, 1, (int)g, Qc, op_colk(w, 1, 0), h, 1, 0, one, zero);                          // h = Q^H w
        gemm((int)g, 1, j + 1, op_colk(Qd, (long long)g, 1), op_colk(h, 1, 0), w, 1, 0, mone, one);  // w -= Q h
      }
      ZOperand wc = op_colk(w, 1, 0);
      wc.cj = 1;
      gemm(1, 1, (int)g, wc, op_colk(w, 1, 0), sc + 1, 1, 0, one, zero);  // beta^2 = w^H w
      double2 hs[2];
      CK(cudaMemcpyAsync(hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, I.stream));
      CK(cudaStreamSynchronize(I.stream));
      const double a = hs[0].x, b = std::sqrt(std::max(0.0, hs[1].x));
      al.push_back(a);
      if (j + 1 == mmax || b <= 1e-14 * (std::fabs(a) + (be.empty() ? 0.0 : be.back()) + 1e-300)) break;
      be.push_back(b);
      zaxpy(Qd + (size_t)(j + 1) * g, w, make_double2(1.0 / b, 0.0), (long long)g, false, I.stream);
    }
    const int mm = (int)al.size();
    std::vector<cd> Tm((size_t)mm * mm, 0.0);
    for (int i = 0; i < mm; ++i) {
      Tm[(size_t)i * mm + i] = al[i];
      if (i + 1 < mm) { Tm[(size_t)i * mm + i + 1] = be[i]; Tm[(size_t)(i + 1) * mm + i] = be[i]; }
    }
    std::vector<double> tw;
    std::vector<cd> Y;
    herm_eig_host(Tm, mm, tw, Y);
    const std::vector<cd> Q = down(Qd, (size_t)mm * g);
    sv.clear();
    vecs.clear();
    for (int j = 0; j < std::min(k, mm); ++j) {
      std::vector<cd> z(g, 0.0);
      for (int i = 0; i < mm; ++i)
        for (size_t r = 0; r < g; ++r) z[r] += Y[(size_t)i * mm + j] * Q[(size_t)i * g + r];
      const double s2 = tw[j];
      sv.push_back(s2 > 0.0 ? std::sqrt(s2) : 0.0);
      if (right == !small_left) { vecs.push_back(z); continue; }
      const double s = sv.back();
      const size_t len = right ? n : m;
      if (!(s > 0.0)) { vecs.push_back(std::vector<cd>(len, 0.0)); continue; }
      DevBuf ob;
      ob.alloc((len + g) * sizeof(double2));
      double2* zd = ob.as<double2>() + len;
      up(zd, z);
      if (right) {  // o(c) = sum_r conj M(r, c) z(r) / s
        ZOperand A = op_colk(M, (long long)n, 1);
        A.cj = 1;
        gemm((int)n, 1, (int)m, A, op_colk(zd, 1, 0), ob.as<double2>(), 1, 0, make_double2(1.0 / s, 0.0), zero);
      } else {      // o(r) = sum_c M(r, c) z(c) / s
        gemm((int)m, 1, (int)n, op_rowmajor(M, (long long)n), op_colk(zd, 1, 0), ob.as<double2>(), 1, 0,
             make_double2(1.0 / s, 0.0), zero);
      }
      vecs.push_back(down(ob.as<double2>(), len));
    }
  }

  // dominant singular values and (right or left) vectors of M (m x n), at most k; Gpre: the
  // Gram matrix of the smaller side when already formed
  static void dominant(const std::vector<cd>& M, size_t m, size_t n, int k, bool right, std::vector<double>& sv,
                       std::vector<std::vector<cd>>& vecs, const std::vector<cd>* Gpre = nullptr) {
    const bool small_left = m <= n;
    const size_t g = small_left ? m : n;
    std::vector<cd> G;
    if (Gpre) G = *Gpre;
    else {
      G.assign(g * g, 0.0);
      for (size_t i = 0; i < g; ++i)
        for (size_t j = 0; j < g; ++j) {
          cd s = 0.0;
          if (small_left) for (size_t c = 0; c < n; ++c) s += M[i * n + c] * std::conj(M[j * n + c]);
          else for (size_t rr = 0; rr < m; ++rr) s += std::conj(M[rr * n + i]) * M[rr * n + j];
          G[i * g + j] = s;
        }
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
      const double s = sv.back();
      std::vector<cd> o(right ? n : m, 0.0);
      if (s > 0.0) {
        if (right) for (size_t c = 0; c < n; ++c) { cd t = 0.0; for (size_t rr = 0; rr < m; ++rr) t += std::conj(M[rr * n + c]) * z[rr]; o[c] = t / s; }
        else for (size_t rr = 0; rr < m; ++rr) { cd t = 0.0; for (size_t c = 0; c < n; ++c) t += M[rr * n + c] * z[c]; o[rr] = t / s; }
      }
      vecs.push_back(o);
    }
  }

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
  std::vector<std::vector<cd>> parent_slices(ttn_state* S, int C) {
    const Tree& T = I.T;
    const int P = T.parent[C], mu = T.slot[C];
    long long pre, post; int d;
    I.r3(P, mu, pre, d, post);
    const std::vector<cd> a = down(S->node(P), (size_t)T.size(P));
    std::vector<std::vector<cd>> s(d, std::vector<cd>((size_t)(pre * post)));
    for (long long x = 0; x < pre; ++x)
      for (int i = 0; i < d; ++i)
        for (long long b = 0; b < post; ++b) s[i][(size_t)(x * post + b)] = a[(size_t)((x * d + i) * post + b)];
    return s;
  }
  std::vector<std::vector<cd>> child_columns(ttn_state* S, int C) {
    const Tree& T = I.T;
    const int r = T.hrank[C];
    const long long m = T.dimen[C];
    const std::vector<cd> a = down(S->node(C), (size_t)T.size(C));
    std::vector<std::vector<cd>> s(r, std::vector<cd>((size_t)m));
    for (long long x = 0; x < m; ++x)
      for (int k = 0; k < r; ++k) s[k][(size_t)x] = a[(size_t)(x * r + k)];
    return s;
  }

  // grow the bond above C by parent slices (down) or child columns (up); the other side
  // and the gauge factor (rmat of P going down, of C going up) gain zeros
  void grow(ttn_state* S, int C, const std::vector<std::vector<cd>>& pslices, const std::vector<std::vector<cd>>& ccols,
            bool down_dir) {
    Tree& T = I.T;
    const int P = T.parent[C], mu = T.slot[C];
    const int nadd = (int)(down_dir ? pslices.size() : ccols.size());
    const int r0 = T.hrank[C], r1 = r0 + nadd;
    TTN_REQUIRE(r1 <= I.cap[C], TTN_ECAPACITY, "subspace expansion beyond a bond's capacity");
    long long pre, post; int d;
    I.r3(P, mu, pre, d, post);
    const long long mC = T.dimen[C];
    const std::vector<cd> ac = down(S->node(C), (size_t)(mC * r0));
    const std::vector<cd> ap = down(S->node(P), (size_t)(pre * r0 * post));
    double2* Rd = I.rmat[down_dir ? P : C];
    const std::vector<cd> R = down(Rd, (size_t)r0 * r0);
    std::vector<cd> nc((size_t)(mC * r1), 0.0), np((size_t)(pre * r1 * post), 0.0), nr((size_t)r1 * r1, 0.0);
    for (long long x = 0; x < mC; ++x) {
      for (int k = 0; k < r0; ++k) nc[(size_t)(x * r1 + k)] = ac[(size_t)(x * r0 + k)];
      if (!down_dir) for (int k = 0; k < nadd; ++k) nc[(size_t)(x * r1 + r0 + k)] = ccols[k][(size_t)x];
    }
    for (long long a = 0; a < pre; ++a)
      for (long long b = 0; b < post; ++b) {
        for (int i = 0; i < r0; ++i) np[(size_t)((a * r1 + i) * post + b)] = ap[(size_t)((a * r0 + i) * post + b)];
        if (down_dir) for (int j = 0; j < nadd; ++j) np[(size_t)((a * r1 + r0 + j) * post + b)] = pslices[j][(size_t)(a * post + b)];
      }
    for (int i = 0; i < r0; ++i)
      for (int j = 0; j < r0; ++j) nr[(size_t)i * r1 + j] = R[(size_t)i * r0 + j];
    T.set_bond(C, r1);
    S->T.set_bond(C, r1);
    up(S->node(C), nc);
    up(S->node(P), np);
    up(Rd, nr);
    I.compile_programs();
  }

  // subspace_expansion_down: C below P after P's decomposition towards C (r = rmat[P])
  bool expand_down(ttn_state* S, int C) {
    const Tree& T = I.T;
    const int P = T.parent[C], mu = T.slot[C], d = T.hrank[C];
    if (d >= I.cap[C]) return false;
    long long pre, post; int dd;
    I.r3(P, mu, pre, dd, post);
    const long long outer = pre * post;
    if (d >= outer) return false;
    const std::vector<double> pops = svals(down(I.rmat[P], (size_t)d * d), d);
    const int nunocc = n_unoccupied(pops);
    if (only_when_no_unoccupied && nunocc >= minimum_unoccupied) return false;
    const int max_add = (int)std::min<long long>(std::min<long long>(I.cap[C] - d, outer - d),
                                                 T.dimen[C] > d ? T.dimen[C] - d : 0);
    const int required = nunocc < minimum_unoccupied ? std::min(minimum_unoccupied - nunocc, max_add) : 0;
    int nadd = 0;
    if (d < T.dimen[C] && d != 1) {
      std::vector<double> sv;
      std::vector<std::vector<cd>> V;
      const size_t mm = (size_t)T.dimen[C], nn = (size_t)outer;
      if (std::min(mm, nn) > 96) {
        two_site_matrix(S, C, I.rmat[P], false);
        dominant_dev(mm, nn, neigenvalues, true, sv, V);
      } else {
        const std::vector<cd> M = two_site_matrix(S, C, I.rmat[P]);
        dominant(M, mm, nn, neigenvalues, true, sv, V);
      }
      for (double s : sv)
        if (s > 0.0 && std::isfinite(s) && s * I.dt / 2.0 > spawning_threshold) ++nadd;
      nadd = std::min(nadd, max_add);
      if (nadd) {
        std::vector<std::vector<cd>> f(nadd);
        for (int j = 0; j < nadd; ++j) {
          f[j] = V[j];
          for (auto& z : f[j]) z = std::conj(z);
        }
        grow(S, C, f, {}, true);
      }
      ++n_twosite;  // down counts every two-site attempt
    } else {
      while (nadd < required) {
        const std::vector<cd> x = random_orthogonal((size_t)outer, parent_slices(S, C));
        grow(S, C, {x}, {}, true);
        ++nadd;
      }
      ++n_onesite;
    }
    return nadd > 0;
  }

  // subspace_expansion_up: C below P after C's leaf-to-root decomposition (r = rmat[C])
  bool expand_up(ttn_state* S, int C) {
    const Tree& T = I.T;
    const int P = T.parent[C], mu = T.slot[C], d = T.hrank[C];
    if (d >= I.cap[C]) return false;
    const long long mC = T.dimen[C];
    if (d >= mC) return false;
    const std::vector<double> pops = svals(down(I.rmat[C], (size_t)d * d), d);
    const int nunocc = n_unoccupied(pops);
    if (only_when_no_unoccupied && nunocc >= minimum_unoccupied) return false;
    long long pre, post; int dd;
    I.r3(P, mu, pre, dd, post);
    const int max_add = (int)std::min<long long>(std::min<long long>(I.cap[C] - d, mC - d),
                                                 pre * post > d ? pre * post - d : 0);
    const int required = nunocc < minimum_unoccupied ? std::min(minimum_unoccupied - nunocc, max_add) : 0;
    int nadd = 0;
    if (d < pre * post && d != 1) {
      std::vector<double> sv;
      std::vector<std::vector<cd>> U;
      const size_t mm = (size_t)mC, nn = (size_t)(pre * post);
      if (std::min(mm, nn) > 96) {
        two_site_matrix(S, C, I.rmat[C], false);
        dominant_dev(mm, nn, neigenvalues, false, sv, U);
      } else {
        const std::vector<cd> M = two_site_matrix(S, C, I.rmat[C]);
        dominant(M, mm, nn, neigenvalues, false, sv, U);
      }
      for (double s : sv)
        if (s > 0.0 && std::isfinite(s) && s * I.dt / 2.0 > spawning_threshold) ++nadd;
      nadd = std::min(nadd, max_add);
      if (nadd) {
        U.resize(nadd);
        grow(S, C, {}, U, false);
        ++n_twosite;  // up counts only the attempts that grew the bond
      }
    } else {
      while (nadd < required) {
        const std::vector<cd> x = random_orthogonal((size_t)mC, child_columns(S, C));
        grow(S, C, {}, {x}, false);
        ++nadd;
      }
      ++n_onesite;
    }
    return nadd > 0;
  }

  void hooks(bool down_on, bool up_on) {
    I.expand_down_fn = down_on ? std::function<bool(ttn_state*, int)>([this](ttn_state* s, int c) { return expand_down(s, c); })
                               : nullptr;
    I.expand_up_fn = up_on ? std::function<bool(ttn_state*, int)>([this](ttn_state* s, int c) { return expand_up(s, c); })
                           : nullptr;
  }
  struct HookReset {
    DevExpander* x;
    ~HookReset() { x->hooks(false, false); }
  };
  // prepare_evolution: environments, then expansion half-sweeps without evolution until
  // nothing grows
  bool prepare(ttn_state* S) {
    HookReset hr{this};
    for (int id = I.T.n - 1; id >= 1; --id) I.update_spf(id, S->node(id));
    bool any = false;
    for (int it = 0; it < 1000; ++it) {
      I.expanded = false;
      hooks(true, false);
      I.forward(S, false);
      const bool f = I.expanded;
      I.expanded = false;
      hooks(false, true);
      I.backward(S, false);
      const bool b = I.expanded;
      any = any || f || b;
      if (!f && !b) break;
    }
    return any;
  }
  void sweep(ttn_state* S) {
    HookReset hr{this};
    hooks(true, false);
    I.forward(S, true);
    I.t_engine += I.dt / 2.0;
    hooks(false, true);
    I.backward(S, true);
    I.t_engine += I.dt / 2.0;
  }
  // subspace_expansion_projector_splitting_integrator::operator()
  void step(ttn_state* S, double step_dt, cd cf) {
    TTN_REQUIRE(S == state, TTN_EINVAL, "with subspace expansion, step the state given to ttn_integrator_set_expansion");
    I.coeff = cf;
    if (I.nsteps == 0) {
      I.dt = step_dt;
      prepare(S);
      double tevolve = 0.0, sdt = step_dt / 1e5;
      while (tevolve < step_dt) {
        I.dt = (sdt + tevolve <= step_dt) ? sdt : step_dt - tevolve;
        I.t_engine = tevolve;
        sweep(S);
        tevolve += sdt;
        sdt *= 10.0;
      }
    } else {
      I.dt = step_dt;
      I.t_engine = I.nsteps * step_dt;
      sweep(S);
    }
    ++I.nsteps;
    I.dt = step_dt;
  }
};
