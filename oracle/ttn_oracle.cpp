// ttn_oracle.cpp -- CPU FP64 restatement of ttns_lib's one-site projector-splitting
// TDVP sweep.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
// bench's CPU-baseline leg load this library as the checker.  The product path
// (ttns_lib_gb300) never links or calls it.
//
// Parity status: the reference's arithmetic lives in two git submodules (linalg,
// utils_cpp) that are empty in the reference checkout, so the reference cannot be
// compiled or run.  This restatement is therefore "parity unpinned" against the
// reference itself; it is pinned instead by known-answer tests (dense exp(-iHt)
// on full-rank trees, the zero-coupling spin precession, norm/energy conservation).
//
// What each part restates (paths are relative to the reference project root):
//   * sweep order ........ include/ttns_lib/tdvp_core/tdvp_algorithm_engine.hpp:208-501
//   * Euler tour ......... include/ttns_lib/tdvp_core/tdvp_tree_traversal.hpp:38-87
//   * node / bond exps ... include/ttns_lib/tdvp_core/projector_splitting_engine.hpp:117-165
//   * H_eff actions ...... include/ttns_lib/tdvp_core/projector_splitting_evolution_functions.hpp:6-258
//   * mode contraction ... include/ttns_lib/tdvp_core/kronecker_product_operator_helper.hpp:212-315
//   * bottom-up env ...... include/ttns_lib/tdvp_core/single_particle_operator.hpp:26-103
//   * top-down env ....... include/ttns_lib/tdvp_core/mean_field_operator.hpp:37-184
//   * gauge moves ........ include/ttns_lib/tdvp_core/root_to_leaf_decomposition.hpp:113-233,
//                          include/ttns_lib/tdvp_core/leaf_to_root_decomposition.hpp:57-138
//   * term compression ... include/ttns_lib/tdvp_core/operator_container.hpp:43-664,
//                          include/ttns_lib/tdvp_core/operator_compression.hpp:373-489
//   * first-step schedule  include/ttns_lib/integrators/projector_splitting_integrator.hpp:136-169
//   * <O> on one mode .... include/ttns_lib/observables/matrix_element.hpp:264-314
//   * adjoint sweep ...... ttn_adjoint.hpp (no counterpart in the reference: the reverse
//                          of the sweep above, checked against finite differences)
//
// Two definitions are ours because the reference's versions live in the absent
// submodules:
//   * gauge moves use Householder QR with LAPACK zlarfg conventions (the reference
//     calls zgesvd); the sweep is gauge covariant and, for exactly rank-deficient
//     tensors, both complete the basis with the same Householder columns;
//   * the Krylov exponential is the Lanczos form of Sidje's Expokit (ACM TOMS 24,
//     1998: corrected Krylov approximation, local error estimate from the
//     augmented matrix, step-size control with gamma=0.9, delta=1.2) with full
//     re-orthogonalisation and an implicit-QL eigen-solve of the tridiagonal.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cd;

namespace orc {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
enum { OK = 0, EINVAL_ = 1, ECAP = 2, ENUM = 3 };
// operations of a sweep, as reported to Engine::on_op
enum { OP_AFP = 1, OP_R2L, OP_MF, OP_NODE, OP_L2R, OP_SPF, OP_BOND, OP_ATP };

#define ORC_REQUIRE(cond, msg) \
  do { if (!(cond)) throw ::orc::Error(::orc::EINVAL_, msg); } while (0)

// ---------------------------------------------------------------- small dense helpers
static inline cd cmul(cd a, cd b) {
  return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}
static inline cd cmulc(cd a, cd b) {  // conj(a) * b
  return cd(a.real() * b.real() + a.imag() * b.imag(), a.real() * b.imag() - a.imag() * b.real());
}

// out(a,i,b) = sum_j S(i,j) in(a,j,b); shapes (na, d, nb); S is d x d row-major.
static void mode_apply(const cd* S, int d, const cd* in, cd* out, size_t na, size_t nb) {
#pragma omp parallel for schedule(static) if (na * d * nb > 65536)
  for (long long a = 0; a < (long long)na; ++a) {
    for (int i = 0; i < d; ++i) {
      cd* o = out + ((size_t)a * d + i) * nb;
      for (size_t b = 0; b < nb; ++b) o[b] = 0.0;
      for (int j = 0; j < d; ++j) {
        cd s = S[(size_t)i * d + j];
        const cd* x = in + ((size_t)a * d + j) * nb;
        for (size_t b = 0; b < nb; ++b) o[b] += cmul(s, x[b]);
      }
    }
  }
}

// out(x,k) (+)= alpha * sum_l in(x,l) M(k,l)  -- in * M^T on the trailing (rank) index.
static void mf_apply(const cd* in, const cd* M, int r, size_t nx, cd* out, cd alpha, bool accumulate) {
#pragma omp parallel for schedule(static) if (nx * r * r > 65536)
  for (long long x = 0; x < (long long)nx; ++x) {
    const cd* v = in + (size_t)x * r;
    cd* o = out + (size_t)x * r;
    for (int k = 0; k < r; ++k) {
      cd s = 0.0;
      for (int l = 0; l < r; ++l) s += cmul(v[l], M[(size_t)k * r + l]);
      if (accumulate) o[k] += cmul(alpha, s); else o[k] = cmul(alpha, s);
    }
  }
}

// out(i,j) (+)= alpha * sum_x conj(A(x,i)) X(x,j); A, X are (nx, r).
static void adj_mul(const cd* A, const cd* X, size_t nx, int r, cd* out, cd alpha, bool accumulate) {
#pragma omp parallel for schedule(static) if (nx * r * r > 65536)
  for (int ij = 0; ij < r * r; ++ij) {
    int i = ij / r, j = ij % r;
    cd s = 0.0;
    for (size_t x = 0; x < nx; ++x) s += cmulc(A[x * r + i], X[x * r + j]);
    if (accumulate) out[ij] += cmul(alpha, s); else out[ij] = cmul(alpha, s);
  }
}

// out(i,j) (+)= alpha * sum_{a,b} conj(A(a,i,b)) T(a,j,b); shapes (na, d, nb).
static void mode_contract(const cd* A, const cd* T, size_t na, int d, size_t nb, cd* out, cd alpha, bool accumulate) {
#pragma omp parallel for schedule(static) if (na * d * d * nb > 65536)
  for (int ij = 0; ij < d * d; ++ij) {
    int i = ij / d, j = ij % d;
    cd s = 0.0;
    for (size_t a = 0; a < na; ++a) {
      const cd* x = A + (a * d + i) * nb;
      const cd* y = T + (a * d + j) * nb;
      for (size_t b = 0; b < nb; ++b) s += cmulc(x[b], y[b]);
    }
    if (accumulate) out[ij] += cmul(alpha, s); else out[ij] = cmul(alpha, s);
  }
}

// C (n x p) = A (n x q) * B (q x p)
static void matmul(const cd* A, const cd* B, int n, int q, int p, cd* C) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < p; ++j) {
      cd s = 0.0;
      for (int k = 0; k < q; ++k) s += cmul(A[(size_t)i * q + k], B[(size_t)k * p + j]);
      C[(size_t)i * p + j] = s;
    }
}

// ---------------------------------------------------------------- tree
// Pre-order numbered tree; children of a node are ordered by id (the reference's
// tree<T> keeps nodes contiguously in pre-order, include/ttns_lib/tree/tree.hpp:187-192).
struct Tree {
  int n = 0;
  std::vector<int> parent, slot, hrank, leaf_mode, leaf_dim, nmodes;
  std::vector<std::vector<int>> children, dims;
  std::vector<size_t> dimen;
  std::vector<int> traversal;          // Euler tour (tdvp_tree_traversal.hpp:38-87)
  std::vector<int> mode_node, mode_pos, lo, hi, sub_end;
  int nleaves = 0;

  void build(int nn, const int* par, const int* hr, const int* lm, const int* ld) {
    ORC_REQUIRE(nn >= 1, "tree needs at least one node");
    n = nn;
    parent.assign(par, par + n); hrank.assign(hr, hr + n);
    leaf_mode.assign(lm, lm + n); leaf_dim.assign(ld, ld + n);
    ORC_REQUIRE(parent[0] == -1, "node 0 must be the root (parent -1)");
    children.assign(n, {}); slot.assign(n, -1);
    for (int i = 1; i < n; ++i) {
      ORC_REQUIRE(parent[i] >= 0 && parent[i] < i, "nodes must be numbered in pre-order (parent[i] < i)");
      slot[i] = (int)children[parent[i]].size();
      children[parent[i]].push_back(i);
    }
    sub_end.assign(n, 0);
    for (int i = n - 1; i >= 0; --i) {
      sub_end[i] = i + 1;
      for (int c : children[i]) sub_end[i] = std::max(sub_end[i], sub_end[c]);
    }
    for (int i = 0; i < n; ++i)
      for (int c : children[i]) ORC_REQUIRE(c < sub_end[i], "pre-order violated");
    dims.assign(n, {}); dimen.assign(n, 1); nmodes.assign(n, 0);
    nleaves = 0;
    for (int i = 0; i < n; ++i) {
      ORC_REQUIRE(hrank[i] >= 1, "hrank must be >= 1");
      if (children[i].empty()) {
        ORC_REQUIRE(leaf_mode[i] >= 0 && leaf_dim[i] >= 1, "leaf nodes need a mode index and a physical dimension");
        dims[i] = {leaf_dim[i]}; nmodes[i] = 1; ++nleaves;
      } else {
        ORC_REQUIRE(leaf_mode[i] < 0, "branch nodes must have leaf_mode -1");
        for (int c : children[i]) dims[i].push_back(hrank[c]);
        nmodes[i] = (int)children[i].size();
      }
      for (int d : dims[i]) dimen[i] *= (size_t)d;
      ORC_REQUIRE((size_t)hrank[i] <= dimen[i], "hrank exceeds the product of child dimensions (sanitise_tree cap)");
    }
    mode_node.assign(nleaves, -1); mode_pos.assign(nleaves, -1);
    int pos = 0;
    for (int i = 0; i < n; ++i)
      if (children[i].empty()) {
        int m = leaf_mode[i];
        ORC_REQUIRE(m < nleaves && mode_node[m] < 0, "leaf mode indices must be a permutation of 0..nleaves-1");
        mode_node[m] = i; mode_pos[m] = pos++;
      }
    lo.assign(n, 0); hi.assign(n, 0);
    for (int i = n - 1; i >= 0; --i) {
      if (children[i].empty()) { lo[i] = mode_pos[leaf_mode[i]]; hi[i] = lo[i] + 1; }
      else { lo[i] = lo[children[i].front()]; hi[i] = hi[children[i].back()]; }
    }
    // r2l decompositions need the permuted matrix to be tall (d1 >= d2).
    for (int i = 0; i < n; ++i)
      if (!children[i].empty())
        for (int m = 0; m < nmodes[i]; ++m) {
          size_t d2 = dims[i][m], d1 = dimen[i] * hrank[i] / d2;
          ORC_REQUIRE(d1 >= d2, "root-to-leaf matricisation is wide; unsupported tree");
        }
    // Euler tour.
    size_t nsites = 0;
    for (int i = 0; i < n; ++i) nsites += children[i].empty() ? 2 : 1 + children[i].size();
    traversal.resize(nsites);
    std::vector<int> tv(n, 0);
    int cur = 0;
    for (size_t k = 0; k < nsites; ++k) {
      traversal[k] = cur;
      int t = tv[cur];
      int nxt = cur;
      if (t == 0 && children[cur].empty()) nxt = cur;
      else if (t < (int)children[cur].size()) nxt = children[cur][t];
      else if (cur != 0) nxt = parent[cur];
      tv[cur]++;
      cur = nxt;
    }
  }
  size_t size(int i) const { return dimen[i] * (size_t)hrank[i]; }
  bool leaf(int i) const { return children[i].empty(); }
};

// ---------------------------------------------------------------- SOP operator
// H = sum_r c_r prod_nu O_{r,nu}; sop_operator.hpp:234-520, bind :323-392.
struct SOP {
  int nterms = 0, nmodes = 0;
  std::vector<cd> coeff;
  std::vector<int> mode_dim;
  std::vector<std::vector<std::vector<cd>>> ops;  // ops[mode][k] dense d x d
  std::vector<std::vector<int>> opidx;            // opidx[mode][r] = k or -1
  std::vector<std::pair<int, int>> op_order;      // (mode, k) of each operator in creation order
};

// ---------------------------------------------------------------- compiled operator plan
// Terms at a node are partitioned as in operator_container.hpp:426-444 / 648-664:
//   S ("common spf"): terms whose operator below the node is identical (>=2 members);
//   M ("common mf"):  remaining terms sharing the operator outside the node (>=2);
//   1 ("standard"):   the rest.
// S keeps the coefficients in its mean field, M in its single-particle operator,
// singletons apply c_r as a scalar.  Each c_r is applied exactly once.
enum { G_S = 0, G_M = 1, G_1 = 2 };
struct Item { int slot; int grp; };
// a_mem / b_mem: the terms whose coefficients were summed into a / b (empty when the
// scalar is the constant 1); the adjoint sweep maps scalar cotangents back through them.
struct SpfTuple { cd a; std::vector<Item> items; std::vector<int> a_mem; };
struct MfKey { cd b; int pg; std::vector<Item> sib; std::vector<int> b_mem; };
struct Group {
  int type = G_1;
  std::vector<int> members;
  bool id_spf = false, id_mf = false;
  cd s = 1.0;
  std::vector<SpfTuple> spf;
  std::vector<MfKey> mf;
};
struct Plan {
  std::vector<std::vector<Group>> groups;   // per node
  std::vector<std::vector<int>> group_of;   // [node][r]
};

typedef std::vector<std::pair<int, int>> Sig;

static void compile_plan(const Tree& T, const SOP& H, Plan& P) {
  const int n = T.n, R = H.nterms;
  // support of each term, ordered by leaf position
  std::vector<std::vector<std::pair<int, std::pair<int, int>>>> sup(R);  // (pos, (mode, opk))
  for (int m = 0; m < H.nmodes; ++m)
    for (int r = 0; r < R; ++r)
      if (H.opidx[m][r] >= 0) sup[r].push_back({T.mode_pos[m], {m, H.opidx[m][r]}});
  for (auto& s : sup) std::sort(s.begin(), s.end());

  P.groups.assign(n, {});
  P.group_of.assign(n, std::vector<int>(R, -1));
  for (int nd = 0; nd < n; ++nd) {
    std::vector<Sig> Ls(R), Rs(R);
    for (int r = 0; r < R; ++r)
      for (auto& e : sup[r]) {
        if (e.first >= T.lo[nd] && e.first < T.hi[nd]) Ls[r].push_back(e.second);
        else Rs[r].push_back(e.second);
      }
    std::map<Sig, std::vector<int>> lcls;
    for (int r = 0; r < R; ++r) lcls[Ls[r]].push_back(r);
    std::vector<char> isS(R, 0);
    std::vector<std::vector<int>> sgroups, mgroups, singles;
    for (auto& kv : lcls)
      if (kv.second.size() >= 2) { sgroups.push_back(kv.second); for (int r : kv.second) isS[r] = 1; }
    std::map<Sig, std::vector<int>> rcls;
    for (int r = 0; r < R; ++r) if (!isS[r]) rcls[Rs[r]].push_back(r);
    for (auto& kv : rcls) {
      if (kv.second.size() >= 2) mgroups.push_back(kv.second);
      else singles.push_back(kv.second);
    }
    auto by_first = [](const std::vector<int>& a, const std::vector<int>& b) { return a[0] < b[0]; };
    std::sort(sgroups.begin(), sgroups.end(), by_first);
    std::sort(mgroups.begin(), mgroups.end(), by_first);
    std::sort(singles.begin(), singles.end(), by_first);
    auto& G = P.groups[nd];
    auto add = [&](const std::vector<int>& mem, int type) {
      Group g; g.type = type; g.members = mem;
      // the identity below the node only if every member is: an M group may mix a term that
      // acts below with one that does not (the latter contributes its coefficient times I)
      g.id_spf = true;
      for (int r : mem) g.id_spf = g.id_spf && Ls[r].empty();
      g.s = (type == G_1) ? H.coeff[mem[0]] : cd(1.0);
      for (int r : mem) P.group_of[nd][r] = (int)G.size();
      G.push_back(g);
    };
    for (auto& v : sgroups) add(v, G_S);
    for (auto& v : mgroups) add(v, G_M);
    for (auto& v : singles) add(v, G_1);
  }
  // single-particle tuples (bottom-up structure)
  for (int nd = 0; nd < n; ++nd) {
    for (auto& g : P.groups[nd]) {
      if (g.id_spf) continue;
      std::map<std::vector<int>, std::vector<int>> keys;  // key -> members
      for (int r : g.members) {
        std::vector<int> key;
        // at a leaf the key is the term's operator there; a member that is the identity on
        // the leaf (possible in an M group) has an empty key, i.e. a tuple without items
        if (T.leaf(nd)) {
          if (H.opidx[T.leaf_mode[nd]][r] >= 0) key.push_back(H.opidx[T.leaf_mode[nd]][r]);
        }
        else
          for (int s = 0; s < (int)T.children[nd].size(); ++s) {
            int c = T.children[nd][s];
            int cg = P.group_of[c][r];
            if (!P.groups[c][cg].id_spf) { key.push_back(s); key.push_back(cg); }
          }
        keys[key].push_back(r);
      }
      // order tuples by their smallest member for a fixed summation order
      std::vector<std::pair<int, std::vector<int>>> ord;
      for (auto& kv : keys) ord.push_back({kv.second[0], kv.first});
      std::sort(ord.begin(), ord.end());
      for (auto& o : ord) {
        const auto& key = o.second;
        const auto& mem = keys[key];
        SpfTuple t;
        bool carrying = false;
        if (T.leaf(nd)) {
          if (!key.empty()) t.items.push_back({-1, key[0]});
        }
        else
          for (size_t q = 0; q < key.size(); q += 2) {
            int c = T.children[nd][key[q]];
            t.items.push_back({key[q], key[q + 1]});
            if (P.groups[c][key[q + 1]].type == G_M) {
              carrying = true;
              if (P.groups[c][key[q + 1]].members != mem)
                throw Error(EINVAL_, "operator compression invariant violated (spf carrying group)");
            }
          }
        if (g.type == G_M && !carrying) { cd a = 0.0; for (int r : mem) a += H.coeff[r]; t.a = a; t.a_mem = mem; }
        else t.a = 1.0;
        g.spf.push_back(t);
      }
      if (g.type != G_M && g.spf.size() != 1)
        throw Error(EINVAL_, "operator compression invariant violated (non-M group with several tuples)");
    }
  }
  // mean-field keys (top-down structure)
  for (int nd = 0; nd < n; ++nd) {
    if (nd == 0) {
      for (auto& g : P.groups[nd]) g.id_mf = (g.type != G_S);
      continue;
    }
    int p = T.parent[nd];
    for (auto& g : P.groups[nd]) {
      std::map<std::vector<int>, std::vector<int>> keys;
      for (int r : g.members) {
        std::vector<int> key{P.group_of[p][r]};
        for (int s = 0; s < (int)T.children[p].size(); ++s) {
          int c = T.children[p][s];
          if (c == nd) continue;
          int cg = P.group_of[c][r];
          if (!P.groups[c][cg].id_spf) { key.push_back(s); key.push_back(cg); }
        }
        keys[key].push_back(r);
      }
      std::vector<std::pair<int, std::vector<int>>> ord;
      for (auto& kv : keys) ord.push_back({kv.second[0], kv.first});
      std::sort(ord.begin(), ord.end());
      for (auto& o : ord) {
        const auto& key = o.second;
        const auto& mem = keys[key];
        MfKey k; k.pg = key[0];
        const Group& pg = P.groups[p][k.pg];
        bool carrying = (pg.type == G_S);
        const std::vector<int>* carrier = carrying ? &pg.members : nullptr;
        for (size_t q = 1; q < key.size(); q += 2) {
          int c = T.children[p][key[q]];
          k.sib.push_back({key[q], key[q + 1]});
          if (P.groups[c][key[q + 1]].type == G_M) { carrying = true; carrier = &P.groups[c][key[q + 1]].members; }
        }
        if (g.type != G_S && carrying)
          throw Error(EINVAL_, "operator compression invariant violated (mf carrying component)");
        if (carrying && *carrier != mem)
          throw Error(EINVAL_, "operator compression invariant violated (mf carrier members)");
        if (g.type == G_S && !carrying) { cd b = 0.0; for (int r : mem) b += H.coeff[r]; k.b = b; k.b_mem = mem; }
        else k.b = 1.0;
        g.mf.push_back(k);
      }
      g.id_mf = (g.mf.size() == 1 && g.mf[0].b == cd(1.0) && g.mf[0].sib.empty() &&
                 P.groups[p][g.mf[0].pg].id_mf);
    }
  }
}

// ---------------------------------------------------------------- Householder QR
// LAPACK zlarfg conventions: H = I - tau v v^H, v(0) = 1, H^H (alpha, x) = (beta, 0),
// beta real with sign opposite to Re(alpha); tau = 0 when x == 0 and Im(alpha) == 0.
// Scaled 2-norm of a strided complex column (no intermediate underflow / overflow).
static double scaled_norm(const cd* x, size_t cnt, size_t stride) {
  double amax = 0.0;
  for (size_t i = 0; i < cnt; ++i)
    amax = std::max(amax, std::max(std::fabs(x[i * stride].real()), std::fabs(x[i * stride].imag())));
  if (amax == 0.0) return 0.0;
  double s = 0.0;
  for (size_t i = 0; i < cnt; ++i) {
    double a = x[i * stride].real() / amax, b = x[i * stride].imag() / amax;
    s += a * a + b * b;
  }
  return amax * std::sqrt(s);
}
// sqrt(x^2 + y^2 + z^2) without destructive underflow or overflow (LAPACK dlapy3 scheme)
static double lapy3(double x, double y, double z) {
  double w = std::max(std::fabs(x), std::max(std::fabs(y), std::fabs(z)));
  if (w == 0.0) return 0.0;
  double a = x / w, b = y / w, c = z / w;
  return w * std::sqrt(a * a + b * b + c * c);
}

static void householder_qr(cd* M, size_t m, int n, cd* R, std::vector<cd>& tau) {
  const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;
  tau.assign(n, 0.0);
  for (int j = 0; j < n; ++j) {
    cd alpha = M[(size_t)j * n + j];
    cd* x = M + (size_t)(j + 1) * n + j;
    const size_t cnt = m - j - 1;
    double xnorm = scaled_norm(x, cnt, n);
    double ar = alpha.real(), ai = alpha.imag();
    cd beta;
    if (xnorm == 0.0 && ai == 0.0) {
      tau[j] = 0.0; beta = alpha;
    } else {
      double b = -std::copysign(lapy3(ar, ai, xnorm), ar >= 0.0 ? 1.0 : -1.0);
      int knt = 0;
      if (std::fabs(b) < safmin) {
        // rescale tiny columns (zlarfg), at most 20 times
        const double rs = 1.0 / safmin;
        do {
          ++knt;
          for (size_t i = 0; i < cnt; ++i) x[i * n] *= rs;
          b *= rs; ar *= rs; ai *= rs;
        } while (std::fabs(b) < safmin && knt < 20);
        xnorm = scaled_norm(x, cnt, n);
        b = -std::copysign(lapy3(ar, ai, xnorm), ar >= 0.0 ? 1.0 : -1.0);
      }
      tau[j] = cd((b - ar) / b, -ai / b);
      cd scal = 1.0 / (cd(ar, ai) - cd(b, 0.0));
      for (size_t i = 0; i < cnt; ++i) x[i * n] = cmul(x[i * n], scal);
      for (int q = 0; q < knt; ++q) b *= safmin;
      beta = cd(b, 0.0);
    }
    M[(size_t)j * n + j] = beta;
    if (tau[j] != cd(0.0)) {
      cd ct = std::conj(tau[j]);
#pragma omp parallel for schedule(static) if ((m - j) * (n - j) > 65536)
      for (int c = j + 1; c < n; ++c) {
        cd w = M[(size_t)j * n + c];
        for (size_t i = j + 1; i < m; ++i) w += cmulc(M[i * n + j], M[i * n + c]);
        cd f = cmul(ct, w);
        M[(size_t)j * n + c] -= f;
        for (size_t i = j + 1; i < m; ++i) M[i * n + c] -= cmul(M[i * n + j], f);
      }
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) R[(size_t)i * n + j] = (j >= i) ? M[(size_t)i * n + j] : cd(0.0);
  // form Q = H_0 ... H_{n-1} [I; 0] in place (zung2r ordering)
  for (int i = n - 1; i >= 0; --i) {
    if (i < n - 1) {
      M[(size_t)i * n + i] = 1.0;
      if (tau[i] != cd(0.0)) {
#pragma omp parallel for schedule(static) if ((m - i) * (n - i) > 65536)
        for (int c = i + 1; c < n; ++c) {
          cd w = 0.0;
          for (size_t r = i; r < m; ++r) w += cmulc(M[r * n + i], M[r * n + c]);
          cd f = cmul(tau[i], w);
          for (size_t r = i; r < m; ++r) M[r * n + c] -= cmul(M[r * n + i], f);
        }
      }
    }
    for (size_t r = i + 1; r < m; ++r) M[r * n + i] = cmul(-tau[i], M[r * n + i]);
    M[(size_t)i * n + i] = cd(1.0) - tau[i];
    for (int r = 0; r < i; ++r) M[(size_t)r * n + i] = 0.0;
  }
}

// ---------------------------------------------------------------- symmetric tridiagonal eigensolver
// Implicit QL with Wilkinson-type shifts (the EISPACK tql2 scheme).  d: diagonal (n),
// e: sub-diagonal e[0..n-2]; on exit d holds eigenvalues and z (n x n, row-major) the
// eigenvectors as columns.
static void tql2(int n, double* d, const double* e_in, double* z) {
  std::vector<double> e(n, 0.0);
  for (int i = 0; i + 1 < n; ++i) e[i] = e_in[i];
  for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) z[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    for (;;) {
      for (m = l; m < n - 1; ++m) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-300 + 2.220446049250313e-16 * dd) break;
      }
      if (m == l) break;
      if (++iter > 60) {
        std::string msg = "tridiagonal eigensolver did not converge: n=" + std::to_string(n) + " l=" + std::to_string(l) + " d=";
        for (int q = 0; q < n; ++q) msg += std::to_string(d[q]) + ",";
        msg += " e=";
        for (int q = 0; q < n; ++q) { char b[64]; std::snprintf(b, 64, "%.3e,", e[q]); msg += b; }
        throw Error(ENUM, msg);
      }
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? std::fabs(r) : -std::fabs(r)));
      double s = 1.0, c = 1.0, p = 0.0;
      int i;
      bool underflow = false;
      for (i = m - 1; i >= l; --i) {
        double f = s * e[i], b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; underflow = true; break; }
        s = f / r; c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        for (int k = 0; k < n; ++k) {
          f = z[k * n + i + 1];
          z[k * n + i + 1] = s * z[k * n + i] + c * f;
          z[k * n + i] = c * z[k * n + i] - s * f;
        }
      }
      if (underflow) continue;
      d[l] -= p; e[l] = g; e[m] = 0.0;
    }
  }
}

// phi_1(x) = (e^x - 1)/x and phi_2(x) = (e^x - 1 - x)/x^2 for complex x.
static cd phi1(cd x) {
  if (std::abs(x) < 0.5) {
    cd s = 0.0, t = 1.0;
    for (int k = 1; k <= 18; ++k) { s += t; t = t * x / double(k + 1); }
    return s;
  }
  return (std::exp(x) - 1.0) / x;
}
static cd phi2(cd x) {
  if (std::abs(x) < 0.5) {
    cd s = 0.0, t = 0.5;
    for (int k = 2; k <= 20; ++k) { s += t; t = t * x / double(k + 1); }
    return s;
  }
  return (std::exp(x) - 1.0 - x) / (x * x);
}

// ---------------------------------------------------------------- the engine
struct Engine {
  Tree T;
  SOP H;
  Plan P;
  int krylov_dim = 12;
  double krylov_tol = 1e-12;
  // 1: stop the Lanczos recurrence of a sub-step once the residual estimate of the space
  // built so far, for the whole remaining interval, is below krylov_tol (the rule the
  // reference's work counter shows); 0: always the full space with Expokit's step control
  int krylov_stop = 0;
  std::vector<std::vector<cd>> A;                       // node tensors (dimen x hrank)
  std::vector<std::vector<std::vector<cd>>> spf, mf;    // [node][group] r x r
  std::vector<std::vector<cd>> rmat;                    // R tensor per node
  double dt = 0.0, t_engine = 0.0;
  cd coeff = cd(0.0, -1.0);
  long long nsteps = 0, nh = 0;
  std::vector<cd> w1, w2, w3, w4;                       // work buffers (max node size)
  std::vector<std::vector<cd>> V;                       // Krylov basis
  std::vector<double> node_time;                        // seconds spent per node in sweeps
  // Called before every operation of a sweep (kind OP_*, node, auxiliary index) while
  // set; the adjoint sweep uses it to record the operations' inputs.
  std::function<void(int, int, int)> on_op;
  // Subspace expansion hooks (ttn_expansion.hpp): called after the root-to-leaf
  // decomposition towards a child in the forward half-sweep, and after a node's
  // leaf-to-root decomposition in the backward half-sweep; `expanded` records growth.
  std::function<bool(int)> expand_down, expand_up;
  // optional update of the primitive operators of a leaf's mode before its evolution
  // (mode, index within the mode, t, dt/2, matrix in place)
  std::function<void(int, int, double, double, cd*)> op_update;
  bool expanded = false;
  std::chrono::steady_clock::time_point tmark;
  void tick() { tmark = std::chrono::steady_clock::now(); }
  void tock(int id) {
    auto now = std::chrono::steady_clock::now();
    if ((int)node_time.size() < T.n) node_time.assign(T.n, 0.0);
    node_time[id] += std::chrono::duration<double>(now - tmark).count();
    tmark = now;
  }

  void init(const int* par, int nn, const int* hr, const int* lm, const int* ld) {
    T.build(nn, par, hr, lm, ld);
  }
  void finalize() {
    compile_plan(T, H, P);
    A.assign(T.n, {}); spf.assign(T.n, {}); mf.assign(T.n, {}); rmat.assign(T.n, {});
    size_t mx = 0;
    for (int i = 0; i < T.n; ++i) {
      A[i].assign(T.size(i), 0.0);
      mx = std::max(mx, T.size(i));
      int r = T.hrank[i];
      spf[i].assign(P.groups[i].size(), {});
      mf[i].assign(P.groups[i].size(), {});
      for (size_t g = 0; g < P.groups[i].size(); ++g) {
        const Group& G = P.groups[i][g];
        if (!G.id_spf) spf[i][g].assign((size_t)r * r, 0.0);
        if (!G.id_mf) {
          mf[i][g].assign((size_t)r * r, 0.0);
          if (i == 0) {  // root S group: (sum of coefficients) * identity
            cd sum = 0.0; for (int rr : G.members) sum += H.coeff[rr];
            for (int k = 0; k < r; ++k) mf[i][g][(size_t)k * r + k] = sum;
          }
        }
      }
      size_t rmx = (size_t)r;
      for (int d : T.dims[i]) rmx = std::max(rmx, (size_t)d);
      rmat[i].assign(rmx * rmx, 0.0);
    }
    w1.assign(mx, 0.0); w2.assign(mx, 0.0); w3.assign(mx, 0.0); w4.assign(mx, 0.0);
  }

  // rank-3 view of node nd on mode mu: (pre, d_mu, post*hrank)
  void r3(int nd, int mu, size_t& na, int& d, size_t& nb) const {
    na = 1; nb = T.hrank[nd];
    for (int i = 0; i < mu; ++i) na *= T.dims[nd][i];
    d = T.dims[nd][mu];
    for (int i = mu + 1; i < T.nmodes[nd]; ++i) nb *= T.dims[nd][i];
  }
  const std::vector<cd>& leaf_op(int nd, int k) const { return H.ops[T.leaf_mode[nd]][k]; }

  // X = (tensor-product of the items' operators) applied to v; items on distinct modes.
  // Uses two scratch buffers; returns pointer to the result (v itself if no items).
  const cd* apply_items(int nd, const std::vector<Item>& items, const cd* v, cd* b1, cd* b2) {
    const cd* cur = v;
    cd* nxt = b1;
    for (const Item& it : items) {
      size_t na, nb; int d;
      const cd* S;
      if (it.slot < 0) { S = leaf_op(nd, it.grp).data(); na = 1; d = T.dims[nd][0]; nb = T.hrank[nd]; }
      else { S = spf[T.children[nd][it.slot]][it.grp].data(); r3(nd, it.slot, na, d, nb); }
      mode_apply(S, d, cur, nxt, na, nb);
      cur = nxt;
      nxt = (nxt == b1) ? b2 : b1;
    }
    return cur;
  }

  // sibling version: operators from the siblings' spf applied to the parent tensor
  const cd* apply_sibs(int p, const std::vector<Item>& items, const cd* v, cd* b1, cd* b2) {
    const cd* cur = v;
    cd* nxt = b1;
    for (const Item& it : items) {
      size_t na, nb; int d;
      r3(p, it.slot, na, d, nb);
      mode_apply(spf[T.children[p][it.slot]][it.grp].data(), d, cur, nxt, na, nb);
      cur = nxt;
      nxt = (nxt == b1) ? b2 : b1;
    }
    return cur;
  }

  // ---- bottom-up environment (single_particle_operator.hpp:26-103)
  void update_spf(int nd) {
    if (on_op) on_op(OP_SPF, nd, 0);
    const size_t sz = T.size(nd);
    const int r = T.hrank[nd];
    for (size_t g = 0; g < P.groups[nd].size(); ++g) {
      const Group& G = P.groups[nd][g];
      if (G.id_spf) continue;
      bool first = true;
      for (const SpfTuple& t : G.spf) {
        const cd* X = apply_items(nd, t.items, A[nd].data(), w1.data(), w2.data());
        adj_mul(A[nd].data(), X, sz / r, r, spf[nd][g].data(), t.a, !first);
        first = false;
      }
    }
  }

  // ---- top-down environment for child nd (mean_field_operator.hpp:37-184)
  void update_mf(int nd) {
    if (nd == 0) return;
    if (on_op) on_op(OP_MF, nd, 0);
    const int p = T.parent[nd], mu = T.slot[nd];
    size_t na, nb; int d;
    r3(p, mu, na, d, nb);
    const int rp = T.hrank[p];
    const size_t szp = T.size(p);
    for (size_t g = 0; g < P.groups[nd].size(); ++g) {
      const Group& G = P.groups[nd][g];
      if (G.id_mf) continue;
      bool first = true;
      for (const MfKey& k : G.mf) {
        const cd* X = apply_sibs(p, k.sib, A[p].data(), w1.data(), w2.data());
        if (!P.groups[p][k.pg].id_mf) {
          cd* dst = (X == w1.data()) ? w2.data() : w1.data();
          mf_apply(X, mf[p][k.pg].data(), rp, szp / rp, dst, 1.0, false);
          X = dst;
        }
        mode_contract(A[p].data(), X, na, d, nb, mf[nd][g].data(), k.b, !first);
        first = false;
      }
    }
  }

  // ---- effective Hamiltonian on a node tensor (coefficient_evolution_leaf / _branch)
  void heff(int nd, const cd* v, cd* out) {
    const size_t sz = T.size(nd);
    const int r = T.hrank[nd];
    std::fill(out, out + sz, cd(0.0));
    for (size_t g = 0; g < P.groups[nd].size(); ++g) {
      const Group& G = P.groups[nd][g];
      const cd* X;
      if (G.id_spf) X = v;
      else if (G.spf.size() == 1) {
        X = apply_items(nd, G.spf[0].items, v, w1.data(), w2.data());
        if (G.spf[0].a != cd(1.0)) {
          for (size_t i = 0; i < sz; ++i) w3[i] = cmul(G.spf[0].a, X[i]);
          X = w3.data();
        }
      } else {
        std::fill(w3.begin(), w3.begin() + sz, cd(0.0));
        for (const SpfTuple& t : G.spf) {
          const cd* Y = apply_items(nd, t.items, v, w1.data(), w2.data());
          for (size_t i = 0; i < sz; ++i) w3[i] += cmul(t.a, Y[i]);
        }
        X = w3.data();
      }
      if (G.id_mf) { for (size_t i = 0; i < sz; ++i) out[i] += cmul(G.s, X[i]); }
      else mf_apply(X, mf[nd][g].data(), r, sz / r, out, G.s, true);
    }
  }

  // ---- bond Hamiltonian on R (full_hamiltonian_action)
  void kbond(int nd, const cd* R, cd* out) {
    const int r = T.hrank[nd];
    const size_t rr = (size_t)r * r;
    std::vector<cd> t1(rr), t2(rr);
    std::fill(out, out + rr, cd(0.0));
    for (size_t g = 0; g < P.groups[nd].size(); ++g) {
      const Group& G = P.groups[nd][g];
      const cd* X = R;
      if (!G.id_spf) { matmul(spf[nd][g].data(), R, r, r, r, t1.data()); X = t1.data(); }
      if (G.id_mf) { for (size_t i = 0; i < rr; ++i) out[i] += cmul(G.s, X[i]); }
      else mf_apply(X, mf[nd][g].data(), r, r, out, G.s, true);
    }
  }

  // ---- Krylov exponential: y <- exp(coeff * tau * Hop) y  (Expokit-style, Lanczos)
  template <typename Op>
  long long expm(Op&& hop, cd* y, size_t n, double tau, cd cf) {
    const int m = krylov_dim;
    const double tol = krylov_tol, gamma = 0.9, delta = 1.2;
    const int mxreject = 10;
    if ((int)V.size() < m + 1) V.resize(m + 1);
    for (auto& v : V) if (v.size() < n) v.resize(n);
    std::vector<cd> p(n);
    long long napps = 0;
    double t_out = std::fabs(tau), sgn = (tau >= 0.0) ? 1.0 : -1.0;
    double t_now = 0.0, t_new = t_out;
    double beta = 0.0;
    for (size_t i = 0; i < n; ++i) beta += std::norm(y[i]);
    beta = std::sqrt(beta);
    if (beta == 0.0 || t_out == 0.0) return 0;
    std::vector<double> alpha(m + 1), bet(m + 2);
    while (t_now < t_out) {
      double t_step = std::min(t_out - t_now, t_new);
      for (size_t i = 0; i < n; ++i) V[0][i] = y[i] / beta;
      int mb = m, k1 = 2;
      double anorm = 0.0, avnorm = 0.0;
      for (int j = 0; j < m; ++j) {
        hop(V[j].data(), p.data()); ++napps;
        double a = 0.0;
        for (size_t i = 0; i < n; ++i) a += (std::conj(V[j][i]) * p[i]).real();
        alpha[j] = a;
        for (size_t i = 0; i < n; ++i) {
          p[i] -= a * V[j][i];
          if (j > 0) p[i] -= bet[j] * V[j - 1][i];
        }
        // full re-orthogonalisation (one classical Gram-Schmidt pass)
        for (int q = 0; q <= j; ++q) {
          cd h = 0.0;
          for (size_t i = 0; i < n; ++i) h += cmulc(V[q][i], p[i]);
          for (size_t i = 0; i < n; ++i) p[i] -= cmul(h, V[q][i]);
        }
        double s = 0.0;
        for (size_t i = 0; i < n; ++i) s += std::norm(p[i]);
        s = std::sqrt(s);
        anorm = std::max(anorm, std::fabs(a) + bet[j] + s);
        bet[j + 1] = s;
        if (s <= 1e-14 * (1.0 + anorm)) { mb = j + 1; k1 = 0; t_step = t_out - t_now; break; }
        for (size_t i = 0; i < n; ++i) V[j + 1][i] = p[i] / s;
        if (krylov_stop && j + 1 < m) {
          // residual estimate beta * beta_{j+1} * |e_j^T exp(c tau T_{j+1}) e_1| for the
          // remaining interval tau, with the (j+1)-dimensional tridiagonal
          const int jj = j + 1;
          std::vector<double> dd(alpha.begin(), alpha.begin() + jj), ee(std::max(jj - 1, 1)), zz((size_t)jj * jj);
          for (int i = 0; i + 1 < jj; ++i) ee[i] = bet[i + 1];
          tql2(jj, dd.data(), ee.data(), zz.data());
          const double rest = t_out - t_now;
          const cd zc = cf * (sgn * rest);
          cd last = 0.0;
          for (int q = 0; q < jj; ++q) last += zz[(jj - 1) * jj + q] * std::exp(zc * dd[q]) * zz[q];
          if (beta * s * std::abs(last) <= tol) { mb = jj; k1 = 0; t_step = rest; break; }
        }
      }
      if (k1 != 0) {
        hop(V[m].data(), p.data()); ++napps;
        double s = 0.0;
        for (size_t i = 0; i < n; ++i) s += std::norm(p[i]);
        avnorm = std::sqrt(s);
      }
      // eigen-decomposition of the mb x mb tridiagonal
      std::vector<double> d(alpha.begin(), alpha.begin() + mb), e(std::max(mb - 1, 1)), z((size_t)mb * mb);
      for (int i = 0; i + 1 < mb; ++i) e[i] = bet[i + 1];
      tql2(mb, d.data(), e.data(), z.data());
      std::vector<cd> F(mb + 2);
      double err_loc = 0.0, xm = 1.0 / m;
      int ireject = 0;
      for (;;) {
        cd zc = cf * (sgn * t_step);
        for (int i = 0; i < mb; ++i) {
          cd s = 0.0;
          for (int q = 0; q < mb; ++q) s += z[i * mb + q] * std::exp(zc * d[q]) * z[q];
          F[i] = s;
        }
        if (k1 == 0) { err_loc = 1e-14; break; }
        cd f1 = 0.0, f2 = 0.0;
        for (int q = 0; q < mb; ++q) {
          cd x = zc * d[q];
          f1 += z[(mb - 1) * mb + q] * zc * phi1(x) * z[q];
          f2 += z[(mb - 1) * mb + q] * zc * zc * phi2(x) * z[q];
        }
        F[mb] = bet[mb] * f1;
        F[mb + 1] = bet[mb] * f2;
        double p1 = std::abs(F[mb]) * beta, p2 = std::abs(F[mb + 1]) * beta * avnorm;
        if (p1 > 10.0 * p2) { err_loc = p2; xm = 1.0 / m; }
        else if (p1 > p2) { err_loc = p1 * p2 / (p1 - p2); xm = 1.0 / m; }
        else { err_loc = p1; xm = 1.0 / (m - 1); }
        if (err_loc <= delta * t_step * tol) break;
        if (ireject == mxreject) throw Error(ENUM, "Krylov exponential: requested tolerance not reachable");
        t_step = gamma * t_step * std::pow(t_step * tol / err_loc, xm);
        double sc = std::pow(10.0, std::floor(std::log10(t_step)) - 1.0);
        t_step = std::ceil(t_step / sc) * sc;
        ++ireject;
      }
      const int mx = mb + std::max(0, k1 - 1);
      for (size_t i = 0; i < n; ++i) {
        cd s = 0.0;
        for (int q = 0; q < mx; ++q) s += cmul(F[q], V[q][i]);
        y[i] = beta * s;
      }
      beta = 0.0;
      for (size_t i = 0; i < n; ++i) beta += std::norm(y[i]);
      beta = std::sqrt(beta);
      t_now += t_step;
      if (k1 != 0) {
        t_new = gamma * t_step * std::pow(t_step * tol / std::max(err_loc, 1e-300), xm);
        double sc = std::pow(10.0, std::floor(std::log10(t_new)) - 1.0);
        t_new = std::ceil(t_new / sc) * sc;
      }
      if (!std::isfinite(beta)) throw Error(ENUM, "Krylov exponential produced a non-finite vector");
      if (beta == 0.0) break;
    }
    return napps;
  }

  // ---- gauge moves
  // leaf_to_root_decomposition.hpp:57-101: A = Q R, A <- Q, rmat = R
  void l2r(int nd) {
    if (on_op) on_op(OP_L2R, nd, 0);
    const size_t m = T.dimen[nd];
    const int r = T.hrank[nd];
    std::vector<cd> tau;
    householder_qr(A[nd].data(), m, r, rmat[nd].data(), tau);
  }
  // leaf_to_root_decomposition.hpp:105-138: parent mode <- R . parent
  void apply_to_parent(int nd) {
    if (on_op) on_op(OP_ATP, nd, 0);
    const int p = T.parent[nd], mu = T.slot[nd];
    size_t na, nb; int d;
    r3(p, mu, na, d, nb);
    mode_apply(rmat[nd].data(), d, A[p].data(), w4.data(), na, nb);
    std::copy(w4.begin(), w4.begin() + T.size(p), A[p].begin());
  }
  // root_to_leaf_decomposition.hpp:113-183: permute mode mu to the fastest index, QR,
  // store R^T so that the child applies A_c <- A_c R^T.
  void r2l(int nd, int mu) {
    if (on_op) on_op(OP_R2L, nd, mu);
    size_t pre = 1, post = (size_t)T.hrank[nd];
    for (int i = 0; i < mu; ++i) pre *= T.dims[nd][i];
    const int dm = T.dims[nd][mu];
    for (int i = mu + 1; i < T.nmodes[nd]; ++i) post *= T.dims[nd][i];
    const size_t d1 = pre * post;
    cd* M = w4.data();
    const cd* a = A[nd].data();
    for (size_t x = 0; x < pre; ++x)
      for (int i = 0; i < dm; ++i)
        for (size_t y = 0; y < post; ++y) M[(y * pre + x) * dm + i] = a[(x * dm + i) * post + y];
    std::vector<cd> R((size_t)dm * dm), tau;
    householder_qr(M, d1, dm, R.data(), tau);
    cd* an = A[nd].data();
    for (size_t x = 0; x < pre; ++x)
      for (int i = 0; i < dm; ++i)
        for (size_t y = 0; y < post; ++y) an[(x * dm + i) * post + y] = M[(y * pre + x) * dm + i];
    for (int i = 0; i < dm; ++i)
      for (int j = 0; j < dm; ++j) rmat[nd][(size_t)i * dm + j] = R[(size_t)j * dm + i];
  }
  // root_to_leaf_decomposition.hpp:208-233: A <- A . R_parent
  void apply_from_parent(int nd) {
    if (on_op) on_op(OP_AFP, nd, 0);
    const int p = T.parent[nd], r = T.hrank[nd];
    const size_t m = T.dimen[nd];
    matmul(A[nd].data(), rmat[p].data(), (int)m, r, r, w4.data());
    std::copy(w4.begin(), w4.begin() + T.size(nd), A[nd].begin());
  }

  // ---- node and bond evolution (projector_splitting_engine.hpp:117-165)
  void evolve_node(int nd) {
    if (on_op) on_op(OP_NODE, nd, 0);
    // time-dependent primitive operators: op.update(leaf, t, dt/2) before a leaf's
    // evolution (projector_splitting_engine.hpp:139)
    if (op_update && T.leaf(nd)) {
      const int mode = T.leaf_mode[nd];
      for (size_t k = 0; k < H.ops[mode].size(); ++k) op_update(mode, (int)k, t_engine, dt / 2.0, H.ops[mode][k].data());
    }
    nh += expm([&](const cd* v, cd* o) { heff(nd, v, o); }, A[nd].data(), T.size(nd), dt / 2.0, coeff);
  }
  // R: the bond matrix held in rmat[owner] (the node's own after l2r, its parent's after r2l)
  void evolve_bond(int nd, int owner) {
    if (on_op) on_op(OP_BOND, nd, owner);
    std::vector<cd>& R = rmat[owner];
    const size_t rr = (size_t)T.hrank[nd] * T.hrank[nd];
    std::vector<cd> tmp(R.begin(), R.begin() + rr);
    expm([&](const cd* v, cd* o) { kbond(nd, v, o); }, tmp.data(), rr, -dt / 2.0, coeff);
    std::copy(tmp.begin(), tmp.end(), R.begin());
  }

  // ---- optional finiteness checks after every operation (ORC_CHECK=1)
  bool checking = std::getenv("ORC_CHECK") != nullptr;
  void chk(const char* what, int id) {
    if (!checking) return;
    auto bad = [](const std::vector<cd>& v) {
      for (auto& z : v) if (!std::isfinite(z.real()) || !std::isfinite(z.imag())) return true;
      return false;
    };
    for (int i = 0; i < T.n; ++i) {
      if (bad(A[i])) throw Error(ENUM, std::string("non-finite tensor at node ") + std::to_string(i) + " after " + what + " on node " + std::to_string(id));
      if (bad(rmat[i])) throw Error(ENUM, std::string("non-finite R at node ") + std::to_string(i) + " after " + what + " on node " + std::to_string(id));
      for (auto& e : spf[i]) if (bad(e)) throw Error(ENUM, std::string("non-finite spf at node ") + std::to_string(i) + " after " + what + " on node " + std::to_string(id));
      for (auto& e : mf[i]) if (bad(e)) throw Error(ENUM, std::string("non-finite mf at node ") + std::to_string(i) + " after " + what + " on node " + std::to_string(id));
    }
  }

  // ---- half sweeps (tdvp_algorithm_engine.hpp:331-501)
  void forward(bool evolve) {
    std::vector<int> tv(T.n, 0);
    tick();
    for (int id : T.traversal) {
      int t = tv[id]++;
      struct Tk { Engine* e; int id; ~Tk() { e->tock(id); } } tk{this, id};
      if (t != T.nmodes[id]) {
        int mode = t;
        if (t == 0 && id != 0) { apply_from_parent(id); chk("apply_from_parent", id); }
        if (!T.leaf(id)) {
          r2l(id, mode); chk("r2l", id);
          if (expand_down) expanded = expand_down(T.children[id][mode]) || expanded;
          update_mf(T.children[id][mode]); chk("update_mf", id);
        }
      } else {
        if (evolve) { evolve_node(id); chk("evolve_node", id); }
        if (id != 0) {
          l2r(id); chk("l2r", id);
          update_spf(id); chk("update_spf", id);
          if (evolve) { evolve_bond(id, id); chk("evolve_bond", id); }
          apply_to_parent(id); chk("apply_to_parent", id);
        }
      }
    }
  }
  void backward(bool evolve) {
    std::vector<int> tv(T.n, 0);
    tick();
    for (auto it = T.traversal.rbegin(); it != T.traversal.rend(); ++it) {
      int id = *it;
      int t = tv[id]++;
      struct Tk { Engine* e; int id; ~Tk() { e->tock(id); } } tk{this, id};
      if (t != T.nmodes[id]) {
        int mode = T.nmodes[id] - (t + 1);
        if (t == 0) {
          if (id != 0) {
            if (evolve) evolve_bond(id, T.parent[id]);
            apply_from_parent(id);
          }
          if (evolve) evolve_node(id);
        }
        if (!T.leaf(id)) {
          r2l(id, mode);
          update_mf(T.children[id][mode]);
        }
      } else {
        if (id != 0) {
          l2r(id);
          if (expand_up) expanded = expand_up(id) || expanded;
          apply_to_parent(id);
          update_spf(id);
        }
      }
    }
  }
  void sweep() {
    forward(true);
    t_engine += dt / 2.0;
    backward(true);
    t_engine += dt / 2.0;
  }
  // tdvp_algorithm_base::prepare_evolution for the fixed-rank engine
  void prepare() {
    for (int id = T.n - 1; id >= 1; --id) update_spf(id);
    forward(false);
    backward(false);
  }
  // fixed_step_projector_splitting_integrator::operator() (projector_splitting_integrator.hpp:136-169)
  void step(double step_dt, cd cf) {
    coeff = cf;
    if (nsteps == 0) {
      double tevolve = 0.0, sdt = step_dt / 1e5;
      dt = (sdt + tevolve <= step_dt) ? sdt : step_dt - tevolve;
      prepare();
      while (tevolve < step_dt) {
        dt = (sdt + tevolve <= step_dt) ? sdt : step_dt - tevolve;
        t_engine = tevolve;
        sweep();
        tevolve += sdt;
        sdt *= 10.0;
      }
    } else {
      dt = step_dt;
      t_engine = nsteps * step_dt;
      sweep();
    }
    ++nsteps;
  }

  // ---- observables (matrix_element.hpp:264-314): leaf-to-root contraction
  cd expect(int mode, const cd* op) {
    std::vector<std::vector<cd>> mel(T.n);
    for (int id = T.n - 1; id >= 0; --id) {
      const int r = T.hrank[id];
      const size_t sz = T.size(id);
      mel[id].assign((size_t)r * r, 0.0);
      const cd* X = A[id].data();
      std::vector<cd> b1(sz), b2(sz);
      if (T.leaf(id)) {
        if (op && T.leaf_mode[id] == mode) {
          mode_apply(op, T.dims[id][0], A[id].data(), b1.data(), 1, r);
          X = b1.data();
        }
      } else {
        const cd* cur = A[id].data();
        cd* nxt = b1.data();
        for (int s = 0; s < T.nmodes[id]; ++s) {
          size_t na, nb; int d;
          r3(id, s, na, d, nb);
          mode_apply(mel[T.children[id][s]].data(), d, cur, nxt, na, nb);
          cur = nxt; nxt = (nxt == b1.data()) ? b2.data() : b1.data();
        }
        X = cur;
      }
      adj_mul(A[id].data(), X, sz / r, r, mel[id].data(), 1.0, false);
    }
    cd tr = 0.0;
    for (int k = 0; k < T.hrank[0]; ++k) tr += mel[0][(size_t)k * T.hrank[0] + k];
    return tr;
  }

  // Schmidt values across the bond above node nd; valid when every non-root node is an
  // isometry (the orthogonalised form the sweep leaves behind).
  std::vector<double> bond_sv(int nd) {
    std::vector<int> path;
    for (int x = nd; x != 0; x = T.parent[x]) path.push_back(x);
    std::reverse(path.begin(), path.end());
    int r0 = T.hrank[0];
    std::vector<cd> rho((size_t)r0 * r0, 0.0);
    for (int k = 0; k < r0; ++k) rho[(size_t)k * r0 + k] = 1.0;
    int prev = 0;
    for (int c : path) {
      int p = T.parent[c];
      size_t na, nb; int d;
      r3(p, T.slot[c], na, d, nb);
      const size_t sz = T.size(p);
      std::vector<cd> X(sz);
      mf_apply(A[p].data(), rho.data(), T.hrank[p], sz / T.hrank[p], X.data(), 1.0, false);
      std::vector<cd> nr((size_t)d * d);
      mode_contract(A[p].data(), X.data(), na, d, nb, nr.data(), 1.0, false);
      rho.swap(nr);
      prev = c;
    }
    (void)prev;
    // Hermitian Jacobi eigen-solve of rho (Schmidt values are sqrt of eigenvalues)
    int d = T.hrank[nd];
    std::vector<cd> a = rho;
    for (int sweepi = 0; sweepi < 100; ++sweepi) {
      double off = 0.0;
      for (int i = 0; i < d; ++i) for (int j = i + 1; j < d; ++j) off += std::norm(a[(size_t)i * d + j]);
      if (off < 1e-30) break;
      for (int p = 0; p < d; ++p)
        for (int q = p + 1; q < d; ++q) {
          cd apq = a[(size_t)p * d + q];
          double ab = std::abs(apq);
          if (ab < 1e-300) continue;
          double app = a[(size_t)p * d + p].real(), aqq = a[(size_t)q * d + q].real();
          double th = 0.5 * std::atan2(2.0 * ab, aqq - app);
          double c = std::cos(th), s = std::sin(th);
          cd ph = apq / ab;
          // rotation J with J_pp = c, J_qq = c, J_pq = s*ph, J_qp = -s*conj(ph); a <- J^H a J
          for (int k = 0; k < d; ++k) {
            cd akp = a[(size_t)k * d + p], akq = a[(size_t)k * d + q];
            a[(size_t)k * d + p] = c * akp - s * std::conj(ph) * akq;
            a[(size_t)k * d + q] = s * ph * akp + c * akq;
          }
          for (int k = 0; k < d; ++k) {
            cd apk = a[(size_t)p * d + k], aqk = a[(size_t)q * d + k];
            a[(size_t)p * d + k] = c * apk - s * ph * aqk;
            a[(size_t)q * d + k] = s * std::conj(ph) * apk + c * aqk;
          }
        }
    }
    std::vector<double> sv(d);
    for (int i = 0; i < d; ++i) sv[i] = std::sqrt(std::max(0.0, a[(size_t)i * d + i].real()));
    std::sort(sv.begin(), sv.end(), std::greater<double>());
    return sv;
  }

  // all environments from scratch for the current tensors (no gauge change)
  void refresh_env() {
    for (int id = T.n - 1; id >= 1; --id) update_spf(id);
    for (int id = 1; id < T.n; ++id) update_mf(id);
  }
  // orthogonaliser::operator() (include/ttns_lib/decompositions/orthogonaliser.hpp:83-112):
  // children before parents, every non-root node A = Q R, A <- Q and R into the parent's
  // slot, so that every non-root node is an isometry and the root holds the norm; the
  // single-particle environments follow the new gauge when the run has started
  void orthogonalise() {
    for (int id = T.n - 1; id >= 1; --id) {
      l2r(id);
      apply_to_parent(id);
    }
    if (nsteps > 0)
      for (int id = T.n - 1; id >= 1; --id) update_spf(id);
  }
};

#include "ttn_adjoint.hpp"
#include "ttn_expansion.hpp"

}  // namespace orc

// ---------------------------------------------------------------- C API (ctypes)
struct OrcHandle {
  orc::Engine E;
  std::string err;
  std::unique_ptr<orc::Expander> X;  // subspace expansion, when enabled
};

#define ORC_TRY(h, ...)                                   \
  try { __VA_ARGS__; return 0; }                                 \
  catch (const orc::Error& ex) { if (h) (h)->err = ex.what(); return ex.code; } \
  catch (const std::exception& ex) { if (h) (h)->err = ex.what(); return 1; }

extern "C" {

// Tree: pre-order parent array; leaf nodes carry (leaf_mode, leaf_dim), branch nodes -1.
// SOP: nterms coefficients (interleaved complex), nops dense operators (op_mode[k],
// op_data concatenated interleaved row-major d x d), each bound to the terms
// bind_r[bind_ptr[k]..bind_ptr[k+1]).
void* orc_create(int nnodes, const int* parent, const int* hrank, const int* leaf_mode, const int* leaf_dim,
                 int nterms, const double* coeff, int nops, const int* op_mode, const double* op_data,
                 const int* bind_ptr, const int* bind_r, int krylov_dim, double krylov_tol,
                 char* errbuf, int errlen) {
  OrcHandle* h = new OrcHandle();
  try {
    h->E.init(parent, nnodes, hrank, leaf_mode, leaf_dim);
    orc::SOP& H = h->E.H;
    H.nterms = nterms; H.nmodes = h->E.T.nleaves;
    H.coeff.resize(nterms);
    for (int r = 0; r < nterms; ++r) H.coeff[r] = cd(coeff[2 * r], coeff[2 * r + 1]);
    H.mode_dim.resize(H.nmodes);
    for (int m = 0; m < H.nmodes; ++m) H.mode_dim[m] = h->E.T.leaf_dim[h->E.T.mode_node[m]];
    H.ops.assign(H.nmodes, {});
    H.opidx.assign(H.nmodes, std::vector<int>(nterms, -1));
    size_t off = 0;
    for (int k = 0; k < nops; ++k) {
      int m = op_mode[k];
      ORC_REQUIRE(m >= 0 && m < H.nmodes, "operator mode out of range");
      int d = H.mode_dim[m];
      std::vector<cd> M((size_t)d * d);
      for (size_t i = 0; i < M.size(); ++i) M[i] = cd(op_data[2 * (off + i)], op_data[2 * (off + i) + 1]);
      off += M.size();
      int idx = (int)H.ops[m].size();
      H.ops[m].push_back(M);
      H.op_order.push_back({m, idx});
      for (int q = bind_ptr[k]; q < bind_ptr[k + 1]; ++q) {
        int r = bind_r[q];
        ORC_REQUIRE(r >= 0 && r < nterms, "bound term index out of range");
        ORC_REQUIRE(H.opidx[m][r] < 0, "term bound twice on the same mode");
        H.opidx[m][r] = idx;
      }
    }
    h->E.krylov_dim = krylov_dim;
    h->E.krylov_tol = krylov_tol;
    h->E.finalize();
    return h;
  } catch (const std::exception& ex) {
    if (errbuf && errlen > 0) { std::snprintf(errbuf, errlen, "%s", ex.what()); }
    delete h;
    return nullptr;
  }
}

void orc_destroy(void* p) { delete (OrcHandle*)p; }
const char* orc_error(void* p) { return ((OrcHandle*)p)->err.c_str(); }

long long orc_state_size(void* p) {
  OrcHandle* h = (OrcHandle*)p;
  long long s = 0;
  for (int i = 0; i < h->E.T.n; ++i) s += (long long)h->E.T.size(i);
  return s;
}
int orc_set_state(void* p, const double* data) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    size_t off = 0;
    for (int i = 0; i < h->E.T.n; ++i)
      for (auto& z : h->E.A[i]) { z = cd(data[2 * off], data[2 * off + 1]); ++off; }
  })
}
int orc_get_state(void* p, double* data) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    size_t off = 0;
    for (int i = 0; i < h->E.T.n; ++i)
      for (auto& z : h->E.A[i]) { data[2 * off] = z.real(); data[2 * off + 1] = z.imag(); ++off; }
  })
}
int orc_set_threads(void* p, int n) {
  (void)p;
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
  return 0;
}
int orc_step(void* p, double dt, double cre, double cim) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    if (h->X) h->X->step(dt, cd(cre, cim));
    else h->E.step(dt, cd(cre, cim));
  })
}
// Subspace expansion (ttn_expansion.hpp) for the following steps: bond capacities per node
// (cap[0] ignored; >= the current hrank), the reference's spawning / unoccupied thresholds,
// minimum number of unoccupied functions, eigenvalues per expansion, only-when-no-
// unoccupied flag and the random generator's seed.
int orc_set_expansion(void* p, const int* cap, double spawning, double unoccupied, int min_unocc, int neig, int only_when,
                      unsigned seed) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    orc::Engine& E = h->E;
    ORC_REQUIRE(E.nsteps == 0, "subspace expansion must be set before the first step");
    ORC_REQUIRE(neig >= 1 && min_unocc >= 0, "bad expansion parameters");
    h->X.reset(new orc::Expander(E));
    h->X->cap.assign(cap, cap + E.T.n);
    for (int i = 1; i < E.T.n; ++i) ORC_REQUIRE(h->X->cap[i] >= E.T.hrank[i], "capacity below the current bond dimension");
    h->X->spawning_threshold = spawning;
    h->X->unoccupied_threshold = unoccupied;
    h->X->minimum_unoccupied = min_unocc;
    h->X->neigenvalues = neig;
    h->X->only_when_no_unoccupied = only_when != 0;
    h->X->rng.seed(seed);
  })
}
// the k largest eigenpairs of a Hermitian g x g matrix (interleaved, row-major) as the
// subspace expansion computes them (dense Jacobi up to g = 96, Lanczos above)
int orc_top_eig(int g, int k, const double* G, double* vals, double* vecs) {
  try {
    std::vector<cd> A((size_t)g * g);
    for (size_t i = 0; i < A.size(); ++i) A[i] = cd(G[2 * i], G[2 * i + 1]);
    std::vector<double> w;
    std::vector<std::vector<cd>> V;
    orc::Expander::top_eig(A, (size_t)g, k, w, V);
    for (size_t j = 0; j < w.size(); ++j) {
      vals[j] = w[j];
      for (int i = 0; i < g; ++i) { vecs[2 * (j * g + i)] = V[j][i].real(); vecs[2 * (j * g + i) + 1] = V[j][i].imag(); }
    }
    return (int)w.size();
  } catch (...) { return -1; }
}
// Time-dependent primitive operators: fn(user, mode, op, t, dt, mat) is called before every
// leaf evolution for each operator bound on the leaf's mode (op = its binding index; mat
// the d x d matrix, interleaved, updated in place); fn = NULL removes the hook.
typedef void (*orc_op_update_fn)(void* user, int mode, int op, double t, double dt, double* mat);
int orc_set_op_update(void* p, orc_op_update_fn fn, void* user) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    orc::Engine& E = h->E;
    if (!fn) { E.op_update = nullptr; return 0; }
    std::vector<std::vector<int>> global(E.H.nmodes);
    for (int m = 0; m < E.H.nmodes; ++m) global[m].assign(E.H.ops[m].size(), -1);
    for (size_t g = 0; g < E.H.op_order.size(); ++g) global[E.H.op_order[g].first][E.H.op_order[g].second] = (int)g;
    E.op_update = [fn, user, global](int mode, int k, double t, double dt, cd* mat) {
      fn(user, mode, global[mode][k], t, dt, reinterpret_cast<double*>(mat));
    };
  })
}
// the current bond dimension above every node (hrank)
int orc_get_hrank(void* p, int* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, { for (int i = 0; i < h->E.T.n; ++i) out[i] = h->E.T.hrank[i]; })
}
// subspace expansion only (prepare_evolution without evolution); returns 1 if anything grew
int orc_expand_prepare(void* p, double dt, int* grew) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    ORC_REQUIRE(h->X != nullptr, "subspace expansion is not enabled");
    h->E.dt = dt;
    *grew = h->X->prepare() ? 1 : 0;
  })
}
// One plain sweep at the given dt (no first-step sub-stepping); used for bounded timing.
int orc_sweep(void* p, double dt, double cre, double cim) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, { h->E.coeff = cd(cre, cim); h->E.dt = dt; h->E.sweep(); })
}
// Per-node seconds accumulated over all sweeps so far (out: nnodes doubles).
int orc_node_times(void* p, double* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    for (int i = 0; i < h->E.T.n; ++i) out[i] = i < (int)h->E.node_time.size() ? h->E.node_time[i] : 0.0;
  })
}
int orc_reset_node_times(void* p) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, { h->E.node_time.assign(h->E.T.n, 0.0); })
}
int orc_prepare(void* p) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, { h->E.prepare(); })
}
double orc_t(void* p) { OrcHandle* h = (OrcHandle*)p; return h->E.nsteps * h->E.dt; }
long long orc_nh(void* p) { return ((OrcHandle*)p)->E.nh; }
int orc_set_krylov_stop(void* p, int mode) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    ORC_REQUIRE(mode == 0 || mode == 1, "Krylov stop rule: 0 (full space) or 1 (residual)");
    h->E.krylov_stop = mode;
  })
}
int orc_orthogonalise(void* p) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, { h->E.orthogonalise(); })
}
// one-site and two-site expansions so far (subspace_expansion_projector_splitting_engine
// Nonesite / Ntwosite, include/ttns_lib/tdvp_core/subspace_expansion_projector_splitting_
// engine.hpp:513-514); zero without expansion
int orc_expansion_counts(void* p, long long* onesite, long long* twosite) {
  OrcHandle* h = (OrcHandle*)p;
  *onesite = h->X ? h->X->n_onesite : 0;
  *twosite = h->X ? h->X->n_twosite : 0;
  return 0;
}
// The spin-boson driver's start state (src/spin_boson.cpp:584-649), in pre-order over the
// nodes with one std::mt19937(seed) stream: at a leaf, SPF 0 is psi0 (mode 0, when given)
// or the first basis state, and SPFs 1.. are random vectors -- per element a uniform phase
// in [0, 2 pi) then a standard-normal length, both distributions created afresh at every
// leaf -- normalised and Gram-Schmidt orthogonalised against the earlier SPFs, redrawn
// when the remainder is below 1e-12; interior nodes are identities and the root is e_0.
int orc_init_product(void* p, const double* psi0, unsigned seed) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    orc::Engine& E = h->E;
    std::mt19937 rng(seed);
    for (int i = 0; i < E.T.n; ++i) {
      const long long d = E.T.dimen[i];
      const int r = E.T.hrank[i];
      std::vector<cd>& A = E.A[i];
      std::fill(A.begin(), A.end(), cd(0.0));
      if (E.T.leaf(i)) {
        std::vector<std::vector<cd>> spf(r, std::vector<cd>(d, 0.0));
        if (E.T.leaf_mode[i] == 0 && psi0) {
          for (long long j = 0; j < d; ++j) spf[0][j] = cd(psi0[2 * j], psi0[2 * j + 1]);
        } else {
          spf[0][0] = 1.0;
        }
        std::uniform_real_distribution<double> phase(0, 2.0 * std::acos(-1.0));
        std::normal_distribution<double> length(0, 1);
        for (int k = 1; k < r; ++k) {
          for (;;) {
            for (long long j = 0; j < d; ++j) {
              const double th = phase(rng);
              spf[k][j] = length(rng) * cd(std::cos(th), std::sin(th));
            }
            cd n2 = 0.0;
            for (const cd& z : spf[k]) n2 += std::conj(z) * z;
            const cd sn = std::sqrt(n2);
            for (cd& z : spf[k]) z /= sn;
            for (int q = 0; q < k; ++q) {
              cd ov = 0.0;
              for (long long j = 0; j < d; ++j) ov += std::conj(spf[q][j]) * spf[k][j];
              for (long long j = 0; j < d; ++j) spf[k][j] -= ov * spf[q][j];
            }
            double nrm = 0.0;
            for (const cd& z : spf[k]) nrm += std::norm(z);
            nrm = std::sqrt(nrm);
            if (nrm > 1e-12) {
              for (cd& z : spf[k]) z /= nrm;
              break;
            }
          }
        }
        for (long long j = 0; j < d; ++j)
          for (int k = 0; k < r; ++k) A[(size_t)j * r + k] = spf[k][j];
      } else if (i != 0) {
        for (long long j = 0; j < d && j < r; ++j) A[(size_t)j * r + j] = 1.0;
      } else {
        A[0] = 1.0;
      }
    }
  })
}
long long orc_nsteps(void* p) { return ((OrcHandle*)p)->E.nsteps; }

int orc_expect(void* p, int mode, const double* op, double* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    std::vector<cd> M;
    const cd* mp = nullptr;
    if (op) {
      ORC_REQUIRE(mode >= 0 && mode < h->E.H.nmodes, "mode out of range");
      int d = h->E.H.mode_dim[mode];
      M.resize((size_t)d * d);
      for (size_t i = 0; i < M.size(); ++i) M[i] = cd(op[2 * i], op[2 * i + 1]);
      mp = M.data();
    }
    cd v = h->E.expect(mode, mp);
    out[0] = v.real(); out[1] = v.imag();
  })
}
int orc_bond_sv(void* p, int node, double* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    ORC_REQUIRE(node >= 1 && node < h->E.T.n, "node out of range");
    auto sv = h->E.bond_sv(node);
    for (size_t i = 0; i < sv.size(); ++i) out[i] = sv[i];
  })
}
// Kernel-level checks: environments for the current tensors, then H_eff / K_bond.
int orc_refresh_env(void* p) { OrcHandle* h = (OrcHandle*)p; ORC_TRY(h, { h->E.refresh_env(); }) }
int orc_heff(void* p, int node, const double* v, double* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    size_t n = h->E.T.size(node);
    std::vector<cd> x(n), y(n);
    for (size_t i = 0; i < n; ++i) x[i] = cd(v[2 * i], v[2 * i + 1]);
    h->E.heff(node, x.data(), y.data());
    for (size_t i = 0; i < n; ++i) { out[2 * i] = y[i].real(); out[2 * i + 1] = y[i].imag(); }
  })
}
int orc_kbond(void* p, int node, const double* v, double* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    size_t n = (size_t)h->E.T.hrank[node] * h->E.T.hrank[node];
    std::vector<cd> x(n), y(n);
    for (size_t i = 0; i < n; ++i) x[i] = cd(v[2 * i], v[2 * i + 1]);
    h->E.kbond(node, x.data(), y.data());
    for (size_t i = 0; i < n; ++i) { out[2 * i] = y[i].real(); out[2 * i + 1] = y[i].imag(); }
  })
}
// Krylov exponential of H_eff at a node applied to v (uses the current environments).
int orc_expm_node(void* p, int node, double tau, double cre, double cim, double* v, long long* napps) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    size_t n = h->E.T.size(node);
    std::vector<cd> x(n);
    for (size_t i = 0; i < n; ++i) x[i] = cd(v[2 * i], v[2 * i + 1]);
    long long k = h->E.expm([&](const cd* a, cd* o) { h->E.heff(node, a, o); }, x.data(), n, tau, cd(cre, cim));
    for (size_t i = 0; i < n; ++i) { v[2 * i] = x[i].real(); v[2 * i + 1] = x[i].imag(); }
    if (napps) *napps = k;
  })
}
// Environment matrices of one node/group (for parity checks).
int orc_num_groups(void* p, int node) { return (int)((OrcHandle*)p)->E.P.groups[node].size(); }
int orc_group_info(void* p, int node, int g, int* info) {
  OrcHandle* h = (OrcHandle*)p;
  const orc::Group& G = h->E.P.groups[node][g];
  info[0] = G.type; info[1] = G.id_spf; info[2] = G.id_mf; info[3] = (int)G.members.size();
  info[4] = (int)G.spf.size(); info[5] = (int)G.mf.size();
  return 0;
}
int orc_get_env(void* p, int node, int g, int which, double* out) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    const auto& M = which == 0 ? h->E.spf[node][g] : h->E.mf[node][g];
    for (size_t i = 0; i < M.size(); ++i) { out[2 * i] = M[i].real(); out[2 * i + 1] = M[i].imag(); }
  })
}
// Adjoint sweep (ttn_adjoint.hpp): J = sum_k w[k] Re <O_mode>(end of step k) over nsteps
// steps of dt from the current state (prepared first unless skip_prepare), checkpoints
// every ckpt steps.  Out: J; gcoeff[nterms] = dJ/dc_r; gops = cotangent of every operator
// (creation order, interleaved d x d); gstate (optional) = cotangent of the state after
// preparation.  Leaves the oracle at the final state.
int orc_adjoint(void* p, double dt, double cre, double cim, int nsteps, const double* w, int mode, const double* op,
                int ckpt, int skip_prepare, double* J, double* gcoeff, double* gops, double* gstate) {
  OrcHandle* h = (OrcHandle*)p;
  ORC_TRY(h, {
    orc::Engine& E = h->E;
    ORC_REQUIRE(mode >= 0 && mode < E.H.nmodes, "mode out of range");
    const int d = E.H.mode_dim[mode];
    std::vector<cd> O((size_t)d * d);
    for (size_t i = 0; i < O.size(); ++i) O[i] = cd(op[2 * i], op[2 * i + 1]);
    orc::Adjoint adj(E);
    *J = adj.run(dt, cd(cre, cim), nsteps, w, mode, O.data(), ckpt, skip_prepare != 0);
    for (int r = 0; r < E.H.nterms; ++r) gcoeff[r] = adj.gc[r];
    size_t off = 0;
    for (auto& mk : E.H.op_order) {
      const auto& G = adj.gop[mk.first][mk.second];
      for (size_t i = 0; i < G.size(); ++i) { gops[2 * (off + i)] = G[i].real(); gops[2 * (off + i) + 1] = G[i].imag(); }
      off += G.size();
    }
    if (gstate) {
      off = 0;
      for (int i = 0; i < E.T.n; ++i)
        for (auto& z : adj.Ab[i]) { gstate[2 * off] = z.real(); gstate[2 * off + 1] = z.imag(); ++off; }
    }
  })
}
// Householder QR of an m x n row-major complex matrix (in/out: Q), R out (n x n).
int orc_qr(int m, int n, double* a, double* r) {
  try {
    std::vector<cd> M((size_t)m * n), R((size_t)n * n), tau;
    for (size_t i = 0; i < M.size(); ++i) M[i] = cd(a[2 * i], a[2 * i + 1]);
    orc::householder_qr(M.data(), m, n, R.data(), tau);
    for (size_t i = 0; i < M.size(); ++i) { a[2 * i] = M[i].real(); a[2 * i + 1] = M[i].imag(); }
    for (size_t i = 0; i < R.size(); ++i) { r[2 * i] = R[i].real(); r[2 * i + 1] = R[i].imag(); }
    return 0;
  } catch (...) { return 1; }
}
// Symmetric tridiagonal eigen-decomposition (for checking the device solver).
int orc_tql2(int n, double* d, const double* e, double* z) {
  try { orc::tql2(n, d, e, z); return 0; } catch (...) { return 3; }
}

}  // extern "C"
