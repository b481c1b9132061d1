// Host side of the GB300 sweep: tree, sum-of-product operator, the compiled term plan,
// device arenas, the half-sweep schedule and the C-ABI of include/ttn_gb300.h.
//
// The schedule is that of ttns_lib's tdvp_algorithm_base (reference paths relative to
// the ttns_lib root):
//   forward half sweep ... include/ttns_lib/tdvp_core/tdvp_algorithm_engine.hpp:331-414
//   backward half sweep .. include/ttns_lib/tdvp_core/tdvp_algorithm_engine.hpp:417-501
//   prepare_evolution .... include/ttns_lib/tdvp_core/tdvp_algorithm_engine.hpp:257-321
//   first-step schedule .. include/ttns_lib/integrators/projector_splitting_integrator.hpp:136-169
// Every numerical operation is a device kernel (ttn_kernels.cu / ttn_tc.cu); the host only
// walks the schedule and enqueues work on the integrator's stream.  The only
// device-to-host traffic inside a step is one status word per Krylov sub-step.
#include "../../include/ttn_gb300.h"
#include "../../include/ttn_gb300_testing.h"
#include "ttn_kernels.cuh"
#include "ttn_coop.cuh"
#include "ttn_expm.cuh"
#include "ttn_tc.cuh"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <atomic>
#include <thread>
#include <complex>
#include <cstring>
#include <cstdio>
#include <functional>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace ttn {

static thread_local std::string g_err;
void set_error_message(const std::string& msg) { g_err = msg; }

struct Err : std::runtime_error {
  int code;
  Err(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
#define TTN_REQUIRE(cond, code, msg) \
  do { if (!(cond)) throw ::ttn::Err(code, msg); } while (0)
#define CK(x)                                                                                       \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess) throw ::ttn::Err(TTN_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

typedef std::complex<double> cd;

// ------------------------------------------------------------------ tree
struct Tree {
  int n = 0;
  std::vector<int> parent, slot, hrank, leaf_mode, leaf_dim, nmodes, sub_end, lo, hi, mode_node, mode_pos;
  std::vector<std::vector<int>> children, dims;
  std::vector<long long> dimen;
  std::vector<int> euler;  // Euler tour, tdvp_tree_traversal.hpp:38-87
  int nleaves = 0;

  long long size(int i) const { return dimen[i] * hrank[i]; }
  bool leaf(int i) const { return children[i].empty(); }
  // the bond above node c takes dimension r (subspace expansion)
  void set_bond(int c, int r) {
    hrank[c] = r;
    const int p = parent[c];
    dims[p][slot[c]] = r;
    dimen[p] = 1;
    for (int d : dims[p]) dimen[p] *= d;
  }

  void build(int nn, const int* par, const int* hr, const int* lm, const int* ld) {
    TTN_REQUIRE(nn >= 1 && par && hr && lm && ld, TTN_EINVAL, "tree arrays must be non-null");
    n = nn;
    parent.assign(par, par + n);
    hrank.assign(hr, hr + n);
    leaf_mode.assign(lm, lm + n);
    leaf_dim.assign(ld, ld + n);
    TTN_REQUIRE(parent[0] == -1, TTN_EINVAL, "node 0 must be the root (parent -1)");
    children.assign(n, {});
    slot.assign(n, -1);
    for (int i = 1; i < n; ++i) {
      TTN_REQUIRE(parent[i] >= 0 && parent[i] < i, TTN_EINVAL, "nodes must be numbered in pre-order");
      slot[i] = (int)children[parent[i]].size();
      children[parent[i]].push_back(i);
    }
    sub_end.assign(n, 0);
    for (int i = n - 1; i >= 0; --i) {
      sub_end[i] = i + 1;
      for (int c : children[i]) sub_end[i] = std::max(sub_end[i], sub_end[c]);
      for (int c : children[i]) TTN_REQUIRE(c < sub_end[i], TTN_EINVAL, "nodes must be numbered in pre-order");
    }
    dims.assign(n, {});
    dimen.assign(n, 1);
    nmodes.assign(n, 0);
    nleaves = 0;
    for (int i = 0; i < n; ++i) {
      TTN_REQUIRE(hrank[i] >= 1, TTN_EINVAL, "hrank must be >= 1");
      if (children[i].empty()) {
        TTN_REQUIRE(leaf_mode[i] >= 0 && leaf_dim[i] >= 1, TTN_EINVAL, "leaves need leaf_mode >= 0 and leaf_dim >= 1");
        dims[i] = {leaf_dim[i]};
        nmodes[i] = 1;
        ++nleaves;
      } else {
        TTN_REQUIRE(leaf_mode[i] < 0, TTN_EINVAL, "branch nodes must have leaf_mode -1");
        for (int c : children[i]) dims[i].push_back(hrank[c]);
        nmodes[i] = (int)children[i].size();
      }
      for (int d : dims[i]) dimen[i] *= d;
      TTN_REQUIRE(hrank[i] <= dimen[i], TTN_EINVAL, "hrank exceeds the product of the child dimensions");
    }
    mode_node.assign(nleaves, -1);
    mode_pos.assign(nleaves, -1);
    int pos = 0;
    for (int i = 0; i < n; ++i)
      if (children[i].empty()) {
        int m = leaf_mode[i];
        TTN_REQUIRE(m < nleaves && mode_node[m] < 0, TTN_EINVAL, "leaf modes must be a permutation of 0..nleaves-1");
        mode_node[m] = i;
        mode_pos[m] = pos++;
      }
    lo.assign(n, 0);
    hi.assign(n, 0);
    for (int i = n - 1; i >= 0; --i) {
      if (children[i].empty()) {
        lo[i] = mode_pos[leaf_mode[i]];
        hi[i] = lo[i] + 1;
      } else {
        lo[i] = lo[children[i].front()];
        hi[i] = hi[children[i].back()];
      }
    }
    for (int i = 0; i < n; ++i) {
      TTN_REQUIRE(hrank[i] <= kMaxBond, TTN_ENOTSUP, "bond dimensions above 256 are not supported");
      if (!children[i].empty())
        for (int m = 0; m < nmodes[i]; ++m) {
          long long d2 = dims[i][m], d1 = dimen[i] * hrank[i] / d2;
          TTN_REQUIRE(d1 >= d2, TTN_ENOTSUP, "root-to-leaf matricisation is wide; unsupported tree");
        }
    }
    size_t nsites = 0;
    for (int i = 0; i < n; ++i) nsites += children[i].empty() ? 2 : 1 + children[i].size();
    euler.resize(nsites);
    std::vector<int> tv(n, 0);
    int cur = 0;
    for (size_t k = 0; k < nsites; ++k) {
      euler[k] = cur;
      int t = tv[cur], nxt = cur;
      if (t == 0 && children[cur].empty()) nxt = cur;
      else if (t < (int)children[cur].size()) nxt = children[cur][t];
      else if (cur != 0) nxt = parent[cur];
      tv[cur]++;
      cur = nxt;
    }
  }
};

// ------------------------------------------------------------------ operator
// a sparse copy of a leaf operator bound in CSR or diagonal form
struct SparseOp {
  std::vector<int> rowptr, colind;
  std::vector<cd> val;
};
struct Sop {
  int nterms = 0, nmodes = 0;
  std::vector<int> mode_dim;
  std::vector<cd> coeff;
  std::vector<std::vector<std::vector<cd>>> ops;  // [mode][k] dense d x d
  std::vector<std::vector<SparseOp>> sparse;      // [mode][k] CSR form, empty rowptr when bound dense
  std::vector<std::vector<int>> opidx;            // [mode][r]
  std::vector<std::pair<int, int>> op_order;      // (mode, k) of every operator in binding order
};

// ------------------------------------------------------------------ compiled term plan
// Per node the terms split into S (shared operator below the node, >= 2 terms; the
// coefficients go into the mean field), M (remaining terms sharing the operator above
// the node, >= 2; coefficients go into the single-particle operator) and singletons
// (coefficient applied as a scalar) -- the common-spf / common-mf / standard split of
// operator_container.hpp:426-444, 648-664.
enum { G_S = 0, G_M = 1, G_1 = 2 };
struct Item { int slot, grp; };
// a_mem / b_mem: the terms whose coefficients were summed into a / b (empty when the
// scalar is the constant 1); the adjoint sweep returns scalar cotangents through them.
struct SpfTuple { cd a; std::vector<Item> items; std::vector<int> a_mem; };
struct MfKey { cd b; int pg; std::vector<Item> sib; std::vector<int> b_mem; };
// operations of a sweep, as reported to Integrator::on_op
enum { OP_AFP = 1, OP_R2L, OP_MF, OP_NODE, OP_L2R, OP_SPF, OP_BOND, OP_ATP };
struct Group {
  int type = G_1;
  std::vector<int> members;
  bool id_spf = false, id_mf = false;
  cd s = 1.0;
  std::vector<SpfTuple> spf;
  std::vector<MfKey> mf;
  double2* spf_dev = nullptr;
  double2* mf_dev = nullptr;
};

struct SigHash {
  size_t operator()(const std::vector<long long>& v) const {
    size_t h = 1469598103934665603ull;
    for (long long x : v) { h ^= (size_t)x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2); }
    return h;
  }
};

static void compile_plan(const Tree& T, const Sop& H, std::vector<std::vector<Group>>& G,
                         std::vector<std::vector<int>>& gof) {
  const int n = T.n, R = H.nterms;
  // supports sorted by leaf position
  std::vector<std::vector<std::pair<int, long long>>> sup(R);
  for (int m = 0; m < H.nmodes; ++m)
    for (int r = 0; r < R; ++r)
      if (H.opidx[m][r] >= 0) sup[r].push_back({T.mode_pos[m], ((long long)m << 32) | (unsigned)H.opidx[m][r]});
  for (auto& s : sup) std::sort(s.begin(), s.end());
  G.assign(n, {});
  gof.assign(n, std::vector<int>(R, -1));
  std::vector<std::vector<long long>> Ls(R), Rs(R);
  for (int nd = 0; nd < n; ++nd) {
    for (int r = 0; r < R; ++r) {
      Ls[r].clear();
      Rs[r].clear();
      for (auto& e : sup[r]) {
        if (e.first >= T.lo[nd] && e.first < T.hi[nd]) Ls[r].push_back(e.second);
        else Rs[r].push_back(e.second);
      }
    }
    std::unordered_map<std::vector<long long>, std::vector<int>, SigHash> lcls;
    for (int r = 0; r < R; ++r) lcls[Ls[r]].push_back(r);
    std::vector<char> isS(R, 0);
    std::vector<std::vector<int>> sg, mg, sing;
    for (auto& kv : lcls)
      if (kv.second.size() >= 2) {
        sg.push_back(kv.second);
        for (int r : kv.second) isS[r] = 1;
      }
    std::unordered_map<std::vector<long long>, std::vector<int>, SigHash> rcls;
    for (int r = 0; r < R; ++r)
      if (!isS[r]) rcls[Rs[r]].push_back(r);
    for (auto& kv : rcls) (kv.second.size() >= 2 ? mg : sing).push_back(kv.second);
    auto first = [](const std::vector<int>& a, const std::vector<int>& b) { return a[0] < b[0]; };
    std::sort(sg.begin(), sg.end(), first);
    std::sort(mg.begin(), mg.end(), first);
    std::sort(sing.begin(), sing.end(), first);
    auto add = [&](std::vector<int>& mem, int type) {
      std::sort(mem.begin(), mem.end());
      Group g;
      g.type = type;
      g.members = mem;
      // the identity below the node only if every member is: an M group may mix a term that
      // acts below with one that does not (the latter contributes its coefficient times I)
      g.id_spf = true;
      for (int r : mem) g.id_spf = g.id_spf && Ls[r].empty();
      g.s = (type == G_1) ? H.coeff[mem[0]] : cd(1.0);
      for (int r : mem) gof[nd][r] = (int)G[nd].size();
      G[nd].push_back(std::move(g));
    };
    for (auto& v : sg) add(v, G_S);
    for (auto& v : mg) add(v, G_M);
    for (auto& v : sing) add(v, G_1);
  }
  // single-particle tuples
  for (int nd = 0; nd < n; ++nd)
    for (auto& g : G[nd]) {
      if (g.id_spf) continue;
      std::map<std::vector<int>, std::vector<int>> keys;
      for (int r : g.members) {
        std::vector<int> key;
        // at a leaf the key is the term's operator there; a member that is the identity on
        // the leaf (possible in an M group) has an empty key, i.e. a tuple without items
        if (T.leaf(nd)) {
          if (H.opidx[T.leaf_mode[nd]][r] >= 0) key.push_back(H.opidx[T.leaf_mode[nd]][r]);
        }
        else
          for (int s = 0; s < (int)T.children[nd].size(); ++s) {
            int c = T.children[nd][s], cg = gof[c][r];
            if (!G[c][cg].id_spf) { key.push_back(s); key.push_back(cg); }
          }
        keys[key].push_back(r);
      }
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
            if (G[c][key[q + 1]].type == G_M) {
              carrying = true;
              TTN_REQUIRE(G[c][key[q + 1]].members == mem, TTN_EINVAL, "term compression invariant violated");
            }
          }
        if (g.type == G_M && !carrying) {
          cd a = 0.0;
          for (int r : mem) a += H.coeff[r];
          t.a = a;
          t.a_mem = mem;
        } else t.a = 1.0;
        g.spf.push_back(t);
      }
      TTN_REQUIRE(g.type == G_M || g.spf.size() == 1, TTN_EINVAL, "term compression invariant violated");
    }
  // mean-field keys
  for (int nd = 0; nd < n; ++nd) {
    if (nd == 0) {
      for (auto& g : G[nd]) g.id_mf = (g.type != G_S);
      continue;
    }
    int p = T.parent[nd];
    for (auto& g : G[nd]) {
      std::map<std::vector<int>, std::vector<int>> keys;
      for (int r : g.members) {
        std::vector<int> key{gof[p][r]};
        for (int s = 0; s < (int)T.children[p].size(); ++s) {
          int c = T.children[p][s];
          if (c == nd) continue;
          int cg = gof[c][r];
          if (!G[c][cg].id_spf) { key.push_back(s); key.push_back(cg); }
        }
        keys[key].push_back(r);
      }
      std::vector<std::pair<int, std::vector<int>>> ord;
      for (auto& kv : keys) ord.push_back({kv.second[0], kv.first});
      std::sort(ord.begin(), ord.end());
      for (auto& o : ord) {
        const auto& key = o.second;
        const auto& mem = keys[key];
        MfKey k;
        k.pg = key[0];
        const Group& pg = G[p][k.pg];
        bool carrying = (pg.type == G_S);
        const std::vector<int>* carrier = carrying ? &pg.members : nullptr;
        for (size_t q = 1; q < key.size(); q += 2) {
          int c = T.children[p][key[q]];
          k.sib.push_back({key[q], key[q + 1]});
          if (G[c][key[q + 1]].type == G_M) {
            carrying = true;
            carrier = &G[c][key[q + 1]].members;
          }
        }
        TTN_REQUIRE(!(g.type != G_S && carrying), TTN_EINVAL, "term compression invariant violated");
        TTN_REQUIRE(!carrying || *carrier == mem, TTN_EINVAL, "term compression invariant violated");
        if (g.type == G_S && !carrying) {
          cd b = 0.0;
          for (int r : mem) b += H.coeff[r];
          k.b = b;
          k.b_mem = mem;
        } else k.b = 1.0;
        g.mf.push_back(k);
      }
      g.id_mf = (g.mf.size() == 1 && g.mf[0].b == cd(1.0) && g.mf[0].sib.empty() && G[p][g.mf[0].pg].id_mf);
    }
  }
}

// ------------------------------------------------------------------ device helpers
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int device = 0;
  void alloc(size_t b) {
    free();
    if (b == 0) b = 16;
    CK(cudaMalloc(&p, b));
    bytes = b;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  ~DevBuf() { free(); }
  template <typename T> T* as() const { return (T*)p; }
};

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
static inline double2 d2(cd z) { return make_double2(z.real(), z.imag()); }
static const long long kBig = 1LL << 60;

static ZOperand op_rowmajor(const double2* p, long long ld) {  // X(i,k) = p[i*ld + k]
  ZOperand o{p, ld, 0, 1, kBig, 0, 1};
  return o;
}
static ZOperand op_colk(const double2* p, long long sk, long long so) {  // X(o,k) = p[o*so + k*sk]
  ZOperand o{p, so, 0, sk, kBig, 0, sk == 1};
  return o;
}

}  // namespace ttn

// ------------------------------------------------------------------ public objects
struct ttn_tree {
  ttn::Tree T;
};
struct ttn_sop {
  ttn::Sop H;
};
struct ttn_state {
  ttn::Tree T;
  int device = 0;
  ttn::DevBuf arena;
  std::vector<size_t> off;  // element offsets (double2) of each node
  double2* node(int i) const { return arena.as<double2>() + off[i]; }
};

namespace ttn {

struct Integrator {
  Tree T;
  Sop H;
  ttn_integ_cfg cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<std::vector<Group>> G;
  std::vector<std::vector<int>> gof;
  // device arenas
  DevBuf ops_buf, env_buf, r_buf, work_buf, ctl_buf, mel_buf;
  std::vector<std::vector<double2*>> leaf_ops;  // [mode][k]
  // sparse copies of large sparse leaf operators (bound in CSR or diagonal form), used by
  // the matvec programs while no time-dependent update hook is set
  struct LeafCsr {
    const int* rp = nullptr;
    const int* ci = nullptr;
    const double2* val = nullptr;
    long long nnz = 0;
  };
  std::vector<std::vector<LeafCsr>> leaf_csr;  // [mode][k]
  DevBuf csr_buf;
  static bool sparse_worth_it(int d, long long nnz) { return d >= 32 && nnz * 8 <= (long long)d * d; }
  bool csr_enabled() const { return !op_update_fn; }
  std::vector<double2*> rmat, mel;
  double2 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr, *w4 = nullptr, *V = nullptr, *p = nullptr,
          *gws = nullptr, *qtau = nullptr, *scal = nullptr;
  int krylov_stop = 0;     // 1: Lanczos recurrences end on the residual estimate
  size_t gws_bytes = 0;
  long long maxsize = 0, ldv = 0;
  KrylovCtl* ctl = nullptr;
  int* status = nullptr;
  // cooperative kernels: barrier state, scratch, grid limits
  DevBuf coop_buf;
  GridBarrier* bar = nullptr;
  double* qr_scratch = nullptr;
  int num_sms = 0, qr_max_grid = 1, qr_rows_grid = 1, expm_max_grid = 1, expm_max_grid_tc = 1;
  bool mixed = false;                      // tensor-core contractions in the matvec programs
  std::vector<char> heff_tc, kbond_tc;     // program contains tensor-core contractions
  std::vector<char> heff_tail, kbond_tail; // program needs a barrier after it
  int max_tc_images = 0;                   // most tensor-core ops in one program
  DevBuf tc_img_buf;                       // their operator images (kTcImageBytes each)
  // compiled matrix-vector programs for the persistent Krylov kernel
  DevBuf prog_buf, expm_part_buf;
  std::vector<int> heff_off, heff_n, kbond_off, kbond_n;
  std::vector<long long> heff_ext, kbond_ext;  // most elements any op of the program reads or writes
  long long* nh_dev = nullptr;
  double* flops_dev = nullptr;   // matvec flops executed by the persistent kernels
  // host mirrors
  double dt = 0.0, t_engine = 0.0;
  cd coeff = cd(0.0, -1.0);
  long long nsteps = 0, nh = 0;
  double flops = 0.0;        // algorithmic flops enqueued (complex MAC = 8 flops)
  double flops_seen = 0.0;   // device matvec flops already folded into `flops`
  long long h2d_bytes = 0, d2h_bytes = 0;  // host<->device traffic issued by the step path
  // optional breakdown (TTN_PROFILE=1): synchronising wall time per operation kind and
  // node-size class; slows the sweep down, for analysis only
  bool profiling = std::getenv("TTN_PROFILE") != nullptr;
  unsigned long long* phase_dev = nullptr;  // Krylov kernel phase timers (TTN_PROFILE)
  double prof_t[8][4] = {};
  long long prof_n[8][4] = {};
  struct Prof {
    Integrator* I; int kind, cls; std::chrono::steady_clock::time_point t0;
    Prof(Integrator* i, int k, int nd) : I(i), kind(k), cls(0) {
      if (!I->profiling) return;
      long long sz = I->T.size(nd);
      cls = sz < 1024 ? 0 : sz < 65536 ? 1 : sz < (1 << 20) ? 2 : 3;
      cudaStreamSynchronize(I->stream);
      t0 = std::chrono::steady_clock::now();
    }
    ~Prof() {
      if (!I->profiling) return;
      cudaStreamSynchronize(I->stream);
      I->prof_t[kind][cls] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      I->prof_n[kind][cls] += 1;
    }
  };
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // called before every operation of a sweep (OP_*, node, auxiliary index) while set: the
  // adjoint sweep records the operations' inputs through it
  std::function<void(int, int, int)> on_op;
  // subspace expansion (ttn_expansion.hpp): bond capacities and the tree at capacity, which
  // sizes every buffer; the expansion calls inside the half-sweeps and the step that
  // replaces step() while expansion is on
  std::vector<int> cap;
  Tree Tsz;
  std::function<bool(ttn_state*, int)> expand_down_fn, expand_up_fn;
  std::function<void(ttn_state*, double, cd)> expanding_step;
  // time-dependent primitive operators (ttn_integrator_set_op_update)
  ttn_op_update_fn op_update_fn = nullptr;
  void* op_update_user = nullptr;
  std::vector<std::vector<int>> op_global;  // [mode][k] -> binding index
  // op.update(leaf, t, dt/2) before a leaf's evolution (projector_splitting_engine.hpp:139):
  // the user updates each operator of the mode on the host; the device copy follows
  void update_leaf_ops(int mode) {
    for (size_t k = 0; k < H.ops[mode].size(); ++k) {
      std::vector<cd>& M = H.ops[mode][k];
      op_update_fn(op_update_user, mode, op_global[mode][k], t_engine, dt / 2.0, reinterpret_cast<double*>(M.data()));
      std::vector<double2> h(M.size());
      for (size_t i = 0; i < M.size(); ++i) {
        TTN_REQUIRE(std::isfinite(M[i].real()) && std::isfinite(M[i].imag()), TTN_ENUMERIC, "operator update produced a non-finite entry");
        h[i] = d2(M[i]);
      }
      CK(cudaMemcpyAsync(leaf_ops[mode][k], h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, stream));
      CK(cudaStreamSynchronize(stream));  // h is pageable and goes out of scope
    }
  }
  bool expanded = false;

  ~Integrator() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  void setup() {
    CK(cudaSetDevice(device));
    // A blocking stream: its work waits for work issued earlier to the legacy default
    // stream, where the state uploads and downloads of ttn_state (cudaMemcpy) run; with a
    // non-blocking stream a step could start before an upload has landed.
    CK(cudaStreamCreate(&stream));
    compile_plan(T, H, G, gof);
    // leaf operators
    size_t ob = 0;
    for (int m = 0; m < H.nmodes; ++m)
      for (auto& M : H.ops[m]) ob += align256(M.size() * sizeof(double2));
    ops_buf.alloc(ob);
    leaf_ops.assign(H.nmodes, {});
    {
      char* base = ops_buf.as<char>();
      size_t o = 0;
      for (int m = 0; m < H.nmodes; ++m)
        for (auto& M : H.ops[m]) {
          double2* dptr = (double2*)(base + o);
          std::vector<double2> tmp(M.size());
          for (size_t i = 0; i < M.size(); ++i) tmp[i] = d2(M[i]);
          CK(cudaMemcpy(dptr, tmp.data(), tmp.size() * sizeof(double2), cudaMemcpyHostToDevice));
          leaf_ops[m].push_back(dptr);
          o += align256(M.size() * sizeof(double2));
        }
    }
    // sparse leaf operators: row pointers, column indices and values in one buffer
    leaf_csr.assign(H.nmodes, {});
    {
      size_t cb = 0;
      for (int m = 0; m < H.nmodes; ++m)
        for (size_t k = 0; k < H.ops[m].size(); ++k) {
          leaf_csr[m].push_back(LeafCsr());
          if (m >= (int)H.sparse.size() || k >= H.sparse[m].size()) continue;
          const SparseOp& sp = H.sparse[m][k];
          if (sp.rowptr.empty() || !sparse_worth_it(H.mode_dim[m], (long long)sp.val.size())) continue;
          cb += align256(sp.rowptr.size() * sizeof(int)) + align256(std::max<size_t>(1, sp.colind.size()) * sizeof(int)) +
                align256(std::max<size_t>(1, sp.val.size()) * sizeof(double2));
        }
      if (cb) {
        csr_buf.alloc(cb);
        char* base = csr_buf.as<char>();
        size_t o = 0;
        for (int m = 0; m < H.nmodes; ++m)
          for (size_t k = 0; k < H.ops[m].size(); ++k) {
            if (m >= (int)H.sparse.size() || k >= H.sparse[m].size()) continue;
            const SparseOp& sp = H.sparse[m][k];
            if (sp.rowptr.empty() || !sparse_worth_it(H.mode_dim[m], (long long)sp.val.size())) continue;
            LeafCsr& c = leaf_csr[m][k];
            int* rp = (int*)(base + o);
            o += align256(sp.rowptr.size() * sizeof(int));
            int* ci = (int*)(base + o);
            o += align256(std::max<size_t>(1, sp.colind.size()) * sizeof(int));
            double2* val = (double2*)(base + o);
            o += align256(std::max<size_t>(1, sp.val.size()) * sizeof(double2));
            std::vector<double2> v(sp.val.size());
            for (size_t q = 0; q < v.size(); ++q) v[q] = d2(sp.val[q]);
            CK(cudaMemcpy(rp, sp.rowptr.data(), sp.rowptr.size() * sizeof(int), cudaMemcpyHostToDevice));
            if (!sp.colind.empty()) {
              CK(cudaMemcpy(ci, sp.colind.data(), sp.colind.size() * sizeof(int), cudaMemcpyHostToDevice));
              CK(cudaMemcpy(val, v.data(), v.size() * sizeof(double2), cudaMemcpyHostToDevice));
            }
            c.rp = rp; c.ci = ci; c.val = val; c.nnz = (long long)sp.val.size();
          }
      }
    }
    allocate_sized();
    finish_setup();
  }

  // the tree that sizes every buffer: the capacities when bonds may grow, else the tree
  const Tree& sizing() const { return cap.empty() ? T : Tsz; }

  // environment, gauge-factor, observable and work buffers, sized for sizing()
  void allocate_sized() {
    const Tree& Z = sizing();
    // environments: one r x r matrix per non-identity spf / mf
    size_t eb = 0;
    for (int i = 0; i < T.n; ++i) {
      size_t rr = (size_t)Z.hrank[i] * Z.hrank[i] * sizeof(double2);
      for (auto& g : G[i]) eb += (g.id_spf ? 0 : align256(rr)) + (g.id_mf ? 0 : align256(rr));
    }
    env_buf.alloc(eb);
    CK(cudaMemsetAsync(env_buf.p, 0, env_buf.bytes, stream));
    {
      char* base = env_buf.as<char>();
      size_t o = 0;
      for (int i = 0; i < T.n; ++i) {
        size_t rr = (size_t)Z.hrank[i] * Z.hrank[i] * sizeof(double2);
        for (auto& g : G[i]) {
          if (!g.id_spf) { g.spf_dev = (double2*)(base + o); o += align256(rr); }
          if (!g.id_mf) {
            g.mf_dev = (double2*)(base + o);
            o += align256(rr);
            if (i == 0) {  // root S group: (sum of coefficients) * I
              cd sum = 0.0;
              for (int r : g.members) sum += H.coeff[r];
              zscale_identity(g.mf_dev, T.hrank[i], d2(sum), stream);
            }
          }
        }
      }
    }
    // R matrices and observable scratch
    size_t rb = 0, mb = 0;
    for (int i = 0; i < T.n; ++i) {
      long long rmx = Z.hrank[i];
      for (int d : Z.dims[i]) rmx = std::max<long long>(rmx, d);
      rb += align256((size_t)rmx * rmx * sizeof(double2));
      mb += align256((size_t)Z.hrank[i] * Z.hrank[i] * sizeof(double2));
    }
    r_buf.alloc(rb);
    mel_buf.alloc(mb);
    rmat.resize(T.n);
    mel.resize(T.n);
    {
      size_t o = 0, o2 = 0;
      for (int i = 0; i < T.n; ++i) {
        long long rmx = Z.hrank[i];
        for (int d : Z.dims[i]) rmx = std::max<long long>(rmx, d);
        rmat[i] = (double2*)(r_buf.as<char>() + o);
        o += align256((size_t)rmx * rmx * sizeof(double2));
        mel[i] = (double2*)(mel_buf.as<char>() + o2);
        o2 += align256((size_t)Z.hrank[i] * Z.hrank[i] * sizeof(double2));
      }
    }
    // work space
    maxsize = 0;
    for (int i = 0; i < T.n; ++i) maxsize = std::max(maxsize, Z.size(i));
    ldv = (long long)(align256((size_t)maxsize * sizeof(double2)) / sizeof(double2));
    size_t gmax = 0;
    for (int i = 0; i < T.n; ++i) {
      int r = Z.hrank[i];
      gmax = std::max(gmax, zgemm_split_workspace_bytes(r, r, (int)Z.dimen[i]));
      for (int m = 0; m < Z.nmodes[i]; ++m) {
        int d = Z.dims[i][m];
        gmax = std::max(gmax, zgemm_split_workspace_bytes(d, d, (int)(Z.size(i) / d)));
      }
    }
    gws_bytes = align256(gmax + 16);
    const int m = cfg.krylov_dim;
    size_t wb = 0;
    wb += 4 * align256(ldv * sizeof(double2));                   // w1..w4
    wb += (size_t)(m + 1) * ldv * sizeof(double2);               // V
    wb += align256(ldv * sizeof(double2));                        // p
    wb += gws_bytes;                                              // zgemm split-K
    wb += align256(kMaxBond * sizeof(double2));                   // QR tau
    wb += align256(64 * sizeof(double2));                         // scalars
    work_buf.alloc(wb);
    {
      char* b = work_buf.as<char>();
      size_t o = 0;
      auto take = [&](size_t bytes) { char* q = b + o; o += align256(bytes); return (double2*)q; };
      w1 = take(ldv * sizeof(double2));
      w2 = take(ldv * sizeof(double2));
      w3 = take(ldv * sizeof(double2));
      w4 = take(ldv * sizeof(double2));
      V = take((size_t)(m + 1) * ldv * sizeof(double2));
      p = take(ldv * sizeof(double2));
      gws = take(gws_bytes);
      qtau = take(kMaxBond * sizeof(double2));
      scal = take(64 * sizeof(double2));
    }
  }

  // control block, events, cooperative-kernel state and the term programs
  void finish_setup() {
    ctl_buf.alloc(align256(sizeof(KrylovCtl)) + 512);
    ctl = ctl_buf.as<KrylovCtl>();
    status = (int*)(ctl_buf.as<char>() + align256(sizeof(KrylovCtl)));
    if (profiling) phase_dev = (unsigned long long*)(ctl_buf.as<char>() + align256(sizeof(KrylovCtl)) + 256);
    CK(cudaMemsetAsync(ctl_buf.p, 0, ctl_buf.bytes, stream));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    {
      CK(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
      qr_max_grid = std::max(1, std::min(qr_blocked_max_grid(), num_sms));
      qr_rows_grid = std::max(1, std::min(qr_rows_max_grid(), num_sms));
      if (const char* e = std::getenv("TTN_QR_ROWS_TARGET")) qr_rows_target = std::max(1, std::atoi(e));
      size_t qb = align256(sizeof(GridBarrier)) +
                  align256(std::max(qr_blocked_scratch_bytes(qr_max_grid), qr_rows_scratch_bytes(qr_rows_grid)));
      coop_buf.alloc(qb);
      CK(cudaMemsetAsync(coop_buf.p, 0, coop_buf.bytes, stream));
      bar = coop_buf.as<GridBarrier>();
      qr_scratch = (double*)(coop_buf.as<char>() + align256(sizeof(GridBarrier)));
      mixed = (cfg.precision == TTN_PREC_MIXED);
      if (const char* e = std::getenv("TTN_EXPM_CTA_FLOPS")) expm_cta_flops = std::atof(e);
      if (const char* e = std::getenv("TTN_EXPM_ELEMS_PER_CTA")) expm_elems_per_cta = std::max(1, std::atoi(e));
      if (const char* e = std::getenv("TTN_EXPM_TPO")) expm_tpo_max = std::max(1, std::min(8, std::atoi(e)));
      if (const char* e = std::getenv("TTN_EXPM_TPO_MIN_FLOPS")) expm_tpo_min_flops = std::atof(e);
      if (const char* e = std::getenv("TTN_EXPM_SMEM_VECS")) expm_smem_vecs = std::atoi(e) != 0;
      if (const char* e = std::getenv("TTN_QR_ROWS_PER_CTA")) qr_rows_per_cta = std::max(1, std::atoi(e));
      if (const char* e = std::getenv("TTN_EXPM_ELEMS_PER_THREAD")) expm_elems_per_thread = std::max(0.1, std::atof(e));
      expm_max_grid = std::max(1, expm_coop_max_grid(0));
      expm_max_grid_tc = std::max(1, expm_coop_max_grid(1));
      if (mixed) {
        for (int i = 0; i < T.n; ++i)
          TTN_REQUIRE(sizing().hrank[i] <= kQrMaxCols, TTN_ENOTSUP, "mixed precision takes bonds of at most 64");
        // the tensor-core contractions need sm_100-family tensor memory
        cudaDeviceProp prop{};
        CK(cudaGetDeviceProperties(&prop, device));
        TTN_REQUIRE(prop.major >= 10, TTN_ENOTSUP, "mixed precision needs a tcgen05 device (sm_100 family)");
      }
      expm_part_buf.alloc(expm_partial_bytes(expm_max_grid) + 512);
      nh_dev = (long long*)(expm_part_buf.as<char>() + expm_partial_bytes(expm_max_grid));
      flops_dev = (double*)(expm_part_buf.as<char>() + expm_partial_bytes(expm_max_grid) + 256);
      CK(cudaMemsetAsync(expm_part_buf.p, 0, expm_part_buf.bytes, stream));
      compile_programs();
      if (mixed) tc_img_buf.alloc((size_t)std::max(1, max_tc_images) * kTcImageBytes);
    }

    CK(cudaStreamSynchronize(stream));
  }

  // ---------------------------------------------------------------- contractions
  void r3(int nd, int mu, long long& na, int& d, long long& nb) const {
    na = 1;
    nb = T.hrank[nd];
    for (int i = 0; i < mu; ++i) na *= T.dims[nd][i];
    d = T.dims[nd][mu];
    for (int i = mu + 1; i < T.nmodes[nd]; ++i) nb *= T.dims[nd][i];
  }
  // One mode or mean-field product on the tensor cores (mixed precision, eligible
  // shapes): the persistent kernel's apply-only path with a one-contraction program.
  bool tc_apply(int kind, const double2* mat, const double2* in, double2* out, long long na, int d, long long nb,
                cd alpha, bool acc) {
    if (!mixed || !tc_eligible(kind, d, na, nb)) return false;
    ExpmArgs a{};
    a.y = const_cast<double2*>(in); a.p = out; a.n = 0;
    a.V = V; a.ldv = ldv; a.t1 = w1; a.t2 = w2; a.t3 = w3;
    a.prog = nullptr; a.nops = 1;
    MvOp& o = a.op1;
    o.kind = kind; o.in = 0; o.out = 1; o.mat = mat; o.na = na; o.d = d; o.nb = nb;
    o.alpha = d2(alpha); o.beta = acc ? 1 : 0; o.tc = 1; o.img = 0; o.barrier_before = 0;
    a.part = expm_part_buf.as<double2>();
    a.ctl = ctl; a.bar = bar; a.err = status;
    a.m = cfg.krylov_dim; a.tau = 0.0; a.cf_re = 0.0; a.cf_im = -1.0; a.tol = cfg.krylov_tol;
    a.mixed = 1; a.apply_only = 1; a.phase = nullptr;
    a.tc_img = tc_img_buf.as<uint32_t>();
    const long long tiles = kind == MV_MODE ? na * (nb / kTcTileN) : na / kTcTileN;
    const int grid = (int)std::max(1LL, std::min<long long>(tiles, expm_max_grid_tc));
    CK(expm_coop(a, grid, stream));
    return true;
  }
  // out(a,i,b) = alpha sum_j S(i,j) in(a,j,b) (+ out)
  // (allow_tc = false keeps a product in FP64 in mixed precision: the gauge moves, which
  // change the state itself, always run in FP64)
  void mode_apply(const double2* S, int d, const double2* in, double2* out, long long na, long long nb, cd alpha,
                  bool acc, bool allow_tc = true) {
    flops += 8.0 * na * (double)d * d * nb;
    if (allow_tc && tc_apply(MV_MODE, S, in, out, na, d, nb, alpha, acc)) return;
    ZGemm g{};
    g.M = d; g.N = (int)nb; g.K = d;
    g.A = op_rowmajor(S, d);
    g.B = op_colk(in, nb, 1);
    g.C = out; g.ci = nb; g.cj = 1;
    g.bsA = 0; g.bsB = (long long)d * nb; g.bsC = (long long)d * nb;
    g.batch = (int)na;
    g.alpha = d2(alpha);
    g.beta = acc ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
    zgemm(g, gws, gws_bytes, stream);
  }
  // out(x,k) = alpha sum_l in(x,l) M(k,l) (+ out)
  void mf_apply(const double2* in, const double2* M, int r, long long nx, double2* out, cd alpha, bool acc,
                bool allow_tc = true) {
    flops += 8.0 * nx * (double)r * r;
    if (allow_tc && tc_apply(MV_MF, M, in, out, nx, r, 0, alpha, acc)) return;
    ZGemm g{};
    g.M = (int)nx; g.N = r; g.K = r;
    g.A = op_rowmajor(in, r);
    g.B = op_rowmajor(M, r);  // B(l,k) = M[k*r + l]
    g.C = out; g.ci = r; g.cj = 1;
    g.batch = 1;
    g.alpha = d2(alpha);
    g.beta = acc ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
    zgemm(g, gws, gws_bytes, stream);
  }
  // out(i,j) = alpha sum_x conj(A(x,i)) X(x,j) (+ out)
  void adj_mul(const double2* A, const double2* X, long long nx, int r, double2* out, cd alpha, bool acc) {
    flops += 8.0 * nx * (double)r * r;
    ZGemm g{};
    g.M = r; g.N = r; g.K = (int)nx;
    g.A = op_colk(A, r, 1);
    g.A.cj = 1;
    g.B = op_colk(X, r, 1);
    g.C = out; g.ci = r; g.cj = 1;
    g.batch = 1;
    g.alpha = d2(alpha);
    g.beta = acc ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
    zgemm(g, gws, gws_bytes, stream);
  }
  // out(i,j) = alpha sum_{a,b} conj(A(a,i,b)) T(a,j,b) (+ out)
  void mode_contract(const double2* A, const double2* Tt, long long na, int d, long long nb, double2* out, cd alpha,
                     bool acc) {
    flops += 8.0 * na * nb * (double)d * d;
    ZGemm g{};
    g.M = d; g.N = d; g.K = (int)(na * nb);
    ZOperand o{A, nb, (long long)d * nb, 1, nb, 1, 1};
    g.A = o;
    ZOperand o2{Tt, nb, (long long)d * nb, 1, nb, 0, 1};
    g.B = o2;
    g.C = out; g.ci = d; g.cj = 1;
    g.batch = 1;
    g.alpha = d2(alpha);
    g.beta = acc ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
    zgemm(g, gws, gws_bytes, stream);
  }
  // C (m x r) = A (m x r) * R (r x r)
  void right_mul(const double2* A, const double2* R, long long m, int r, double2* C) {
    flops += 8.0 * m * (double)r * r;
    ZGemm g{};
    g.M = (int)m; g.N = r; g.K = r;
    g.A = op_rowmajor(A, r);
    g.B = op_colk(R, r, 1);  // B(k,j) = R[k*r + j]
    g.C = C; g.ci = r; g.cj = 1;
    g.batch = 1;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    zgemm(g, gws, gws_bytes, stream);
  }

  // A chain applies its scalar with its last product; a tuple without items (terms that act
  // as the identity below the node, next to terms that do not) carries it in the
  // accumulation that follows instead.
  static cd chain_scale(const SpfTuple& t) { return t.items.empty() ? t.a : cd(1.0); }
  const double2* apply_items(int nd, const std::vector<Item>& items, const double2* v, double2* b1, double2* b2,
                             cd alpha_last = 1.0) {
    const double2* cur = v;
    double2* nxt = b1;
    for (size_t q = 0; q < items.size(); ++q) {
      const Item& it = items[q];
      long long na, nb;
      int d;
      const double2* S;
      if (it.slot < 0) {
        S = leaf_ops[T.leaf_mode[nd]][it.grp];
        na = 1; d = T.dims[nd][0]; nb = T.hrank[nd];
      } else {
        S = G[T.children[nd][it.slot]][it.grp].spf_dev;
        r3(nd, it.slot, na, d, nb);
      }
      mode_apply(S, d, cur, nxt, na, nb, q + 1 == items.size() ? alpha_last : cd(1.0), false);
      cur = nxt;
      nxt = (nxt == b1) ? b2 : b1;
    }
    return cur;
  }
  const double2* apply_sibs(int p, const std::vector<Item>& items, const double2* v, double2* b1, double2* b2) {
    const double2* cur = v;
    double2* nxt = b1;
    for (const Item& it : items) {
      long long na, nb;
      int d;
      r3(p, it.slot, na, d, nb);
      mode_apply(G[T.children[p][it.slot]][it.grp].spf_dev, d, cur, nxt, na, nb, 1.0, false);
      cur = nxt;
      nxt = (nxt == b1) ? b2 : b1;
    }
    return cur;
  }

  // bottom-up environment (single_particle_operator.hpp:26-103)
  // A group with several tuples sums a_t X_t into w3 first and contracts once:
  // sum_t a_t A^H X_t = A^H (sum_t a_t X_t), one K = dimen reduction instead of one per tuple.
  void update_spf(int nd, const double2* A) {
    if (on_op) on_op(OP_SPF, nd, 0);
    Prof pf(this, 5, nd);
    const long long sz = T.size(nd);
    const int r = T.hrank[nd];
    for (auto& g : G[nd]) {
      if (g.id_spf) continue;
      if (g.spf.size() == 1) {
        const SpfTuple& t = g.spf[0];
        const double2* X = apply_items(nd, t.items, A, w1, w2);
        adj_mul(A, X, sz / r, r, g.spf_dev, t.a, false);
        continue;
      }
      bool first = true;
      for (const SpfTuple& t : g.spf) {
        const double2* X = apply_items(nd, t.items, A, w1, w2);
        mode_identity_axpy(X, w3, sz, t.a, !first);
        first = false;
      }
      adj_mul(A, w3, sz / r, r, g.spf_dev, 1.0, false);
    }
  }
  // top-down environment of child nd (mean_field_operator.hpp:37-184)
  void update_mf(int nd, const double2* Ap) {
    if (nd == 0) return;
    if (on_op) on_op(OP_MF, nd, 0);
    Prof pf(this, 4, T.parent[nd]);
    const int p = T.parent[nd], mu = T.slot[nd];
    long long na, nb;
    int d;
    r3(p, mu, na, d, nb);
    const int rp = T.hrank[p];
    const long long szp = T.size(p);
    for (auto& g : G[nd]) {
      if (g.id_mf) continue;
      if (g.mf.size() == 1) {
        const MfKey& k = g.mf[0];
        const double2* X = apply_sibs(p, k.sib, Ap, w1, w2);
        if (!G[p][k.pg].id_mf) {
          double2* dst = (X == w1) ? w2 : w1;
          mf_apply(X, G[p][k.pg].mf_dev, rp, szp / rp, dst, 1.0, false);
          X = dst;
        }
        mode_contract(Ap, X, na, d, nb, g.mf_dev, k.b, false);
        continue;
      }
      // several keys: sum_k b_k X_k into w3 (the parent's mean field applied on the way),
      // then one contraction with the parent tensor
      bool first = true;
      for (const MfKey& k : g.mf) {
        const double2* X = apply_sibs(p, k.sib, Ap, w1, w2);
        if (!G[p][k.pg].id_mf) mf_apply(X, G[p][k.pg].mf_dev, rp, szp / rp, w3, k.b, !first);
        else mode_identity_axpy(X, w3, szp, k.b, !first);
        first = false;
      }
      mode_contract(Ap, w3, na, d, nb, g.mf_dev, 1.0, false);
    }
  }
  // out = H_eff(nd) v (coefficient_evolution_leaf / _branch)
  void heff(int nd, const double2* v, double2* out) {
    const long long sz = T.size(nd);
    const int r = T.hrank[nd];
    bool first = true;
    for (auto& g : G[nd]) {
      const bool direct = g.id_mf;  // accumulate straight into out
      if (g.id_spf) {
        if (direct) {
          // out (+)= s v
          mode_identity_axpy(v, out, sz, g.s, !first);
        } else {
          mf_apply(v, g.mf_dev, r, sz / r, out, g.s, !first);
        }
      } else if (g.spf.size() == 1) {
        const auto& t = g.spf[0];
        if (direct && t.items.size() == 1) {
          // single contraction straight into out with the combined scalar
          const Item& it = t.items[0];
          long long na, nb;
          int d;
          const double2* S;
          if (it.slot < 0) { S = leaf_ops[T.leaf_mode[nd]][it.grp]; na = 1; d = T.dims[nd][0]; nb = r; }
          else { S = G[T.children[nd][it.slot]][it.grp].spf_dev; r3(nd, it.slot, na, d, nb); }
          mode_apply(S, d, v, out, na, nb, g.s * t.a, !first);
        } else {
          const double2* X = apply_items(nd, t.items, v, w1, w2, t.a);
          if (direct) mode_identity_axpy(X, out, sz, g.s * chain_scale(t), !first);
          else mf_apply(X, g.mf_dev, r, sz / r, out, g.s * chain_scale(t), !first);
        }
      } else {
        // several tuples: sum into w3 then one mean-field product
        if (direct) {
          bool f2 = first;
          for (const SpfTuple& t : g.spf) {
            if (t.items.size() == 1) {
              const Item& it = t.items[0];
              long long na, nb;
              int d;
              const double2* S;
              if (it.slot < 0) { S = leaf_ops[T.leaf_mode[nd]][it.grp]; na = 1; d = T.dims[nd][0]; nb = r; }
              else { S = G[T.children[nd][it.slot]][it.grp].spf_dev; r3(nd, it.slot, na, d, nb); }
              mode_apply(S, d, v, out, na, nb, g.s * t.a, !f2);
            } else {
              const double2* X = apply_items(nd, t.items, v, w1, w2, t.a);
              mode_identity_axpy(X, out, sz, g.s * chain_scale(t), !f2);
            }
            f2 = false;
          }
        } else {
          bool f2 = true;
          for (const SpfTuple& t : g.spf) {
            if (t.items.size() == 1) {
              const Item& it = t.items[0];
              long long na, nb;
              int d;
              const double2* S;
              if (it.slot < 0) { S = leaf_ops[T.leaf_mode[nd]][it.grp]; na = 1; d = T.dims[nd][0]; nb = r; }
              else { S = G[T.children[nd][it.slot]][it.grp].spf_dev; r3(nd, it.slot, na, d, nb); }
              mode_apply(S, d, v, w3, na, nb, t.a, !f2);
            } else {
              const double2* X = apply_items(nd, t.items, v, w1, w2, t.a);
              mode_identity_axpy(X, w3, sz, chain_scale(t), !f2);
            }
            f2 = false;
          }
          mf_apply(w3, g.mf_dev, r, sz / r, out, g.s, !first);
        }
      }
      first = false;
    }
    if (first) zfill(out, make_double2(0.0, 0.0), sz, stream);
  }
  // out (+)= s * x
  void mode_identity_axpy(const double2* x, double2* out, long long sz, cd s, bool acc) {
    zaxpy(out, x, d2(s), sz, acc, stream);
  }
  // algorithmic flops of one H_eff application at nd
  double heff_flops(int nd) {
    double before = flops;
    // count by dry-running the contraction shapes (no launches)
    double f = 0.0;
    const double sz = (double)T.size(nd);
    const int r = T.hrank[nd];
    for (auto& g : G[nd]) {
      if (!g.id_spf)
        for (const SpfTuple& t : g.spf)
          for (const Item& it : t.items) {
            int d = (it.slot < 0) ? T.dims[nd][0] : T.dims[nd][it.slot];
            const LeafCsr* c = item_csr(nd, it);
            f += c ? 8.0 * (sz / d) * (double)c->nnz : 8.0 * sz * d;
          }
      if (!g.id_mf) f += 8.0 * sz * r;
    }
    (void)before;
    return f;
  }
  double kbond_flops(int nd) {
    const double r = T.hrank[nd];
    double f = 0.0;
    for (auto& g : G[nd]) {
      if (!g.id_spf) f += 8.0 * r * r * r;
      if (!g.id_mf) f += 8.0 * r * r * r;
    }
    return f;
  }
  // ---------------------------------------------------------------- matvec programs
  // Barriers go where one contraction reads a buffer another wrote (or overwrites one
  // another read) since the last barrier.  The element-wise FP64 contractions give output
  // element e to the same thread whatever the shape, so two of them may accumulate into
  // one buffer back to back; a tensor-core contraction distributes its output by tiles,
  // so an accumulation that involves one is a hazard too.
  struct ProgBuilder {
    bool mixed = false;
    std::vector<MvOp> ops;
    unsigned dirty = 0, read = 0, dirty_tc = 0;
    int n_img = 0;
    void emit(MvOp op) {
      op.tc = (mixed && tc_eligible(op.kind, op.d, op.na, op.nb)) ? 1 : 0;
      op.img = op.tc ? n_img++ : -1;
      const unsigned in_bit = (op.kind == MV_ZERO) ? 0u : (1u << op.in);
      const unsigned out_bit = 1u << op.out;
      const bool waw = (out_bit & dirty) && (op.tc || (out_bit & dirty_tc));
      op.barrier_before = ((in_bit & dirty) || (out_bit & read) || waw) ? 1 : 0;
      if (op.barrier_before) { dirty = 0; read = 0; dirty_tc = 0; }
      dirty |= out_bit;
      read |= in_bit;
      if (op.tc) dirty_tc |= out_bit;
      ops.push_back(op);
    }
  };
  static MvOp mk(int kind, int in, int out, const double2* mat, long long na, int d, long long nb, cd alpha, bool acc) {
    MvOp o{};
    o.kind = kind; o.in = in; o.out = out; o.mat = mat; o.na = na; o.d = d; o.nb = nb;
    o.alpha = d2(alpha); o.beta = acc ? 1 : 0;
    return o;
  }
  void item_shape(int nd, const Item& it, const double2*& S, long long& na, int& d, long long& nb) {
    if (it.slot < 0) { S = leaf_ops[T.leaf_mode[nd]][it.grp]; na = 1; d = T.dims[nd][0]; nb = T.hrank[nd]; }
    else { S = G[T.children[nd][it.slot]][it.grp].spf_dev; r3(nd, it.slot, na, d, nb); }
  }
  // the product of one item with the vector: a sparse leaf operator's CSR contraction, or
  // the dense mode product
  const LeafCsr* item_csr(int nd, const Item& it) const {
    if (it.slot >= 0 || !csr_enabled()) return nullptr;
    const LeafCsr& c = leaf_csr[T.leaf_mode[nd]][it.grp];
    return c.rp ? &c : nullptr;
  }
  MvOp mk_item(int in, int out, int nd, const Item& it, cd alpha, bool acc) {
    const double2* S; long long na, nb; int d;
    item_shape(nd, it, S, na, d, nb);
    if (const LeafCsr* c = item_csr(nd, it)) {
      MvOp o = mk(MV_CSR, in, out, c->val, na, d, nb, alpha, acc);
      o.rowptr = c->rp;
      o.colind = c->ci;
      return o;
    }
    return mk(MV_MODE, in, out, S, na, d, nb, alpha, acc);
  }
  // chain of mode products ending in a temporary; returns its buffer id
  int emit_chain(ProgBuilder& B, int nd, const std::vector<Item>& items, int in, cd alpha_last) {
    int cur = in;
    for (size_t q = 0; q < items.size(); ++q) {
      int out = (q % 2 == 0) ? 2 : 3;
      B.emit(mk_item(cur, out, nd, items[q], q + 1 == items.size() ? alpha_last : cd(1.0), false));
      cur = out;
    }
    return cur;
  }
  std::vector<MvOp> heff_program(int nd) {
    ProgBuilder B;
    B.mixed = mixed;
    const long long sz = T.size(nd);
    const int r = T.hrank[nd];
    bool first = true;
    for (auto& g : G[nd]) {
      const bool direct = g.id_mf;
      if (g.id_spf) {
        if (direct) B.emit(mk(MV_AXPY, 0, 1, nullptr, sz, 0, 0, g.s, !first));
        else B.emit(mk(MV_MF, 0, 1, g.mf_dev, sz / r, r, 0, g.s, !first));
      } else if (g.spf.size() == 1) {
        const auto& t = g.spf[0];
        if (direct && t.items.size() == 1) {
          B.emit(mk_item(0, 1, nd, t.items[0], g.s * t.a, !first));
        } else {
          int X = emit_chain(B, nd, t.items, 0, t.a);
          if (direct) B.emit(mk(MV_AXPY, X, 1, nullptr, sz, 0, 0, g.s * chain_scale(t), !first));
          else B.emit(mk(MV_MF, X, 1, g.mf_dev, sz / r, r, 0, g.s * chain_scale(t), !first));
        }
      } else {
        bool f2 = true;
        const int acc_buf = direct ? 1 : 4;
        for (const SpfTuple& t : g.spf) {
          const bool accum = direct ? !(first && f2) : !f2;
          const cd sc = direct ? g.s * t.a : t.a;
          if (t.items.size() == 1) {
            B.emit(mk_item(0, acc_buf, nd, t.items[0], sc, accum));
          } else {
            int X = emit_chain(B, nd, t.items, 0, t.a);
            B.emit(mk(MV_AXPY, X, acc_buf, nullptr, sz, 0, 0, (direct ? g.s : cd(1.0)) * chain_scale(t), accum));
          }
          f2 = false;
        }
        if (!direct) B.emit(mk(MV_MF, 4, 1, g.mf_dev, sz / r, r, 0, g.s, !first));
      }
      first = false;
    }
    if (first) B.emit(mk(MV_ZERO, 0, 1, nullptr, sz, 0, 0, 0.0, false));
    return B.ops;
  }
  // K R = sum_g s_g spf_g R mf_g^T.  The spf products of up to three groups go to the
  // temporaries 2, 3, 4 first and the mean-field products follow, so that one grid barrier
  // separates them instead of two per group; the accumulation order is the groups' order.
  std::vector<MvOp> kbond_program(int nd) {
    ProgBuilder B;
    B.mixed = mixed;
    const int r = T.hrank[nd];
    bool first = true;
    const std::vector<Group>& gs = G[nd];
    size_t i0 = 0;
    while (i0 < gs.size()) {
      size_t i1 = i0;
      int used = 0;
      while (i1 < gs.size() && (gs[i1].id_spf || used < 3)) {
        if (!gs[i1].id_spf) ++used;
        ++i1;
      }
      std::vector<int> X(i1 - i0, 0);
      int nb = 0;
      for (size_t k = i0; k < i1; ++k)
        if (!gs[k].id_spf) {
          X[k - i0] = 2 + nb++;
          B.emit(mk(MV_MODE, 0, X[k - i0], gs[k].spf_dev, 1, r, r, 1.0, false));
        }
      for (size_t k = i0; k < i1; ++k) {
        const Group& g = gs[k];
        if (g.id_mf) B.emit(mk(MV_AXPY, X[k - i0], 1, nullptr, (long long)r * r, 0, 0, g.s, !first));
        else B.emit(mk(MV_MF, X[k - i0], 1, g.mf_dev, r, r, 0, g.s, !first));
        first = false;
      }
      i0 = i1;
    }
    if (first) B.emit(mk(MV_ZERO, 0, 1, nullptr, (long long)r * r, 0, 0, 0.0, false));
    return B.ops;
  }
  void compile_programs() {
    std::vector<MvOp> all;
    heff_off.assign(T.n, 0); heff_n.assign(T.n, 0); kbond_off.assign(T.n, 0); kbond_n.assign(T.n, 0);
    heff_tc.assign(T.n, 0); kbond_tc.assign(T.n, 0);
    heff_tail.assign(T.n, 0); kbond_tail.assign(T.n, 0);
    heff_ext.assign(T.n, 0); kbond_ext.assign(T.n, 0);
    max_tc_images = 0;
    auto extent = [](const std::vector<MvOp>& ops) {
      long long e = 0;
      for (const auto& o : ops) {
        long long t = o.na;
        if (o.kind == MV_MODE || o.kind == MV_CSR) t = o.na * o.d * o.nb;
        else if (o.kind == MV_MF) t = o.na * o.d;
        e = std::max(e, t);
      }
      return e;
    };
    // a tensor-core op wrote the result buffer (1) after the program's last barrier
    auto tail_needed = [](const std::vector<MvOp>& ops) {
      bool pending = false;
      for (const auto& o : ops) {
        if (o.barrier_before) pending = false;
        if (o.tc && o.out == 1) pending = true;
      }
      return pending;
    };
    auto mark = [&](const std::vector<MvOp>& ops) {
      int n = 0;
      for (const auto& o : ops) n += o.tc ? 1 : 0;
      max_tc_images = std::max(max_tc_images, n);
      return n > 0;
    };
    for (int i = 0; i < T.n; ++i) {
      auto h = heff_program(i);
      heff_tc[i] = mark(h);
      heff_tail[i] = tail_needed(h);
      heff_ext[i] = extent(h);
      heff_off[i] = (int)all.size(); heff_n[i] = (int)h.size();
      all.insert(all.end(), h.begin(), h.end());
      auto k = kbond_program(i);
      kbond_tc[i] = mark(k);
      kbond_tail[i] = tail_needed(k);
      kbond_ext[i] = extent(k);
      kbond_off[i] = (int)all.size(); kbond_n[i] = (int)k.size();
      all.insert(all.end(), k.begin(), k.end());
    }
    prog_buf.alloc(all.size() * sizeof(MvOp) + 16);
    CK(cudaMemcpyAsync(prog_buf.p, all.data(), all.size() * sizeof(MvOp), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));  // `all` is pageable and goes out of scope
  }
  // CTAs of a Krylov launch: at most one per expm_elems_per_cta vector elements and one per
  // expm_cta_flops of matvec work.  Small problems run on few CTAs (one CTA synchronises
  // with __syncthreads alone, several need grid barriers of a few microseconds each),
  // large ones on the whole device.
  double expm_cta_flops = 5.0e4;
  long long expm_elems_per_cta = 64;  // at least this many vector elements per CTA
  int expm_tpo_max = 8;               // most lanes per output element of the element-wise ops
  double expm_tpo_min_flops = 2000.0; // matvec flops per vector element from which they are split
  bool expm_smem_vecs = true;         // one-CTA launches with the vectors in shared memory
  // threads per CTA: about expm_elems_per_thread vector elements per thread, 64..256 (the
  // FP64 warp reductions cost the same per warp whatever the data, so tiny problems run on
  // fewer warps)
  double expm_elems_per_thread = 1.0;
  int expm_threads(long long n, int grid) const {
    long long t = (long long)std::ceil((double)n / ((double)grid * expm_elems_per_thread));
    t = (t + 31) / 32 * 32;
    return (int)std::max(64LL, std::min(256LL, t));
  }
  int expm_grid(long long n, bool tc, double flops_per_app) const {
    long long g = (n + expm_elems_per_cta - 1) / expm_elems_per_cta;
    if (expm_cta_flops > 0.0) {
      const long long gw = (long long)std::ceil(flops_per_app / expm_cta_flops);
      if (gw < g) g = gw;
    }
    if (g < 1) g = 1;
    const int mx = tc ? expm_max_grid_tc : expm_max_grid;
    if (g > mx) g = mx;
    return (int)g;
  }
  // persistent Krylov exponential of one node tensor (kind 0) or bond matrix (kind 1)
  void expm_dev(int nd, int kind, double2* y, long long n, double tau, cd cf, bool count, bool tally = true,
                bool apply_only = false) {
    if (tau == 0.0 && !apply_only) return;
    ExpmArgs a{};
    a.y = y; a.n = n; a.V = V; a.ldv = ldv; a.p = p; a.t1 = w1; a.t2 = w2; a.t3 = w3;
    a.prog = prog_buf.as<MvOp>() + (kind == 0 ? heff_off[nd] : kbond_off[nd]);
    a.nops = kind == 0 ? heff_n[nd] : kbond_n[nd];
    a.part = expm_part_buf.as<double2>();
    a.ctl = ctl; a.bar = bar; a.err = status;
    a.napps_total = count ? nh_dev : nullptr;
    a.flops_total = tally ? flops_dev : nullptr;
    a.flops_per_app = (kind == 0) ? heff_flops(nd) : kbond_flops(nd);
    a.m = cfg.krylov_dim; a.tau = tau; a.cf_re = cf.real(); a.cf_im = cf.imag(); a.tol = cfg.krylov_tol;
    a.krylov_stop = krylov_stop;
    a.mixed = (kind == 0 ? heff_tc[nd] : kbond_tc[nd]) ? 1 : 0;
    a.tail_barrier = (kind == 0 ? heff_tail[nd] : kbond_tail[nd]) ? 1 : 0;
    a.apply_only = apply_only ? 1 : 0;
    a.phase = phase_dev;
    a.tc_img = tc_img_buf.as<uint32_t>();
    const int grid = expm_grid(n, a.mixed, a.flops_per_app);
    int threads = expm_threads(n, grid);
    // launches with threads to spare give each output element of the element-wise ops
    // several lanes (ExpmArgs::tpo) when the program has many terms per element (bond
    // matrices: 6 products of 64 terms; measured: 11 % faster); with few terms per element
    // (leaves, 256 x 64 nodes) the wider CTAs cost the Lanczos reductions more than the
    // split saves
    if (!a.mixed && expm_tpo_max > 1 && a.flops_per_app >= expm_tpo_min_flops * (double)n) {
      const long long cap = (long long)grid * 256;
      int tpo = 1;
      while (tpo < expm_tpo_max && n * tpo * 2 <= cap) tpo *= 2;
      if (tpo > 1) {
        a.tpo = tpo;
        a.tail_barrier = 1;
        threads = (int)std::min<long long>(256, ((n * tpo + grid - 1) / grid + 31) / 32 * 32);
      }
    }
    // one-CTA launches keep their vectors in shared memory when they fit
    if (grid == 1 && expm_smem_vecs && !a.mixed && !apply_only) {
      const long long ext = kind == 0 ? heff_ext[nd] : kbond_ext[nd];
      const long long ldt = (std::max(ext, n) + 1) / 2 * 2;
      if (expm_smem_vecs_bytes(a.m, ldt) <= expm_smem_vecs_max_bytes()) {
        a.smem_vecs = 1;
        a.ldt = ldt;
      }
    }
    CK(expm_coop(a, grid, stream, threads));
    // Lanczos vector passes of one sub-step (the matvec flops are tallied on the device)
    if (tally) flops += lanczos_vec_flops(n);
  }
  double lanczos_vec_flops(long long n) const {
    const int m = cfg.krylov_dim;
    double vec = 0.0;
    for (int j = 0; j < m; ++j) vec += (8.0 + 8.0 + 16.0 * (j + 1) + 4.0 + 2.0) * n;
    vec += (4.0 + 8.0 * (m + 1)) * n;
    return vec;
  }

  // ---------------------------------------------------------------- gauge moves
  // Householder QR on as many CTAs as the height allows (one row block per CTA)
  int qr_rows_per_cta = 32;  // rows of the matrix per CTA of the panel-blocked QR (tall matrices)
  int qr_rows_target = 8;    // rows per CTA of the shared-memory QR
  void qr(double2* M, long long m, int n, double2* R, int Rt) {
    TTN_REQUIRE(n >= 1 && n <= kMaxBond, TTN_ECAPACITY, "a gauge move wider than 256 columns");
    // rows resident in shared memory: about qr_rows_target rows per CTA (one CTA while the
    // rows fit), as long as the grid holds every row; else the panel-blocked kernel
    {
      const long long cap = qr_rows_max_rows(n);
      long long g = m <= cap ? 1 : (m + qr_rows_target - 1) / qr_rows_target;
      if (g > qr_rows_grid) g = qr_rows_grid;
      if (cap > 0 && (m + g - 1) / g <= cap) {
        CK(householder_qr_rows(M, m, n, R, Rt, qtau, qr_scratch, bar, status, (int)g, stream));
        return;
      }
    }
    int g = (int)std::max(1LL, std::min<long long>(m / qr_rows_per_cta, qr_max_grid));
    CK(householder_qr_blocked(M, m, n, R, Rt, qtau, qr_scratch, bar, status, g, stream));
  }
  static double qr_flops(double m, double n) { return 2.0 * 8.0 * (m * n * n - n * n * n / 3.0); }
  void l2r(int nd, double2* A) {
    if (on_op) on_op(OP_L2R, nd, 0);
    Prof pf(this, 3, nd);
    const long long m = T.dimen[nd];
    const int r = T.hrank[nd];
    flops += qr_flops((double)m, (double)r);
    qr(A, m, r, rmat[nd], 0);
  }
  void apply_to_parent(int nd, double2* Ap, int p) {
    if (on_op) on_op(OP_ATP, nd, 0);
    Prof pf(this, 6, p);
    long long na, nb;
    int d;
    r3(p, T.slot[nd], na, d, nb);
    mode_apply(rmat[nd], d, Ap, w4, na, nb, 1.0, false, false);
    zcopy(Ap, w4, T.size(p), stream);
  }
  void r2l(int nd, int mu, double2* A) {
    if (on_op) on_op(OP_R2L, nd, mu);
    Prof pf(this, 2, nd);
    long long pre = 1, post = T.hrank[nd];
    for (int i = 0; i < mu; ++i) pre *= T.dims[nd][i];
    const int dm = T.dims[nd][mu];
    for (int i = mu + 1; i < T.nmodes[nd]; ++i) post *= T.dims[nd][i];
    flops += qr_flops((double)(pre * post), (double)dm);
    permute_mode_last(A, w4, pre, dm, post, stream);
    qr(w4, pre * post, dm, rmat[nd], 1);
    unpermute_mode_last(w4, A, pre, dm, post, stream);
  }
  void apply_from_parent(int nd, double2* A) {
    if (on_op) on_op(OP_AFP, nd, 0);
    Prof pf(this, 7, nd);
    const int p = T.parent[nd], r = T.hrank[nd];
    right_mul(A, rmat[p], T.dimen[nd], r, w4);
    zcopy(A, w4, T.size(nd), stream);
  }

  // ---------------------------------------------------------------- sweep
  void evolve_node(ttn_state* S, int nd) {
    if (on_op) on_op(OP_NODE, nd, 0);
    if (op_update_fn && T.leaf(nd)) update_leaf_ops(T.leaf_mode[nd]);
    Prof pf(this, 0, nd);
    expm_dev(nd, 0, S->node(nd), T.size(nd), dt / 2.0, coeff, true);
  }
  // the bond matrix held in rmat[owner]: the node's own after l2r, its parent's after r2l
  void evolve_bond(int nd, int owner) {
    if (on_op) on_op(OP_BOND, nd, owner);
    double2* R = rmat[owner];
    Prof pf(this, 1, nd);
    const long long rr = (long long)T.hrank[nd] * T.hrank[nd];
    expm_dev(nd, 1, R, rr, -dt / 2.0, coeff, false);
  }
  void forward(ttn_state* S, bool evolve) {
    std::vector<int> tv(T.n, 0);
    for (int id : T.euler) {
      int t = tv[id]++;
      double2* A = S->node(id);
      if (t != T.nmodes[id]) {
        if (t == 0 && id != 0) apply_from_parent(id, A);
        if (!T.leaf(id)) {
          r2l(id, t, A);
          if (expand_down_fn) expanded = expand_down_fn(S, T.children[id][t]) || expanded;
          update_mf(T.children[id][t], A);
        }
      } else {
        if (evolve) evolve_node(S, id);
        if (id != 0) {
          l2r(id, A);
          update_spf(id, A);
          if (evolve) evolve_bond(id, id);
          apply_to_parent(id, S->node(T.parent[id]), T.parent[id]);
        }
      }
    }
  }
  void backward(ttn_state* S, bool evolve) {
    std::vector<int> tv(T.n, 0);
    for (auto it = T.euler.rbegin(); it != T.euler.rend(); ++it) {
      int id = *it;
      int t = tv[id]++;
      double2* A = S->node(id);
      if (t != T.nmodes[id]) {
        int mode = T.nmodes[id] - (t + 1);
        if (t == 0) {
          if (id != 0) {
            if (evolve) evolve_bond(id, T.parent[id]);
            apply_from_parent(id, A);
          }
          if (evolve) evolve_node(S, id);
        }
        if (!T.leaf(id)) {
          r2l(id, mode, A);
          update_mf(T.children[id][mode], A);
        }
      } else if (id != 0) {
        l2r(id, A);
        if (expand_up_fn) expanded = expand_up_fn(S, id) || expanded;
        apply_to_parent(id, S->node(T.parent[id]), T.parent[id]);
        update_spf(id, A);
      }
    }
  }
  void sweep(ttn_state* S) {
    forward(S, true);
    t_engine += dt / 2.0;
    backward(S, true);
    t_engine += dt / 2.0;
  }
  void prepare(ttn_state* S) {
    for (int id = T.n - 1; id >= 1; --id) update_spf(id, S->node(id));
    forward(S, false);
    backward(S, false);
  }
  // orthogonaliser::operator() (include/ttns_lib/decompositions/orthogonaliser.hpp:83-112):
  // children before parents, A = Q R on the device, A <- Q, R applied to the parent's slot;
  // the single-particle environments follow the new gauge once the run has started
  void orthogonalise(ttn_state* S) {
    for (int id = T.n - 1; id >= 1; --id) {
      l2r(id, S->node(id));
      apply_to_parent(id, S->node(T.parent[id]), T.parent[id]);
    }
    if (nsteps > 0)
      for (int id = T.n - 1; id >= 1; --id) update_spf(id, S->node(id));
  }
  void step(ttn_state* S, double step_dt, cd cf) {
    if (expanding_step) {
      expanding_step(S, step_dt, cf);
      finish_check(S);
      return;
    }
    coeff = cf;
    if (nsteps == 0) {
      double tevolve = 0.0, sdt = step_dt / 1e5;
      dt = (sdt + tevolve <= step_dt) ? sdt : step_dt - tevolve;
      prepare(S);
      while (tevolve < step_dt) {
        dt = (sdt + tevolve <= step_dt) ? sdt : step_dt - tevolve;
        t_engine = tevolve;
        sweep(S);
        tevolve += sdt;
        sdt *= 10.0;
      }
    } else {
      dt = step_dt;
      t_engine = nsteps * step_dt;
      sweep(S);
    }
    ++nsteps;
    dt = step_dt;
    finish_check(S);
  }
  // environments and gauge passes of the first step without its evolution; later
  // steps are then full dt steps (used to time steady-state sweeps)
  void prepare_only(ttn_state* S) {
    prepare(S);
    nsteps = std::max<long long>(nsteps, 1);
    finish_check(S);
  }
  void finish_check(ttn_state* S) {
    check_finite(S->arena.as<double2>(), (long long)(S->arena.bytes / sizeof(double2)), status, kErrNonFinite, stream);
    int h = 0;
    long long napps = 0;
    double mvf = 0.0;
    CK(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&napps, nh_dev, sizeof(long long), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&mvf, flops_dev, sizeof(double), cudaMemcpyDeviceToHost, stream));
    d2h_bytes += sizeof(int) + sizeof(long long) + sizeof(double);
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    nh = napps;
    flops += mvf - flops_seen;
    flops_seen = mvf;
    CK(cudaMemsetAsync(status, 0, sizeof(int), stream));
    TTN_REQUIRE(!(h & kErrBarrierTimeout), TTN_ETIMEOUT, "a device-side grid barrier gave up waiting");
    TTN_REQUIRE(!(h >> kKrylovErrShift), TTN_ENUMERIC,
                "Krylov exponential failed (status " + std::to_string(h >> kKrylovErrShift) +
                    ": 1 tolerance unreachable, 2 non-finite vector, 4 eigen-solve, 8 step size, 16 sub-step limit)");
    TTN_REQUIRE(h == 0, TTN_ENUMERIC, "the state holds non-finite values after the step");
  }

  // ---------------------------------------------------------------- observables
  // (always FP64, also in mixed precision)

  // Schmidt values across the bond above node nd, for the orthogonalised form the sweep
  // leaves (every non-root node an isometry): the bond's density matrix from the root down
  // the path (mean-field product and mode contraction per node, FP64 on the device), then a
  // cyclic Hermitian Jacobi eigen-solve on the host; sqrt of the eigenvalues, descending
  // (matrix_element / decomposition_engine singular values of the reference, S() = "pops").
  std::vector<double> bond_sv(ttn_state* S, int nd) {
    std::vector<int> path;
    for (int x = nd; x != 0; x = T.parent[x]) path.push_back(x);
    std::reverse(path.begin(), path.end());
    const int r0 = T.hrank[0];
    std::vector<double2> eye((size_t)r0 * r0, make_double2(0.0, 0.0));
    for (int k = 0; k < r0; ++k) eye[(size_t)k * r0 + k] = make_double2(1.0, 0.0);
    CK(cudaMemcpyAsync(w2, eye.data(), eye.size() * sizeof(double2), cudaMemcpyHostToDevice, stream));
    h2d_bytes += (long long)eye.size() * sizeof(double2);
    for (int c : path) {
      const int p = T.parent[c];
      long long na, nb;
      int d;
      r3(p, T.slot[c], na, d, nb);
      const long long sz = T.size(p);
      mf_apply(S->node(p), w2, T.hrank[p], sz / T.hrank[p], w1, 1.0, false, false);
      mode_contract(S->node(p), w1, na, d, nb, w2, 1.0, false);
    }
    const int d = T.hrank[nd];
    std::vector<cd> a((size_t)d * d);
    CK(cudaMemcpyAsync(a.data(), w2, a.size() * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    d2h_bytes += (long long)a.size() * sizeof(double2);
    CK(cudaStreamSynchronize(stream));
    for (int sweepi = 0; sweepi < 100; ++sweepi) {
      double off = 0.0;
      for (int i = 0; i < d; ++i)
        for (int j = i + 1; j < d; ++j) off += std::norm(a[(size_t)i * d + j]);
      if (off < 1e-30) break;
      for (int pp = 0; pp < d; ++pp)
        for (int q = pp + 1; q < d; ++q) {
          const cd apq = a[(size_t)pp * d + q];
          const double ab = std::abs(apq);
          if (ab < 1e-300) continue;
          const double app = a[(size_t)pp * d + pp].real(), aqq = a[(size_t)q * d + q].real();
          const double th = 0.5 * std::atan2(2.0 * ab, aqq - app);
          const double c = std::cos(th), sn = std::sin(th);
          const cd ph = apq / ab;
          // a <- J^H a J with J_pp = J_qq = c, J_pq = sn ph, J_qp = -sn conj(ph)
          for (int k = 0; k < d; ++k) {
            const cd akp = a[(size_t)k * d + pp], akq = a[(size_t)k * d + q];
            a[(size_t)k * d + pp] = c * akp - sn * std::conj(ph) * akq;
            a[(size_t)k * d + q] = sn * ph * akp + c * akq;
          }
          for (int k = 0; k < d; ++k) {
            const cd apk = a[(size_t)pp * d + k], aqk = a[(size_t)q * d + k];
            a[(size_t)pp * d + k] = c * apk - sn * ph * aqk;
            a[(size_t)q * d + k] = sn * std::conj(ph) * apk + c * aqk;
          }
        }
    }
    std::vector<double> sv(d);
    for (int i = 0; i < d; ++i) sv[i] = std::sqrt(std::max(0.0, a[(size_t)i * d + i].real()));
    std::sort(sv.begin(), sv.end(), std::greater<double>());
    return sv;
  }
  // <B| prod_m O_m |K> for states of this tree (B may be K): the leaf-to-root contraction
  // of matrix_element.hpp:223-259 / :441-481 with a dense operator on each mode that has
  // one (op_of_mode[m] != nullptr, d_m x d_m on the device) and the identity elsewhere
  cd contract(ttn_state* B, ttn_state* K, const std::vector<const double2*>& op_of_mode) {
    for (int id = T.n - 1; id >= 0; --id) {
      const int r = T.hrank[id];
      const long long sz = T.size(id);
      const double2* Ab = B->node(id);
      const double2* Ak = K->node(id);
      const double2* X = Ak;
      if (T.leaf(id)) {
        const double2* op = op_of_mode[T.leaf_mode[id]];
        if (op) {
          mode_apply(op, T.dims[id][0], Ak, w1, 1, r, 1.0, false, false);
          X = w1;
        }
      } else {
        const double2* cur = Ak;
        double2* nxt = w1;
        for (int s = 0; s < T.nmodes[id]; ++s) {
          long long na, nb;
          int d;
          r3(id, s, na, d, nb);
          mode_apply(mel[T.children[id][s]], d, cur, nxt, na, nb, 1.0, false, false);
          cur = nxt;
          nxt = (nxt == w1) ? w2 : w1;
        }
        X = cur;
      }
      adj_mul(Ab, X, sz / r, r, mel[id], 1.0, false);
    }
    ztrace(mel[0], T.hrank[0], scal + 1, stream);
    double2 h;
    CK(cudaMemcpyAsync(&h, scal + 1, sizeof(double2), cudaMemcpyDeviceToHost, stream));
    d2h_bytes += sizeof(double2);
    CK(cudaStreamSynchronize(stream));
    return cd(h.x, h.y);
  }
  cd expect(ttn_state* S, int mode, const double2* op_dev) {
    for (int id = T.n - 1; id >= 0; --id) {
      const int r = T.hrank[id];
      const long long sz = T.size(id);
      const double2* A = S->node(id);
      const double2* X = A;
      if (T.leaf(id)) {
        if (op_dev && T.leaf_mode[id] == mode) {
          mode_apply(op_dev, T.dims[id][0], A, w1, 1, r, 1.0, false, false);
          X = w1;
        }
      } else {
        const double2* cur = A;
        double2* nxt = w1;
        for (int s = 0; s < T.nmodes[id]; ++s) {
          long long na, nb;
          int d;
          r3(id, s, na, d, nb);
          mode_apply(mel[T.children[id][s]], d, cur, nxt, na, nb, 1.0, false, false);
          cur = nxt;
          nxt = (nxt == w1) ? w2 : w1;
        }
        X = cur;
      }
      adj_mul(A, X, sz / r, r, mel[id], 1.0, false);
    }
    ztrace(mel[0], T.hrank[0], scal + 1, stream);
    double2 h;
    CK(cudaMemcpyAsync(&h, scal + 1, sizeof(double2), cudaMemcpyDeviceToHost, stream));
    d2h_bytes += sizeof(double2);
    CK(cudaStreamSynchronize(stream));
    return cd(h.x, h.y);
  }
};

#include "ttn_adjoint.hpp"
#include "ttn_expansion.hpp"

static void check_same_tree(const Tree& a, const Tree& b) {
  TTN_REQUIRE(a.parent == b.parent && a.hrank == b.hrank && a.leaf_dim == b.leaf_dim && a.leaf_mode == b.leaf_mode,
              TTN_EINVAL, "state and integrator were built for different trees");
}

}  // namespace ttn

struct ttn_integrator {
  ttn::Integrator I;
  std::unique_ptr<ttn::DevExpander> X;  // subspace expansion, when enabled
};

// ====================================================================== C-ABI
#define TTN_API_BEGIN try {
#define TTN_API_END                                   \
  return TTN_OK;                                      \
  }                                                   \
  catch (const ttn::Err& e) {                         \
    ttn::g_err = e.what();                            \
    return e.code;                                    \
  }                                                   \
  catch (const std::bad_alloc&) {                     \
    ttn::g_err = "host allocation failed";            \
    return TTN_ECAPACITY;                             \
  }                                                   \
  catch (const std::exception& e) {                   \
    ttn::g_err = e.what();                            \
    return TTN_EINVAL;                                \
  }

extern "C" {

const char* ttn_last_error(void) { return ttn::g_err.c_str(); }
const char* ttn_version(void) { return "ttn_gb300 1.0 (sm_103a)"; }

int ttn_tree_create(int nnodes, const int* parent, const int* hrank, const int* leaf_mode, const int* leaf_dim,
                    ttn_tree** out) {
  TTN_API_BEGIN
  TTN_REQUIRE(out, TTN_EINVAL, "out is null");
  auto* t = new ttn_tree();
  try { t->T.build(nnodes, parent, hrank, leaf_mode, leaf_dim); } catch (...) { delete t; throw; }
  *out = t;
  TTN_API_END
}
int ttn_tree_destroy(ttn_tree* t) { delete t; return TTN_OK; }
int ttn_tree_num_nodes(const ttn_tree* t, int* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(t && out, TTN_EINVAL, "null argument");
  *out = t->T.n;
  TTN_API_END
}
int ttn_tree_node_shape(const ttn_tree* t, int node, long long* dimen, int* hrank) {
  TTN_API_BEGIN
  TTN_REQUIRE(t && node >= 0 && node < t->T.n, TTN_EINVAL, "node out of range");
  if (dimen) *dimen = t->T.dimen[node];
  if (hrank) *hrank = t->T.hrank[node];
  TTN_API_END
}
int ttn_tree_state_size(const ttn_tree* t, long long* n) {
  TTN_API_BEGIN
  TTN_REQUIRE(t && n, TTN_EINVAL, "null argument");
  long long s = 0;
  for (int i = 0; i < t->T.n; ++i) s += t->T.size(i);
  *n = s;
  TTN_API_END
}

int ttn_sop_create(int nterms, int nmodes, const int* mode_dims, ttn_sop** out) {
  TTN_API_BEGIN
  TTN_REQUIRE(out && nterms >= 1 && nmodes >= 1 && mode_dims, TTN_EINVAL, "bad operator shape");
  auto* s = new ttn_sop();
  s->H.nterms = nterms;
  s->H.nmodes = nmodes;
  s->H.mode_dim.assign(mode_dims, mode_dims + nmodes);
  for (int d : s->H.mode_dim)
    if (d < 1) { delete s; throw ttn::Err(TTN_EINVAL, "mode dimensions must be >= 1"); }
  s->H.coeff.assign(nterms, 1.0);
  s->H.ops.assign(nmodes, {});
  s->H.sparse.assign(nmodes, {});
  s->H.opidx.assign(nmodes, std::vector<int>(nterms, -1));
  *out = s;
  TTN_API_END
}
int ttn_sop_destroy(ttn_sop* s) { delete s; return TTN_OK; }

static void sop_bind(ttn_sop* s, int mode, std::vector<ttn::cd>&& M, const int* r, int nr,
                     ttn::SparseOp&& sp = ttn::SparseOp()) {
  TTN_REQUIRE(s && mode >= 0 && mode < s->H.nmodes, TTN_EINVAL, "mode out of range");
  TTN_REQUIRE(r && nr >= 1, TTN_EINVAL, "an operator must be bound to at least one term");
  for (int q = 0; q < nr; ++q) {
    TTN_REQUIRE(r[q] >= 0 && r[q] < s->H.nterms, TTN_EINVAL, "term index out of range");
    TTN_REQUIRE(s->H.opidx[mode][r[q]] < 0, TTN_EINVAL, "term already has an operator on this mode");
  }
  for (auto& z : M) TTN_REQUIRE(std::isfinite(z.real()) && std::isfinite(z.imag()), TTN_EINVAL, "non-finite operator entry");
  int k = (int)s->H.ops[mode].size();
  s->H.ops[mode].push_back(std::move(M));
  if (s->H.sparse.size() < (size_t)s->H.nmodes) s->H.sparse.resize(s->H.nmodes);
  s->H.sparse[mode].push_back(std::move(sp));
  s->H.op_order.push_back({mode, k});
  for (int q = 0; q < nr; ++q) s->H.opidx[mode][r[q]] = k;
}
int ttn_sop_bind_dense(ttn_sop* s, int mode, const double* mat, const int* r, int nr) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && mat && mode >= 0 && mode < s->H.nmodes, TTN_EINVAL, "bad argument");
  int d = s->H.mode_dim[mode];
  std::vector<ttn::cd> M((size_t)d * d);
  for (size_t i = 0; i < M.size(); ++i) M[i] = ttn::cd(mat[2 * i], mat[2 * i + 1]);
  sop_bind(s, mode, std::move(M), r, nr);
  TTN_API_END
}
int ttn_sop_bind_diag(ttn_sop* s, int mode, const double* diag, const int* r, int nr) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && diag && mode >= 0 && mode < s->H.nmodes, TTN_EINVAL, "bad argument");
  int d = s->H.mode_dim[mode];
  std::vector<ttn::cd> M((size_t)d * d, 0.0);
  ttn::SparseOp sp;
  sp.rowptr.resize(d + 1);
  for (int i = 0; i < d; ++i) {
    M[(size_t)i * d + i] = ttn::cd(diag[2 * i], diag[2 * i + 1]);
    sp.rowptr[i] = i;
    sp.colind.push_back(i);
    sp.val.push_back(M[(size_t)i * d + i]);
  }
  sp.rowptr[d] = d;
  sop_bind(s, mode, std::move(M), r, nr, std::move(sp));
  TTN_API_END
}
int ttn_sop_bind_csr(ttn_sop* s, int mode, const int* rowptr, const int* colind, const double* vals, const int* r,
                     int nr) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && rowptr && mode >= 0 && mode < s->H.nmodes, TTN_EINVAL, "bad argument");
  int d = s->H.mode_dim[mode];
  TTN_REQUIRE(rowptr[0] == 0, TTN_EINVAL, "CSR row pointers must start at 0");
  for (int i = 0; i < d; ++i) TTN_REQUIRE(rowptr[i + 1] >= rowptr[i], TTN_EINVAL, "CSR row pointers must not decrease");
  std::vector<ttn::cd> M((size_t)d * d, 0.0);
  ttn::SparseOp sp;
  sp.rowptr.assign(rowptr, rowptr + d + 1);
  for (int i = 0; i < d; ++i)
    for (int q = rowptr[i]; q < rowptr[i + 1]; ++q) {
      TTN_REQUIRE(colind && vals && colind[q] >= 0 && colind[q] < d, TTN_EINVAL, "CSR column out of range");
      M[(size_t)i * d + colind[q]] += ttn::cd(vals[2 * q], vals[2 * q + 1]);
      sp.colind.push_back(colind[q]);
      sp.val.push_back(ttn::cd(vals[2 * q], vals[2 * q + 1]));
    }
  sop_bind(s, mode, std::move(M), r, nr, std::move(sp));
  TTN_API_END
}
int ttn_sop_set_coeff(ttn_sop* s, int r, double re, double im) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && r >= 0 && r < s->H.nterms, TTN_EINVAL, "term index out of range");
  TTN_REQUIRE(std::isfinite(re) && std::isfinite(im), TTN_EINVAL, "non-finite coefficient");
  s->H.coeff[r] = ttn::cd(re, im);
  TTN_API_END
}

int ttn_state_create(const ttn_tree* t, int device, ttn_state** out) {
  TTN_API_BEGIN
  TTN_REQUIRE(t && out, TTN_EINVAL, "null argument");
  CK(cudaSetDevice(device));
  auto* s = new ttn_state();
  try {
    s->T = t->T;
    s->device = device;
    s->off.resize(t->T.n + 1);
    size_t o = 0;
    for (int i = 0; i < t->T.n; ++i) {
      s->off[i] = o;
      o += ttn::align256((size_t)t->T.size(i) * sizeof(double2)) / sizeof(double2);
    }
    s->off[t->T.n] = o;
    s->arena.alloc(o * sizeof(double2));
    CK(cudaMemset(s->arena.p, 0, s->arena.bytes));
  } catch (...) {
    delete s;
    throw;
  }
  *out = s;
  TTN_API_END
}
int ttn_state_destroy(ttn_state* s) { delete s; return TTN_OK; }
int ttn_state_upload_node(ttn_state* s, int node, const double* data) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && data && node >= 0 && node < s->T.n, TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(s->device));
  CK(cudaMemcpy(s->node(node), data, s->T.size(node) * sizeof(double2), cudaMemcpyHostToDevice));
  TTN_API_END
}
int ttn_state_download_node(ttn_state* s, int node, double* data) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && data && node >= 0 && node < s->T.n, TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(s->device));
  CK(cudaMemcpy(data, s->node(node), s->T.size(node) * sizeof(double2), cudaMemcpyDeviceToHost));
  TTN_API_END
}
int ttn_state_upload(ttn_state* s, const double* data) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && data, TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(s->device));
  size_t o = 0;
  for (int i = 0; i < s->T.n; ++i) {
    CK(cudaMemcpy(s->node(i), data + 2 * o, s->T.size(i) * sizeof(double2), cudaMemcpyHostToDevice));
    o += s->T.size(i);
  }
  TTN_API_END
}
int ttn_state_download(ttn_state* s, double* data) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && data, TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(s->device));
  size_t o = 0;
  for (int i = 0; i < s->T.n; ++i) {
    CK(cudaMemcpy(data + 2 * o, s->node(i), s->T.size(i) * sizeof(double2), cudaMemcpyDeviceToHost));
    o += s->T.size(i);
  }
  TTN_API_END
}

// The spin-boson driver's start state, src/spin_boson.cpp:584-649.
int ttn_state_init_product(ttn_state* s, const double* psi0, unsigned int seed) {
  TTN_API_BEGIN
  TTN_REQUIRE(s, TTN_EINVAL, "null state");
  const ttn::Tree& T = s->T;
  std::mt19937 rng(seed);
  std::vector<double> host;
  for (int i = 0; i < T.n; ++i) {
    const long long d = T.dimen[i];
    const int r = T.hrank[i];
    std::vector<ttn::cd> A((size_t)d * r, 0.0);
    if (T.leaf(i)) {
      std::vector<std::vector<ttn::cd>> ct(r, std::vector<ttn::cd>(d, 0.0));
      if (T.leaf_mode[i] == 0 && psi0) {
        for (long long j = 0; j < d; ++j) ct[0][j] = ttn::cd(psi0[2 * j], psi0[2 * j + 1]);
      } else {
        ct[0][0] = 1.0;
      }
      std::uniform_real_distribution<double> dist(0, 2.0 * std::acos(-1.0));
      std::normal_distribution<double> length_dist(0, 1);
      for (int k = 1; k < r; ++k) {
        bool done = false;
        while (!done) {
          for (long long j = 0; j < d; ++j) {
            double theta = dist(rng);
            ct[k][j] = length_dist(rng) * ttn::cd(std::cos(theta), std::sin(theta));
          }
          ttn::cd nn = 0.0;
          for (auto& z : ct[k]) nn += std::conj(z) * z;
          ttn::cd sn = std::sqrt(nn);
          for (auto& z : ct[k]) z /= sn;
          for (int q = 0; q < k; ++q) {
            ttn::cd dp = 0.0;
            for (long long j = 0; j < d; ++j) dp += std::conj(ct[q][j]) * ct[k][j];
            for (long long j = 0; j < d; ++j) ct[k][j] -= dp * ct[q][j];
          }
          double norm = 0.0;
          for (auto& z : ct[k]) norm += (std::conj(z) * z).real();
          norm = std::sqrt(norm);
          if (norm > 1e-12) {
            for (auto& z : ct[k]) z /= norm;
            done = true;
          }
        }
      }
      for (long long j = 0; j < d; ++j)
        for (int k = 0; k < r; ++k) A[(size_t)j * r + k] = ct[k][j];
    } else if (i != 0) {
      for (long long j = 0; j < d; ++j)
        for (int k = 0; k < r; ++k) A[(size_t)j * r + k] = (j == k) ? 1.0 : 0.0;
    } else {
      A[0] = 1.0;
    }
    for (auto& z : A) { host.push_back(z.real()); host.push_back(z.imag()); }
  }
  int rc = ttn_state_upload(s, host.data());
  if (rc != TTN_OK) return rc;
  TTN_API_END
}

int ttn_integrator_create(const ttn_tree* t, const ttn_sop* h, const ttn_integ_cfg* cfg, ttn_integrator** out) {
  TTN_API_BEGIN
  TTN_REQUIRE(t && h && cfg && out, TTN_EINVAL, "null argument");
  TTN_REQUIRE(cfg->krylov_dim >= 2 && cfg->krylov_dim <= ttn::kKrylovMax, TTN_EINVAL, "krylov_dim must be in [2, 64]");
  TTN_REQUIRE(cfg->krylov_tol > 0.0, TTN_EINVAL, "krylov_tol must be positive");
  TTN_REQUIRE(cfg->precision == TTN_PREC_FP64 || cfg->precision == TTN_PREC_MIXED, TTN_EINVAL, "unknown precision");
  TTN_REQUIRE(h->H.nmodes == t->T.nleaves, TTN_EINVAL, "operator and tree disagree on the number of modes");
  for (int m = 0; m < h->H.nmodes; ++m)
    TTN_REQUIRE(h->H.mode_dim[m] == t->T.leaf_dim[t->T.mode_node[m]], TTN_EINVAL, "operator and tree disagree on a mode dimension");
  auto* it = new ttn_integrator();
  try {
    it->I.T = t->T;
    it->I.H = h->H;
    it->I.cfg = *cfg;
    it->I.device = cfg->device;
    it->I.setup();
  } catch (...) {
    delete it;
    throw;
  }
  *out = it;
  TTN_API_END
}
int ttn_integrator_destroy(ttn_integrator* it) { delete it; return TTN_OK; }
int ttn_integrator_set_dt(ttn_integrator* it, double dt) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && std::isfinite(dt) && dt > 0.0, TTN_EINVAL, "dt must be positive");
  it->I.dt = dt;
  TTN_API_END
}
int ttn_integrator_dt(const ttn_integrator* it, double* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && out, TTN_EINVAL, "null argument");
  *out = it->I.dt;
  TTN_API_END
}
int ttn_integrator_t(const ttn_integrator* it, double* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && out, TTN_EINVAL, "null argument");
  *out = it->I.dt * it->I.nsteps;
  TTN_API_END
}
int ttn_integrator_step(ttn_integrator* it, ttn_state* psi, double cre, double cim, double* dt_out) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi, TTN_EINVAL, "null argument");
  TTN_REQUIRE(it->I.dt > 0.0, TTN_EINVAL, "set dt before stepping");
  ttn::check_same_tree(it->I.T, psi->T);
  CK(cudaSetDevice(it->I.device));
  double dt = it->I.dt;
  it->I.step(psi, dt, ttn::cd(cre, cim));
  if (dt_out) *dt_out = dt;
  TTN_API_END
}
int ttn_batch_step(ttn_integrator* const* its, ttn_state* const* states, int n, double cre, double cim, int threads,
                   int* failed) {
  TTN_API_BEGIN
  TTN_REQUIRE(its && states && n >= 0, TTN_EINVAL, "null argument");
  if (failed) *failed = -1;
  if (n == 0) return TTN_OK;
  for (int k = 0; k < n; ++k) {
    TTN_REQUIRE(its[k] && states[k], TTN_EINVAL, "null instance");
    for (int q = 0; q < k; ++q)
      TTN_REQUIRE(its[q] != its[k] && states[q] != states[k], TTN_EINVAL,
                  "instances must use distinct integrators and states");
  }
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  nt = std::max(1, std::min(nt, n));
  std::atomic<int> next{0};
  std::vector<int> rc(n, TTN_OK);
  std::vector<std::string> msg(n);
  // every worker steps whole instances (each integrator has its own stream, so instances
  // run concurrently on the device and their kernel launches are issued in parallel)
  auto work = [&]() {
    for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
      rc[k] = ttn_integrator_step(its[k], states[k], cre, cim, nullptr);
      if (rc[k] != TTN_OK) msg[k] = ttn::g_err;
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < nt; ++w) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  for (int k = 0; k < n; ++k)
    if (rc[k] != TTN_OK) {
      if (failed) *failed = k;
      throw ttn::Err(rc[k], "instance " + std::to_string(k) + ": " + msg[k]);
    }
  TTN_API_END
}
int ttn_integrator_nh_applications(const ttn_integrator* it, long long* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && out, TTN_EINVAL, "null argument");
  *out = it->I.nh;
  TTN_API_END
}
int ttn_integrator_set_krylov_stop(ttn_integrator* it, int mode) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && (mode == 0 || mode == 1), TTN_EINVAL, "Krylov stop rule: 0 (full space) or 1 (residual)");
  it->I.krylov_stop = mode;
  TTN_API_END
}
int ttn_state_orthogonalise(ttn_integrator* it, ttn_state* psi) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi, TTN_EINVAL, "null argument");
  TTN_REQUIRE(psi->T.n == it->I.T.n, TTN_EINVAL, "state and integrator trees differ");
  for (int i = 0; i < it->I.T.n; ++i)
    TTN_REQUIRE(psi->T.hrank[i] == it->I.T.hrank[i] && psi->T.dimen[i] == it->I.T.dimen[i], TTN_EINVAL,
                "state and integrator trees differ");
  it->I.orthogonalise(psi);
  it->I.finish_check(psi);
  TTN_API_END
}
int ttn_integrator_expansion_counts(const ttn_integrator* it, long long* onesite, long long* twosite) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && onesite && twosite, TTN_EINVAL, "null argument");
  *onesite = it->X ? it->X->n_onesite : 0;
  *twosite = it->X ? it->X->n_twosite : 0;
  TTN_API_END
}
// ---- checkpoints: integrator scalars and the state in one little-endian file
namespace {
const char kCkptMagic[8] = {'T', 'T', 'N', 'C', 'K', 'P', 'T', '1'};
struct FileCloser {
  FILE* f;
  ~FileCloser() { if (f) std::fclose(f); }
};
void put_raw(FILE* f, const void* p, size_t elem, size_t n) {
  TTN_REQUIRE(std::fwrite(p, elem, n, f) == n, TTN_EINVAL, "checkpoint: write failed");
}
void get_raw(FILE* f, void* p, size_t elem, size_t n) {
  TTN_REQUIRE(std::fread(p, elem, n, f) == n, TTN_EINVAL, "checkpoint: truncated file");
}
#define CKPT_PUT(f, p, n) put_raw(f, p, sizeof(*(p)), n)
#define CKPT_GET(f, p, n) get_raw(f, p, sizeof(*(p)), n)
}  // namespace
int ttn_integrator_save(ttn_integrator* it, ttn_state* psi, const char* path) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi && path, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  ttn::Integrator& I = it->I;
  CK(cudaSetDevice(I.device));
  CK(cudaStreamSynchronize(I.stream));
  FileCloser fc{std::fopen(path, "wb")};
  TTN_REQUIRE(fc.f, TTN_EINVAL, std::string("checkpoint: cannot open ") + path);
  CKPT_PUT(fc.f, kCkptMagic, 8);
  const int n = I.T.n;
  CKPT_PUT(fc.f, &n, 1);
  CKPT_PUT(fc.f, I.T.parent.data(), n);
  CKPT_PUT(fc.f, I.T.hrank.data(), n);
  CKPT_PUT(fc.f, I.T.leaf_mode.data(), n);
  CKPT_PUT(fc.f, I.T.leaf_dim.data(), n);
  const long long nsteps = I.nsteps, nh = I.nh;
  const double sc[3] = {I.dt, I.t_engine, I.coeff.real()};
  const double ci = I.coeff.imag();
  CKPT_PUT(fc.f, &nsteps, 1);
  CKPT_PUT(fc.f, &nh, 1);
  CKPT_PUT(fc.f, sc, 3);
  CKPT_PUT(fc.f, &ci, 1);
  for (int i = 0; i < n; ++i) {
    std::vector<double2> h((size_t)psi->T.size(i));
    CK(cudaMemcpyAsync(h.data(), psi->node(i), h.size() * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
    CK(cudaStreamSynchronize(I.stream));
    CKPT_PUT(fc.f, h.data(), h.size());
  }
  TTN_API_END
}
int ttn_integrator_load(ttn_integrator* it, ttn_state* psi, const char* path) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi && path, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  ttn::Integrator& I = it->I;
  TTN_REQUIRE(!it->X, TTN_EINVAL, "checkpoint: not supported with subspace expansion");
  CK(cudaSetDevice(I.device));
  FileCloser fc{std::fopen(path, "rb")};
  TTN_REQUIRE(fc.f, TTN_EINVAL, std::string("checkpoint: cannot open ") + path);
  char magic[8];
  CKPT_GET(fc.f, magic, 8);
  TTN_REQUIRE(std::memcmp(magic, kCkptMagic, 8) == 0, TTN_EINVAL, "checkpoint: not a checkpoint file");
  int n = 0;
  CKPT_GET(fc.f, &n, 1);
  TTN_REQUIRE(n == I.T.n, TTN_EINVAL, "checkpoint: different tree");
  std::vector<int> a(n);
  for (const std::vector<int>* want : {&I.T.parent, &I.T.hrank, &I.T.leaf_mode, &I.T.leaf_dim}) {
    CKPT_GET(fc.f, a.data(), n);
    TTN_REQUIRE(a == *want, TTN_EINVAL, "checkpoint: different tree");
  }
  long long nsteps = 0, nh = 0;
  double sc[3], ci = 0.0;
  CKPT_GET(fc.f, &nsteps, 1);
  CKPT_GET(fc.f, &nh, 1);
  CKPT_GET(fc.f, sc, 3);
  CKPT_GET(fc.f, &ci, 1);
  for (int i = 0; i < n; ++i) {
    std::vector<double2> h((size_t)psi->T.size(i));
    CKPT_GET(fc.f, h.data(), h.size());
    for (const double2& z : h) TTN_REQUIRE(std::isfinite(z.x) && std::isfinite(z.y), TTN_EINVAL, "checkpoint: non-finite tensor");
    CK(cudaMemcpyAsync(psi->node(i), h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
    CK(cudaStreamSynchronize(I.stream));
  }
  I.nsteps = nsteps;
  I.nh = nh;
  I.dt = sc[0];
  I.t_engine = sc[1];
  I.coeff = ttn::cd(sc[2], ci);
  // the single-particle environments the next step carries in: consistent with the state
  // (each was last written from its node's final tensor), so recomputed bottom-up they
  // equal the saved run's
  if (nsteps > 0)
    for (int id = I.T.n - 1; id >= 1; --id) I.update_spf(id, psi->node(id));
  CK(cudaMemcpyAsync(I.nh_dev, &nh, sizeof(long long), cudaMemcpyHostToDevice, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  TTN_API_END
}
#undef CKPT_PUT
#undef CKPT_GET
int ttn_integrator_reset(ttn_integrator* it) {
  TTN_API_BEGIN
  TTN_REQUIRE(it, TTN_EINVAL, "null argument");
  it->I.nsteps = 0;
  it->I.nh = 0;
  CK(cudaMemset(it->I.nh_dev, 0, sizeof(long long)));
  TTN_API_END
}
int ttn_integrator_synchronize(ttn_integrator* it) {
  TTN_API_BEGIN
  TTN_REQUIRE(it, TTN_EINVAL, "null argument");
  CK(cudaStreamSynchronize(it->I.stream));
  TTN_API_END
}

int ttn_expect_leaf(ttn_integrator* it, ttn_state* psi, int mode, const double* op, double* re, double* im) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  CK(cudaSetDevice(it->I.device));
  const double2* dop = nullptr;
  if (op) {
    TTN_REQUIRE(mode >= 0 && mode < it->I.H.nmodes, TTN_EINVAL, "mode out of range");
    int d = it->I.H.mode_dim[mode];
    TTN_REQUIRE((long long)d * d <= it->I.ldv, TTN_ECAPACITY, "observable operator larger than the work buffer");
    CK(cudaMemcpyAsync(it->I.w3, op, (size_t)d * d * sizeof(double2), cudaMemcpyHostToDevice, it->I.stream));
    it->I.h2d_bytes += (long long)d * d * sizeof(double2);
    dop = it->I.w3;
  }
  ttn::cd v = it->I.expect(psi, mode, dop);
  if (re) *re = v.real();
  if (im) *im = v.imag();
  TTN_API_END
}
// dense operators uploaded for one call: ops[k] (d_k x d_k interleaved) on modes[k]
static std::vector<const double2*> upload_ops(ttn::Integrator& I, ttn::DevBuf& buf, int nops, const int* modes,
                                              const double* ops) {
  std::vector<const double2*> by_mode(I.H.nmodes, nullptr);
  size_t total = 0;
  for (int k = 0; k < nops; ++k) {
    TTN_REQUIRE(modes[k] >= 0 && modes[k] < I.H.nmodes, TTN_EINVAL, "mode out of range");
    TTN_REQUIRE(!by_mode[modes[k]], TTN_EINVAL, "one operator per mode");
    by_mode[modes[k]] = reinterpret_cast<const double2*>(1);
    total += (size_t)I.H.mode_dim[modes[k]] * I.H.mode_dim[modes[k]];
  }
  std::fill(by_mode.begin(), by_mode.end(), nullptr);
  if (nops == 0) return by_mode;
  for (size_t i = 0; i < 2 * total; ++i) TTN_REQUIRE(std::isfinite(ops[i]), TTN_EINVAL, "non-finite operator entry");
  buf.alloc(total * sizeof(double2));
  CK(cudaMemcpyAsync(buf.p, ops, total * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  size_t off = 0;
  for (int k = 0; k < nops; ++k) {
    by_mode[modes[k]] = buf.as<double2>() + off;
    off += (size_t)I.H.mode_dim[modes[k]] * I.H.mode_dim[modes[k]];
  }
  return by_mode;
}
int ttn_overlap(ttn_integrator* it, ttn_state* bra, ttn_state* ket, double* re, double* im) {
  return ttn_expect_product(it, bra, ket, 0, nullptr, nullptr, re, im);
}
int ttn_expect_product(ttn_integrator* it, ttn_state* bra, ttn_state* ket, int nops, const int* modes, const double* ops,
                       double* re, double* im) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && bra && ket && nops >= 0 && (nops == 0 || (modes && ops)), TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, bra->T);
  ttn::check_same_tree(it->I.T, ket->T);
  CK(cudaSetDevice(it->I.device));
  ttn::DevBuf buf;
  const auto by_mode = upload_ops(it->I, buf, nops, modes, ops);
  const ttn::cd v = it->I.contract(bra, ket, by_mode);
  if (re) *re = v.real();
  if (im) *im = v.imag();
  TTN_API_END
}
int ttn_expect_sop(ttn_integrator* it, ttn_state* bra, ttn_state* ket, const ttn_sop* op, double* re, double* im) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && bra && ket && op, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, bra->T);
  ttn::check_same_tree(it->I.T, ket->T);
  const ttn::Sop& H = op->H;
  TTN_REQUIRE(H.nmodes == it->I.H.nmodes && H.mode_dim == it->I.H.mode_dim, TTN_EINVAL, "operator modes differ from the tree's");
  CK(cudaSetDevice(it->I.device));
  // every primitive operator on the device once, then one contraction per term
  size_t total = 0;
  for (int m = 0; m < H.nmodes; ++m)
    for (auto& M : H.ops[m]) total += M.size();
  ttn::DevBuf buf;
  buf.alloc(std::max<size_t>(total, 1) * sizeof(double2));
  std::vector<std::vector<const double2*>> dev(H.nmodes);
  {
    std::vector<double2> h(total);
    size_t off = 0;
    for (int m = 0; m < H.nmodes; ++m)
      for (auto& M : H.ops[m]) {
        dev[m].push_back(buf.as<double2>() + off);
        for (size_t i = 0; i < M.size(); ++i) h[off + i] = ttn::d2(M[i]);
        off += M.size();
      }
    CK(cudaMemcpyAsync(buf.p, h.data(), total * sizeof(double2), cudaMemcpyHostToDevice, it->I.stream));
    CK(cudaStreamSynchronize(it->I.stream));
  }
  ttn::cd sum = 0.0;
  std::vector<const double2*> by_mode(H.nmodes);
  for (int r = 0; r < H.nterms; ++r) {
    for (int m = 0; m < H.nmodes; ++m) by_mode[m] = H.opidx[m][r] >= 0 ? dev[m][H.opidx[m][r]] : nullptr;
    sum += H.coeff[r] * it->I.contract(bra, ket, by_mode);
  }
  if (re) *re = sum.real();
  if (im) *im = sum.imag();
  TTN_API_END
}
int ttn_bond_singular_values(ttn_integrator* it, ttn_state* psi, int node, double* out, int* n) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi && out, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  TTN_REQUIRE(node >= 1 && node < it->I.T.n, TTN_EINVAL, "node must name a bond (1 <= node < nodes)");
  CK(cudaSetDevice(it->I.device));
  const auto sv = it->I.bond_sv(psi, node);
  for (size_t k = 0; k < sv.size(); ++k) out[k] = sv[k];
  if (n) *n = (int)sv.size();
  TTN_API_END
}
int ttn_adjoint_grad(ttn_integrator* it, ttn_state* psi, double dt, double coeff_re, double coeff_im, int nsteps,
                     const double* weights, int mode, const double* op, int checkpoint_every, int skip_prepare,
                     double* J, double* grad_coeff, double* grad_ops, double* grad_state) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi && weights && op && J && grad_coeff && grad_ops, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  ttn::Integrator& I = it->I;
  TTN_REQUIRE(nsteps >= 1, TTN_EINVAL, "nsteps must be >= 1");
  TTN_REQUIRE(std::isfinite(dt) && dt > 0.0, TTN_EINVAL, "dt must be positive and finite");
  TTN_REQUIRE(mode >= 0 && mode < I.H.nmodes, TTN_EINVAL, "mode out of range");
  TTN_REQUIRE(!I.mixed, TTN_EINVAL, "the adjoint sweep needs an FP64 integrator (TTN_PREC_FP64)");
  TTN_REQUIRE(I.nsteps == 0, TTN_EINVAL, "the adjoint sweep starts from step 0 (a fresh or reset integrator)");
  TTN_REQUIRE(!it->X, TTN_EINVAL, "the adjoint sweep needs fixed bond dimensions (no subspace expansion)");
  TTN_REQUIRE(!I.krylov_stop, TTN_EINVAL, "the adjoint sweep uses the full Krylov space (Krylov stop rule 0)");
  TTN_REQUIRE(!I.op_update_fn, TTN_EINVAL, "the adjoint sweep needs time-independent operators");
  for (int k = 0; k < nsteps; ++k) TTN_REQUIRE(std::isfinite(weights[k]), TTN_EINVAL, "non-finite weight");
  CK(cudaSetDevice(I.device));
  const int d = I.H.mode_dim[mode];
  std::vector<double2> oh((size_t)d * d);
  for (size_t i = 0; i < oh.size(); ++i) {
    TTN_REQUIRE(std::isfinite(op[2 * i]) && std::isfinite(op[2 * i + 1]), TTN_EINVAL, "non-finite operator entry");
    oh[i] = make_double2(op[2 * i], op[2 * i + 1]);
  }
  ttn::DevBuf opd;
  opd.alloc(oh.size() * sizeof(double2));
  CK(cudaMemcpyAsync(opd.p, oh.data(), oh.size() * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  ttn::DevAdjoint adj(I, psi);
  *J = adj.run(dt, ttn::cd(coeff_re, coeff_im), nsteps, weights, mode, opd.as<double2>(), checkpoint_every,
               skip_prepare != 0);
  for (int r = 0; r < I.H.nterms; ++r) grad_coeff[r] = adj.gc[r];
  size_t off = 0;
  for (const auto& mk : I.H.op_order) {
    const auto& G = adj.gop[mk.first][mk.second];
    for (size_t i = 0; i < G.size(); ++i) {
      grad_ops[2 * (off + i)] = G[i].real();
      grad_ops[2 * (off + i) + 1] = G[i].imag();
    }
    off += G.size();
  }
  if (grad_state) {
    size_t o = 0;
    for (int i = 0; i < I.T.n; ++i) {
      const long long sz = I.T.size(i);
      CK(cudaMemcpyAsync(grad_state + 2 * o, adj.ab[i], sz * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
      o += sz;
    }
    CK(cudaStreamSynchronize(I.stream));
  }
  TTN_API_END
}
int ttn_integrator_set_expansion(ttn_integrator* it, ttn_state* psi, const int* capacity, double spawning_threshold,
                                 double unoccupied_threshold, int minimum_unoccupied, int neigenvalues,
                                 int only_when_no_unoccupied, unsigned seed) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi && capacity, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  ttn::Integrator& I = it->I;
  TTN_REQUIRE(I.nsteps == 0, TTN_EINVAL, "subspace expansion must be enabled before the first step");
  TTN_REQUIRE(!I.mixed, TTN_EINVAL, "subspace expansion needs an FP64 integrator (TTN_PREC_FP64)");
  TTN_REQUIRE(!it->X, TTN_EINVAL, "subspace expansion is already enabled");
  TTN_REQUIRE(neigenvalues >= 1 && minimum_unoccupied >= 0, TTN_EINVAL, "bad expansion parameters");
  TTN_REQUIRE(capacity[0] == I.T.hrank[0], TTN_EINVAL, "the root's rank does not grow (capacity[0] must equal it)");
  for (int i = 1; i < I.T.n; ++i)
    TTN_REQUIRE(capacity[i] >= I.T.hrank[i], TTN_EINVAL, "capacity below the current bond dimension");
  CK(cudaSetDevice(I.device));
  ttn::Tree Z;
  Z.build(I.T.n, I.T.parent.data(), capacity, I.T.leaf_mode.data(), I.T.leaf_dim.data());
  I.cap.assign(capacity, capacity + I.T.n);
  I.Tsz = Z;
  I.allocate_sized();
  I.compile_programs();
  // the state in slabs sized for the capacities (the tensors at the start of each slab)
  {
    std::vector<size_t> off(Z.n + 1);
    size_t o = 0;
    for (int i = 0; i < Z.n; ++i) {
      off[i] = o;
      o += ttn::align256((size_t)Z.size(i) * sizeof(double2)) / sizeof(double2);
    }
    off[Z.n] = o;
    ttn::DevBuf na;
    na.alloc(o * sizeof(double2));
    CK(cudaMemsetAsync(na.p, 0, na.bytes, I.stream));
    for (int i = 0; i < Z.n; ++i)
      CK(cudaMemcpyAsync(na.as<double2>() + off[i], psi->node(i), (size_t)psi->T.size(i) * sizeof(double2),
                         cudaMemcpyDeviceToDevice, I.stream));
    CK(cudaStreamSynchronize(I.stream));
    std::swap(psi->arena.p, na.p);
    std::swap(psi->arena.bytes, na.bytes);
    psi->off = off;
  }
  it->X.reset(new ttn::DevExpander(I));
  ttn::DevExpander* X = it->X.get();
  X->state = psi;
  X->spawning_threshold = spawning_threshold;
  X->unoccupied_threshold = unoccupied_threshold;
  X->minimum_unoccupied = minimum_unoccupied;
  X->neigenvalues = neigenvalues;
  X->only_when_no_unoccupied = only_when_no_unoccupied != 0;
  X->rng.seed(seed);
  I.expanding_step = [X](ttn_state* S, double dt, ttn::cd cf) { X->step(S, dt, cf); };
  TTN_API_END
}
int ttn_integrator_set_op_update(ttn_integrator* it, ttn_op_update_fn fn, void* user) {
  TTN_API_BEGIN
  TTN_REQUIRE(it, TTN_EINVAL, "null argument");
  ttn::Integrator& I = it->I;
  TTN_REQUIRE(!fn || !I.mixed, TTN_EINVAL, "time-dependent operators need an FP64 integrator");
  const bool recompile = (I.op_update_fn == nullptr) != (fn == nullptr);
  I.op_update_fn = fn;
  I.op_update_user = user;
  if (recompile) I.compile_programs();  // sparse leaf copies are used only without the hook
  I.op_global.assign(I.H.nmodes, {});
  for (int m = 0; m < I.H.nmodes; ++m) I.op_global[m].assign(I.H.ops[m].size(), -1);
  for (size_t g = 0; g < I.H.op_order.size(); ++g) I.op_global[I.H.op_order[g].first][I.H.op_order[g].second] = (int)g;
  TTN_API_END
}
int ttn_state_hrank(const ttn_state* s, int* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(s && out, TTN_EINVAL, "null argument");
  for (int i = 0; i < s->T.n; ++i) out[i] = s->T.hrank[i];
  TTN_API_END
}
int ttn_norm2(ttn_integrator* it, ttn_state* psi, double* out) {
  double re = 0, im = 0;
  int rc = ttn_expect_leaf(it, psi, 0, nullptr, &re, &im);
  if (rc == TTN_OK && out) *out = re;
  return rc;
}

int ttn_integrator_prepare(ttn_integrator* it, ttn_state* psi) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  CK(cudaSetDevice(it->I.device));
  if (it->X) {
    // prepare_evolution with subspace expansion: the expansion half-sweeps use dt
    TTN_REQUIRE(psi == it->X->state, TTN_EINVAL, "with subspace expansion, prepare the state given to ttn_integrator_set_expansion");
    TTN_REQUIRE(it->I.dt > 0.0, TTN_EINVAL, "set dt before preparing an expanding integrator");
    it->X->prepare(psi);
    it->I.nsteps = std::max<long long>(it->I.nsteps, 1);
    it->I.finish_check(psi);
  } else {
    it->I.prepare_only(psi);
  }
  TTN_API_END
}
int ttn_integrator_flops(const ttn_integrator* it, double* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && out, TTN_EINVAL, "null argument");
  *out = it->I.flops;
  TTN_API_END
}
int ttn_integrator_timer(ttn_integrator* it, int start, double* ms) {
  TTN_API_BEGIN
  TTN_REQUIRE(it, TTN_EINVAL, "null argument");
  CK(cudaSetDevice(it->I.device));
  if (start) {
    CK(cudaEventRecord(it->I.ev0, it->I.stream));
  } else {
    CK(cudaEventRecord(it->I.ev1, it->I.stream));
    CK(cudaEventSynchronize(it->I.ev1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, it->I.ev0, it->I.ev1));
    if (ms) *ms = f;
  }
  TTN_API_END
}
int ttn_bench_node_op(ttn_integrator* it, ttn_state* psi, int node, int kind, int reps, double* ms_per_rep,
                      double* flops_per_rep) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi && reps >= 1, TTN_EINVAL, "bad argument");
  auto& I = it->I;
  TTN_REQUIRE(node >= 0 && node < I.T.n, TTN_EINVAL, "node out of range");
  ttn::check_same_tree(I.T, psi->T);
  CK(cudaSetDevice(I.device));
  const long long n = I.T.size(node);
  double f0 = I.flops;
  ttn::zcopy(I.w4, psi->node(node), n, I.stream);
  auto run = [&]() {
    switch (kind) {
      case 0: I.heff(node, psi->node(node), I.p); break;
      case 1: {
        ttn::zcopy(I.w4, psi->node(node), n, I.stream);
        I.expm_dev(node, 0, I.w4, n, I.dt > 0 ? I.dt / 2 : 0.01, ttn::cd(0.0, -1.0), false, false);
        break;
      }
      case 3: {
        const long long rr = (long long)I.T.hrank[node] * I.T.hrank[node];
        ttn::zcopy(I.w4, I.rmat[node], rr, I.stream);
        I.expm_dev(node, 1, I.w4, rr, I.dt > 0 ? -I.dt / 2 : -0.01, ttn::cd(0.0, -1.0), false, false);
        break;
      }
      case 2: {
        ttn::zcopy(I.w4, psi->node(node), n, I.stream);
        I.flops += I.qr_flops((double)I.T.dimen[node], (double)I.T.hrank[node]);
        I.qr(I.w4, I.T.dimen[node], I.T.hrank[node], I.w3, 0);
        break;
      }
      default: throw ttn::Err(TTN_EINVAL, "unknown benchmark kind");
    }
  };
  run();  // warm-up
  CK(cudaStreamSynchronize(I.stream));
  f0 = I.flops;
  CK(cudaEventRecord(I.ev0, I.stream));
  for (int k = 0; k < reps; ++k) run();
  CK(cudaEventRecord(I.ev1, I.stream));
  CK(cudaEventSynchronize(I.ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, I.ev0, I.ev1));
  CK(cudaGetLastError());
  double fl = (I.flops - f0) / reps;
  if (kind == 1 || kind == 3) {
    // the persistent kernel's matvecs: H applications of the last repetition times the
    // flops of one application, plus the Lanczos vector passes already counted
    long long k = 0;
    int subs = 0;
    CK(cudaMemcpy(&k, &I.ctl->napps, sizeof(long long), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&subs, &I.ctl->substeps, sizeof(int), cudaMemcpyDeviceToHost));
    const long long nn = (kind == 1) ? n : (long long)I.T.hrank[node] * I.T.hrank[node];
    fl = I.lanczos_vec_flops(nn) * (subs > 0 ? subs : 1) + (double)k * (kind == 1 ? I.heff_flops(node) : I.kbond_flops(node));
  }
  if (ms_per_rep) *ms_per_rep = ms / reps;
  if (flops_per_rep) *flops_per_rep = fl;
  I.flops = f0;
  TTN_API_END
}
int ttn_integrator_set_profiling(ttn_integrator* it, int on) {
  TTN_API_BEGIN
  TTN_REQUIRE(it, TTN_EINVAL, "null argument");
  CK(cudaSetDevice(it->I.device));
  CK(cudaStreamSynchronize(it->I.stream));
  it->I.profiling = on != 0;
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 4; ++c) {
      it->I.prof_t[k][c] = 0.0;
      it->I.prof_n[k][c] = 0;
    }
  TTN_API_END
}
int ttn_integrator_profile(ttn_integrator* it, double* seconds, long long* counts) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && seconds && counts, TTN_EINVAL, "null argument");
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 4; ++c) {
      seconds[k * 4 + c] = it->I.prof_t[k][c];
      counts[k * 4 + c] = it->I.prof_n[k][c];
    }
  TTN_API_END
}
int ttn_integrator_io_bytes(const ttn_integrator* it, long long* h2d, long long* d2h) {
  TTN_API_BEGIN
  TTN_REQUIRE(it, TTN_EINVAL, "null argument");
  if (h2d) *h2d = it->I.h2d_bytes;
  if (d2h) *d2h = it->I.d2h_bytes;
  TTN_API_END
}
int ttn_host_alloc(long long bytes, void** out) {
  TTN_API_BEGIN
  TTN_REQUIRE(out && bytes > 0, TTN_EINVAL, "bad argument");
  CK(cudaMallocHost(out, (size_t)bytes));
  TTN_API_END
}
int ttn_host_free(void* p) {
  TTN_API_BEGIN
  if (p) CK(cudaFreeHost(p));
  TTN_API_END
}
int ttn_launch_count(unsigned long long* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(out, TTN_EINVAL, "null argument");
  *out = ttn::g_launches.load();
  TTN_API_END
}
int ttn_device_fp64_peak(int device, double* tflops) {
  TTN_API_BEGIN
  TTN_REQUIRE(tflops, TTN_EINVAL, "null argument");
  CK(cudaSetDevice(device));
  *tflops = ttn::measure_fp64_fma_tflops();
  TTN_API_END
}

int ttn_debug_refresh_env(ttn_integrator* it, ttn_state* psi) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && psi, TTN_EINVAL, "null argument");
  ttn::check_same_tree(it->I.T, psi->T);
  CK(cudaSetDevice(it->I.device));
  auto& I = it->I;
  for (int id = I.T.n - 1; id >= 1; --id) I.update_spf(id, psi->node(id));
  for (int id = 1; id < I.T.n; ++id) I.update_mf(id, psi->node(I.T.parent[id]));
  CK(cudaStreamSynchronize(I.stream));
  CK(cudaGetLastError());
  TTN_API_END
}
int ttn_debug_heff(ttn_integrator* it, int node, const double* v, double* out) {
  TTN_API_BEGIN
  auto& I = it->I;
  TTN_REQUIRE(node >= 0 && node < I.T.n && v && out, TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(I.device));
  const long long n = I.T.size(node);
  CK(cudaMemcpyAsync(I.V, v, n * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
  I.heff(node, I.V, I.p);
  CK(cudaMemcpyAsync(out, I.p, n * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  CK(cudaGetLastError());
  TTN_API_END
}
int ttn_debug_expm_node(ttn_integrator* it, int node, double tau, double cre, double cim, double* v, long long* napps) {
  TTN_API_BEGIN
  auto& I = it->I;
  TTN_REQUIRE(node >= 0 && node < I.T.n && v, TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(I.device));
  const long long n = I.T.size(node);
  CK(cudaMemcpyAsync(I.w4, v, n * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
  // w4 is a gauge scratch; the exponential itself uses V, p, w1-w3
  long long k = 0;
  I.expm_dev(node, 0, I.w4, n, tau, ttn::cd(cre, cim), false, false);
  CK(cudaMemcpyAsync(v, I.w4, n * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
  CK(cudaMemcpyAsync(&k, &I.ctl->napps, sizeof(long long), cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  int h = 0;
  CK(cudaMemcpy(&h, I.status, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemset(I.status, 0, sizeof(int)));
  TTN_REQUIRE(h == 0, TTN_ENUMERIC, "Krylov exponential failed on the device");
  if (napps) *napps = (tau == 0.0) ? 0 : k;
  TTN_API_END
}
int ttn_integrator_kernel_phases(ttn_integrator* it, double* out) {
  TTN_API_BEGIN
  auto& I = it->I;
  TTN_REQUIRE(out, TTN_EINVAL, "null output");
  for (int k = 0; k < ttn::kPhases; ++k) out[k] = 0.0;
  if (!I.phase_dev) return TTN_OK;
  CK(cudaSetDevice(I.device));
  CK(cudaStreamSynchronize(I.stream));
  unsigned long long h[ttn::kPhases];
  CK(cudaMemcpy(h, I.phase_dev, sizeof(h), cudaMemcpyDeviceToHost));
  CK(cudaMemset(I.phase_dev, 0, sizeof(h)));
  for (int k = 0; k < ttn::kPhases; ++k) out[k] = (k < 8 || (k >= 10 && k < 14) || k == 15) ? 1e-6 * (double)h[k] : (double)h[k];
  TTN_API_END
}
int ttn_debug_program_apply(ttn_integrator* it, int node, int kind, const double* v, double* out) {
  TTN_API_BEGIN
  auto& I = it->I;
  TTN_REQUIRE(node >= 0 && node < I.T.n && v && out && (kind == 0 || kind == 1), TTN_EINVAL, "bad argument");
  CK(cudaSetDevice(I.device));
  const long long n = kind == 0 ? I.T.size(node) : (long long)I.T.hrank[node] * I.T.hrank[node];
  CK(cudaMemcpyAsync(I.w4, v, n * sizeof(double2), cudaMemcpyHostToDevice, I.stream));
  I.expm_dev(node, kind, I.w4, n, 0.0, ttn::cd(0.0, -1.0), false, false, true);
  CK(cudaMemcpyAsync(out, I.p, n * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  CK(cudaGetLastError());
  int h = 0;
  CK(cudaMemcpy(&h, I.status, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemset(I.status, 0, sizeof(int)));
  TTN_REQUIRE(h == 0, TTN_ETIMEOUT, "program application reported a device-side wait failure");
  TTN_API_END
}
int ttn_debug_num_groups(ttn_integrator* it, int node, int* out) {
  TTN_API_BEGIN
  TTN_REQUIRE(it && out && node >= 0 && node < it->I.T.n, TTN_EINVAL, "bad argument");
  *out = (int)it->I.G[node].size();
  TTN_API_END
}
int ttn_debug_get_env(ttn_integrator* it, int node, int group, int which, double* out) {
  TTN_API_BEGIN
  auto& I = it->I;
  TTN_REQUIRE(node >= 0 && node < I.T.n && group >= 0 && group < (int)I.G[node].size() && out, TTN_EINVAL, "bad argument");
  const auto& g = I.G[node][group];
  const double2* p = which == 0 ? g.spf_dev : g.mf_dev;
  TTN_REQUIRE(p, TTN_EINVAL, "that environment matrix is the identity");
  const int r = I.T.hrank[node];
  CK(cudaMemcpyAsync(out, p, (size_t)r * r * sizeof(double2), cudaMemcpyDeviceToHost, I.stream));
  CK(cudaStreamSynchronize(I.stream));
  TTN_API_END
}
int ttn_debug_tc_gemm(const double* A, const double* B, double* D, int K, int N, int device) {
  TTN_API_BEGIN
  TTN_REQUIRE(A && B && D, TTN_EINVAL, "null argument");
  TTN_REQUIRE(K >= 8 && K % 8 == 0 && N >= 16 && N <= 256 && N % 16 == 0, TTN_EINVAL, "bad tensor-core test shape");
  TTN_REQUIRE((size_t)2 * (128 + N) * K * 4 <= 196608, TTN_EINVAL, "operands do not fit in shared memory");
  CK(cudaSetDevice(device));
  ttn::DevBuf buf;
  size_t na = (size_t)128 * K, nb = (size_t)N * K, nd = (size_t)128 * N;
  buf.alloc((na + nb + nd) * sizeof(double) + 256);
  double* dA = buf.as<double>();
  double* dB = dA + na;
  double* dD = dB + nb;
  int* derr = (int*)(dD + nd);
  CK(cudaMemcpy(dA, A, na * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dB, B, nb * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemset(derr, 0, sizeof(int)));
  CK(ttn::tc_gemm_test(dA, dB, dD, K, N, derr, 0));
  CK(cudaDeviceSynchronize());
  int herr = 0;
  CK(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost));
  TTN_REQUIRE(herr == 0, TTN_ETIMEOUT, "tensor-core test: MMA completion wait gave up");
  CK(cudaMemcpy(D, dD, nd * sizeof(double), cudaMemcpyDeviceToHost));
  TTN_API_END
}
static int debug_qr_impl(int m, int n, double* a, double* r, int device, double* phases) {
  TTN_API_BEGIN
  TTN_REQUIRE(a && r && m >= n && n >= 1 && n <= ttn::kMaxBond, TTN_EINVAL, "bad QR shape");
  CK(cudaSetDevice(device));
  ttn::DevBuf buf;
  buf.alloc(((size_t)m * n + (size_t)n * n + ttn::kMaxBond) * sizeof(double2));
  double2* dA = buf.as<double2>();
  double2* dR = dA + (size_t)m * n;
  double2* dt = dR + (size_t)n * n;
  CK(cudaMemcpy(dA, a, (size_t)m * n * sizeof(double2), cudaMemcpyHostToDevice));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  // the sweep's choice: the shared-memory kernel (8 rows per CTA, one CTA up to 64 rows)
  // when the grid holds every row, else the panel-blocked kernel
  long long target = 8;
  if (const char* e = std::getenv("TTN_QR_ROWS_TARGET")) target = std::max(1, std::atoi(e));
  const long long cap = ttn::qr_rows_max_rows(n);
  long long gr = m <= cap ? 1 : (m + target - 1) / target;
  gr = std::min<long long>(gr, std::max(1, std::min(ttn::qr_rows_max_grid(), sms)));
  const bool rows = cap > 0 && (m + gr - 1) / gr <= cap;
  int g = rows ? (int)gr : std::min(ttn::coop_qr_grid(m, sms), std::max(1, std::min(ttn::qr_blocked_max_grid(), sms)));
  const size_t sb = rows ? ttn::qr_rows_scratch_bytes(g) : ttn::qr_blocked_scratch_bytes(g);
  ttn::DevBuf cb;
  cb.alloc(ttn::align256(sizeof(ttn::GridBarrier)) + ttn::align256(sb) + 256);
  CK(cudaMemset(cb.p, 0, cb.bytes));
  auto* bar = cb.as<ttn::GridBarrier>();
  double* scr = (double*)(cb.as<char>() + ttn::align256(sizeof(ttn::GridBarrier)));
  int* err = (int*)(cb.as<char>() + ttn::align256(sizeof(ttn::GridBarrier)) + ttn::align256(sb));
  unsigned long long* ph = nullptr;
  ttn::DevBuf pb;
  if (phases && rows) {
    pb.alloc(ttn::kQrPhases * sizeof(unsigned long long));
    CK(cudaMemset(pb.p, 0, pb.bytes));
    ph = pb.as<unsigned long long>();
  }
  if (rows) CK(ttn::householder_qr_rows(dA, m, n, dR, 0, dt, scr, bar, err, g, 0, ph));
  else CK(ttn::householder_qr_blocked(dA, m, n, dR, 0, dt, scr, bar, err, g, 0));
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  int herr = 0;
  CK(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
  TTN_REQUIRE(herr == 0, TTN_ETIMEOUT, "device QR barrier gave up waiting");
  CK(cudaGetLastError());
  CK(cudaMemcpy(a, dA, (size_t)m * n * sizeof(double2), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(r, dR, (size_t)n * n * sizeof(double2), cudaMemcpyDeviceToHost));
  if (phases) {
    unsigned long long h[ttn::kQrPhases] = {};
    if (ph) CK(cudaMemcpy(h, ph, sizeof(h), cudaMemcpyDeviceToHost));
    for (int k = 0; k < ttn::kQrPhases; ++k) phases[k] = (k == 8) ? (double)h[k] : 1e-3 * (double)h[k];
  }
  TTN_API_END
}
int ttn_debug_qr(int m, int n, double* a, double* r, int device) { return debug_qr_impl(m, n, a, r, device, nullptr); }
int ttn_debug_qr_phases(int m, int n, double* a, double* r, int device, double* phases) {
  return debug_qr_impl(m, n, a, r, device, phases);
}

}  // extern "C"
