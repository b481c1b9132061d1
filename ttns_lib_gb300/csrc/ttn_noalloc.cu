// ttn_qr_noalloc: the cooperative Householder QR on a matrix that already lives in the
// caller's device memory, with every byte of workspace taken from one file-scope device
// array instead of cudaMalloc.
//
// Who needs it: callers that cannot allocate device memory at the point where they
// factorise.  A host framework that hands all device memory out of its own pool (a
// caching allocator, or one arena shared by several solvers sized up front) must not
// have a library take and return memory behind its back, and cudaMalloc / cudaFree
// synchronise the whole device, which a caller that interleaves this call with work on
// other streams cannot afford.  Such a caller passes the matrix and R in memory it
// owns; the per-CTA partial norms and products, the Householder scalars, the
// grid-barrier state and the status word sit in g_qr_scratch below.
//
// Limits: n <= 64 columns (wider matrices are rejected with TTN_ECAPACITY); the grid is
// capped at kMaxGrid CTAs, which is what the array holds partials for.  The first call on
// a device looks up the array's address there (cudaGetSymbolAddress) and the launch
// limits; make that first call before any stream capture.  Every call shares the one
// array: calls whose kernels overlap on the GPU (two host threads, or two streams without
// an ordering between them) race on it.  Each call clears the barrier state and the
// status word before its launch; the rest of the workspace is written before it is read.
#include "ttn_gb300.h"
#include "ttn_coop.cuh"
#include "ttn_kernels.cuh"

#include <cuda_runtime.h>

#include <cstdint>
#include <exception>
#include <mutex>
#include <string>

namespace ttn {

void set_error_message(const std::string& msg);  // ttn_host.cpp: text of ttn_last_error()

namespace {

constexpr int kMaxGrid = 256;         // CTAs the workspace holds partials for
constexpr int kMaxDevices = 64;
// layout (bytes): [0, 256) barrier + status word (cleared by each call), [256, 1280) tau,
// [2048, ...) partials of the cooperative QR for up to kMaxGrid CTAs
constexpr size_t kZeroBytes = 256;
constexpr size_t kTauOffset = 256;
constexpr size_t kPartOffset = 2048;
constexpr size_t kPartBytes = (size_t)(4 * kMaxGrid + 4 + 4 * (size_t)kMaxGrid * kQrMaxCols) * sizeof(double);
constexpr size_t kScratchBytes = kPartOffset + kPartBytes;  // 534,560 bytes
static_assert(sizeof(GridBarrier) + sizeof(int) <= kZeroBytes, "barrier and status word exceed their slot");
static_assert(kTauOffset + kQrMaxCols * sizeof(double2) <= kPartOffset, "tau overlaps the partials");

__device__ __align__(256) static unsigned char g_qr_scratch[kScratchBytes];

struct DeviceSetup {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of g_qr_scratch on this device
  int max_grid = 1;               // co-resident CTAs of the cooperative QR
  int sms = 1;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

struct Fail {
  int code;
  std::string msg;
};

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Fail{TTN_ECUDA, std::string("ttn_qr_noalloc: ") + what + ": " + cudaGetErrorString(e)};
}

const DeviceSetup& setup(int device) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[device];
  if (!s.ready) {
    void* p = nullptr;
    check(cudaGetSymbolAddress(&p, g_qr_scratch), "cudaGetSymbolAddress of the workspace");
    if (coop_qr_scratch_bytes(kMaxGrid) > kPartBytes)
      throw Fail{TTN_ECAPACITY, "ttn_qr_noalloc: workspace smaller than the QR's partials"};
    check(cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, device), "multiprocessor count");
    check(coop_qr_max_grid(&s.max_grid), "occupancy query");
    s.base = static_cast<unsigned char*>(p);
    s.ready = true;
  }
  return s;
}

// Puts back the caller's current device on every return path: the entry point works on
// `device`, but the caller (a framework with its own notion of the current device) must
// not find it changed afterwards.
struct DeviceGuard {
  int saved = -1;
  ~DeviceGuard() {
    if (saved >= 0) cudaSetDevice(saved);
  }
};

}  // namespace
}  // namespace ttn

extern "C" int ttn_qr_noalloc(int m, int n, double* a, double* r, void* stream, int device) {
  using namespace ttn;
  try {
    if (!a || !r || m < n || n < 1)
      throw Fail{TTN_EINVAL, "ttn_qr_noalloc: needs device pointers a, r and m >= n >= 1"};
    if (n > kQrMaxCols)
      throw Fail{TTN_ECAPACITY, "ttn_qr_noalloc: n = " + std::to_string(n) + " exceeds the " +
                                    std::to_string(kQrMaxCols) + " columns its static workspace holds"};
    if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(r)) % 16 != 0)
      throw Fail{TTN_EINVAL, "ttn_qr_noalloc: a and r must be 16-byte aligned (complex double)"};
    int ndev = 0;
    check(cudaGetDeviceCount(&ndev), "device count");
    if (device < 0 || device >= ndev || device >= kMaxDevices)
      throw Fail{TTN_EINVAL, "ttn_qr_noalloc: no such device"};
    DeviceGuard guard;
    check(cudaGetDevice(&guard.saved), "cudaGetDevice");
    check(cudaSetDevice(device), "cudaSetDevice");
    const DeviceSetup& s = setup(device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int grid = coop_qr_grid(m, s.sms);
    if (grid > s.max_grid) grid = s.max_grid;
    if (grid > kMaxGrid) grid = kMaxGrid;
    auto* bar = reinterpret_cast<GridBarrier*>(s.base);
    int* err = reinterpret_cast<int*>(s.base + sizeof(GridBarrier));
    auto* tau = reinterpret_cast<double2*>(s.base + kTauOffset);
    auto* part = reinterpret_cast<double*>(s.base + kPartOffset);
    check(cudaMemsetAsync(s.base, 0, kZeroBytes, st), "clearing the barrier state");
    check(householder_qr_coop(reinterpret_cast<double2*>(a), m, n, reinterpret_cast<double2*>(r), 0, tau, part, bar,
                              err, grid, st),
          "QR launch");
    int h = 0;
    check(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st), "reading the status word");
    check(cudaStreamSynchronize(st), "QR");
    if (h != 0) throw Fail{TTN_ETIMEOUT, "ttn_qr_noalloc: a grid barrier of the QR gave up waiting"};
    return TTN_OK;
  } catch (const Fail& f) {
    set_error_message(f.msg);
    return f.code;
  } catch (const std::exception& e) {
    set_error_message(std::string("ttn_qr_noalloc: ") + e.what());
    return TTN_EINVAL;
  }
}
