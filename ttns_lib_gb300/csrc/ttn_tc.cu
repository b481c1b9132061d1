// Mixed-precision contraction engine.  Not yet available in this build: creating it
// fails with TTN_ENOTSUP so that a caller asking for the mixed form never silently
// gets the FP64 kernels instead.
#include "ttn_tc.cuh"

#include <stdexcept>

namespace ttn {

struct TcEngine {
  int device;
};

TcEngine* tc_create(int, long long, cudaStream_t) {
  throw std::runtime_error("mixed-precision contractions are not available in this build");
}
void tc_destroy(TcEngine* e) { delete e; }
bool tc_mode_apply(TcEngine*, const double2*, int, const double2*, double2*, long long, long long, double2, bool,
                   cudaStream_t) { return false; }
bool tc_mf_apply(TcEngine*, const double2*, const double2*, int, long long, double2*, double2, bool, cudaStream_t) {
  return false;
}
bool tc_adj_mul(TcEngine*, const double2*, const double2*, long long, int, double2*, double2, bool, cudaStream_t) {
  return false;
}
bool tc_mode_contract(TcEngine*, const double2*, const double2*, long long, int, long long, double2*, double2, bool,
                      cudaStream_t) { return false; }

}  // namespace ttn
