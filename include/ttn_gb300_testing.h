/* Test-only entry points of libttn_gb300: kernel-level calls that the parity tests use to
 * check one operation of the sweep against the oracle.  They are not part of the drop-in
 * boundary (ttn_gb300.h) and a caller of the sweep has no use for them; the library
 * exports them so that the device tests can reach single kernels through the same C-ABI. */
#ifndef TTN_GB300_TESTING_H
#define TTN_GB300_TESTING_H
#include "ttn_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* recompute every environment for the current node tensors, without gauge moves */
int ttn_debug_refresh_env(ttn_integrator* it, ttn_state* psi);
/* out = H_eff(node) v with the current environments; v, out are host buffers */
int ttn_debug_heff(ttn_integrator* it, int node, const double* v, double* out);
/* out = the compiled matrix-vector program of a node (kind 0: H_eff, kind 1: bond
 * Hamiltonian on the node's R matrix) applied once by the persistent kernel, in the
 * integrator's precision */
int ttn_debug_program_apply(ttn_integrator* it, int node, int kind, const double* v, double* out);
/* v <- exp(coeff * tau * H_eff(node)) v; returns the number of H applications */
int ttn_debug_expm_node(ttn_integrator* it, int node, double tau, double cre, double cim,
                        double* v, long long* napps);
/* environment matrix of one node group (which: 0 spf, 1 mean field) */
int ttn_debug_num_groups(ttn_integrator* it, int node, int* out);
int ttn_debug_get_env(ttn_integrator* it, int node, int group, int which, double* out);
/* tensor-core check: D (128 x N) = A (128 x K) B^T with B stored N x K, real fp64 in and out,
 * computed with split-TF32 tcgen05 MMAs and FP32 accumulation */
int ttn_debug_tc_gemm(const double* A, const double* B, double* D, int K, int N, int device);
/* Householder QR of an m x n row-major matrix on the device: a <- Q, r <- R */
int ttn_debug_qr(int m, int n, double* a, double* r, int device);
/* the same QR with the shared-memory kernel's phase clock: phases[16] microseconds as seen
 * by thread 0 of CTA 0 (0 column barriers, 1 column sums, 2 reflectors, 3 projections,
 * 4 row updates, 5 next partials, 6 panel updates, 7 R and Q formation; phases[8] columns);
 * zeros when the panel-blocked kernel ran */
int ttn_debug_qr_phases(int m, int n, double* a, double* r, int device, double* phases);

#ifdef __cplusplus
}
#endif
#endif
