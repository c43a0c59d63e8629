// Multi-part assemblies coupled by kinematic constraints (Assembly.solve,
// src/torchfem/assembly.py:378-650).  The parts keep their own FP64 CSR
// matrices; a coupling map T [n_dofs x n_retained] eliminates the secondary
// DOFs (u = T q), so the solved system is the Galerkin product
//   K_r = T^T blockdiag(K_parts) T
// with the Dirichlet condensation of Assembly._stiffness (assembly.py:295-334).
//
// The sparsity of K_r and, for each of its entries, the list of part-matrix
// entries that sum into it (with the product of the two T coefficients) are
// fixed by the couplings and the part patterns: the host builds them once and
// keeps them while the couplings and parts do not change.  Every solve then
// forms the values with one kernel here, a thread per entry summing its
// contributions in a fixed order, and the residual T^T (F_int - F_ext) and the
// expansion u = T q are rectangular CSR products by the second kernel.
#include "fem_common.cuh"

namespace tfg {
namespace {

constexpr int kThreads = 256;

// out[e] = sum_c coef[c] * kval[src[c]], c in [ptr[e], ptr[e+1]); then the
// condensation: fix 1 zeroes a constrained row or column, fix 2 puts 1 on a
// constrained diagonal.
__global__ void k_coupled_values(int64_t n_out, const int64_t* __restrict__ ptr, const int64_t* __restrict__ src,
                                 const double* __restrict__ coef, const double* __restrict__ kval,
                                 const uint8_t* __restrict__ fix, double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_out) return;
  double s = 0.0;
  for (int64_t c = ptr[e]; c < ptr[e + 1]; ++c) s = fma(coef[c], kval[src[c]], s);
  if (fix) {
    if (fix[e] == 1) s = 0.0;
    else if (fix[e] == 2) s = 1.0;
  }
  out[e] = s;
}

// y = A x for a rectangular FP64 CSR matrix, a warp per row (rows of a
// coupling map hold one to four entries; the transposed map's row of a
// reference point holds every coupled DOF).
__global__ void k_csr_apply(int64_t n_rows, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                            const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n_rows) return;
  double s = 0.0;
  for (int64_t q = row_ptr[w] + lane; q < row_ptr[w + 1]; q += 32) s = fma(val[q], x[col[q]], s);
  s = warp_sum(s);
  if (lane == 0) y[w] = s;
}

}  // namespace
}  // namespace tfg

using namespace tfg;

extern "C" {

int fem_coupled_values(int64_t n_out, const int64_t* ptr, const int64_t* src, const double* coef,
                       const double* kval, const uint8_t* fix, double* out, void* stream) {
  if (n_out < 0 || (n_out > 0 && (!ptr || !out))) {
    set_last_error("fem_coupled_values: bad arguments");
    return FEM_INVALID;
  }
  if (n_out == 0) return FEM_OK;
  k_coupled_values<<<grid_for(n_out, kThreads), kThreads, 0, as_stream(stream)>>>(n_out, ptr, src, coef, kval, fix,
                                                                                  out);
  ::tfg::note_launch();
  return check_cuda("fem_coupled_values");
}

int fem_csr_apply(int64_t n_rows, const int64_t* row_ptr, const int32_t* col, const double* val, const double* x,
                  double* y, void* stream) {
  if (n_rows < 0 || (n_rows > 0 && (!row_ptr || !y))) {
    set_last_error("fem_csr_apply: bad arguments");
    return FEM_INVALID;
  }
  if (n_rows == 0) return FEM_OK;
  k_csr_apply<<<grid_for(n_rows * 32, kThreads), kThreads, 0, as_stream(stream)>>>(n_rows, row_ptr, col, val, x, y);
  ::tfg::note_launch();
  return check_cuda("fem_csr_apply");
}

}  // extern "C"
