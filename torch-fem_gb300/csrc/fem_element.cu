// Gauss-point element integration for small-strain mechanics:
//   geometry   eval_shape_functions            src/torchfem/base.py:293-314
//   stiffness  k += w detJ t B^T C B            src/torchfem/base.py:1085-1090
//   forces     f += w detJ t B^T sigma          src/torchfem/base.py:1050-1083
//   vjp        the adjoint replay of the residual (sparse.py:690-705), written
//              out by hand instead of recorded by autograd.
//
// Layouts (device):
//   bt   [nip][n_elem][n_e][dim]   physical gradients dN_a/dx_J
//   detj [nip][n_elem]
//   ke   [n_elem][n_e*dim][n_e*dim] row-major, row p = a*dim + i — the layout
//        of the reference's k tensor, so its values can be assembled as is.
#include "fem_common.cuh"

namespace tfg {

int etype_info(int etype, int* ne, int* d, int* nip) {
  switch (etype) {
    case FEM_QUAD1: *ne = 4; *d = 2; *nip = 4; return FEM_OK;
    case FEM_HEXA1: *ne = 8; *d = 3; *nip = 8; return FEM_OK;
    case FEM_TETRA2: *ne = 10; *d = 3; *nip = 4; return FEM_OK;
    case FEM_TETRA1: *ne = 4; *d = 3; *nip = 1; return FEM_OK;
    case FEM_TRIA1: *ne = 3; *d = 2; *nip = 1; return FEM_OK;
    case FEM_QUAD2: *ne = 8; *d = 2; *nip = 4; return FEM_OK;
    case FEM_TRIA2: *ne = 6; *d = 2; *nip = 3; return FEM_OK;
    case FEM_SHELL3: *ne = 3; *d = 6; *nip = 1; return FEM_OK;  // d: DOFs per node
    case FEM_HEXA2: *ne = 20; *d = 3; *nip = 8; return FEM_OK;
    default: return FEM_INVALID;
  }
}

// ---------------------------------------------------------------- geometry --
template <int NE, int D, int NIP>
__global__ void k_geometry(const double* __restrict__ nodes, const int32_t* __restrict__ elements,
                           int64_t n_elem, const double* __restrict__ dndxi, double* __restrict__ bt,
                           double* __restrict__ detj, int32_t* status) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elem * NIP) return;
  const int ip = (int)(t / n_elem);
  const int64_t e = t % n_elem;
  double X[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a) {
    const int64_t nd = elements[e * NE + a];
#pragma unroll
    for (int j = 0; j < D; ++j) X[a][j] = nodes[nd * D + j];
  }
  const double* b = dndxi + ip * D * NE;  // [D][NE]
  double J[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < NE; ++a) s += b[i * NE + a] * X[a][j];
      J[i][j] = s;
    }
  double det, inv[D][D];
  if constexpr (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double r = 1.0 / det;
    inv[0][0] = J[1][1] * r;
    inv[0][1] = -J[0][1] * r;
    inv[1][0] = -J[1][0] * r;
    inv[1][1] = J[0][0] * r;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    const double r = 1.0 / det;
    inv[0][0] = c00 * r;
    inv[1][0] = c01 * r;
    inv[2][0] = c02 * r;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  }
  if (!(det > 0.0)) flag_status(status, kStatBadJacobian);
  detj[t] = det;
  double* out = bt + t * (NE * D);
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) s += inv[i][j] * b[j * NE + a];
      out[a * D + i] = s;
    }
}

// ---------------------------------------------------------------- material --
// sigma = C : e for the three material layouts (e need not be symmetric).
template <int D, typename T>
__device__ __forceinline__ void apply_c(int kind, const T* cm, const T (&e)[D][D], T (&s)[D][D]) {
  if (kind == FEM_MAT_ISO) {
    const T lam = cm[0], G = cm[1];
    T tr = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) tr += e[i][i];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) s[i][j] = G * (e[i][j] + e[j][i]) + (i == j ? lam * tr : T(0));
  } else {
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T acc = 0;
#pragma unroll
        for (int k = 0; k < D; ++k)
#pragma unroll
          for (int l = 0; l < D; ++l) acc += cm[((i * D + j) * D + k) * D + l] * e[k][l];
        s[i][j] = acc;
      }
  }
}

// Pointer to the material data of element e at integration point ip.
template <int D, int NIP>
__device__ __forceinline__ const double* mat_ptr(int kind, const double* data, int64_t n_elem,
                                                 int64_t e, int ip) {
  constexpr int C4 = D * D * D * D;
  if (kind == FEM_MAT_ISO) return data + e * 2;
  if (kind == FEM_MAT_GENERAL) return data + e * C4;
  return data + ((int64_t)ip * n_elem + e) * C4;
}

// --------------------------------------------------------------- stiffness --
// Thread per (element, node a): accumulates the d x (n_e d) row block of a
// over all integration points, then writes it contiguously.
template <int NE, int D, int NIP, typename T>
__global__ void __launch_bounds__(128)
k_stiffness(const double* __restrict__ bt, const double* __restrict__ detj,
            const double* __restrict__ weights, const double* __restrict__ thickness,
            int kind, const double* __restrict__ mat, int64_t n_elem, T* __restrict__ ke) {
  constexpr int ND = NE * D;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elem * NE) return;
  const int64_t e = t / NE;
  const int a = (int)(t % NE);
  T acc[D][ND];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int q = 0; q < ND; ++q) acc[i][q] = T(0);
  const T th = thickness ? (T)thickness[e] : T(1);
  for (int ip = 0; ip < NIP; ++ip) {
    const double* g = bt + ((int64_t)ip * n_elem + e) * ND;
    const T s = (T)weights[ip] * (T)detj[(int64_t)ip * n_elem + e] * th;
    T ga[D];
#pragma unroll
    for (int J = 0; J < D; ++J) ga[J] = (T)g[a * D + J];
    const double* cmd = mat_ptr<D, NIP>(kind, mat, n_elem, e, ip);
    if (kind == FEM_MAT_ISO) {
      const T lam = (T)cmd[0] * s, G = (T)cmd[1] * s;
#pragma unroll
      for (int b = 0; b < NE; ++b) {
        T gb[D];
#pragma unroll
        for (int J = 0; J < D; ++J) gb[J] = (T)g[b * D + J];
        T dot = T(0);
#pragma unroll
        for (int J = 0; J < D; ++J) dot += ga[J] * gb[J];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int k = 0; k < D; ++k)
            acc[i][b * D + k] += lam * ga[i] * gb[k] + G * ga[k] * gb[i] + (i == k ? G * dot : T(0));
      }
    } else {
      // t[i][k][L] = sum_J ga[J] C[i][J][k][L]
      T tt[D][D][D];
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int k = 0; k < D; ++k)
#pragma unroll
          for (int L = 0; L < D; ++L) {
            T v = T(0);
#pragma unroll
            for (int J = 0; J < D; ++J) v += ga[J] * (T)cmd[((i * D + J) * D + k) * D + L];
            tt[i][k][L] = v * s;
          }
#pragma unroll
      for (int b = 0; b < NE; ++b) {
        T gb[D];
#pragma unroll
        for (int J = 0; J < D; ++J) gb[J] = (T)g[b * D + J];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int k = 0; k < D; ++k) {
            T v = T(0);
#pragma unroll
            for (int L = 0; L < D; ++L) v += tt[i][k][L] * gb[L];
            acc[i][b * D + k] += v;
          }
      }
    }
  }
  T* out = ke + (e * ND + (int64_t)a * D) * ND;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int q = 0; q < ND; ++q) out[i * ND + q] = acc[i][q];
}

// FP64 element matrices of an isotropic material by moments, for the FP64
// copy of the mixed solvers' sliced matrix.  For C = lambda I(x)I + 2 G Isym
// the (a, b) block of Ke is
//   K_ab[i][k] = lambda M[i][k] + G M[k][i] + G tr(M) delta_ik,
//   M = sum_ip w detJ t g_a g_b^T,
// the same sum as k_stiffness's, regrouped.  A CTA takes iso_epb(NE)
// elements: it stages their gradients g and the scaled gradients
// w detJ t g of every integration point in shared memory once, then a thread
// per (element, node pair a <= b) accumulates the 3x3 (2x2) moment and writes
// K_ab and K_ba = K_ab^T.  NE (NE + 1) / 2 pairs of D^2 FMAs per point
// instead of NE^2 rows of products: this GPU's FP64 pipe is narrow.
__host__ __device__ constexpr int iso_pairs(int ne) { return ne * (ne + 1) / 2; }
__host__ __device__ constexpr int iso_epb(int ne) { return iso_pairs(ne) >= 128 ? 1 : 128 / iso_pairs(ne); }

template <int NE, int D, int NIP>
__global__ void __launch_bounds__(iso_epb(NE) * iso_pairs(NE))
k_stiffness_iso64(const double* __restrict__ bt, const double* __restrict__ detj,
                  const double* __restrict__ weights, const double* __restrict__ thickness,
                  const double* __restrict__ mat, int64_t n_elem, double* __restrict__ ke) {
  constexpr int ND = NE * D;
  constexpr int NP = iso_pairs(NE);
  constexpr int EPB = iso_epb(NE);
  __shared__ double g_s[EPB][NIP][ND];   // g
  __shared__ double sg_s[EPB][NIP][ND];  // w detJ t g
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  for (int q = threadIdx.x; q < EPB * NIP * ND; q += blockDim.x) {
    const int le = q / (NIP * ND);
    const int ip = (q / ND) % NIP;
    const int c = q % ND;
    const int64_t e = e0 + le;
    double g = 0.0, sc = 0.0;
    if (e < n_elem) {
      g = bt[((int64_t)ip * n_elem + e) * ND + c];
      sc = weights[ip] * detj[(int64_t)ip * n_elem + e] * (thickness ? thickness[e] : 1.0);
    }
    g_s[le][ip][c] = g;
    sg_s[le][ip][c] = sc * g;
  }
  __syncthreads();
  const int le = threadIdx.x / NP;
  const int64_t e = e0 + le;
  if (le >= EPB || e >= n_elem) return;
  int p = threadIdx.x - le * NP;
  int a = 0;
  while (p >= NE - a) {  // pairs of row a: (a, a) .. (a, NE - 1)
    p -= NE - a;
    ++a;
  }
  const int b = a + p;
  double M[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int k = 0; k < D; ++k) M[i][k] = 0.0;
#pragma unroll
  for (int ip = 0; ip < NIP; ++ip) {
    double ga[D], gb[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      ga[i] = sg_s[le][ip][a * D + i];
      gb[i] = g_s[le][ip][b * D + i];
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int k = 0; k < D; ++k) M[i][k] = fma(ga[i], gb[k], M[i][k]);
  }
  const double lam = mat[e * 2], G = mat[e * 2 + 1];
  double tr = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) tr += M[i][i];
  double* kab = ke + (e * ND + (int64_t)a * D) * ND + b * D;
  double* kba = ke + (e * ND + (int64_t)b * D) * ND + a * D;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const double v = lam * M[i][k] + G * M[k][i] + (i == k ? G * tr : 0.0);
      kab[i * ND + k] = v;
      kba[k * ND + i] = v;
    }
}

// ------------------------------------------------------------------ forces --
template <int NE, int D>
__device__ __forceinline__ void load_field(const double* __restrict__ v, const int32_t* __restrict__ conn,
                                           const uint8_t* __restrict__ con_mask,
                                           const double* __restrict__ con_values, int con_mode,
                                           double (&ve)[NE][D]) {
#pragma unroll
  for (int a = 0; a < NE; ++a) {
    const int64_t nd = conn[a];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const int64_t dof = nd * D + c;
      double x = v ? v[dof] : 0.0;
      if (con_mode != 0 && con_mask[dof]) x = (con_mode == 1) ? con_values[dof] : 0.0;
      ve[a][c] = x;
    }
  }
}

// Thread per element.  Linear stress update for ISO/GENERAL materials,
// linearised product C:grad(v) for per-point tangents.
template <int NE, int D, int NIP>
__global__ void __launch_bounds__(128)
k_force(const double* __restrict__ bt, const double* __restrict__ detj,
        const double* __restrict__ weights, const double* __restrict__ thickness,
        const int32_t* __restrict__ elements, int kind, const double* __restrict__ mat,
        int64_t n_elem, const double* __restrict__ v, const uint8_t* __restrict__ con_mask,
        const double* __restrict__ con_values, int con_mode, const double* __restrict__ sigma_prev,
        const double* __restrict__ de0, double* __restrict__ fe, double* __restrict__ flux,
        double* __restrict__ hgrad, int32_t* status) {
  constexpr int ND = NE * D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  double ve[NE][D];
  load_field<NE, D>(v, elements + e * NE, con_mask, con_values, con_mode, ve);
  double f[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) f[a][c] = 0.0;
  double e0[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) e0[i][j] = de0 ? de0[e * D * D + i * D + j] : 0.0;
  const double th = thickness ? thickness[e] : 1.0;
  bool finite = true;
  for (int ip = 0; ip < NIP; ++ip) {
    const double* g = bt + ((int64_t)ip * n_elem + e) * ND;
    double gl[NE][D];
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int j = 0; j < D; ++j) gl[a][j] = g[a * D + j];
    // H[c][j] = sum_a v[a][c] dN_a/dx_j   (H_inc = du @ B^T, base.py:1052)
    double H[D][D];
#pragma unroll
    for (int c = 0; c < D; ++c)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < NE; ++a) s += ve[a][c] * gl[a][j];
        H[c][j] = s;
      }
    if (hgrad) {
      double* ho = hgrad + ((int64_t)ip * n_elem + e) * D * D;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) ho[i * D + j] = H[i][j];
    }
    double eps[D][D], sig[D][D];
    if (kind == FEM_MAT_TANGENT_IP) {
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) eps[i][j] = H[i][j];
    } else {
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) eps[i][j] = 0.5 * (H[j][i] + H[i][j]) - e0[i][j];
    }
    apply_c<D, double>(kind, mat_ptr<D, NIP>(kind, mat, n_elem, e, ip), eps, sig);
    if (sigma_prev) {
      const double* sp = sigma_prev + ((int64_t)ip * n_elem + e) * D * D;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) sig[i][j] += sp[i * D + j];
    }
    if (flux) {
      double* fo = flux + ((int64_t)ip * n_elem + e) * D * D;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) fo[i * D + j] = sig[i][j];
    }
    const double s = weights[ip] * detj[(int64_t)ip * n_elem + e] * th;
    // f[a][c] += s * sum_j dN_a/dx_j sigma[c][j]   (solid.py:56-58)
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) acc += gl[a][j] * sig[c][j];
        f[a][c] += s * acc;
      }
  }
  double* out = fe + e * ND;
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) {
      out[a * D + c] = f[a][c];
      finite = finite && isfinite(f[a][c]);
    }
  if (!finite) flag_status(status, kStatNonFinite);
}

// --------------------------------------------------------------------- vjp --
template <int NE, int D, int NIP>
__global__ void __launch_bounds__(128)
k_vjp(const double* __restrict__ bt, const double* __restrict__ detj,
      const double* __restrict__ weights, const double* __restrict__ thickness,
      const int32_t* __restrict__ elements, int kind, const double* __restrict__ mat,
      int64_t n_elem, const double* __restrict__ v, const uint8_t* __restrict__ con_mask,
      const double* __restrict__ con_values, int con_mode, const double* __restrict__ sigma_prev,
      const double* __restrict__ de0, const double* __restrict__ g,
      const double* __restrict__ gflux, const double* __restrict__ gh, double* __restrict__ gsig,
      double* __restrict__ gmat,
      double* __restrict__ gthick, double* __restrict__ gde0, double* __restrict__ gve) {
  constexpr int ND = NE * D;
  constexpr int C4 = D * D * D * D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int32_t* conn = elements + e * NE;
  double ve[NE][D], ge[NE][D];
  load_field<NE, D>(v, conn, con_mask, con_values, con_mode, ve);
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) ge[a][c] = g ? g[(int64_t)conn[a] * D + c] : 0.0;
  double e0[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) e0[i][j] = de0 ? de0[e * D * D + i * D + j] : 0.0;
  const double th = thickness ? thickness[e] : 1.0;
  double gv[NE][D];
#pragma unroll
  for (int a = 0; a < NE; ++a)
#pragma unroll
    for (int c = 0; c < D; ++c) gv[a][c] = 0.0;
  double glam = 0.0, gG = 0.0, gt = 0.0;
  double gd0[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) gd0[i][j] = 0.0;
  if (gmat && kind == FEM_MAT_GENERAL)
    for (int k = 0; k < C4; ++k) gmat[e * C4 + k] = 0.0;
  for (int ip = 0; ip < NIP; ++ip) {
    const double* gp = bt + ((int64_t)ip * n_elem + e) * ND;
    double gl[NE][D];
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int j = 0; j < D; ++j) gl[a][j] = gp[a * D + j];
    const double wd = weights[ip] * detj[(int64_t)ip * n_elem + e];
    const double s = wd * th;
    const double* cm = mat_ptr<D, NIP>(kind, mat, n_elem, e, ip);
    // forward quantities at this point
    double H[D][D], eps[D][D], sig[D][D];
#pragma unroll
    for (int c = 0; c < D; ++c)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double acc = 0.0;
#pragma unroll
        for (int a = 0; a < NE; ++a) acc += ve[a][c] * gl[a][j];
        H[c][j] = acc;
      }
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j)
        eps[i][j] = (kind == FEM_MAT_TANGENT_IP) ? H[i][j] : 0.5 * (H[j][i] + H[i][j]) - e0[i][j];
    apply_c<D, double>(kind, cm, eps, sig);
    if (sigma_prev) {
      const double* sp = sigma_prev + ((int64_t)ip * n_elem + e) * D * D;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) sig[i][j] += sp[i * D + j];
    }
    // cotangent of sigma: from the forces and from the flux output
    double gradg[D][D], sb[D][D];
#pragma unroll
    for (int c = 0; c < D; ++c)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double acc = 0.0;
#pragma unroll
        for (int a = 0; a < NE; ++a) acc += ge[a][c] * gl[a][j];
        gradg[c][j] = acc;
        sb[c][j] = s * acc + (gflux ? gflux[((int64_t)ip * n_elem + e) * D * D + c * D + j] : 0.0);
      }
    if (gthick) {
      double acc = 0.0;
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int j = 0; j < D; ++j) acc += gradg[c][j] * sig[c][j];
      gt += wd * acc;
    }
    if (gsig) {
      double* o = gsig + ((int64_t)ip * n_elem + e) * D * D;
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int j = 0; j < D; ++j) o[c * D + j] = sb[c][j];
    }
    if (gmat) {
      if (kind == FEM_MAT_ISO) {
        double trs = 0.0, tre = 0.0, sym = 0.0;
#pragma unroll
        for (int i = 0; i < D; ++i) {
          trs += sb[i][i];
          tre += eps[i][i];
        }
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) sym += sb[i][j] * (eps[i][j] + eps[j][i]);
        glam += trs * tre;
        gG += sym;
      } else if (kind == FEM_MAT_GENERAL) {
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j)
            for (int k = 0; k < D; ++k)
              for (int l = 0; l < D; ++l) gmat[e * C4 + ((i * D + j) * D + k) * D + l] += sb[i][j] * eps[k][l];
      } else {
        double* o = gmat + ((int64_t)ip * n_elem + e) * C4;
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j)
            for (int k = 0; k < D; ++k)
              for (int l = 0; l < D; ++l) o[((i * D + j) * D + k) * D + l] = sb[i][j] * eps[k][l];
      }
    }
    // ebar = C^T : sb
    double eb[D][D];
    if (kind == FEM_MAT_ISO) {
      apply_c<D, double>(kind, cm, sb, eb);  // isotropic C is major-symmetric
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k)
#pragma unroll
        for (int l = 0; l < D; ++l) {
          double acc = 0.0;
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) acc += cm[((i * D + j) * D + k) * D + l] * sb[i][j];
          eb[k][l] = acc;
        }
    }
    double Hb[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        if (kind == FEM_MAT_TANGENT_IP) {
          Hb[i][j] = eb[i][j];
        } else {
          gd0[i][j] -= eb[i][j];
          Hb[i][j] = 0.5 * (eb[i][j] + eb[j][i]);
        }
        if (gh) Hb[i][j] += gh[((int64_t)ip * n_elem + e) * D * D + i * D + j];
      }
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) acc += gl[a][j] * Hb[c][j];
        gv[a][c] += acc;
      }
  }
  if (gmat && kind == FEM_MAT_ISO) {
    gmat[e * 2 + 0] = glam;
    gmat[e * 2 + 1] = gG;
  }
  if (gthick) gthick[e] = gt;
  if (gde0) {
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) gde0[e * D * D + i * D + j] = gd0[i][j];
  }
  if (gve) {
#pragma unroll
    for (int a = 0; a < NE; ++a)
#pragma unroll
      for (int c = 0; c < D; ++c) gve[e * ND + a * D + c] = gv[a][c];
  }
}

// ------------------------------------------------------------ nodal gather --
// out[dof] = sum_{(e,a) incident to node, ascending} fe[e][a][c]; optional
// subtraction, constrained-DOF handling and a deterministic ||out||^2.
__global__ void k_gather(const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                         int64_t n_nod, int D, const double* __restrict__ fe,
                         const double* __restrict__ sub, const uint8_t* __restrict__ con_mask,
                         int con_mode, const double* __restrict__ con_src, double* __restrict__ out,
                         double* __restrict__ partial) {
  __shared__ double red[32];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double sq = 0.0;
  if (t < n_nod * D) {
    const int64_t a = t / D;
    const int c = (int)(t % D);
    double s = 0.0;
    for (int64_t q = inc_ptr[a]; q < inc_ptr[a + 1]; ++q) s += fe[(int64_t)inc[q] * D + c];
    if (sub) s -= sub[t];
    if (con_mode != 0 && con_mask[t]) s = (con_mode == 1) ? 0.0 : con_src[t];
    out[t] = s;
    sq = s * s;
  }
  if (partial) {
    const double b = block_sum(sq, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = b;
  }
}

__global__ void k_sum_partials(const double* __restrict__ partial, int64_t n, double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

}  // namespace tfg

using namespace tfg;

extern "C" {

int fem_geometry(const fem_mesh* m, const double* dndxi, double* bt, double* detj, int32_t* status,
                 void* stream) {
  cudaStream_t st = as_stream(stream);
  if (!m || m->n_elem < 0) {
    set_last_error("fem_geometry: bad mesh");
    return FEM_INVALID;
  }
  if (m->n_elem == 0) return FEM_OK;
#define TFG_BODY                                                                          \
  k_geometry<NE, D, NIP><<<grid_for(m->n_elem * NIP, 128), 128, 0, st>>>(                 \
      m->nodes, m->elements, m->n_elem, dndxi, bt, detj, status);
      ::tfg::note_launch();
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_geometry");
}

int fem_element_stiffness_iso64(const fem_mesh* m, const fem_material* mat, double* ke, int32_t* status,
                                void* stream) {
  (void)status;
  cudaStream_t st = as_stream(stream);
  if (!m || !mat || mat->kind != FEM_MAT_ISO) {
    set_last_error("fem_element_stiffness_iso64: needs an isotropic material");
    return FEM_INVALID;
  }
  if (m->n_elem == 0) return FEM_OK;
#define TFG_BODY                                                                                  \
  k_stiffness_iso64<NE, D, NIP><<<(unsigned)((m->n_elem + iso_epb(NE) - 1) / iso_epb(NE)),          \
                                  iso_epb(NE) * iso_pairs(NE), 0, st>>>(                           \
      m->bt, m->detj, m->weights, m->thickness, mat->data, m->n_elem, ke);
      ::tfg::note_launch();
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_element_stiffness_iso64");
}

int fem_element_stiffness(const fem_mesh* m, const fem_material* mat, int out_dtype, void* ke,
                          int32_t* status, void* stream) {
  (void)status;
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
  if (mat->kind == FEM_MAT_CONDUCTIVITY) return fem_heat_stiffness(m, mat->data, out_dtype, ke, status, stream);
  if (mat->kind != FEM_MAT_ISO && mat->kind != FEM_MAT_GENERAL && mat->kind != FEM_MAT_TANGENT_IP) {
    set_last_error("fem_element_stiffness: unknown material kind %d", mat->kind);
    return FEM_INVALID;
  }
  if (out_dtype == FEM_F64) {
#define TFG_BODY                                                                               \
  k_stiffness<NE, D, NIP, double><<<grid_for(m->n_elem * NE, 128), 128, 0, st>>>(              \
      m->bt, m->detj, m->weights, m->thickness, mat->kind, mat->data, m->n_elem, (double*)ke);
      ::tfg::note_launch();
    TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  } else if (out_dtype == FEM_F32) {
#define TFG_BODY                                                                               \
  k_stiffness<NE, D, NIP, float><<<grid_for(m->n_elem * NE, 128), 128, 0, st>>>(               \
      m->bt, m->detj, m->weights, m->thickness, mat->kind, mat->data, m->n_elem, (float*)ke);
      ::tfg::note_launch();
    TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  } else {
    set_last_error("fem_element_stiffness: bad dtype %d", out_dtype);
    return FEM_INVALID;
  }
  return check_cuda("fem_element_stiffness");
}

int fem_element_force(const fem_mesh* m, const fem_material* mat, const double* v,
                      const uint8_t* con_mask, const double* con_values, int con_mode,
                      const double* sigma_prev, const double* de0, double* fe, double* flux,
                      double* hgrad, int32_t* status, void* stream) {
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
  if (mat->kind == FEM_MAT_CONDUCTIVITY)
    return fem_heat_force(m, mat->data, v, con_mask, con_values, con_mode, sigma_prev, de0, fe, flux, hgrad,
                          status, stream);
  if (con_mode != 0 && !con_mask) {
    set_last_error("fem_element_force: con_mode needs con_mask");
    return FEM_INVALID;
  }
#define TFG_BODY                                                                               \
  k_force<NE, D, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                               \
      m->bt, m->detj, m->weights, m->thickness, m->elements, mat->kind, mat->data, m->n_elem, v, \
      con_mask, con_values, con_mode, sigma_prev, de0, fe, flux, hgrad, status);
      ::tfg::note_launch();
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_element_force");
}

int fem_element_vjp(const fem_mesh* m, const fem_material* mat, const double* v,
                    const uint8_t* con_mask, const double* con_values, int con_mode,
                    const double* sigma_prev, const double* de0, const double* g,
                    const double* gflux, const double* ghgrad, double* gsig, double* gmat,
                    double* gthick, double* gde0, double* gve, int32_t* status, void* stream) {
  (void)status;
  cudaStream_t st = as_stream(stream);
  if (m->n_elem == 0) return FEM_OK;
  if (mat->kind == FEM_MAT_CONDUCTIVITY)
    return fem_heat_vjp(m, mat->data, v, con_mask, con_values, con_mode, sigma_prev, de0, g, gflux, ghgrad, gsig,
                        gmat, gthick, gde0, gve, stream);
#define TFG_BODY                                                                                 \
  k_vjp<NE, D, NIP><<<grid_for(m->n_elem, 128), 128, 0, st>>>(                                   \
      m->bt, m->detj, m->weights, m->thickness, m->elements, mat->kind, mat->data, m->n_elem, v,   \
      con_mask, con_values, con_mode, sigma_prev, de0, g, gflux, ghgrad, gsig, gmat, gthick, gde0, \
      gve);
      ::tfg::note_launch();
  TFG_DISPATCH_ETYPE(m->etype)
#undef TFG_BODY
  return check_cuda("fem_element_vjp");
}

size_t fem_gather_workspace_bytes(int64_t n) { return (size_t)(grid_for(n, 256) + 1) * sizeof(double); }

int fem_gather_nodal(const fem_mesh* m, const double* fe, const double* sub, const uint8_t* con_mask,
                     int con_mode, const double* con_src, double* out, double* sumsq, void* ws,
                     size_t ws_bytes, void* stream) {
  cudaStream_t st = as_stream(stream);
  int ne, d, nip;
  if (etype_info(m->etype, &ne, &d, &nip) != FEM_OK) {
    set_last_error("fem_gather_nodal: unsupported element type %d", m->etype);
    return FEM_INVALID;
  }
  if (m->dof_per_node > 0) d = m->dof_per_node;
  const int64_t n = m->n_nod * d;
  double* partial = nullptr;
  if (sumsq) {
    if (ws_bytes < fem_gather_workspace_bytes(n)) {
      set_last_error("fem_gather_nodal: workspace too small");
      return FEM_INVALID;
    }
    partial = reinterpret_cast<double*>(ws);
  }
  const unsigned g = grid_for(n, 256);
  k_gather<<<g, 256, 0, st>>>(m->inc_ptr, m->inc, m->n_nod, d, fe, sub, con_mask, con_mode, con_src,
                              out, partial);
                              ::tfg::note_launch();
  if (sumsq) k_sum_partials<<<1, 1024, 0, st>>>(partial, g, sumsq);
  ::tfg::note_launch();
  return check_cuda("fem_gather_nodal");
}

}  // extern "C"
