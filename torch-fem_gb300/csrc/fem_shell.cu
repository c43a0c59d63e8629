// Tria1 flat-facet shell (src/torchfem/shell.py): element matrices, internal
// forces with the through-thickness station stresses, and the vector-Jacobian
// product for the section and material parameters.
//
// Each node carries six DOFs (three translations, three rotations).  Per
// element the kernels rebuild the local frame (material axis projected on the
// facet, shell.py:358-380), the in-plane shape gradients of the linear
// triangle and the transverse-shear operator averaged over the three cyclic
// node orderings (shell.py:310-356); the section integrates the plane-stress
// tangent over Simpson stations (A, B, D matrices, shell.py:474-504).  The
// element matrix is  T^T (km + kb + kc + ks + kd) T  (shell.py:506-586).
// Thread per element: shells are small structural models, the kernels are
// FP64 and keep the 18 x 18 local matrix in per-thread local memory.
#include "fem_common.cuh"

namespace tfg {

struct ShellGeom {
  double t[3][3];        // rows: material axis 1, material axis 2, normal
  double bx[3], by[3];   // in-plane shape gradients of the three nodes
  double ds[2][3][3];    // transverse shear rows x nodes x (w, rx, ry)
  double detj;
};

// Frame, gradients and shear operator of element e; false if detJ <= 0.
__device__ bool shell_geometry(const double* __restrict__ nodes, const int32_t* __restrict__ el, int64_t e,
                               const double* __restrict__ orient, ShellGeom& g) {
  double X[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int64_t n = el[3 * e + a];
#pragma unroll
    for (int k = 0; k < 3; ++k) X[a][k] = nodes[3 * n + k];
  }
  double e1[3], e2[3], nr[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    e1[k] = X[1][k] - X[0][k];
    e2[k] = X[2][k] - X[1][k];
  }
  nr[0] = e1[1] * e2[2] - e1[2] * e2[1];
  nr[1] = e1[2] * e2[0] - e1[0] * e2[2];
  nr[2] = e1[0] * e2[1] - e1[1] * e2[0];
  double ln = sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
#pragma unroll
  for (int k = 0; k < 3; ++k) nr[k] /= ln;
  double o[3] = {1.0, 0.0, 0.0};
  if (orient) {
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = orient[3 * e + k];
  }
  const double on = o[0] * nr[0] + o[1] * nr[1] + o[2] * nr[2];
  double a1[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) a1[k] = o[k] - on * nr[k];
  double la = sqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
  if (la < 1e-8) {  // reference direction normal to the facet: first edge
#pragma unroll
    for (int k = 0; k < 3; ++k) a1[k] = e1[k];
    la = sqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) a1[k] /= la;
  double a2[3] = {nr[1] * a1[2] - nr[2] * a1[1], nr[2] * a1[0] - nr[0] * a1[2], nr[0] * a1[1] - nr[1] * a1[0]};
  const double l2 = sqrt(a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2]);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a2[k] /= l2;
    g.t[0][k] = a1[k];
    g.t[1][k] = a2[k];
    g.t[2][k] = nr[k];
  }
  // in-plane coordinates relative to node 0
  double x[3], y[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double dx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dx[k] = X[a][k] - X[0][k];
    x[a] = g.t[0][0] * dx[0] + g.t[0][1] * dx[1] + g.t[0][2] * dx[2];
    y[a] = g.t[1][0] * dx[0] + g.t[1][1] * dx[1] + g.t[1][2] * dx[2];
  }
  // J = dN/dxi . x with dN/dxi = [[-1, 1, 0], [-1, 0, 1]]
  const double j00 = x[1] - x[0], j01 = y[1] - y[0], j10 = x[2] - x[0], j11 = y[2] - y[0];
  const double det = j00 * j11 - j01 * j10;
  g.detj = det;
  if (!(det > 0.0)) return false;
  const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
  const double d0[3] = {-1.0, 1.0, 0.0}, d1[3] = {-1.0, 0.0, 1.0};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    g.bx[a] = i00 * d0[a] + i01 * d1[a];
    g.by[a] = i10 * d0[a] + i11 * d1[a];
  }
  // transverse shear operator, averaged over the orderings (0,1,2), (1,2,0), (2,0,1)
  const double A = det / 2.0;
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) g.ds[r][a][c] = 0.0;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const int p0 = s, p1 = (s + 1) % 3, p2 = (s + 2) % 3;
    const double a = x[p1] - x[p0], b = y[p1] - y[p0], c = x[p2] - x[p0], d = y[p2] - y[p0];
    g.ds[0][p0][0] += b - d;
    g.ds[0][p0][2] += A;
    g.ds[1][p0][0] += c - a;
    g.ds[1][p0][1] += -A;
    g.ds[0][p1][0] += d;
    g.ds[0][p1][1] += -b * d / 2.0;
    g.ds[0][p1][2] += a * d / 2.0;
    g.ds[1][p1][0] += -c;
    g.ds[1][p1][1] += b * c / 2.0;
    g.ds[1][p1][2] += -a * c / 2.0;
    g.ds[0][p2][0] += -b;
    g.ds[0][p2][1] += b * d / 2.0;
    g.ds[0][p2][2] += -b * c / 2.0;
    g.ds[1][p2][0] += a;
    g.ds[1][p2][1] += -a * d / 2.0;
    g.ds[1][p2][2] += a * c / 2.0;
  }
  const double inv = 1.0 / (3.0 * 2.0 * A);
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) g.ds[r][a][c] *= inv;
  return true;
}

// Columns of the membrane, curvature and shear operators for local DOF p.
__device__ __forceinline__ void shell_columns(const ShellGeom& g, int p, double m[3], double b[3], double s[2]) {
  const int a = p / 6, c = p % 6;
  m[0] = m[1] = m[2] = b[0] = b[1] = b[2] = s[0] = s[1] = 0.0;
  if (c == 0) {
    m[0] = g.bx[a];
    m[2] = g.by[a];
  } else if (c == 1) {
    m[1] = g.by[a];
    m[2] = g.bx[a];
  } else if (c == 3) {
    b[1] = -g.by[a];
    b[2] = -g.bx[a];
  } else if (c == 4) {
    b[0] = g.bx[a];
    b[2] = g.by[a];
  }
  if (c >= 2 && c <= 4) {
    s[0] = g.ds[0][a][c - 2];
    s[1] = g.ds[1][a][c - 2];
  }
}

// Generalised strains of a local DOF vector: membrane (Voigt, engineering
// shear), curvature and transverse shear.
__device__ __forceinline__ void shell_strains(const ShellGeom& g, const double v[18], double em[3], double kb[3],
                                              double gs[2]) {
  em[0] = em[1] = em[2] = kb[0] = kb[1] = kb[2] = gs[0] = gs[1] = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    em[0] += g.bx[a] * v[6 * a];
    em[1] += g.by[a] * v[6 * a + 1];
    em[2] += g.by[a] * v[6 * a] + g.bx[a] * v[6 * a + 1];
    kb[0] += g.bx[a] * v[6 * a + 4];
    kb[1] += -g.by[a] * v[6 * a + 3];
    kb[2] += -g.bx[a] * v[6 * a + 3] + g.by[a] * v[6 * a + 4];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      gs[0] += g.ds[0][a][c] * v[6 * a + 2 + c];
      gs[1] += g.ds[1][a][c] * v[6 * a + 2 + c];
    }
  }
}

// v_local = T v_global for one element (six 3-blocks rotated by t).
__device__ __forceinline__ void shell_to_local(const ShellGeom& g, const double vg[18], double vl[18]) {
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      vl[3 * k + i] = g.t[i][0] * vg[3 * k] + g.t[i][1] * vg[3 * k + 1] + g.t[i][2] * vg[3 * k + 2];
}

__device__ __forceinline__ void shell_to_global(const ShellGeom& g, const double vl[18], double vg[18]) {
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      vg[3 * k + i] = g.t[0][i] * vl[3 * k] + g.t[1][i] * vl[3 * k + 1] + g.t[2][i] * vl[3 * k + 2];
}

struct ShellSection {
  double Am[3][3], Bm[3][3], Dm[3][3];  // integrated plane-stress tangent (A, B, D)
  double As[2];                        // psi * h * (G_xz, G_yz)
  double C[3][3];
  double G[2];
};

// Section of element e: A, B, D from the stations (z_j, w_j normalised to
// the thickness) and the psi-scaled transverse shear (shell.py:540-572).
__device__ void shell_section(const fem_shell* S, const double* __restrict__ mat, int64_t e, double detj,
                              ShellSection& sec, double* psi_out = nullptr, double* dpsih_out = nullptr) {
  const double h = S->thickness[e];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      sec.C[i][j] = mat[11 * e + 3 * i + j];
      sec.Am[i][j] = sec.Bm[i][j] = sec.Dm[i][j] = 0.0;
    }
  sec.G[0] = mat[11 * e + 9];
  sec.G[1] = mat[11 * e + 10];
  for (int k = 0; k < S->n_z; ++k) {
    const double z = S->z[k] * h, w = S->w[k] * h;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        sec.Am[i][j] += sec.C[i][j] * w;
        sec.Bm[i][j] += sec.C[i][j] * w * z;
        sec.Dm[i][j] += sec.C[i][j] * w * z * z;
      }
  }
  const double A = detj / 2.0;
  const double he2 = 2.0 * A;  // (sqrt(2) sqrt(A))^2
  const double alpha = S->kappa / (2.0 * (1.0 + S->nu_t));
  const double den = h * h + alpha * he2;
  const double psi = S->kappa * h * h / den;
  sec.As[0] = psi * h * sec.G[0];
  sec.As[1] = psi * h * sec.G[1];
  if (psi_out) *psi_out = psi;
  if (dpsih_out) *dpsih_out = S->kappa * h * h * (h * h + 3.0 * alpha * he2) / (den * den);
}

__global__ void __launch_bounds__(128) k_shell_stiffness(fem_shell S, const double* __restrict__ mat,
                                                         double* __restrict__ ke, int32_t* status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= S.n_elem) return;
  ShellGeom g;
  if (!shell_geometry(S.nodes, S.elements, e, S.orientation, g)) {
    flag_status(status, kStatBadJacobian);
    return;
  }
  ShellSection sec;
  shell_section(&S, mat, e, g.detj, sec);
  const double wd = 0.5 * g.detj;  // Tria1 weight 1/2 times detJ
  double kl[18][18];
  for (int q = 0; q < 18; ++q) {
    double mq[3], bq[3], sq[2];
    shell_columns(g, q, mq, bq, sq);
    double M[3], N[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      M[i] = 0.0;
      N[i] = 0.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        M[i] += sec.Am[i][j] * mq[j] + sec.Bm[i][j] * bq[j];
        N[i] += sec.Bm[i][j] * mq[j] + sec.Dm[i][j] * bq[j];
      }
    }
    const double Sq0 = sec.As[0] * sq[0], Sq1 = sec.As[1] * sq[1];
    for (int p = 0; p < 18; ++p) {
      double mp[3], bp[3], sp[2];
      shell_columns(g, p, mp, bp, sp);
      double v = mp[0] * M[0] + mp[1] * M[1] + mp[2] * M[2] + bp[0] * N[0] + bp[1] * N[1] + bp[2] * N[2];
      v = wd * v + wd * (sp[0] * Sq0 + sp[1] * Sq1);
      if (p == q && p % 6 == 5) v += S.drill;
      kl[p][q] = v;
    }
  }
  // global element matrix: ke = T^T kl T with T = diag(t, t, t, t, t, t)
  double* out = ke + e * 324;
  for (int I = 0; I < 6; ++I)
    for (int J = 0; J < 6; ++J) {
      double tmp[3][3];  // kl_IJ t
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          tmp[p][j] = kl[3 * I + p][3 * J] * g.t[0][j] + kl[3 * I + p][3 * J + 1] * g.t[1][j] +
                      kl[3 * I + p][3 * J + 2] * g.t[2][j];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          out[(3 * I + i) * 18 + 3 * J + j] = g.t[0][i] * tmp[0][j] + g.t[1][i] * tmp[1][j] + g.t[2][i] * tmp[2][j];
    }
}

// fe = ke u_e; optional station stresses C (eps_m + z_j h kappa) (local frame).
__global__ void __launch_bounds__(128) k_shell_force(fem_shell S, const double* __restrict__ mat,
                                                     const double* __restrict__ ke, const double* __restrict__ u,
                                                     double* __restrict__ fe, double* __restrict__ stress) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= S.n_elem) return;
  double ue[18];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int64_t n = S.elements[3 * e + a];
#pragma unroll
    for (int c = 0; c < 6; ++c) ue[6 * a + c] = u[6 * n + c];
  }
  if (fe) {
    const double* k = ke + e * 324;
    for (int i = 0; i < 18; ++i) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 18; ++j) s += k[i * 18 + j] * ue[j];
      fe[e * 18 + i] = s;
    }
  }
  if (stress) {
    ShellGeom g;
    if (!shell_geometry(S.nodes, S.elements, e, S.orientation, g)) return;
    double ul[18], em[3], kb[3], gs[2];
    shell_to_local(g, ue, ul);
    shell_strains(g, ul, em, kb, gs);
    const double h = S.thickness[e];
    for (int k = 0; k < S.n_z; ++k) {
      const double z = S.z[k] * h;
      double ev[3], sv[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) ev[i] = em[i] + z * kb[i];
#pragma unroll
      for (int i = 0; i < 3; ++i)
        sv[i] = mat[11 * e + 3 * i] * ev[0] + mat[11 * e + 3 * i + 1] * ev[1] + mat[11 * e + 3 * i + 2] * ev[2];
      double* o = stress + ((int64_t)k * S.n_elem + e) * 4;
      o[0] = sv[0];
      o[1] = sv[2];
      o[2] = sv[2];
      o[3] = sv[1];
    }
  }
}

// d/d(mat, h, u) of  a^T f(u) + sum_j <gstress_j, sigma_j(u)>  per element,
// with f = k(mat, h) u (a: cotangent of the element forces, gathered from the
// nodal cotangent) and sigma_j the station stresses.  The force part's
// u-derivative (k a) is not formed here: k is symmetric and the caller gets it
// from k_shell_force with u := a.
__global__ void __launch_bounds__(128) k_shell_vjp(fem_shell S, const double* __restrict__ mat,
                                                   const double* __restrict__ u, const double* __restrict__ a,
                                                   const double* __restrict__ gstress, double* __restrict__ gmat,
                                                   double* __restrict__ gthick, double* __restrict__ gue) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= S.n_elem) return;
  ShellGeom g;
  if (!shell_geometry(S.nodes, S.elements, e, S.orientation, g)) return;
  double ue[18], ae[18];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int64_t n = S.elements[3 * e + q];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      ue[6 * q + c] = u[6 * n + c];
      ae[6 * q + c] = a ? a[6 * n + c] : 0.0;
    }
  }
  double ul[18], al[18];
  shell_to_local(g, ue, ul);
  shell_to_local(g, ae, al);
  double emu[3], kbu[3], gsu[2], ema[3], kba[3], gsa[2];
  shell_strains(g, ul, emu, kbu, gsu);
  shell_strains(g, al, ema, kba, gsa);
  ShellSection sec;
  double psi, dpsih;
  shell_section(&S, mat, e, g.detj, sec, &psi, &dpsih);
  const double h = S.thickness[e];
  double S0 = 0.0, S1 = 0.0, S2 = 0.0;  // station moments of the weights
  for (int k = 0; k < S.n_z; ++k) {
    S0 += S.w[k];
    S1 += S.w[k] * S.z[k];
    S2 += S.w[k] * S.z[k] * S.z[k];
  }
  const double wd = 0.5 * g.detj;
  double gC[3][3], gh = 0.0;
  double gul[18];
#pragma unroll
  for (int i = 0; i < 18; ++i) gul[i] = 0.0;
  // force part: a^T k u
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int s = 0; s < 3; ++s)
      gC[r][s] = wd * (h * S0 * ema[r] * emu[s] + h * h * S1 * (ema[r] * kbu[s] + kba[r] * emu[s]) +
                       h * h * h * S2 * kba[r] * kbu[s]);
  double qmm = 0.0, qmb = 0.0, qbb = 0.0;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      qmm += ema[r] * sec.C[r][s] * emu[s];
      qmb += ema[r] * sec.C[r][s] * kbu[s] + kba[r] * sec.C[r][s] * emu[s];
      qbb += kba[r] * sec.C[r][s] * kbu[s];
    }
  const double gg0 = gsa[0] * gsu[0], gg1 = gsa[1] * gsu[1];
  gh += wd * (S0 * qmm + 2.0 * h * S1 * qmb + 3.0 * h * h * S2 * qbb) + wd * dpsih * (sec.G[0] * gg0 + sec.G[1] * gg1);
  double gG0 = wd * psi * h * gg0, gG1 = wd * psi * h * gg1;
  // station-stress part
  if (gstress) {
    for (int k = 0; k < S.n_z; ++k) {
      const double* gs = gstress + ((int64_t)k * S.n_elem + e) * 4;
      const double v[3] = {gs[0], gs[3], gs[1] + gs[2]};
      const double z = S.z[k] * h;
      double ev[3], Ctv[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) ev[i] = emu[i] + z * kbu[i];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int s = 0; s < 3; ++s) gC[r][s] += v[r] * ev[s];
#pragma unroll
      for (int s = 0; s < 3; ++s) Ctv[s] = sec.C[0][s] * v[0] + sec.C[1][s] * v[1] + sec.C[2][s] * v[2];
      gh += (Ctv[0] * kbu[0] + Ctv[1] * kbu[1] + Ctv[2] * kbu[2]) * S.z[k];
      // u-derivative: (Dm + z Db)^T C^T v
      for (int p = 0; p < 18; ++p) {
        double mp[3], bp[3], sp[2];
        shell_columns(g, p, mp, bp, sp);
        gul[p] += (mp[0] + z * bp[0]) * Ctv[0] + (mp[1] + z * bp[1]) * Ctv[1] + (mp[2] + z * bp[2]) * Ctv[2];
      }
    }
  }
  if (gmat) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int s = 0; s < 3; ++s) gmat[11 * e + 3 * r + s] = gC[r][s];
    gmat[11 * e + 9] = gG0;
    gmat[11 * e + 10] = gG1;
  }
  if (gthick) gthick[e] = gh;
  if (gue) {
    double gug[18];
    shell_to_global(g, gul, gug);
#pragma unroll
    for (int i = 0; i < 18; ++i) gue[e * 18 + i] = gug[i];
  }
}

static int shell_check(const fem_shell* S, const char* what) {
  if (!S || S->n_elem < 0 || S->n_nod < 0 || !S->nodes || !S->elements || !S->thickness || S->n_z < 1 || !S->z ||
      !S->w) {
    set_last_error("%s: invalid shell description", what);
    return FEM_INVALID;
  }
  return FEM_OK;
}

}  // namespace tfg

using namespace tfg;

extern "C" {

int fem_shell_stiffness(const fem_shell* shell, const double* mat, double* ke, int32_t* status, void* stream) {
  if (int rc = shell_check(shell, "fem_shell_stiffness")) return rc;
  if (shell->n_elem == 0) return FEM_OK;
  k_shell_stiffness<<<grid_for(shell->n_elem, 128), 128, 0, as_stream(stream)>>>(*shell, mat, ke, status);
  note_launch();
  return check_cuda("fem_shell_stiffness");
}

int fem_shell_force(const fem_shell* shell, const double* mat, const double* ke, const double* u, double* fe,
                    double* stress, void* stream) {
  if (int rc = shell_check(shell, "fem_shell_force")) return rc;
  if (shell->n_elem == 0) return FEM_OK;
  k_shell_force<<<grid_for(shell->n_elem, 128), 128, 0, as_stream(stream)>>>(*shell, mat, ke, u, fe, stress);
  note_launch();
  return check_cuda("fem_shell_force");
}

int fem_shell_vjp(const fem_shell* shell, const double* mat, const double* u, const double* a,
                  const double* gstress, double* gmat, double* gthick, double* gue, void* stream) {
  if (int rc = shell_check(shell, "fem_shell_vjp")) return rc;
  if (shell->n_elem == 0) return FEM_OK;
  k_shell_vjp<<<grid_for(shell->n_elem, 128), 128, 0, as_stream(stream)>>>(*shell, mat, u, a, gstress, gmat, gthick,
                                                                          gue);
  note_launch();
  return check_cuda("fem_shell_vjp");
}

}  // extern "C"
