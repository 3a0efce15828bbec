// dr_device.cuh -- device-side HEX8 shape functions, Jacobian and the
// directional-residual (DR) test function, templated on the arithmetic type.
//
// Mathematics (restated, not translated):
//   N_i(xi,eta,zeta) = (1 +- xi)(1 +- eta)(1 +- zeta)/8 with the node signs
//     of par_3d (vanadis_full_DR_OpenMP_timing.for:297-338);
//   J = dX/dxi, detJ, J^-1 by cofactors, grad N = J^-T grad_xi N
//     (gauss_point_hex8DR, :1567-1640);
//   W_i = N_i + tau (v . grad N_i), tau = h/(2|v|) beta(Pe), Pe = |v| h/(2 lambda_s)
//   with three ways of taking h, lambda_s and beta (DR variants):
//     OT  h = 2/(sum_k |v_k|/dl_k + 1e-14) from axis edge lengths,
//         lambda_s = lambda, beta = coth(Pe) - 1/Pe through exp  (:1652-1700)
//     GP  h = 2/|J^-1 e|, lambda_s = lambda, beta through exp
//         (src_updates/gauss_point_hex8DR.for:104-160)
//     VF  h = 2/|J^-1 e|, lambda_s = e^T Lambda e, beta by series /
//         1 - 1/Pe / 1/tanh - 1/Pe  (src_v2026_2_1/VANADIS.FOR:1954-2012)
//   The diffusion term uses grad W := grad N in every variant.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace vdr {

enum { DR_OT = 0, DR_GP = 1, DR_VF = 2 };

// Gauss abscissa exactly as the reference writes it (not 1/sqrt(3)).
#define VDR_GAUSS_C 0.577350269189626

__device__ __forceinline__ double dr_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dr_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dr_abs(double x) { return fabs(x); }
__device__ __forceinline__ float dr_abs(float x) { return fabsf(x); }

// beta(Pe) = coth(Pe) - 1/Pe for the OT and GP variants.
//   double: through exp, as the reference does; exp(Pe) overflows for
//           Pe > 709.78 and the result is NaN, exactly as in the reference.
//   float:  the same function evaluated safely (series below 0.05, tanh
//           above), with the reference's NaN kept for Pe > 709.78 so both
//           precisions agree on which elements are undefined.
__device__ __forceinline__ double beta_exp(double pe) {
  const double epos = exp(pe), eneg = exp(-pe);
  const double c = 0.5 * (epos + eneg), s = 0.5 * (epos - eneg);
  return c / s - 1.0 / pe;
}
__device__ __forceinline__ float beta_exp(float pe) {
  if (pe > 709.782712893384f) return __int_as_float(0x7fc00000);
  if (pe < 0.05f) {
    const float p2 = pe * pe;
    return pe * (1.0f / 3.0f - p2 * (1.0f / 45.0f - p2 * (2.0f / 945.0f)));
  }
  return 1.0f / tanhf(pe) - 1.0f / pe;
}
// VF variant: series for Pe < 1e-3, 1 - 1/Pe for Pe > 50, else 1/tanh - 1/Pe.
template <typename T>
__device__ __forceinline__ T beta_safe(T pe) {
  if (pe < T(1.0e-3)) {
    const T p3 = pe * pe * pe;
    const T p5 = (pe * pe) * (pe * pe) * pe;
    return pe / T(3) - p3 / T(45) + T(2) * p5 / T(945);
  }
  if (pe > T(50)) return T(1) - T(1) / pe;
  return T(1) / tanh(pe) - T(1) / pe;
}
template <>
__device__ __forceinline__ float beta_safe<float>(float pe) {
  if (pe < 1.0e-3f) {
    const float p3 = pe * pe * pe;
    const float p5 = (pe * pe) * (pe * pe) * pe;
    return pe / 3.0f - p3 / 45.0f + 2.0f * p5 / 945.0f;
  }
  if (pe > 50.0f) return 1.0f - 1.0f / pe;
  return 1.0f / tanhf(pe) - 1.0f / pe;
}

// Local node signs of the reference cube.
__device__ __forceinline__ float node_sx(int i) { return ((i + 1) & 2) ? 1.f : -1.f; }  // 1,2,5,6 -> +
__device__ __forceinline__ float node_sy(int i) { return (i & 2) ? 1.f : -1.f; }        // 2,3,6,7 -> +
__device__ __forceinline__ float node_sz(int i) { return (i & 4) ? 1.f : -1.f; }

template <typename T>
struct GPData {
  T detj;
  T n[8], w[8], gx[8], gy[8], gz[8];
};

// Shape functions and their reference-cube derivatives at one point
// (shape_hex8DR, vanadis_full_DR_OpenMP_timing.for:1398-1474).
template <typename T>
__device__ __forceinline__ void shape_at(const T xi, const T eta, const T zeta,
                                         T *n, T *d0, T *d1, T *d2) {
  const T xm = T(1) - xi, xp = T(1) + xi;
  const T ym = T(1) - eta, yp = T(1) + eta;
  const T zm = T(1) - zeta, zp = T(1) + zeta;
  n[0] = T(0.125) * xm * ym * zm;
  n[1] = T(0.125) * xp * ym * zm;
  n[2] = T(0.125) * xp * yp * zm;
  n[3] = T(0.125) * xm * yp * zm;
  n[4] = T(0.125) * xm * ym * zp;
  n[5] = T(0.125) * xp * ym * zp;
  n[6] = T(0.125) * xp * yp * zp;
  n[7] = T(0.125) * xm * yp * zp;
  d0[0] = -(T(0.125) * ym * zm);
  d0[1] = T(0.125) * ym * zm;
  d0[2] = T(0.125) * yp * zm;
  d0[3] = -(T(0.125) * yp * zm);
  d0[4] = -(T(0.125) * ym * zp);
  d0[5] = T(0.125) * ym * zp;
  d0[6] = T(0.125) * yp * zp;
  d0[7] = -(T(0.125) * yp * zp);
  d1[0] = -(T(0.125) * xm * zm);
  d1[1] = -(T(0.125) * xp * zm);
  d1[2] = T(0.125) * xp * zm;
  d1[3] = T(0.125) * xm * zm;
  d1[4] = -(T(0.125) * xm * zp);
  d1[5] = -(T(0.125) * xp * zp);
  d1[6] = T(0.125) * xp * zp;
  d1[7] = T(0.125) * xm * zp;
  d2[0] = -(T(0.125) * xm * ym);
  d2[1] = -(T(0.125) * xp * ym);
  d2[2] = -(T(0.125) * xp * yp);
  d2[3] = -(T(0.125) * xm * yp);
  d2[4] = T(0.125) * xm * ym;
  d2[5] = T(0.125) * xp * ym;
  d2[6] = T(0.125) * xp * yp;
  d2[7] = T(0.125) * xm * yp;
}

// The OT streamline length from the element's axis edge lengths
// dl = |x2-x1|, |y4-y1|, |z5-z1| (local nodes 1, 2, 4, 5).
template <typename T>
__device__ __forceinline__ T dr_h_axes(const T vx, const T vy, const T vz,
                                       const T vmag, const T dlx, const T dly,
                                       const T dlz) {
  const T eps = T(1.0e-14);
  return (vmag > eps)
             ? T(2) / (dr_abs(vx) / dlx + dr_abs(vy) / dly + dr_abs(vz) / dlz + eps)
             : T(0);
}

// tau from the streamline length h, |v| and the streamline diffusivity:
// Pe = |v| h / (2 lambda_s), tau = h/(2|v|) beta(Pe), zero unless |v| and
// lambda_s exceed 1e-14 and Pe exceeds 1e-12.
template <typename T>
__device__ __forceinline__ T dr_tau_from(const int variant, const T h,
                                         const T vmag, const T lams) {
  const T eps = T(1.0e-14);
  T pe = 0;
  if (vmag > eps && lams > eps) pe = vmag * h / (T(2) * lams);
  T tau = 0;
  if (pe > T(1.0e-12) && vmag > eps) {
    const T beta = (variant == DR_VF) ? beta_safe<T>(pe) : beta_exp(pe);
    tau = T(0.5) * h / vmag * beta;
  }
  return tau;
}

// The DR stabilization parameter tau at one point from the inverse
// Jacobian (i_ab = d xi_a / d x_b) and the element's velocity and
// diffusivity: streamline length h (OT: axis edge lengths; GP/VF: 2/|J^-1 e|,
// e = v/|v|), streamline diffusivity (VF: e^T Lambda e), Peclet number and
// beta(Pe) as the three reference variants define them.
template <typename T>
__device__ __forceinline__ T dr_tau(const int variant, const T i11, const T i12,
                                    const T i13, const T i21, const T i22,
                                    const T i23, const T i31, const T i32,
                                    const T i33, const T (&xe)[8],
                                    const T (&ye)[8], const T (&ze)[8],
                                    const T lam, const T vx, const T vy,
                                    const T vz) {
  const T eps = T(1.0e-14);
  const T vmag = dr_sqrt(vx * vx + vy * vy + vz * vz);
  T h, lams;
  if (variant == DR_OT) {
    h = dr_h_axes<T>(vx, vy, vz, vmag, dr_abs(xe[1] - xe[0]),
                     dr_abs(ye[3] - ye[0]), dr_abs(ze[4] - ze[0]));
    lams = lam;
  } else {
    T ex = 0, ey = 0, ez = 0;
    if (vmag > eps) {
      const T iv = T(1) / vmag;
      ex = vx * iv;
      ey = vy * iv;
      ez = vz * iv;
    }
    const T gx = i11 * ex + i12 * ey + i13 * ez;
    const T gy = i21 * ex + i22 * ey + i23 * ez;
    const T gz = i31 * ex + i32 * ey + i33 * ez;
    const T gn = dr_sqrt(gx * gx + gy * gy + gz * gz);
    h = (gn > eps) ? T(2) / gn : T(0);
    lams = (variant == DR_VF) ? (lam * ex * ex + lam * ey * ey + lam * ez * ez) : lam;
  }
  return dr_tau_from<T>(variant, h, vmag, lams);
}

// Geometry and DR weight of one point given its shape data: detJ, grad N
// (x,y,z) and W.  xe/ye/ze hold the 8 node coordinates in local order;
// (vx,vy,vz), lam are the element's velocity and isotropic diffusivity.
template <typename T>
__device__ __forceinline__ void gp_core(const int variant, const T *nsh,
                                        const T *d0, const T *d1, const T *d2,
                                        const T (&xe)[8], const T (&ye)[8],
                                        const T (&ze)[8], const T lam,
                                        const T vx, const T vy, const T vz,
                                        GPData<T> &o) {
  T j11 = 0, j12 = 0, j13 = 0, j21 = 0, j22 = 0, j23 = 0, j31 = 0, j32 = 0,
    j33 = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    o.n[i] = nsh[i];
    j11 += xe[i] * d0[i];
    j12 += xe[i] * d1[i];
    j13 += xe[i] * d2[i];
    j21 += ye[i] * d0[i];
    j22 += ye[i] * d1[i];
    j23 += ye[i] * d2[i];
    j31 += ze[i] * d0[i];
    j32 += ze[i] * d1[i];
    j33 += ze[i] * d2[i];
  }
  const T c11 = j22 * j33 - j23 * j32;
  const T c12 = j21 * j33 - j23 * j31;
  const T c13 = j21 * j32 - j22 * j31;
  const T detj = j11 * c11 - j12 * c12 + j13 * c13;
  const T r = T(1) / detj;
  const T i11 = r * c11;
  const T i12 = r * (j13 * j32 - j12 * j33);
  const T i13 = r * (j12 * j23 - j13 * j22);
  const T i21 = -r * c12;
  const T i22 = r * (j11 * j33 - j13 * j31);
  const T i23 = r * (j13 * j21 - j11 * j23);
  const T i31 = r * c13;
  const T i32 = r * (j12 * j31 - j11 * j32);
  const T i33 = r * (j11 * j22 - j12 * j21);
#pragma unroll
  for (int i = 0; i < 8; i++) {
    o.gx[i] = i11 * d0[i] + i21 * d1[i] + i31 * d2[i];
    o.gy[i] = i12 * d0[i] + i22 * d1[i] + i32 * d2[i];
    o.gz[i] = i13 * d0[i] + i23 * d1[i] + i33 * d2[i];
  }

  const T tau = dr_tau<T>(variant, i11, i12, i13, i21, i22, i23, i31, i32, i33,
                          xe, ye, ze, lam, vx, vy, vz);
#pragma unroll
  for (int i = 0; i < 8; i++)
    o.w[i] = o.n[i] + tau * (vx * o.gx[i] + vy * o.gy[i] + vz * o.gz[i]);
  o.detj = detj;
}

// Evaluates one Gauss (or face) point of an element: shape functions at
// (xi,eta,zeta), then gp_core.
template <typename T>
__device__ __forceinline__ void gp_eval(const int variant, const T xi,
                                        const T eta, const T zeta,
                                        const T (&xe)[8], const T (&ye)[8],
                                        const T (&ze)[8], const T lam,
                                        const T vx, const T vy, const T vz,
                                        GPData<T> &o) {
  T n[8], d0[8], d1[8], d2[8];
  shape_at<T>(xi, eta, zeta, n, d0, d1, d2);
  gp_core<T>(variant, n, d0, d1, d2, xe, ye, ze, lam, vx, vy, vz, o);
}

// Surface Jacobian of the xi = -1 face (nodes 1,4,8,5 of the element) at
// face coordinates (r,s) = (eta,zeta): |dX/dr x dX/ds| (quad4_3d,
// vanadis_full_DR_OpenMP_timing.for:1199-1261).
template <typename T>
__device__ __forceinline__ T face3_detjs(const T (&xe)[8], const T (&ye)[8],
                                         const T (&ze)[8], const T r,
                                         const T s) {
  const int f[4] = {0, 3, 7, 4};
  const T dr[4] = {-(T(0.25) * (T(1) - s)), T(0.25) * (T(1) - s),
                   T(0.25) * (T(1) + s), -(T(0.25) * (T(1) + s))};
  const T ds[4] = {-(T(0.25) * (T(1) - r)), -(T(0.25) * (T(1) + r)),
                   T(0.25) * (T(1) + r), T(0.25) * (T(1) - r)};
  T xr = 0, xs = 0, yr = 0, ys = 0, zr = 0, zs = 0;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    xr += dr[a] * xe[f[a]];
    xs += ds[a] * xe[f[a]];
    yr += dr[a] * ye[f[a]];
    ys += ds[a] * ye[f[a]];
    zr += dr[a] * ze[f[a]];
    zs += ds[a] * ze[f[a]];
  }
  const T cx = yr * zs - zr * ys;
  const T cy = zr * xs - xr * zs;
  const T cz = xr * ys - yr * xs;
  return dr_sqrt(cx * cx + cy * cy + cz * cz);
}

}  // namespace vdr
