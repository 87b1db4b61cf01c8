// Flat-shell spectral element: per-element K_e*u_e, sum-factorised.
//
// One element = 6x6 GLL nodes (order 5), 5 DOF per node in the reference's
// order (u, phi_x, v, phi_y, w; main_flat_shell.m:432-436).  The reference
// applies block-diagonal sparse operators Npx = I (x) D and Npy = D (x) I
// (shape2D_prim.m:45-58) to element-local vectors; here the same 6x6 matrix D
// is applied along element rows and columns in registers.
//
// Thread mapping (both kernels): a CTA owns 32 elements and 6 warps; warp w
// holds "line" w of all 32 elements, lane = element.  Work goes in three
// phases separated by __syncthreads():
//   A  row thread (element e, eta-row j): the 6 nodes (i=0..5, j) of its row,
//      xi-derivatives in registers, values + derivatives to shared memory;
//   B  column thread (element e, xi-column i): the 6 nodes (i, k=0..5),
//      eta-derivatives in registers, strains -> resultants -> weighted fluxes
//      (main_flat_shell.m:674-681), eta-part of the transposed operator
//      (Npyt*..., :683-689) in registers, xi-fluxes to shared memory;
//   C  row thread again: xi-part of the transposed operator + column part.
// Shared layout per element: buf[f*36 + i*6 + j] for node (i, j); the element
// stride is odd, so every warp access (fixed line, 32 elements) is
// bank-conflict free for both 4- and 8-byte words.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace shm {

constexpr int NP = 6;            // GLL nodes per direction
constexpr int NPE = 36;          // nodes per element
constexpr int ELEM_STRIDE = 181; // odd shared-memory stride per element (>= 5*36)
constexpr int CTA_ELEMS = 32;    // elements per CTA (one per lane)
constexpr int CTA_THREADS = 192; // 6 warps

// GLL derivative matrix D[r][c] = l_c'(x_r) and weights, filled at set-up.
// Internal linkage: every translation unit that includes this header owns
// (and initialises) its own copy.
static __constant__ double c_D64[NP * NP];
static __constant__ float c_D32[NP * NP];
static __constant__ double c_w64[NP];
static __constant__ float c_w32[NP];

template <typename T> __device__ __forceinline__ T Dm(int r, int c);
template <> __device__ __forceinline__ double Dm<double>(int r, int c) { return c_D64[r * NP + c]; }
template <> __device__ __forceinline__ float Dm<float>(int r, int c) { return c_D32[r * NP + c]; }
template <typename T> __device__ __forceinline__ T Wg(int r);
template <> __device__ __forceinline__ double Wg<double>(int r) { return c_w64[r]; }
template <> __device__ __forceinline__ float Wg<float>(int r) { return c_w32[r]; }

// Wavefield frames (main_flat_shell.m:765-885).  Every frm_int steps the
// displacement u_n (kind 0), the velocity a1*(u_{n+1} - u_{n-1}) (kind 1)
// and/or the acceleration a0*(u_{n-1} - 2 u_n + u_{n+1}) (kind 2) of the
// selected DOF components are stored as fields [frame][field][node_pad];
// slot[kind*5 + dof] is the field index of (kind, dof) or -1.  Frame c
// (0-based) is taken at loop index nn = (c + fc0) * frm_int, fc0 being the
// first multiple of frm_int at or after the loop's first index.
struct FrameSpec {
  int frm_int, nframes, nfields, fc0;
  int guard_int;  // blow-up guard also every guard_int steps (0: at frame steps only)
  signed char slot[15];
};

// Steps at which the update checks for blow-up: the frame steps, as the
// reference does (main_flat_shell.m:786-804), and every guard_int steps, so
// that runs without frames are guarded too.
__device__ __forceinline__ bool guard_step(const FrameSpec& fs, int nn) {
  return (fs.frm_int > 0 && nn % fs.frm_int == 0) || (fs.guard_int > 0 && nn % fs.guard_int == 0);
}

template <typename T>
__device__ __forceinline__ void store_frame(const FrameSpec& fs, T* __restrict__ frames, int64_t npad,
                                            int64_t node, int f, int nn, T u, T uo, T un, T a0, T a1) {
  const int fc = nn / fs.frm_int - fs.fc0;
  if (fc < 0 || fc >= fs.nframes) return;
  T* base = frames + (int64_t)fc * fs.nfields * npad + node;
  const int sU = fs.slot[f], sV = fs.slot[5 + f], sA = fs.slot[10 + f];
  if (sU >= 0) base[sU * npad] = u;
  if (sV >= 0) base[sV * npad] = a1 * (un - uo);
  if (sA >= 0) base[sA * npad] = a0 * (uo - T(2) * u + un);
}

// Pressure loading: nodal frames pf[k][node_pad], lumped area parea[node],
// per step (row nn-1 of pcoef) the two frames and their weights
// {f0, f1, c0, c1}; the load on w is parea * (c0 pf[f0] + c1 pf[f1]).
template <typename T> struct PressureArgs {
  int npf;                          // 0 = no pressure loading
  const T* __restrict__ pf;
  const T* __restrict__ parea;
  const double* __restrict__ pcoef;
};

template <typename T>
__device__ __forceinline__ T pressure_load(const PressureArgs<T>& pr, int nn, int64_t npad, int64_t node) {
  const double* c = pr.pcoef + 4 * (int64_t)(nn - 1);
  const T p = (T)c[2] * pr.pf[(int64_t)c[0] * npad + node] + (T)c[3] * pr.pf[(int64_t)c[1] * npad + node];
  return pr.parea[node] * p;
}

// Laminate coefficients of one element (composite_plate*.m outputs).
template <typename T> struct Lam {
  T a11, a12, a16, a22, a26, a66, a44, a45, a55;
  T b11, b12, b16, b22, b26, b66;
  T d11, d12, d16, d22, d26, d66;
};

// Material table row: 23 values (21 stiffness + m11 + I11), stored with a
// stride of 24 on the device.
constexpr int MAT_STRIDE_DEV = 24;

template <typename T>
__device__ __forceinline__ Lam<T> load_lam(const T* __restrict__ row, T keep) {
  Lam<T> L;
  L.a11 = row[0] * keep; L.a12 = row[1] * keep; L.a16 = row[2] * keep;
  L.a22 = row[3] * keep; L.a26 = row[4] * keep; L.a66 = row[5] * keep;
  L.a44 = row[6] * keep; L.a45 = row[7] * keep; L.a55 = row[8] * keep;
  L.b11 = row[9] * keep; L.b12 = row[10] * keep; L.b16 = row[11] * keep;
  L.b22 = row[12] * keep; L.b26 = row[13] * keep; L.b66 = row[14] * keep;
  L.d11 = row[15] * keep; L.d12 = row[16] * keep; L.d16 = row[17] * keep;
  L.d22 = row[18] * keep; L.d26 = row[19] * keep; L.d66 = row[20] * keep;
  return L;
}

// Geometry at node (i, k) of an element: inverse Jacobian (reference naming,
// inv_jacp_2D.m: invJ11 = dxi/dx, invJ12 = dxi/dy, invJ21 = deta/dx,
// invJ22 = deta/dy) and w_i w_k det J (WWDetJ, main_flat_shell.m:418).
template <typename T> struct NodeGeo {
  T i11, i12, i21, i22, W;
};

// General geometry: per local node arrays [5][36][fen_pad] (i11,i12,i21,i22,W).
template <typename T> struct GeoGeneral {
  static constexpr bool kAffineRect = false;
  const T* __restrict__ g;
  int64_t fen_pad;
  int e;
  __device__ __forceinline__ NodeGeo<T> at(int i, int k) const {
    const int c = k * NP + i;
    NodeGeo<T> r;
    r.i11 = g[(0 * NPE + c) * fen_pad + e];
    r.i12 = g[(1 * NPE + c) * fen_pad + e];
    r.i21 = g[(2 * NPE + c) * fen_pad + e];
    r.i22 = g[(3 * NPE + c) * fen_pad + e];
    r.W = g[(4 * NPE + c) * fen_pad + e];
    return r;
  }
};

// Axis-aligned rectangular elements of size ax x ay: invJ = diag(2/ax, 2/ay),
// det J = ax*ay/4.  The zero off-diagonal terms are compile-time zeros.
template <typename T> struct GeoRect {
  static constexpr bool kAffineRect = true;
  T sx, sy, area4;  // 2/ax, 2/ay, ax*ay/4
  __device__ __forceinline__ NodeGeo<T> at(int i, int k) const {
    NodeGeo<T> r;
    r.i11 = sx; r.i12 = T(0); r.i21 = T(0); r.i22 = sy;
    r.W = Wg<T>(i) * Wg<T>(k) * area4;
    return r;
  }
};

// PZT sensor constants (main_flat_shell.m:690-692).
template <typename T> struct SensorConst {
  T k0;   // pzt_thickness / g33
  T e31, e32;
  T hh;   // h/2
};

// Phase B for one column thread.  v[f][k] are the column's values (node (i,k)),
// dxi(f,k) reads the xi-derivative from shared memory.  Writes the weighted
// xi-fluxes Gxi[f] of node (i,k) to `xo[f*36 + i*6 + k]` and accumulates the
// eta-part of the transposed operator plus the pointwise shear terms into
// Fe[f][m] (column nodes m).  Returns the column's PZT voltage partial sum.
template <typename T, class Geo, bool kSensor>
__device__ __forceinline__ T shell_column(const T (&v)[5][NP], const T* __restrict__ ysm, T* xo, int i,
                                          const Lam<T>& L, const Geo& geo, T (&Fe)[5][NP],
                                          const SensorConst<T>& sc) {
  T vpart = T(0);
#pragma unroll
  for (int f = 0; f < 5; ++f)
#pragma unroll
    for (int m = 0; m < NP; ++m) Fe[f][m] = T(0);
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    T de[5], dx[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      T s = T(0);
#pragma unroll
      for (int m = 0; m < NP; ++m) s = fma(Dm<T>(k, m), v[f][m], s);
      de[f] = s;                               // Npy * field at (i,k)
      dx[f] = ysm[f * NPE + i * NP + k];       // Npx * field at (i,k)
    }
    const NodeGeo<T> G = geo.at(i, k);
    // physical derivatives d/dx = Npx*invJ11 + Npy*invJ21, d/dy = Npx*invJ12 + Npy*invJ22
    T gx[5], gy[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      if (Geo::kAffineRect) {
        gx[f] = dx[f] * G.i11;
        gy[f] = de[f] * G.i22;
      } else {
        gx[f] = dx[f] * G.i11 + de[f] * G.i21;
        gy[f] = dx[f] * G.i12 + de[f] * G.i22;
      }
    }
    // fields: 0 u, 1 phi_x, 2 v, 3 phi_y, 4 w
    const T ex = gx[0], ey = gy[2], gxy = gy[0] + gx[2];
    const T kx = gx[1], ky = gy[3], kxy = gy[1] + gx[3];
    const T gyz = v[3][k] + gy[4];  // phi_y + dw/dy
    const T gxz = v[1][k] + gx[4];  // phi_x + dw/dx
    const T Nxx = L.a11 * ex + L.a12 * ey + L.a16 * gxy + L.b11 * kx + L.b12 * ky + L.b16 * kxy;
    const T Nyy = L.a12 * ex + L.a22 * ey + L.a26 * gxy + L.b12 * kx + L.b22 * ky + L.b26 * kxy;
    const T Nxy = L.a16 * ex + L.a26 * ey + L.a66 * gxy + L.b16 * kx + L.b26 * ky + L.b66 * kxy;
    const T Mxx = L.b11 * ex + L.b12 * ey + L.b16 * gxy + L.d11 * kx + L.d12 * ky + L.d16 * kxy;
    const T Myy = L.b12 * ex + L.b22 * ey + L.b26 * gxy + L.d12 * kx + L.d22 * ky + L.d26 * kxy;
    const T Mxy = L.b16 * ex + L.b26 * ey + L.b66 * gxy + L.d16 * kx + L.d26 * ky + L.d66 * kxy;
    const T Qy = L.a44 * gyz + L.a45 * gxz;  // Syz
    const T Qx = L.a45 * gyz + L.a55 * gxz;  // Sxz
    // (Sx, Sy) pair per output field: u:(Nxx,Nxy) phi_x:(Mxx,Mxy) v:(Nxy,Nyy)
    // phi_y:(Mxy,Myy) w:(Qx,Qy).  Gxi = W(i11 Sx + i12 Sy), Geta = W(i21 Sx + i22 Sy).
    const T Sx[5] = {Nxx, Mxx, Nxy, Mxy, Qx};
    const T Sy[5] = {Nxy, Mxy, Nyy, Myy, Qy};
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      T gxi, geta;
      if (Geo::kAffineRect) {
        gxi = G.W * (G.i11 * Sx[f]);
        geta = G.W * (G.i22 * Sy[f]);
      } else {
        gxi = G.W * (G.i11 * Sx[f] + G.i12 * Sy[f]);
        geta = G.W * (G.i21 * Sx[f] + G.i22 * Sy[f]);
      }
      xo[f * NPE + i * NP + k] = gxi;
#pragma unroll
      for (int m = 0; m < NP; ++m) Fe[f][m] = fma(Dm<T>(k, m), geta, Fe[f][m]);
    }
    Fe[1][k] += G.W * Qx;  // + Sxz.*WWDetJ into mx
    Fe[3][k] += G.W * Qy;  // + Syz.*WWDetJ into my
    if (kSensor) {
      // reference quirk kept: invJ12 with d/deta in the x-derivative and
      // invJ21 with d/dxi in the y-derivative (main_flat_shell.m:691-692)
      const T dux = dx[0] * G.i11 + de[0] * G.i12, dfxx = dx[1] * G.i11 + de[1] * G.i12;
      const T dvy = dx[2] * G.i21 + de[2] * G.i22, dfyy = dx[3] * G.i21 + de[3] * G.i22;
      vpart += sc.k0 * (sc.e31 * (dux + sc.hh * dfxx) + sc.e32 * (dvy + sc.hh * dfyy));
    }
  }
  return vpart;
}

// xi-derivative of the row values in registers: d[f][i] = sum_k D[i][k] u[f][k]
template <typename T>
__device__ __forceinline__ void row_deriv_store(const T (&u)[5][NP], T* xs, T* ys, int j) {
#pragma unroll
  for (int f = 0; f < 5; ++f)
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < NP; ++k) s = fma(Dm<T>(i, k), u[f][k], s);
      xs[f * NPE + i * NP + j] = u[f][i];
      ys[f * NPE + i * NP + j] = s;
    }
}

// Phase C: out[f][i'] = sum_i D[i][i'] Gxi[f](i,j) + column part (i',j).
template <typename T>
__device__ __forceinline__ void row_transpose_apply(const T* xs, const T* ys, int j, T (&out)[5][NP]) {
#pragma unroll
  for (int f = 0; f < 5; ++f) {
    T g[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) g[i] = xs[f * NPE + i * NP + j];
#pragma unroll
    for (int ip = 0; ip < NP; ++ip) {
      T s = ys[f * NPE + ip * NP + j];
#pragma unroll
      for (int i = 0; i < NP; ++i) s = fma(Dm<T>(i, ip), g[i], s);
      out[f][ip] = s;
    }
  }
}

}  // namespace shm
