// 3D solid spectral element: 6 x 6 x 3 GLL nodes (order 5 in plane, order 2
// through the ply), 3 DOF per node (u, v, w), general hexahedral geometry.
//
// Restates the per-step work of the reference's 3D solver
// (src/models/solid3D/main_spec3Dcuda_global_cpu_gpu3_wave_sens_opt_single_PCT_mat.m:922-1010):
//   strains_spec_p.m   Exx..Exz from the 9 derivative products,
//   stresses_spec_p.m  Sxx..Sxz = D * E with D11..D66 (Voigt xx yy zz xy yz xz),
//   forces             fu, fv, fw = sum of 27 transposed products (:944-954),
// as one element kernel: the element's displacements, derivatives and
// weighted fluxes staged in shared memory, the three 1D derivative matrices
// (6-point along xi and eta, 3-point along zeta) applied along node lines --
// a thread per line in FP32 (k_elem_solid), a thread per node in FP64
// (k_elem_solid_nodes).  Element-local forces go to scratch and are assembled
// by the node kernel exactly like the flat shell's general path.  Per-element
// arrays are element-major ([e][108]), so a CTA's threads read and write
// consecutive words.
#pragma once
#include <type_traits>

#include "shell_element.cuh"

namespace shm {

constexpr int S_NZ = 3;
constexpr int S_NPE = NP * NP * S_NZ;   // 108 nodes per element
constexpr int S_EPB = 48;               // element padding (a multiple of the elements per CTA)
constexpr int S_MAT = 14;               // D11 D12 D13 D14 D22 D23 D24 D33 D34 D44 D55 D56 D66 rho
constexpr int S_MAT_DEV = 16;

static __constant__ double c_D3_64[S_NZ * S_NZ];
static __constant__ float c_D3_32[S_NZ * S_NZ];
static __constant__ double c_w3_64[S_NZ];
static __constant__ float c_w3_32[S_NZ];
template <typename T> __device__ __forceinline__ T W3m(int r);
template <> __device__ __forceinline__ double W3m<double>(int r) { return c_w3_64[r]; }
template <> __device__ __forceinline__ float W3m<float>(int r) { return c_w3_32[r]; }
template <typename T> __device__ __forceinline__ T D3m(int r, int c);
template <> __device__ __forceinline__ double D3m<double>(int r, int c) { return c_D3_64[r * S_NZ + c]; }
template <> __device__ __forceinline__ float D3m<float>(int r, int c) { return c_D3_32[r * S_NZ + c]; }

template <typename T> struct SolidArgs {
  int64_t fen_pad, nnode_pad, plane;
  int nnode, fen, nn_first, nft;
  T* UA;
  T* UB;
  T* F2;                           // [3][plane], element slots e*108 + c, then force slots
  const int* __restrict__ conn;    // [fen_pad][108]
  const T* __restrict__ geo;       // [10][fen_pad][108]: invJ_ab (a = xi,eta,zeta; b = x,y,z) row-major, W
  const T* __restrict__ gbox;      // box elements: [4][fen_pad] dxi/dx, deta/dy, dzeta/dz, |det J|
  const int* __restrict__ emat;
  const T* __restrict__ ekeep;
  const T* __restrict__ mat;       // [nmat][16]
  const int* __restrict__ row_ptr;
  const int* __restrict__ slots;
  const T* __restrict__ minv;      // [nnode_pad]
  T k1[3], k2[3];
  int nforce;
  const int* __restrict__ fq_field;
  const int* __restrict__ fq_scen;
  const double* __restrict__ fq_val;
  const double* __restrict__ st;
  int nout;
  const int* __restrict__ out_node;
  const int* __restrict__ out_field;
  double* displ;
  FrameSpec fs;
  T* frames;
  T a0, a1, blowup;
  int* flag;
  const int* d_base;
};

// Element step by node lines.  18 threads per element: thread t = 6a + b owns
// the xi line (cz = a, cy = b), the eta line (cz = a, cx = b) and the zeta
// lines of the in-plane positions q = t and t + 18, and the nodes
// c = t + 18 j (j = 0..5) in the pointwise parts.  Per element in shared
// memory: the displacements in node order (xi lines contiguous) and in
// eta-major order (eta lines contiguous), and the nine derivatives of each
// node, overwritten in place by its nine fluxes (along xi and zeta in node
// order, along eta in eta-major order).  Each line is read as three pairs and
// gives all six of its outputs, so a line's values are read once instead of
// once per node.  The element stride is 18 mod 32 words: consecutive threads
// then touch consecutive banks across an element boundary too, which the
// per-node accesses (most of the shared-memory traffic) need.
//   phase 0  stage the element group's u, gathered through the connectivity
//            while the previous group was computed, in both orders
//   phase 1  derivatives along the thread's xi, eta and zeta lines
//   phase 2  per node: physical gradient, strains, stresses, weighted fluxes
//   phase 3  transposed operators along the xi and eta lines (into the u
//            buffers, which are free by then)
//   phase 4  per node: the two line sums + the zeta transposed operator,
//            written to the element-local force slots
// kBox: every element is an axis-aligned box, so the inverse Jacobian is the
// constant diagonal (sx, sy, sz) and w_i w_j w_k |det J| the weights times a
// constant volume factor: four numbers per element replace the 1 080 per-node
// geometry values.
constexpr int S_TPE = 18;                       // threads per element
constexpr int S_ES = 1650;                      // element stride in shared memory (values)
static_assert(S_ES >= 15 * S_NPE && S_ES % 32 == 18, "element stride");
template <typename T> struct SolidLines {   // (instantiated for FP32)
  // elements per CTA: 12 (79 KB, two CTAs per SM) leaves ~98 KB of L1 for the
  // connectivity gathers and measured faster than 8 (four CTAs, ~45 KB of L1)
  // and 16 (two CTAs, ~45 KB)
  static constexpr int EPB = 12;
  static constexpr int THREADS = S_TPE * EPB;
  static constexpr size_t SMEM = sizeof(T) * (size_t)S_ES * EPB;
};
static_assert(S_EPB % SolidLines<float>::EPB == 0, "element padding");

template <typename T, bool kBox>
__global__ void __launch_bounds__(SolidLines<T>::THREADS) k_elem_solid(SolidArgs<T> a, int kstep) {
  using T2 = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
  constexpr int EPB = SolidLines<T>::EPB;
  extern __shared__ __align__(16) unsigned char s_raw[];
  __shared__ T sW[NP], sW3[S_NZ], sD3[S_NZ * S_NZ];
  if (threadIdx.x < NP) sW[threadIdx.x] = Wg<T>(threadIdx.x);
  if (threadIdx.x < S_NZ) sW3[threadIdx.x] = W3m<T>(threadIdx.x);
  if (threadIdx.x < S_NZ * S_NZ) sD3[threadIdx.x] = D3m<T>(threadIdx.x / S_NZ, threadIdx.x % S_NZ);
  const int nn = *a.d_base + kstep;
  const T* __restrict__ cur = ((nn - a.nn_first) & 1) ? a.UB : a.UA;
  if (blockIdx.x == 0) {
    const int64_t p0 = (int64_t)S_NPE * a.fen_pad;
    for (int q = threadIdx.x; q < a.nforce; q += blockDim.x) {
      const double s = a.st[(int64_t)a.fq_scen[q] * a.nft + (nn - 1)];
      const T val = (T)(-a.fq_val[q] * s);
#pragma unroll
      for (int f = 0; f < 3; ++f) a.F2[f * a.plane + p0 + q] = (f == a.fq_field[q]) ? val : T(0);
    }
    for (int q = threadIdx.x; q < a.nout; q += blockDim.x)
      a.displ[(int64_t)q * a.nft + (nn - 1)] = (double)cur[a.out_field[q] * a.nnode_pad + a.out_node[q]];
  }
  const int le = threadIdx.x / S_TPE;
  const int t = threadIdx.x % S_TPE;
  T* const base = reinterpret_cast<T*>(s_raw) + le * S_ES;
  T* const su = base;                 // [3][108] node order, later the xi-line forces
  T* const suT = base + 3 * S_NPE;    // [3][108] eta-major, later the eta-line forces
  T* const sd = base + 6 * S_NPE;     // [9][108] derivative / flux (f, direction)
  // the thread's nodes c = t + 18 j: layer j / 2, in-plane position
  // t + 18 (j % 2) = (cy_h, cx_h); eta-major index cT = 36 (j / 2) + cTh
  int cxh[2], cyh[2], cTh[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int q = t + S_TPE * h;
    cyh[h] = q / NP;
    cxh[h] = q - NP * cyh[h];
    cTh[h] = cxh[h] * NP + cyh[h];
  }

  // The CTA takes element groups blockIdx.x, + gridDim.x, ... (the grid is
  // what stays resident), and gathers the next group's nodal values into
  // registers while it computes the current one: the connectivity two groups
  // ahead, the displacements one group ahead.
  const int ngroups = (int)(a.fen_pad / EPB);
  const int G = gridDim.x;
  int nd[NP];      // node numbers of the next group to gather
  T uv[NP][3];     // gathered displacements of the group to stage next
  auto load_conn = [&](int grp) {
#pragma unroll
    for (int j = 0; j < NP; ++j) nd[j] = a.conn[((int64_t)grp * EPB + le) * S_NPE + t + S_TPE * j];
  };
  auto load_u = [&]() {
#pragma unroll
    for (int j = 0; j < NP; ++j)
#pragma unroll
      for (int f = 0; f < 3; ++f) uv[j][f] = cur[f * a.nnode_pad + nd[j]];
  };
  if (blockIdx.x < ngroups) {
    load_conn(blockIdx.x);
    load_u();
    if (blockIdx.x + G < ngroups) load_conn(blockIdx.x + G);
  }
  for (int grp = blockIdx.x; grp < ngroups; grp += G) {
    const int e = grp * EPB + le;
    __syncthreads();  // the previous group is done with the shared buffers
    // phase 0: stage the gathered values in both orders, start the next gathers
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      const int c = t + S_TPE * j;
      const int cT = 36 * (j / 2) + cTh[j % 2];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        su[f * S_NPE + c] = uv[j][f];
        suT[f * S_NPE + cT] = uv[j][f];
      }
    }
    if (grp + G < ngroups) {
      load_u();
      if (grp + 2 * G < ngroups) load_conn(grp + 2 * G);
    }
    // this group's per-element numbers for phase 2, ahead of phase 1
    const int mat_e = a.emat[e];
    const T kp = a.ekeep[e];
    T bx = T(0), by = T(0), bz = T(0), bv = T(0);
    if constexpr (kBox) {
      bx = a.gbox[e];
      by = a.gbox[a.fen_pad + e];
      bz = a.gbox[2 * a.fen_pad + e];
      bv = a.gbox[3 * a.fen_pad + e];
    }
    __syncthreads();

    const int lo = (t / NP) * 36 + (t % NP) * NP;  // first value of the thread's xi line (node order)
                                                   // and of its eta line (eta-major order)
    auto ld6 = [](const T* p, T (&o)[NP]) {
#pragma unroll
      for (int k = 0; k < NP / 2; ++k) {
        const T2 v = reinterpret_cast<const T2*>(p)[k];
        o[2 * k] = v.x;
        o[2 * k + 1] = v.y;
      }
    };
    auto st6 = [](T* p, const T (&o)[NP]) {
#pragma unroll
      for (int k = 0; k < NP / 2; ++k) {
        T2 v;
        v.x = o[2 * k];
        v.y = o[2 * k + 1];
        reinterpret_cast<T2*>(p)[k] = v;
      }
    };
    // phase 1: reference derivatives (Npx*U, Npy*U, Npz*U) along lines
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      T u[NP], d[NP];
      ld6(su + f * S_NPE + lo, u);
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        T s = T(0);
#pragma unroll
        for (int m = 0; m < NP; ++m) s = fma(Dm<T>(i, m), u[m], s);
        d[i] = s;
      }
      st6(sd + (f * 3 + 0) * S_NPE + lo, d);
      ld6(suT + f * S_NPE + lo, u);
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        T s = T(0);
#pragma unroll
        for (int m = 0; m < NP; ++m) s = fma(Dm<T>(i, m), u[m], s);
        d[i] = s;
      }
      st6(sd + (f * 3 + 1) * S_NPE + lo, d);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = t + S_TPE * h;
        T z[S_NZ];
#pragma unroll
        for (int m = 0; m < S_NZ; ++m) z[m] = su[f * S_NPE + m * 36 + q];
#pragma unroll
        for (int i = 0; i < S_NZ; ++i) {
          T s = T(0);
#pragma unroll
          for (int m = 0; m < S_NZ; ++m) s = fma(D3m<T>(i, m), z[m], s);
          sd[(f * 3 + 2) * S_NPE + i * 36 + q] = s;
        }
      }
    }
    __syncthreads();

    // phase 2: per node, strains_spec_p.m / stresses_spec_p.m and the fluxes
    {
      const T* __restrict__ Dm_ = a.mat + (int64_t)mat_e * S_MAT_DEV;
      const T D11 = Dm_[0] * kp, D12 = Dm_[1] * kp, D13 = Dm_[2] * kp, D14 = Dm_[3] * kp, D22 = Dm_[4] * kp;
      const T D23 = Dm_[5] * kp, D24 = Dm_[6] * kp, D33 = Dm_[7] * kp, D34 = Dm_[8] * kp, D44 = Dm_[9] * kp;
      const T D55 = Dm_[10] * kp, D56 = Dm_[11] * kp, D66 = Dm_[12] * kp;
#pragma unroll 2
      for (int j = 0; j < NP; ++j) {
        const int c = t + S_TPE * j;
        const int cT = 36 * (j / 2) + cTh[j % 2];
        const int cx = cxh[j % 2], cy = cyh[j % 2], cz = j / 2;
        T iJ[3][3];
        T W;
        if constexpr (kBox) {
#pragma unroll
          for (int q = 0; q < 9; ++q) iJ[q / 3][q % 3] = T(0);
          iJ[0][0] = bx;
          iJ[1][1] = by;
          iJ[2][2] = bz;
          W = sW[cx] * sW[cy] * sW3[cz] * bv;
        } else {
#pragma unroll
          for (int q = 0; q < 9; ++q) iJ[q / 3][q % 3] = a.geo[((int64_t)q * a.fen_pad + e) * S_NPE + c];
          W = a.geo[((int64_t)9 * a.fen_pad + e) * S_NPE + c];
        }
        T g[3][3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          const T d0 = sd[(f * 3 + 0) * S_NPE + c], d1 = sd[(f * 3 + 1) * S_NPE + cT], d2 = sd[(f * 3 + 2) * S_NPE + c];
#pragma unroll
          for (int b = 0; b < 3; ++b)
            g[f][b] = kBox ? (b == 0 ? d0 : b == 1 ? d1 : d2) * iJ[b][b] : d0 * iJ[0][b] + d1 * iJ[1][b] + d2 * iJ[2][b];
        }
        const T Exx = g[0][0], Eyy = g[1][1], Ezz = g[2][2];
        const T Exy = g[0][1] + g[1][0];
        const T Eyz = g[1][2] + g[2][1];
        const T Exz = g[0][2] + g[2][0];
        const T Sxx = Exx * D11 + Eyy * D12 + Ezz * D13 + Exy * D14;
        const T Syy = Exx * D12 + Eyy * D22 + Ezz * D23 + Exy * D24;
        const T Szz = Exx * D13 + Eyy * D23 + Ezz * D33 + Exy * D34;
        const T Sxy = Exx * D14 + Eyy * D24 + Ezz * D34 + Exy * D44;
        const T Syz = Eyz * D55 + Exz * D56;
        const T Sxz = Eyz * D56 + Exz * D66;
        // fluxes: field u uses (Sxx, Sxy, Sxz), v (Sxy, Syy, Syz), w (Sxz, Syz, Szz)
        const T S[3][3] = {{Sxx, Sxy, Sxz}, {Sxy, Syy, Syz}, {Sxz, Syz, Szz}};
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
          for (int aa = 0; aa < 3; ++aa)
            sd[(f * 3 + aa) * S_NPE + (aa == 1 ? cT : c)] =
                kBox ? W * (S[f][aa] * iJ[aa][aa]) : W * (S[f][0] * iJ[aa][0] + S[f][1] * iJ[aa][1] + S[f][2] * iJ[aa][2]);
      }
    }
    __syncthreads();

    // phase 3: transposed operators Npx' and Npy' along the thread's lines
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      T gl[NP], o[NP];
      ld6(sd + (f * 3 + 0) * S_NPE + lo, gl);
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        T s = T(0);
#pragma unroll
        for (int m = 0; m < NP; ++m) s = fma(Dm<T>(m, i), gl[m], s);
        o[i] = s;
      }
      st6(su + f * S_NPE + lo, o);
      ld6(sd + (f * 3 + 1) * S_NPE + lo, gl);
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        T s = T(0);
#pragma unroll
        for (int m = 0; m < NP; ++m) s = fma(Dm<T>(m, i), gl[m], s);
        o[i] = s;
      }
      st6(suT + f * S_NPE + lo, o);
    }
    __syncthreads();

    // phase 4: per node, + Npz' and out to the element-local force slots
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      const int c = t + S_TPE * j;
      const int cT = 36 * (j / 2) + cTh[j % 2];
      const int cz = j / 2, q = t + S_TPE * (j % 2);
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        T s = su[f * S_NPE + c] + suT[f * S_NPE + cT];
#pragma unroll
        for (int m = 0; m < S_NZ; ++m) s = fma(sD3[m * S_NZ + cz], sd[(f * 3 + 2) * S_NPE + m * 36 + q], s);
        a.F2[f * a.plane + (int64_t)e * S_NPE + c] = s;
      }
    }
  }  // element groups
}

// Element step with a thread per element node (the FP64 path: the line
// kernel's per-element staging, 13 KB in FP64, leaves too few warps per SM to
// keep the FP64 pipe busy).  Each thread applies the three 1D derivative
// matrices along its own node lines; the nodal values and the eta fluxes are
// also kept eta-major so that xi and eta lines are read as pairs.
constexpr int S_NODE_EPB = 2;                       // elements per CTA
constexpr int S_NODE_THREADS = S_NPE * S_NODE_EPB;
static_assert(S_EPB % S_NODE_EPB == 0, "element padding");
template <typename T, bool kBox>
__global__ void __launch_bounds__(S_NODE_THREADS) k_elem_solid_nodes(SolidArgs<T> a, int kstep) {
  using T2 = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
  // node values in two orders: su[c] with c = cz*36 + cy*6 + cx (xi lines
  // contiguous) and suT[cz*36 + cx*6 + cy] (eta lines contiguous), so that
  // both 6-point contractions read pairs; fluxes along xi are kept in node
  // order, fluxes along eta in eta-major order, for the same reason
  __shared__ __align__(16) T su[S_NODE_EPB][3][S_NPE];
  __shared__ __align__(16) T suT[S_NODE_EPB][3][S_NPE];
  __shared__ __align__(16) T sg[S_NODE_EPB][9][S_NPE];   // flux of field f along direction d at [f*3+d]
  // D and D' (6x6), D3 (3x3) and the GLL weights: each thread indexes them by
  // its own node position, which the constant cache would serialise per
  // distinct address; shared memory serves a warp's distinct addresses in one pass
  constexpr int kTab = 2 * NP * NP + S_NZ * S_NZ + NP + S_NZ;
  __shared__ __align__(16) T sD[kTab];
  {
    const int t = threadIdx.x;
    if (t < NP * NP) {
      sD[t] = Dm<T>(t / NP, t % NP);
      sD[NP * NP + t] = Dm<T>(t % NP, t / NP);
    } else if (t < NP * NP + S_NZ * S_NZ) {
      sD[NP * NP + t] = D3m<T>((t - NP * NP) / S_NZ, (t - NP * NP) % S_NZ);
    } else if (t < NP * NP + S_NZ * S_NZ + NP) {
      sD[NP * NP + t] = Wg<T>(t - NP * NP - S_NZ * S_NZ);
    } else if (t < NP * NP + S_NZ * S_NZ + NP + S_NZ) {
      sD[NP * NP + t] = W3m<T>(t - NP * NP - S_NZ * S_NZ - NP);
    }
  }
  const T* sDT = sD + NP * NP;     // sDT[i * NP + m] = D[m][i]
  const T* sD3 = sDT + NP * NP;
  const T* sW = sD3 + S_NZ * S_NZ;
  const T* sW3 = sW + NP;
  // six consecutive values from an even (16-byte aligned for FP64) index
  auto ld6 = [](const T* p, T (&o)[NP]) {
#pragma unroll
    for (int k = 0; k < NP / 2; ++k) {
      const T2 v = reinterpret_cast<const T2*>(p)[k];
      o[2 * k] = v.x;
      o[2 * k + 1] = v.y;
    }
  };
  const int nn = *a.d_base + kstep;
  const T* __restrict__ cur = ((nn - a.nn_first) & 1) ? a.UB : a.UA;
  if (blockIdx.x == 0) {
    const int64_t p0 = (int64_t)S_NPE * a.fen_pad;
    for (int q = threadIdx.x; q < a.nforce; q += blockDim.x) {
      const double s = a.st[(int64_t)a.fq_scen[q] * a.nft + (nn - 1)];
      const T val = (T)(-a.fq_val[q] * s);
#pragma unroll
      for (int f = 0; f < 3; ++f) a.F2[f * a.plane + p0 + q] = (f == a.fq_field[q]) ? val : T(0);
    }
    for (int q = threadIdx.x; q < a.nout; q += blockDim.x)
      a.displ[(int64_t)q * a.nft + (nn - 1)] = (double)cur[a.out_field[q] * a.nnode_pad + a.out_node[q]];
  }
  const int le = threadIdx.x / S_NPE;
  const int c = threadIdx.x % S_NPE;
  const int e = blockIdx.x * S_NODE_EPB + le;
  const int cx = c % NP, cy = (c / NP) % NP, cz = c / (NP * NP);
  const int node = a.conn[(int64_t)e * S_NPE + c];
  const int cT = cz * 36 + cx * NP + cy;  // this node's eta-major index
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const T v = cur[f * a.nnode_pad + node];
    su[le][f][c] = v;
    suT[le][f][cT] = v;
  }
  __syncthreads();
  // reference derivatives (Npx*U, Npy*U, Npz*U)
  T d[3][3];
  {
    T Dx[NP], Dy[NP];
    ld6(sD + cx * NP, Dx);
    ld6(sD + cy * NP, Dy);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      T sx = T(0), sy = T(0), sz = T(0);
      T ux[NP], uy[NP];
      ld6(&su[le][f][cz * 36 + cy * NP], ux);
      ld6(&suT[le][f][cz * 36 + cx * NP], uy);
#pragma unroll
      for (int m = 0; m < NP; ++m) {
        sx = fma(Dx[m], ux[m], sx);
        sy = fma(Dy[m], uy[m], sy);
      }
#pragma unroll
      for (int m = 0; m < S_NZ; ++m) sz = fma(sD3[cz * S_NZ + m], su[le][f][m * 36 + cy * NP + cx], sz);
      d[f][0] = sx;
      d[f][1] = sy;
      d[f][2] = sz;
    }
  }
  T iJ[3][3];
  T W;
  if constexpr (kBox) {
#pragma unroll
    for (int q = 0; q < 9; ++q) iJ[q / 3][q % 3] = T(0);
    iJ[0][0] = a.gbox[e];
    iJ[1][1] = a.gbox[a.fen_pad + e];
    iJ[2][2] = a.gbox[2 * a.fen_pad + e];
    W = sW[cx] * sW[cy] * sW3[cz] * a.gbox[3 * a.fen_pad + e];
  } else {
#pragma unroll
    for (int q = 0; q < 9; ++q) iJ[q / 3][q % 3] = a.geo[((int64_t)q * a.fen_pad + e) * S_NPE + c];
    W = a.geo[((int64_t)9 * a.fen_pad + e) * S_NPE + c];
  }
  // physical gradient g[f][b] = sum_a d[f][a] * invJ_ab  (strains_spec_p.m)
  T g[3][3];
#pragma unroll
  for (int f = 0; f < 3; ++f)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      g[f][b] = kBox ? d[f][b] * iJ[b][b] : d[f][0] * iJ[0][b] + d[f][1] * iJ[1][b] + d[f][2] * iJ[2][b];
  const T Exx = g[0][0], Eyy = g[1][1], Ezz = g[2][2];
  const T Exy = g[0][1] + g[1][0];
  const T Eyz = g[1][2] + g[2][1];
  const T Exz = g[0][2] + g[2][0];
  const T* __restrict__ Dm_ = a.mat + (int64_t)a.emat[e] * S_MAT_DEV;
  const T kp = a.ekeep[e];
  const T D11 = Dm_[0] * kp, D12 = Dm_[1] * kp, D13 = Dm_[2] * kp, D14 = Dm_[3] * kp, D22 = Dm_[4] * kp;
  const T D23 = Dm_[5] * kp, D24 = Dm_[6] * kp, D33 = Dm_[7] * kp, D34 = Dm_[8] * kp, D44 = Dm_[9] * kp;
  const T D55 = Dm_[10] * kp, D56 = Dm_[11] * kp, D66 = Dm_[12] * kp;
  // stresses_spec_p.m
  const T Sxx = Exx * D11 + Eyy * D12 + Ezz * D13 + Exy * D14;
  const T Syy = Exx * D12 + Eyy * D22 + Ezz * D23 + Exy * D24;
  const T Szz = Exx * D13 + Eyy * D23 + Ezz * D33 + Exy * D34;
  const T Sxy = Exx * D14 + Eyy * D24 + Ezz * D34 + Exy * D44;
  const T Syz = Eyz * D55 + Exz * D56;
  const T Sxz = Eyz * D56 + Exz * D66;
  // fluxes: field u uses (Sxx, Sxy, Sxz), v (Sxy, Syy, Syz), w (Sxz, Syz, Szz)
  const T S[3][3] = {{Sxx, Sxy, Sxz}, {Sxy, Syy, Syz}, {Sxz, Syz, Szz}};
#pragma unroll
  for (int f = 0; f < 3; ++f)
#pragma unroll
    for (int aa = 0; aa < 3; ++aa)
      sg[le][f * 3 + aa][aa == 1 ? cT : c] =
          kBox ? W * (S[f][aa] * iJ[aa][aa]) : W * (S[f][0] * iJ[aa][0] + S[f][1] * iJ[aa][1] + S[f][2] * iJ[aa][2]);
  __syncthreads();
  // transposed operators: Npx' (xi), Npy' (eta), Npz' (zeta)
  T Tx[NP], Ty[NP];
  ld6(sDT + cx * NP, Tx);
  ld6(sDT + cy * NP, Ty);
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    T s = T(0);
    T gxi[NP], geta[NP];
    ld6(&sg[le][f * 3 + 0][cz * 36 + cy * NP], gxi);
    ld6(&sg[le][f * 3 + 1][cz * 36 + cx * NP], geta);
#pragma unroll
    for (int m = 0; m < NP; ++m) {
      s = fma(Tx[m], gxi[m], s);
      s = fma(Ty[m], geta[m], s);
    }
#pragma unroll
    for (int m = 0; m < S_NZ; ++m) s = fma(sD3[m * S_NZ + cz], sg[le][f * 3 + 2][m * 36 + cy * NP + cx], s);
    a.F2[f * a.plane + (int64_t)e * S_NPE + c] = s;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_node_solid(SolidArgs<T> a, int kstep) {
  const int nn = *a.d_base + kstep;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.nnode) return;
  const bool odd = ((nn - a.nn_first) & 1);
  const T* __restrict__ cur = odd ? a.UB : a.UA;
  T* prev = odd ? a.UA : a.UB;
  T F[3] = {T(0), T(0), T(0)};
  // the copies in runs of up to four: their slot numbers, then their values,
  // are read together; the sum keeps the basket order
  const int s0 = a.row_ptr[g], s1 = a.row_ptr[g + 1];
  for (int s = s0; s < s1; s += 4) {
    const int n = min(4, s1 - s);
    int64_t sl[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) sl[k] = k < n ? a.slots[s + k] : 0;
    T v[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int f = 0; f < 3; ++f) v[k][f] = k < n ? a.F2[f * a.plane + sl[k]] : T(0);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < n) {
#pragma unroll
        for (int f = 0; f < 3; ++f) F[f] += v[k][f];
      }
  }
  const T im = a.minv[g];
  const bool frame = a.fs.frm_int > 0 && (nn % a.fs.frm_int) == 0;
  const bool guard = guard_step(a.fs, nn);
  bool bad = false;
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const T u = cur[f * a.nnode_pad + g];
    const T uo = prev[f * a.nnode_pad + g];
    const T un = u + a.k1[f] * (u - uo) - a.k2[f] * (im * F[f]);
    prev[f * a.nnode_pad + g] = un;
    if (frame) store_frame(a.fs, a.frames, a.nnode_pad, g, f, nn, u, uo, un, a.a0, a.a1);
    if (guard && !isfinite(un)) bad = true;
  }
  if (bad) atomicOr(a.flag, 1);
}

}  // namespace shm
