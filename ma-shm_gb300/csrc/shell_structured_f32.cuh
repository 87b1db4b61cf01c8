// Structured fused flat-shell step, FP32 specialisation for sm_103a.
//
// Same decomposition as k_struct_step (shell_structured.cuh: strips of EW-1
// element columns swept bottom to top, shared-memory force band, every node
// owned by one task), restructured for throughput:
//  * u_n of the strip lives in a shared-memory ring of 11 node rows; the 5 new
//    node rows of the next element row are copied with cp.async while the
//    current row is computed, so the gather never waits on memory;
//  * the 6x6 contractions, resultants and fluxes run on packed FP32x2 FMA
//    (__ffma2_rn, two lanes of a 64-bit register pair per instruction);
//  * the force band is a 6-row ring (the shared node row is carried by
//    re-labelling, not copied);
//  * the update's loads of u_{n-1} and 1/M are issued before phase C so that
//    their latency overlaps the transposed operator;
//  * the laminate pairs are copied with cp.async one row ahead
//    (double-buffered); the material index is read two rows ahead and the
//    stiffness factor one row ahead into registers.
// Results equal the generic kernel's up to FP32 rounding order.
#pragma once
#include <cuda_fp16.h>

#include "shell_element.cuh"
#include "shell_structured.cuh"

namespace shm {

// c_Dp[k][p]  = (D[2p][k], D[2p+1][k])   for out[i]  += D[i][k] * in[k]
// c_DTp[k][p] = (D[k][2p], D[k][2p+1])   for out[m]  += D[k][m] * in[k]
static __constant__ float2 c_Dp[NP][3];
static __constant__ float2 c_DTp[NP][3];

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

// laminate coefficient pairs, in the order the resultant pairs use them
// (Nxx,Nyy): (a11,a12) (a12,a22) (a16,a26) (b11,b12) (b12,b22) (b16,b26)
// (Nxy,Mxx): (a16,b11) (a26,b12) (a66,b16) (b16,d11) (b26,d12) (b66,d16)
// (Myy,Mxy): (b12,b16) (b22,b26) (b26,b66) (d12,d16) (d22,d26) (d26,d66)
// (Qy,Qx):   (a44,a45) (a45,a55)
constexpr int LAMP = 20;
#ifndef SHM_F32_KB
#define SHM_F32_KB 3
#endif
constexpr int KB = SHM_F32_KB;  // column nodes per laminate read in phase B (divides 6)

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int EW> struct F32Geom {
  static constexpr int G = 32 / EW;
  static constexpr int W = 5 * EW + 1;          // band columns
  static constexpr int OWN = 5 * (EW - 1);      // owned columns
  static constexpr int URING = 11;              // u_n node rows kept
  static constexpr int URAW = URING * 5 * W;
  static constexpr int UGS = URAW + ((16 - URAW % 32) + 64) % 32;   // group stride = 16 mod 32
  static constexpr int FRAW = 6 * 5 * W;
  static constexpr int FGS = FRAW + ((16 - FRAW % 32) + 64) % 32;
};

template <int EW>
constexpr size_t struct_f32_smem_bytes() {
  using GM = F32Geom<EW>;
  return sizeof(float) * (2 * CTA_ELEMS * ELEM_STRIDE + NP * CTA_ELEMS + GM::G * (GM::UGS + GM::FGS)) +
         sizeof(float2) * 2 * LAMP * CTA_ELEMS;
}

struct F32Args {
  const PlateDesc* __restrict__ plates;
  const TaskDesc* __restrict__ tasks;
  int ntask, H, nn_first, nft;
  int64_t nnode_pad;
  float* UA;
  float* UB;
  float* outp;  // u_{n+1} destination; null = over u_{n-1}
  PressureArgs<float> pr;
  const float* __restrict__ minv;
  float k1[5], k2[5];
  const float2* __restrict__ matp;  // [nmat][20] coefficient pairs
  const int* __restrict__ emat_g;
  const float* __restrict__ ekeep_g;
  const int* __restrict__ esens_g;
  const int* __restrict__ f_xl;
  const int* __restrict__ f_iy;
  const int* __restrict__ f_field;
  const double* __restrict__ f_val;
  const double* __restrict__ st;
  int nout;
  const int* __restrict__ out_node;
  const int* __restrict__ out_field;
  double* displ;
  double* vsum;
  SensorConst<float> sc;
  FrameSpec fs;
  float* frames;
  float a0, a1, blowup;
  int* flag;
  const int* d_base;
  // adjoint step (kAdj): residual forces at the point outputs each task owns,
  // forward state u_{n-1} for the damage gradient, gradient in plan order
  const int* __restrict__ o_xl;
  const int* __restrict__ o_iy;
  const int* __restrict__ o_field;
  const int* __restrict__ o_q;
  const double* __restrict__ asig;  // [nout][nft] residuals in reversed time
  const float* __restrict__ um;
  double* grad;
  const int* __restrict__ e_of_g;   // grid-order element -> plan element
};

// per-group task facts, uniform inside the group
struct GroupTask {
  int has, nrows, eyA, block, strip, plate, ney, nex, NX, f0, fn, scen, o0, on;
  long long node0, egrid0;
  float sx, sy, area4;
};

__device__ __forceinline__ GroupTask load_group_task(const F32Args& a, int tid) {
  GroupTask t{};
  if (tid >= a.ntask) return t;
  const TaskDesc tk = a.tasks[tid];
  const PlateDesc pl = a.plates[tk.plate];
  t.has = 1;
  t.nrows = tk.nrows;
  t.block = tk.block;
  t.eyA = tk.block == 0 ? 0 : tk.block * a.H - 1;
  t.strip = tk.strip;
  t.plate = tk.plate;
  t.ney = pl.ney;
  t.nex = pl.nex;
  t.NX = pl.NX;
  t.f0 = tk.f0;
  t.fn = tk.fn;
  t.o0 = tk.o0;
  t.on = tk.on;
  t.scen = pl.scen;
  t.node0 = pl.node0;
  t.egrid0 = pl.egrid0;
  t.sx = (float)pl.sx;
  t.sy = (float)pl.sy;
  t.area4 = (float)pl.area4;
  return t;
}

template <int G>
__device__ __forceinline__ const GroupTask& pick(const GroupTask* gt, int g) {
  if constexpr (G == 1) {
    return gt[0];
  } else {
    return gt[g];
  }
}

// copy node rows [r0, r0+NR) (relative to the task's first node row) of u_n
// into ring slots slot0, slot0+1, ... (mod URING); warp f < 5 copies field f
// of every lane group; columns outside the plate are left untouched (never
// read).  colmask bit (gg*8 + chunk) says whether this lane's column
// chunk*32 + lane of group gg lies on the plate (fixed for a task).
template <int EW>
__device__ __forceinline__ unsigned ring_colmask(const GroupTask* gt) {
  using GM = F32Geom<EW>;
  const int lane = threadIdx.x & 31;
  unsigned m = 0;
#pragma unroll
  for (int gg = 0; gg < GM::G; ++gg) {
    const GroupTask& t = pick<GM::G>(gt, gg);
    const int col0 = 5 * (t.strip * (EW - 1) - 1);
#pragma unroll
    for (int ch = 0; ch * 32 < GM::W; ++ch) {
      const int c = ch * 32 + lane;
      if (t.has && c < GM::W && (unsigned)(col0 + c) < (unsigned)t.NX) m |= 1u << (gg * 8 + ch);
    }
  }
  return m;
}

template <int EW, int NR>
__device__ __forceinline__ void ring_load(float* ring, const float* __restrict__ cur, int64_t nnode_pad,
                                          const GroupTask* gt, int r0, int slot0, unsigned colmask) {
  using GM = F32Geom<EW>;
  constexpr int G = GM::G, W = GM::W, UR = GM::URING;
  const int f = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (f >= 5) return;
#pragma unroll
  for (int gg = 0; gg < G; ++gg) {
    const GroupTask& t = pick<G>(gt, gg);
    if (!t.has) continue;
    const int col0 = 5 * (t.strip * (EW - 1) - 1);
    const int row0 = 5 * t.eyA + r0;
    const int NX = t.NX, rmax = 5 * t.ney;
    const float* src = cur + f * nnode_pad + t.node0 + (int64_t)row0 * NX + col0 + lane;
    const unsigned dbase =
        static_cast<unsigned>(__cvta_generic_to_shared(ring + gg * GM::UGS + f * W + lane));
    int sl = slot0;
#pragma unroll
    for (int rr = 0; rr < NR; ++rr) {
      if (row0 + rr <= rmax) {
        const unsigned drow = dbase + (unsigned)(sl * 5 * W) * 4u;
#pragma unroll
        for (int ch = 0; ch * 32 < W; ++ch)
          if (colmask & (1u << (gg * 8 + ch)))
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(drow + ch * 128u), "l"(src + ch * 32)
                         : "memory");
      }
      src += NX;
      if (++sl == UR) sl = 0;
    }
  }
}

// kAdj: the adjoint step of the same operator (K symmetric): lambda in
// place of u, residual forces r(n) at the point outputs instead of the
// excitation, and dJ/dd_e -= lambda_n' K_e^0 u_{n-1} accumulated per element
// (FP32 line products, FP64 per-element and across-step sums).
template <int EW, bool kSensor, bool kAdj = false>
__global__ void __launch_bounds__(CTA_THREADS, 2) k_struct_step_f32(F32Args a, int kstep) {
  using GM = F32Geom<EW>;
  constexpr int G = GM::G;
  constexpr int W = GM::W;
  constexpr int OWN = GM::OWN;
  constexpr int NCOL = (OWN + 31) / 32;  // update passes over a band row's owned columns
  constexpr int UR = GM::URING;
  extern __shared__ __align__(16) unsigned char smraw[];
  float* sm = reinterpret_cast<float*>(smraw);
  float* vred = sm + 2 * CTA_ELEMS * ELEM_STRIDE;
  float* ring = vred + NP * CTA_ELEMS;
  float* band = ring + G * GM::UGS;
  // laminate pairs of a row's elements, two buffers [2][LAMP][lane] (row r in
  // buffer r & 1, copied at the top of row r - 1)
  float2* lsm = reinterpret_cast<float2*>(band + G * GM::FGS);

  const int nn = *a.d_base + kstep;
  const bool odd = ((nn - a.nn_first) & 1);
  const float* __restrict__ cur = odd ? a.UB : a.UA;
  float* prev = odd ? a.UA : a.UB;
  float* dst = a.outp ? a.outp : prev;
  if (blockIdx.x == 0)
    for (int q = threadIdx.x; q < a.nout; q += blockDim.x)
      a.displ[(int64_t)q * a.nft + (nn - 1)] = (double)cur[a.out_field[q] * a.nnode_pad + a.out_node[q]];

  const int j = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int g = lane / EW;
  const int q = lane % EW;
  float* xs = sm + lane * ELEM_STRIDE;
  float* ys = sm + (CTA_ELEMS + lane) * ELEM_STRIDE;
  const bool frame = a.fs.frm_int > 0 && (nn % a.fs.frm_int) == 0;
  const bool guard = guard_step(a.fs, nn);
  const int ntg = (a.ntask + G - 1) / G;
  bool bad = false;
  // update prefetch: warp j finalises logical band row j of every lane group,
  // owned columns c = lane + 32*s
  float uo_r[G][NCOL][5];
  float mt_r[G][NCOL], mr_r[G][NCOL];
  bool gpend = false;      // adjoint: an element's gradient partials await reduction
  long long gpend_e = 0;   // (its grid-order index)

  // copy the lane's element's laminate pairs (warp j: pairs j, j+6, ...)
  auto lam_load = [&](int buf, int mat) {
    const float2* mp = a.matp + (int64_t)mat * LAMP;
    float2* d = lsm + buf * LAMP * CTA_ELEMS + lane;
    for (int c = j; c < LAMP; c += CTA_THREADS / 32) {
      const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(d + c * CTA_ELEMS));
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(mp + c) : "memory");
    }
  };

  __shared__ GroupTask gt[G];  // task facts of the lane groups (shared, not in registers)
  for (int tg = blockIdx.x; tg < ntg; tg += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < G) gt[threadIdx.x] = load_group_task(a, tg * G + threadIdx.x);
    __syncthreads();
    int maxrows = 0;
#pragma unroll
    for (int gg = 0; gg < G; ++gg) maxrows = max(maxrows, gt[gg].nrows);
    // this lane's element column, kept in registers for the whole task
    const GroupTask& t = pick<G>(gt, g);
    const int t_nrows = t.nrows, t_nex = t.nex;
    const int ex = t.strip * (EW - 1) - 1 + q;
    const bool colok = ex >= 0 && ex < t_nex;
    const long long eg0 = t.egrid0 + (long long)t.eyA * t_nex + ex;
    const float t_sx = t.sx, t_sy = t.sy, t_area4 = t.area4;
    float* ub = ring + g * GM::UGS;
    float* fb = band + g * GM::FGS;
    const float2 wsxy = make_float2(t_sx, t_sy);
    // band row j of group gg is final at element rows r in [ulo, uhi), and
    // for j == 5 only at the plate's last element row; node of column c at
    // element row r: ub0 + r*ustr + c, valid for c < ucol
    long long ub0[G];
    int ustr[G], ulo[G], uhi[G], ucol[G];
#pragma unroll
    for (int gg = 0; gg < G; ++gg) {
      const GroupTask& t2 = pick<G>(gt, gg);
      const int ix0 = 5 * t2.strip * (EW - 1);
      ub0[gg] = t2.node0 + (long long)(5 * t2.eyA + j) * t2.NX + ix0;
      ustr[gg] = 5 * t2.NX;
      ulo[gg] = t2.block > 0 ? 1 : 0;
      uhi[gg] = t2.has ? t2.nrows : 0;
      if (j == 5) {  // the top node row is shared with the next element row
        const int last = t2.ney - 1 - t2.eyA;
        ulo[gg] = max(ulo[gg], last);
        uhi[gg] = min(uhi[gg], last + 1);
      }
      ucol[gg] = min(OWN, t2.NX - ix0);
    }
    int fcur[G];  // next force entry of each lane group's task (warp j's node rows)
#pragma unroll
    for (int gg = 0; gg < G; ++gg) fcur[gg] = pick<G>(gt, gg).f0;

    for (int i = threadIdx.x; i < G * GM::FGS; i += blockDim.x) band[i] = 0.f;
    const unsigned colmask = ring_colmask<EW>(gt);
    ring_load<EW, 6>(ring, cur, a.nnode_pad, gt, 0, 0, colmask);
    // row 0's laminate pairs; the material index two rows ahead and the
    // stiffness factor one row ahead are read into registers
    int mnext = 0;
    float keep = 1.f, knext = 1.f;
    if (t_nrows > 0 && colok) {
      lam_load(0, a.emat_g[eg0]);
      keep = a.ekeep_g[eg0];
    }
    if (t_nrows > 1 && colok) mnext = a.emat_g[eg0 + t_nex];
    cp_async_commit();

    int rb = 0;   // ring slot of the element row's first node row, (5 r) mod 11
    int rb6 = 0;  // r mod 6
    for (int r = 0; r < maxrows; ++r) {
      // this row's node rows have landed (the only copy group in flight); the
      // barrier also ends the previous row's update for every warp, so the
      // ring slots of the previous row's first five node rows are free: the
      // next element row's five new node rows (5r+6 .. 5r+10) go there
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      __syncthreads();
      if (kAdj && gpend) {  // previous element row's gradient partials are complete
        double sum = 0.0;
#pragma unroll
        for (int i = 0; i < NP; ++i) sum += (double)vred[i * CTA_ELEMS + lane];
        a.grad[a.e_of_g[gpend_e]] -= sum;
        gpend = false;
      }
      const bool rowact = r < t_nrows;
      const bool valid = rowact && colok;
      const long long egrid = eg0 + (long long)r * t_nex;
      // the next row's laminate pairs go to the other buffer (last read in the
      // previous row's phase B)
      if (r + 1 < maxrows) {
        ring_load<EW, 5>(ring, cur, a.nnode_pad, gt, 5 * r + 6, rb + 6 >= UR ? rb + 6 - UR : rb + 6, colmask);
        if (r + 1 < t_nrows && colok) lam_load((r + 1) & 1, mnext);
      }
      cp_async_commit();
      if (r + 1 < t_nrows && colok) knext = a.ekeep_g[egrid + t_nex];
      if (r + 2 < t_nrows && colok) mnext = a.emat_g[egrid + 2 * t_nex];
      auto slot = [rb](int k) { const int s = rb + k; return s >= UR ? s - UR : s; };

      // phase A: row j, xi-derivatives (scaled by 2/ax) to ys
      if (valid) {
        const float* urow = ub + slot(j) * 5 * W + 5 * q;
        float2 acc[5][3];
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int p = 0; p < 3; ++p) acc[f][p] = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NP; ++k)
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            const float2 u2 = bc2(urow[f * W + k]);
#pragma unroll
            for (int p = 0; p < 3; ++p) acc[f][p] = fma2(c_Dp[k][p], u2, acc[f][p]);
          }
        const float2 sx2 = bc2(t_sx);
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int p = 0; p < 3; ++p) {
            const float2 d = mul2(acc[f][p], sx2);
            ys[f * NPE + (2 * p) * NP + j] = d.x;
            ys[f * NPE + (2 * p + 1) * NP + j] = d.y;
          }
      }
      __syncthreads();
      // phase B: column i = j
      if (valid) {
        const int i = j;
        float v[5][NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
          const float* urow = ub + slot(k) * 5 * W + 5 * q + i;
#pragma unroll
          for (int f = 0; f < 5; ++f) v[f][k] = urow[f * W];
        }
        // eta-derivatives, packed over node pairs, scaled by 2/ay
        float2 de2[5][3];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
#pragma unroll
          for (int p = 0; p < 3; ++p) de2[f][p] = make_float2(0.f, 0.f);
#pragma unroll
          for (int m = 0; m < NP; ++m) {
            const float2 v2 = bc2(v[f][m]);
#pragma unroll
            for (int p = 0; p < 3; ++p) de2[f][p] = fma2(c_Dp[m][p], v2, de2[f][p]);
          }
#pragma unroll
          for (int p = 0; p < 3; ++p) de2[f][p] = mul2(de2[f][p], bc2(t_sy));
        }
        const float2* L = lsm + (r & 1) * LAMP * CTA_ELEMS + lane;  // pair c at L[c * CTA_ELEMS]
        // the stiffness factor scales the element's fluxes (K_e^0 for the adjoint)
        const float akeep = kAdj ? t_area4 : t_area4 * keep;
        float2 Fe2[5][3];
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int p = 0; p < 3; ++p) Fe2[f][p] = make_float2(0.f, 0.f);
        float vp = 0.f;
        // nodes k of the column in blocks of KB: each laminate pair is read
        // from shared memory once per block (the products keep their order)
#pragma unroll
        for (int k0 = 0; k0 < NP; k0 += KB) {
          // strains: ex, ey, gxy, kx, ky, kxy, gyz, gxz
          float sn[KB][8];
#pragma unroll
          for (int kk = 0; kk < KB; ++kk) {
            const int k = k0 + kk;
            float gx[5], gy[5];
#pragma unroll
            for (int f = 0; f < 5; ++f) {
              gx[f] = ys[f * NPE + i * NP + k];
              gy[f] = (k & 1) ? de2[f][k >> 1].y : de2[f][k >> 1].x;
            }
            sn[kk][0] = gx[0];
            sn[kk][1] = gy[2];
            sn[kk][2] = gy[0] + gx[2];
            sn[kk][3] = gx[1];
            sn[kk][4] = gy[3];
            sn[kk][5] = gy[1] + gx[3];
            sn[kk][6] = v[3][k] + gy[4];
            sn[kk][7] = v[1][k] + gx[4];
            if (kSensor) {
              vp += a.sc.k0 * (a.sc.e31 * (gx[0] + a.sc.hh * gx[1]) + a.sc.e32 * (gy[2] + a.sc.hh * gy[3]));
            }
          }
          // R[0] = (Nxx, Nyy), R[1] = (Nxy, Mxx), R[2] = (Myy, Mxy), R[3] = (Qy, Qx)
          float2 R[4][KB];
#pragma unroll
          for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              const float2 l = L[(6 * b + c) * CTA_ELEMS];
#pragma unroll
              for (int kk = 0; kk < KB; ++kk)
                R[b][kk] = c == 0 ? mul2(l, bc2(sn[kk][c])) : fma2(l, bc2(sn[kk][c]), R[b][kk]);
            }
          {
            const float2 l18 = L[18 * CTA_ELEMS], l19 = L[19 * CTA_ELEMS];
#pragma unroll
            for (int kk = 0; kk < KB; ++kk) R[3][kk] = fma2(l19, bc2(sn[kk][7]), mul2(l18, bc2(sn[kk][6])));
          }
#pragma unroll
          for (int kk = 0; kk < KB; ++kk) {
            const int k = k0 + kk;
            const float2 NN = R[0][kk], NM = R[1][kk], MM = R[2][kk], QQ = R[3][kk];
            const float Wn = c_w32[i] * c_w32[k] * akeep;
            const float2 W2 = mul2(bc2(Wn), wsxy);  // (W*2/ax, W*2/ay)
            // (Gxi, Geta) per field: Sx = (Nxx, Mxx, Nxy, Mxy, Qx), Sy = (Nxy, Mxy, Nyy, Myy, Qy)
            const float2 G0 = mul2(W2, make_float2(NN.x, NM.x));
            const float2 G1 = mul2(W2, make_float2(NM.y, MM.y));
            const float2 G2 = mul2(W2, make_float2(NM.x, NN.y));
            const float2 G3 = mul2(W2, make_float2(MM.y, MM.x));
            const float2 G4 = mul2(W2, make_float2(QQ.y, QQ.x));
            const float2 Gs[5] = {G0, G1, G2, G3, G4};
#pragma unroll
            for (int f = 0; f < 5; ++f) {
              ys[f * NPE + i * NP + k] = Gs[f].x;
              const float2 ge = bc2(Gs[f].y);
#pragma unroll
              for (int p = 0; p < 3; ++p) Fe2[f][p] = fma2(c_DTp[k][p], ge, Fe2[f][p]);
            }
            if (k & 1) {
              Fe2[1][k >> 1].y += Wn * QQ.y;   // + Sxz.*WWDetJ into mx
              Fe2[3][k >> 1].y += Wn * QQ.x;   // + Syz.*WWDetJ into my
            } else {
              Fe2[1][k >> 1].x += Wn * QQ.y;
              Fe2[3][k >> 1].x += Wn * QQ.x;
            }
          }
        }
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int p = 0; p < 3; ++p) {
            xs[f * NPE + i * NP + 2 * p] = Fe2[f][p].x;
            xs[f * NPE + i * NP + 2 * p + 1] = Fe2[f][p].y;
          }
        if (kSensor) vred[i * CTA_ELEMS + lane] = vp;
      }
      __syncthreads();

      // the update's global loads for band row j, issued before phase C
      bool rowok[G];
      long long rowbase[G];
#pragma unroll
      for (int gg = 0; gg < G; ++gg) {
        rowok[gg] = r >= ulo[gg] && r < uhi[gg];
        rowbase[gg] = ub0[gg] + (long long)r * ustr[gg];
#pragma unroll
        for (int s = 0; s < NCOL; ++s) {
          const int c = lane + 32 * s;
          if (rowok[gg] && c < ucol[gg]) {
            const long long node = rowbase[gg] + c;
            mt_r[gg][s] = a.minv[node];
            mr_r[gg][s] = a.minv[a.nnode_pad + node];
#pragma unroll
            for (int f = 0; f < 5; ++f) uo_r[gg][s][f] = prev[f * a.nnode_pad + node];
          }
        }
      }

      // phase C: xi-part of the transposed operator + column part
      float out[5][NP];
      if (valid) {
#pragma unroll
        for (int f = 0; f < 5; ++f) {
          float2 o2[3];
#pragma unroll
          for (int p = 0; p < 3; ++p) o2[p] = make_float2(xs[f * NPE + (2 * p) * NP + j], xs[f * NPE + (2 * p + 1) * NP + j]);
#pragma unroll
          for (int ii = 0; ii < NP; ++ii) {
            const float2 gg2 = bc2(ys[f * NPE + ii * NP + j]);
#pragma unroll
            for (int p = 0; p < 3; ++p) o2[p] = fma2(c_DTp[ii][p], gg2, o2[p]);
          }
#pragma unroll
          for (int p = 0; p < 3; ++p) {
            out[f][2 * p] = o2[p].x;
            out[f][2 * p + 1] = o2[p].y;
          }
        }
        if constexpr (kAdj) {
          // line j's share of lambda' K_e^0 u_{n-1}, then keep_e K_e^0 lambda
          const float* umr = a.um + t.node0 + (int64_t)(5 * (t.eyA + r) + j) * t.NX + 5 * ex;
          float dl = 0.f;
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int i = 0; i < NP; ++i) {
              dl += out[f][i] * umr[f * a.nnode_pad + i];
              out[f][i] *= keep;
            }
          vred[j * CTA_ELEMS + lane] = dl;
        }
      } else {
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int i = 0; i < NP; ++i) out[f][i] = 0.f;
      }
      // band accumulation.  Logical row j of this element row is physical row
      // (j - r) mod 6.  Row 0 carries the previous element row's top line and
      // is added to; rows 1..5 start here and are stored.  Column i = 5 of a
      // lane's element is column 0 of the next lane's: it moves one lane up
      // by shuffle (lanes of a group are consecutive), and the strip's last
      // lane writes it itself.
      int prow = j - rb6;
      if (prow < 0) prow += 6;
      {
        float* dst = fb + prow * 5 * W + 5 * q;
#pragma unroll
        for (int f = 0; f < 5; ++f) {
          const float from_left = __shfl_up_sync(0xffffffffu, out[f][5], 1);
          if (q > 0) out[f][0] += from_left;
        }
        if (j == 0) {
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int i = 0; i < 5; ++i) dst[f * W + i] += out[f][i];
          if (q == EW - 1) {
#pragma unroll
            for (int f = 0; f < 5; ++f) dst[f * W + 5] += out[f][5];
          }
        } else {
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int i = 0; i < 5; ++i) dst[f * W + i] = out[f][i];
          if (q == EW - 1) {
#pragma unroll
            for (int f = 0; f < 5; ++f) dst[f * W + 5] = out[f][5];
          }
        }
        // band row j is now complete and written by this warp alone (row 0
        // adds the previous element row's line 5, stored before this row's
        // first barrier), and warp j updates exactly band row j: a warp
        // barrier suffices.  (The adjoint's gradient partials are reduced
        // after the next CTA barrier.)
        __syncwarp();
      }
      if constexpr (!kAdj) {
        // excitation of this band row's owned nodes: the task's forces are
        // ordered by node row (merged per DOF), warp j walks them with one
        // cursor per lane group and its lanes subtract a row's entries from
        // the completed band row (distinct DOFs: no two lanes meet)
#pragma unroll
        for (int gg = 0; gg < G; ++gg) {
          const GroupTask& t2 = pick<G>(gt, gg);
          if (t2.fn == 0 || !(r >= ulo[gg] && r < uhi[gg])) continue;
          const int iy = 5 * (t2.eyA + r) + j;
          const int fend = t2.f0 + t2.fn;
          int c0 = fcur[gg];
          while (c0 < fend && a.f_iy[c0] < iy) ++c0;
          int c1 = c0;
          while (c1 < fend && a.f_iy[c1] == iy) ++c1;
          fcur[gg] = c1;
          if (c1 > c0) {
            const double sv = a.st[(int64_t)t2.scen * a.nft + (nn - 1)];
            float* brow = band + gg * GM::FGS + prow * 5 * W;
            for (int fi = c0 + lane; fi < c1; fi += 32)
              brow[a.f_field[fi] * W + a.f_xl[fi]] -= (float)(a.f_val[fi] * sv);
            __syncwarp();
          }
        }
      }
      const bool owned_row = rowact && (t.block == 0 || r > 0);
      if (kAdj && j == 0) {  // reduced after the next CTA barrier
        gpend = valid && owned_row && q > 0;
        gpend_e = egrid;
      }
      if (kSensor && j == 0 && valid && owned_row && q > 0) {
        const int sl = a.esens_g[egrid];
        if (sl >= 0) {
          double sum = 0.0;
#pragma unroll
          for (int i = 0; i < NP; ++i) sum += (double)vred[i * CTA_ELEMS + lane];
          a.vsum[(int64_t)sl * a.nft + (nn - 1)] = sum;
        }
      }
      // update owned, complete nodes of band row j (excitation added here by
      // the node's owner)
#pragma unroll
      for (int gg = 0; gg < G; ++gg)
#pragma unroll
        for (int s = 0; s < NCOL; ++s) {
          const int c = lane + 32 * s;
          if (!(rowok[gg] && c < ucol[gg])) continue;
          const float* bnd = band + gg * GM::FGS + prow * 5 * W + 5 + c;
          const float* urow = ring + gg * GM::UGS + slot(j) * 5 * W + 5 + c;
          const long long node = rowbase[gg] + c;
          float F[5];
#pragma unroll
          for (int f = 0; f < 5; ++f) F[f] = bnd[f * W];
          const GroupTask& t2 = pick<G>(gt, gg);
          if (kAdj && t2.on > 0) {
            const int iy = 5 * (t2.eyA + r) + j;
            for (int oi = t2.o0; oi < t2.o0 + t2.on; ++oi)
              if (a.o_iy[oi] == iy && a.o_xl[oi] == 5 + c) {
                const float rv = (float)a.asig[(int64_t)a.o_q[oi] * a.nft + (nn - 1)];
#pragma unroll
                for (int f = 0; f < 5; ++f)
                  if (f == a.o_field[oi]) F[f] += rv;
              }
          }
          if (!kAdj && a.pr.npf > 0) F[4] -= pressure_load(a.pr, nn, a.nnode_pad, node);
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            const float u = urow[f * W];
            const float uo = uo_r[gg][s][f];
            const float im = (f == 1 || f == 3) ? mr_r[gg][s] : mt_r[gg][s];
            const float un = u + a.k1[f] * (u - uo) - a.k2[f] * (im * F[f]);
            dst[f * a.nnode_pad + node] = un;
            if (frame) store_frame(a.fs, a.frames, a.nnode_pad, node, f, nn, u, uo, un, a.a0, a.a1);
            if (guard && (!isfinite(un) || (f == 4 && u > a.blowup))) bad = true;
          }
        }
      // (the next row's first barrier separates this update from the ring
      // refill and the next band accumulation)
      keep = knext;
      rb += 5;
      if (rb >= UR) rb -= UR;
      if (++rb6 == 6) rb6 = 0;
    }
    cp_async_wait_all();
    __syncthreads();
    if (kAdj && gpend) {  // the task's last element row
      double sum = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) sum += (double)vred[i * CTA_ELEMS + lane];
      a.grad[a.e_of_g[gpend_e]] -= sum;
      gpend = false;
    }
  }
  if (bad) atomicOr(a.flag, 1);
}

}  // namespace shm
