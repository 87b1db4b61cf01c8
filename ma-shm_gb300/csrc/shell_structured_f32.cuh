// Structured fused flat-shell step, FP32 specialisation for sm_103a.
//
// Same decomposition as k_struct_step (shell_structured.cuh: strips of EW-1
// element columns swept bottom to top, shared-memory force band, every node
// owned by one task), restructured for throughput:
//  * u_n of the strip lives in a shared-memory ring of 11 node rows; the 5 new
//    node rows of the next element row arrive by TMA bulk copies
//    (cp.async.bulk, one per node row and field, completed on an mbarrier)
//    while the current row is computed, so the gather never waits on memory;
//  * the update's global loads (u_{n-1}, inverse mass) are issued before the
//    transposed operator so that their latency overlaps it;
//  * the 6x6 contractions, resultants and fluxes run on packed FP32x2 FMA
//    (__ffma2_rn, two lanes of a 64-bit register pair per instruction);
//  * the force band is a 6-row ring (the shared node row is carried by
//    re-labelling, not copied); the column part of the transposed operator is
//    written into it directly (phase B), the row part added on top (phase C);
//  * the laminate pairs are read through the read-only data cache (the table
//    holds a few materials, so all lanes of a warp usually read the same
//    pair); material index and stiffness factor come one row ahead;
//  * lanes without an element (the strip's left halo at the plate edge,
//    lanes past the plate, rows past the task) run the same code on finite
//    data with a zero stiffness factor, so the phases have no divergent
//    branches and such lanes contribute exact zeros.
// Every bulk copy starts and ends on a 16-byte boundary: it covers the needed
// columns rounded out to 4 floats, and a per-row offset locates column 0.
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
#define SHM_F32_KB 6
#endif
constexpr int KB = SHM_F32_KB;  // column nodes per laminate read in phase B (divides 6)
static_assert(NP % KB == 0, "laminate blocks cover the column");


// --- mbarrier and bulk copies (one CTA, no cluster) -------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
// waits for the phase with the given parity; gives up after a bounded number
// of polls (returns false) instead of spinning for ever
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (int it = 0; it < (1 << 16); ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// One line of floats to copy: global element indices [lo, hi) of `base`
// (lo >= 0), to be read back as column c of the line at smem[c + off] where
// `origin` is the global index of column 0.  The copy is rounded out to
// 16-byte boundaries (base is 16-byte aligned): it starts at lo & ~3 and
// moves whole 16-byte units, so off = origin - (lo & ~3).
struct Line {
  const float* src;
  unsigned bytes;
  int off;
};
__device__ __forceinline__ Line line_of(const float* base, long long origin, long long lo, long long hi) {
  Line l;
  const long long a = lo & ~3LL, e = (hi + 3) & ~3LL;
  l.src = base + a;
  l.bytes = hi > lo ? (unsigned)((e - a) * 4) : 0u;
  l.off = (int)(origin - a);
  return l;
}

template <int EW> struct F32Geom {
  static constexpr int G = 32 / EW;
  static constexpr int W = 5 * EW + 1;               // band columns
  static constexpr int OWN = 5 * (EW - 1);           // owned columns
  static constexpr int WP = (W + 6 + 3) / 4 * 4;     // ring line stride (floats): W + alignment slack
  static constexpr int URING = 11;                   // u_n node rows kept
  static constexpr int URAW = URING * 5 * WP;
  static constexpr int UGS = URAW + ((16 - URAW % 32) + 64) % 32;   // group stride = 16 mod 32 (a multiple of 4)
  static constexpr int FRAW = 6 * 5 * W;
  static constexpr int FGS = FRAW + ((16 - FRAW % 32) + 64) % 32;
  static constexpr int EDGE = 6 * 5 * CTA_ELEMS;     // column part of each lane's column 5 [row][field][lane]
  static_assert(UGS % 4 == 0 && WP % 4 == 0, "bulk-copy targets stay 16-byte aligned");
};

// shared-memory layout (floats): ys, vred, edge | ring | band
template <int EW> struct F32Smem {
  using GM = F32Geom<EW>;
  static constexpr int YS = 0;
  static constexpr int VRED = CTA_ELEMS * ELEM_STRIDE;
  static constexpr int EDGE = VRED + NP * CTA_ELEMS;
  static constexpr int RING = (EDGE + GM::EDGE + 3) / 4 * 4;
  static constexpr int BAND = RING + GM::G * GM::UGS;
  static constexpr int END = BAND + GM::G * GM::FGS;
};

template <int EW>
constexpr size_t struct_f32_smem_bytes() {
  return sizeof(float) * F32Smem<EW>::END;
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
  const int* __restrict__ f_rowptr;  // node-row pointer tables of the task force and output lists
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
  int has, nrows, eyA, block, strip, plate, ney, nex, NX, f0, fn, fr0, scen, o0, on, or0;
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
  t.fr0 = tk.fr0;
  t.o0 = tk.o0;
  t.on = tk.on;
  t.or0 = tk.or0;
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

// Issues, from one warp, the bulk copies of one phase of the CTA's mbarrier
// and arrives on it with their byte count: u_n node rows [r0, r0 + nr) of
// each lane group's task (relative to its first node row 5 eyA), all five
// fields, into ring slots slot0, slot0 + 1, ...  Rows off the plate are
// skipped; the slot's column offset goes to roff.
template <int EW>
__device__ __forceinline__ void issue_lines(const F32Args& a, const GroupTask* gt, const float* cur, float* ring,
                                            int* roff, unsigned bar, int r0, int nr, int slot0) {
  using GM = F32Geom<EW>;
  constexpr int G = GM::G, UR = GM::URING;
  const int lane = threadIdx.x & 31;
  const int ntot = G * nr * 5;
  unsigned bytes = 0;
  for (int k = lane; k < ntot; k += 32) {
    const int gg = k / (nr * 5), rem = k % (nr * 5), rr = rem / 5, f = rem % 5;
    const GroupTask& t = gt[gg];
    const int row = 5 * t.eyA + r0 + rr;
    int sl = slot0 + rr;
    if (sl >= UR) sl -= UR;
    const long long rowbeg = t.node0 + (long long)row * t.NX;
    const long long origin = rowbeg + 5 * (t.strip * (EW - 1) - 1);
    const long long lo = max(origin, rowbeg), hi = min(origin + GM::W, rowbeg + t.NX);
    const Line l = line_of(cur + f * a.nnode_pad, origin, lo, (t.has && row <= 5 * t.ney) ? hi : lo);
    if (f == 0) roff[gg * UR + sl] = l.off;
    bytes += l.bytes;
    if (l.bytes) bulk_g2s(smem_u32(ring + gg * GM::UGS + (sl * 5 + f) * GM::WP), l.src, l.bytes, bar);
  }
  bytes = __reduce_add_sync(0xffffffffu, bytes);
  if (lane == 0) mbar_arrive_tx(bar, bytes);
}

// kAdj: the adjoint step of the same operator (K symmetric): lambda in
// place of u, residual forces r(n) at the point outputs instead of the
// excitation, and dJ/dd_e -= lambda_n' K_e^0 u_{n-1} accumulated per element
// (FP32 line products, FP64 per-element and across-step sums).
//
// One time step of every task the CTA takes (tasks blockIdx.x, + gridDim.x,
// ...).  `bar` is the CTA's initialised mbarrier and `phase` the parity of its
// next phase: both persist across calls, so a persistent kernel can run many
// steps on one mbarrier.  reuse: the CTA takes the same single task group as
// in its previous call, whose task facts and ring padding are still in shared
// memory.
template <int EW, bool kSensor, bool kAdj>
__device__ __forceinline__ void struct_f32_step(const F32Args& a, int kstep, unsigned bar, unsigned& phase,
                                                bool reuse = false) {
  using GM = F32Geom<EW>;
  using SM = F32Smem<EW>;
  constexpr int G = GM::G;
  constexpr int W = GM::W;
  constexpr int WP = GM::WP;
  constexpr int OWN = GM::OWN;
  constexpr int NCOL = (OWN + 31) / 32;  // update passes over a band row's owned columns
  constexpr int UR = GM::URING;
  extern __shared__ __align__(16) unsigned char smraw[];
  float* sm = reinterpret_cast<float*>(smraw);
  float* vred = sm + SM::VRED;
  float* edge = sm + SM::EDGE;
  float* ring = sm + SM::RING;
  float* band = sm + SM::BAND;
  __shared__ int roff[G * UR];  // ring slot -> smem offset of relative column 0
  __shared__ GroupTask gt[G];   // task facts of the lane groups (shared, not in registers)

  const int nn = *a.d_base + kstep;
  const bool odd = ((nn - a.nn_first) & 1);
  const float* cur = odd ? a.UB : a.UA;
  float* prev = odd ? a.UA : a.UB;
  float* dst = a.outp ? a.outp : prev;
  // (read through L2: in a persistent launch other CTAs wrote these words
  // in the previous step, and this SM's L1 may hold an older copy)
  if (blockIdx.x == 0)
    for (int q = threadIdx.x; q < a.nout; q += blockDim.x)
      a.displ[(int64_t)q * a.nft + (nn - 1)] = (double)__ldcg(cur + a.out_field[q] * a.nnode_pad + a.out_node[q]);

  const int j = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int g = lane / EW;
  const int q = lane % EW;
  float* ys = sm + SM::YS + lane * ELEM_STRIDE;
  const bool frame = !kAdj && a.fs.frm_int > 0 && (nn % a.fs.frm_int) == 0;  // (no frames in the adjoint)
  const bool guard = guard_step(a.fs, nn);
  const int ntg = (a.ntask + G - 1) / G;
  bool bad = false, late = false;
  bool gpend = false;      // adjoint: an element's gradient partials await reduction
  long long gpend_e = 0;   // (its grid-order index)

  for (int tg = blockIdx.x; tg < ntg; tg += gridDim.x) {
    __syncthreads();
    if (!reuse) {
      if (threadIdx.x < G) gt[threadIdx.x] = load_group_task(a, tg * G + threadIdx.x);
      // columns that no copy of this task writes stay finite (lanes without
      // an element read them); the copies write the same columns every step
      for (int i = threadIdx.x; i < G * GM::UGS; i += blockDim.x) ring[i] = 0.f;
      // the bulk copies (async proxy) write ring words just zeroed through
      // the generic proxy: order the two
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    // band row 0 is the one the first element row adds to (the column part
    // of the others is stored, not added)
    for (int g2 = 0; g2 < G; ++g2)
      for (int i = threadIdx.x; i < 5 * GM::W; i += blockDim.x) band[g2 * GM::FGS + i] = 0.f;
    __syncthreads();
    int maxrows = 0;
#pragma unroll
    for (int gg = 0; gg < G; ++gg) maxrows = max(maxrows, gt[gg].nrows);
    // the task's first six node rows (one mbarrier phase, waited at row 0)
    if (j == 0 && maxrows > 0) issue_lines<EW>(a, gt, cur, ring, roff, bar, 0, 6, 0);
    // this lane's element column, kept in registers for the whole task; a lane
    // without an element reads the columns of the nearest lane that has one
    const GroupTask& t = pick<G>(gt, g);
    const int t_nrows = t.nrows, t_nex = t.nex;
    const int ex = t.strip * (EW - 1) - 1 + q;
    const bool colok = ex >= 0 && ex < t_nex;
    const int qc = min(max(q, t.strip == 0 ? 1 : 0), t_nex - (t.strip * (EW - 1) - 1) - 1);
    const long long eg0 = t.egrid0 + (long long)t.eyA * t_nex + ex;
    const float t_sx = t.sx, t_sy = t.sy, t_area4 = t.area4;
    float* ub = ring + g * GM::UGS + 5 * qc;
    const int* uoff = roff + g * UR;
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
    // material and stiffness factor of the lane's element in the current
    // row (factor 0 where there is no element), the next row's read ahead
    int mcur = 0, mnext = 0;
    float keep = 0.f, knext = 0.f;
    if (t_nrows > 0 && colok) {
      mcur = a.emat_g[eg0];
      keep = a.ekeep_g[eg0];
    }

    int rb = 0;   // ring slot of the element row's first node row, (5 r) mod 11
    int rb6 = 0;  // r mod 6
    for (int r = 0; r < maxrows; ++r) {
      // this row's node rows have landed (the phase issued at the previous
      // row's start); the barrier also ends the previous row's update for
      // every warp, so the ring slots of the previous row's first five node
      // rows are free
      if (!late) late = !mbar_wait(bar, phase);  // after one timeout, no further waits
      phase ^= 1u;
      __syncthreads();
      if (kAdj && gpend) {  // previous element row's gradient partials are complete
        double sum = 0.0;
#pragma unroll
        for (int i = 0; i < NP; ++i) sum += (double)vred[i * CTA_ELEMS + lane];
        atomicAdd(&a.grad[a.e_of_g[gpend_e]], -sum);  // one thread per element: no waiting on a read
        gpend = false;
      }
      // the next element row's five new node rows (5r+6 .. 5r+10)
      if (j == 5 && r + 1 < maxrows)  // warp 5: it has no band row to update in most rows
        issue_lines<EW>(a, gt, cur, ring, roff, bar, 5 * r + 6, 5, rb + 6 >= UR ? rb + 6 - UR : rb + 6);
      const bool rowact = r < t_nrows;
      const bool valid = rowact && colok;
      const long long egrid = eg0 + (long long)r * t_nex;
      if (r + 1 < t_nrows && colok) {
        mnext = a.emat_g[egrid + t_nex];
        knext = a.ekeep_g[egrid + t_nex];
      } else {
        mnext = 0;
        knext = 0.f;
      }
      auto slot = [rb](int k) { const int s = rb + k; return s >= UR ? s - UR : s; };

      // phase A: row j, xi-derivatives (scaled by 2/ax) to ys
      {
        const int sj = slot(j);
        const float* urow = ub + sj * 5 * WP + uoff[sj];
        float2 acc[5][3];
#pragma unroll
        for (int k = 0; k < NP; ++k)
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            const float2 u2 = bc2(urow[f * WP + k]);
#pragma unroll
            for (int p = 0; p < 3; ++p) acc[f][p] = k == 0 ? mul2(c_Dp[0][p], u2) : fma2(c_Dp[k][p], u2, acc[f][p]);
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
      // band row of logical row m of this element row (row 0 carries the
      // previous element row's top line)
      auto prow_of = [rb6](int m) { const int p = m - rb6; return p < 0 ? p + 6 : p; };
      float dl = 0.f;  // adjoint: this thread's share of the element's gradient partial
      // phase B: column i = j; the column part of the transposed operator goes
      // straight into the band (column 5 of a lane is column 0 of the next
      // lane's element: kept in `edge` for it, except at the strip's end)
      {
        const int i = j;
        float2 Fe2[5][3];
        float vp = 0.f;
        float v[5][NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
          const int sk = slot(k);
          const float* urow = ub + sk * 5 * WP + uoff[sk] + i;
#pragma unroll
          for (int f = 0; f < 5; ++f) v[f][k] = urow[f * WP];
        }
        // eta-derivatives, packed over node pairs, scaled by 2/ay
        float2 de2[5][3];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
#pragma unroll
          for (int m = 0; m < NP; ++m) {
            const float2 v2 = bc2(v[f][m]);
#pragma unroll
            for (int p = 0; p < 3; ++p) de2[f][p] = m == 0 ? mul2(c_Dp[0][p], v2) : fma2(c_Dp[m][p], v2, de2[f][p]);
          }
#pragma unroll
          for (int p = 0; p < 3; ++p) de2[f][p] = mul2(de2[f][p], bc2(t_sy));
        }
        // laminate pairs of the element's material (read-only data cache)
        const float2* __restrict__ L = a.matp + mcur * LAMP;
        // the stiffness factor scales the element's fluxes (K_e^0 for the
        // adjoint); zero for lanes and rows without an element
        const float akeep = valid ? (kAdj ? t_area4 : t_area4 * keep) : 0.f;
        // nodes k of the column in blocks of KB: each laminate pair is read
        // once per block (the products keep their order)
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
              const float2 l = __ldg(L + 6 * b + c);
#pragma unroll
              for (int kk = 0; kk < KB; ++kk)
                R[b][kk] = c == 0 ? mul2(l, bc2(sn[kk][c])) : fma2(l, bc2(sn[kk][c]), R[b][kk]);
            }
          {
            const float2 l18 = __ldg(L + 18), l19 = __ldg(L + 19);
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
              for (int p = 0; p < 3; ++p) Fe2[f][p] = k == 0 ? mul2(c_DTp[0][p], ge) : fma2(c_DTp[k][p], ge, Fe2[f][p]);
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
        if (kSensor) vred[i * CTA_ELEMS + lane] = vp;
        if constexpr (kAdj) {
          // lambda' K_e^0 u_{n-1} over the element's nodes: here only row 0's
          // column part (row 0 joins the carried band row, so it is scaled by
          // keep_e now).  Rows 1-5 of the column part stay unscaled in the
          // band (and in `edge`): phase C adds the row part there, takes the
          // node's whole term and scales.
          if (valid) {
            const float* umc = a.um + t.node0 + (int64_t)(5 * (t.eyA + r)) * t.NX + 5 * ex + i;
#pragma unroll
            for (int f = 0; f < 5; ++f) dl += Fe2[f][0].x * umc[f * a.nnode_pad];
          }
#pragma unroll
          for (int f = 0; f < 5; ++f) Fe2[f][0].x *= keep;
        }
        // column part at rows m = 0..5 of column i (zeros from lanes without
        // an element, so that stale band values never survive)
        if (i < 5 || q == EW - 1) {
          float* col = fb + 5 * q + i;
          int pr[6];
#pragma unroll
          for (int m = 0; m < 6; ++m) pr[m] = prow_of(m) * 5 * W;
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            col[pr[0] + f * W] += Fe2[f][0].x;   // the carried row: added to
            col[pr[1] + f * W] = Fe2[f][0].y;
            col[pr[2] + f * W] = Fe2[f][1].x;
            col[pr[3] + f * W] = Fe2[f][1].y;
            col[pr[4] + f * W] = Fe2[f][2].x;
            col[pr[5] + f * W] = Fe2[f][2].y;
          }
        } else {
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int p = 0; p < 3; ++p) {
              edge[((2 * p) * 5 + f) * CTA_ELEMS + lane] = Fe2[f][p].x;
              edge[((2 * p + 1) * 5 + f) * CTA_ELEMS + lane] = Fe2[f][p].y;
            }
        }
      }
      __syncthreads();

      // the update's global loads for band row j, issued before phase C
      float uo_r[G][NCOL][5], mt_r[G][NCOL], mr_r[G][NCOL];
#pragma unroll
      for (int gg = 0; gg < G; ++gg) {
        const bool rok = r >= ulo[gg] && r < uhi[gg];
        const long long rbase = ub0[gg] + (long long)r * ustr[gg];
#pragma unroll
        for (int s2 = 0; s2 < NCOL; ++s2) {
          const int c = lane + 32 * s2;
          if (rok && c < ucol[gg]) {
            const long long node = rbase + c;
            mt_r[gg][s2] = a.minv[node];
            mr_r[gg][s2] = a.minv[a.nnode_pad + node];
#pragma unroll
            for (int f = 0; f < 5; ++f) uo_r[gg][s2][f] = prev[f * a.nnode_pad + node];
          }
        }
      }
      // phase C: xi-part of the transposed operator, added to the band
      float out[5][NP];
#pragma unroll
      for (int f = 0; f < 5; ++f) {
        float2 o2[3];
#pragma unroll
        for (int ii = 0; ii < NP; ++ii) {
          const float2 gg2 = bc2(ys[f * NPE + ii * NP + j]);
#pragma unroll
          for (int p = 0; p < 3; ++p) o2[p] = ii == 0 ? mul2(c_DTp[0][p], gg2) : fma2(c_DTp[ii][p], gg2, o2[p]);
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          out[f][2 * p] = o2[p].x;
          out[f][2 * p + 1] = o2[p].y;
        }
      }
      if constexpr (kAdj) {
        // K_e^0 lambda at the element's nodes of line j: the row part plus,
        // for j > 0, the element's own column part (unscaled in the band, in
        // `edge` for column 5 unless this is the strip's last lane); its
        // product with u_{n-1} is the line's share of lambda' K_e^0 u_{n-1};
        // then keep_e K_e^0 lambda for the band
        const float* bsrc = fb + prow_of(j) * 5 * W + 5 * q;
        const float* umr = a.um + t.node0 + (int64_t)(5 * (t.eyA + r) + j) * t.NX + 5 * ex;
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int i = 0; i < NP; ++i) {
            float tot = out[f][i];
            if (j > 0) tot += (i < 5 || q == EW - 1) ? bsrc[f * W + i] : edge[(j * 5 + f) * CTA_ELEMS + lane];
            if (valid) dl += tot * umr[f * a.nnode_pad + i];
            out[f][i] = keep * tot;
          }
        if (valid) vred[j * CTA_ELEMS + lane] = dl;
      }
      // band accumulation: logical row j of this element row is physical row
      // (j - r) mod 6 and already holds the column part (phase B).  Column
      // i = 5 of a lane's element is column 0 of the next lane's: its row
      // part moves one lane up by shuffle and its column part comes from
      // `edge`; the strip's last lane adds it itself.
      const int prow = prow_of(j);
      {
        float* bdst = fb + prow * 5 * W + 5 * q;
        if (kAdj && j > 0) {
          // out holds keep_e x (column + row part) of the element's nodes: it
          // replaces the band entries; column 5 is the next lane's column 0
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            const float from_left = __shfl_up_sync(0xffffffffu, out[f][5], 1);
            if (q > 0) out[f][0] += from_left;
          }
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int i = 0; i < 5; ++i) bdst[f * W + i] = out[f][i];
          if (q == EW - 1) {
#pragma unroll
            for (int f = 0; f < 5; ++f) bdst[f * W + 5] = out[f][5];
          }
        } else {
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            const float from_left = __shfl_up_sync(0xffffffffu, out[f][5], 1);
            if (q > 0) out[f][0] += from_left + edge[(j * 5 + f) * CTA_ELEMS + lane - 1];
          }
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int i = 0; i < 5; ++i) bdst[f * W + i] += out[f][i];
          if (q == EW - 1) {
#pragma unroll
            for (int f = 0; f < 5; ++f) bdst[f * W + 5] += out[f][5];
          }
        }
        // band row j is now complete and written by this warp alone (the
        // column parts of all warps were stored before the third barrier),
        // and warp j updates exactly band row j: a warp barrier suffices.
        // (The adjoint's gradient partials are reduced after the next CTA
        // barrier.)
        __syncwarp();
      }
      if constexpr (!kAdj) {
        // excitation of this band row's owned nodes: the task's forces are
        // ordered by node row (merged per DOF) and indexed by node row, and
        // the warp's lanes subtract the row's entries from the completed
        // band row (distinct DOFs: no two lanes meet)
#pragma unroll
        for (int gg = 0; gg < G; ++gg) {
          const GroupTask& t2 = pick<G>(gt, gg);
          if (t2.fn == 0 || !(r >= ulo[gg] && r < uhi[gg])) continue;
          const int c0 = a.f_rowptr[t2.fr0 + 5 * r + j], c1 = a.f_rowptr[t2.fr0 + 5 * r + j + 1];
          if (c1 > c0) {
            const double sv = a.st[(int64_t)t2.scen * a.nft + (nn - 1)];
            float* brow = band + gg * GM::FGS + prow * 5 * W;
            for (int fi = c0 + lane; fi < c1; fi += 32)
              brow[a.f_field[fi] * W + a.f_xl[fi]] -= (float)(a.f_val[fi] * sv);
            __syncwarp();
          }
        }
      } else {
        // the adjoint's residual forces at the point outputs of this band row
        // (a few entries: one lane adds them in list order)
#pragma unroll
        for (int gg = 0; gg < G; ++gg) {
          const GroupTask& t2 = pick<G>(gt, gg);
          if (t2.on == 0 || !(r >= ulo[gg] && r < uhi[gg])) continue;
          const int c0 = a.f_rowptr[t2.or0 + 5 * r + j], c1 = a.f_rowptr[t2.or0 + 5 * r + j + 1];
          if (c1 > c0) {
            if (lane == 0) {
              float* brow = band + gg * GM::FGS + prow * 5 * W;
              for (int oi = c0; oi < c1; ++oi)
                brow[a.o_field[oi] * W + a.o_xl[oi]] += (float)a.asig[(int64_t)a.o_q[oi] * a.nft + (nn - 1)];
            }
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
      // update owned, complete nodes of band row j (excitation subtracted
      // above by the node's owner)
#pragma unroll
      for (int gg = 0; gg < G; ++gg) {
        if (!(r >= ulo[gg] && r < uhi[gg])) continue;
        const long long rowbase = ub0[gg] + (long long)r * ustr[gg];
        const float* urow = ring + gg * GM::UGS + slot(j) * 5 * WP + roff[gg * UR + slot(j)] + 5;
        const float* bnd = band + gg * GM::FGS + prow * 5 * W + 5;
#pragma unroll
        for (int s = 0; s < NCOL; ++s) {
          const int c = lane + 32 * s;
          if (c >= ucol[gg]) continue;
          const long long node = rowbase + c;
          float F[5];
#pragma unroll
          for (int f = 0; f < 5; ++f) F[f] = bnd[f * W + c];
          if (!kAdj && a.pr.npf > 0) F[4] -= pressure_load(a.pr, nn, a.nnode_pad, node);
#pragma unroll
          for (int f = 0; f < 5; ++f) {
            const float u = urow[f * WP + c];
            const float uo = uo_r[gg][s][f];
            const float im = (f == 1 || f == 3) ? mr_r[gg][s] : mt_r[gg][s];
            const float un = u + a.k1[f] * (u - uo) - a.k2[f] * (im * F[f]);
            dst[f * a.nnode_pad + node] = un;
            if (frame) store_frame(a.fs, a.frames, a.nnode_pad, node, f, nn, u, uo, un, a.a0, a.a1);
            if (guard && (!isfinite(un) || (f == 4 && u > a.blowup))) bad = true;
          }
        }
      }
      // (the next row's first barrier separates this update from the ring
      // refill and the next band accumulation)
      mcur = mnext;
      keep = knext;
      rb += 5;
      if (rb >= UR) rb -= UR;
      if (++rb6 == 6) rb6 = 0;
    }
    __syncthreads();
    if (kAdj && gpend) {  // the task's last element row
      double sum = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) sum += (double)vred[i * CTA_ELEMS + lane];
      atomicAdd(&a.grad[a.e_of_g[gpend_e]], -sum);
      gpend = false;
    }
  }
  if (bad) atomicOr(a.flag, 1);
  if (late) atomicOr(a.flag, 2);  // a bounded wait gave up: reported as SHM_ERR_TIMEOUT
}

// One time step per launch (CUDA-graph chunks of launches advance a plan).
template <int EW, bool kSensor, bool kAdj = false>
__global__ void __launch_bounds__(CTA_THREADS, 2) k_struct_step_f32(F32Args a, int kstep) {
  __shared__ __align__(8) unsigned long long bar_mem;
  const unsigned bar = smem_u32(&bar_mem);
  if (threadIdx.x == 0) mbar_init(bar, 1);  // (made visible by the step's first CTA barrier)
  unsigned phase = 0;
  struct_f32_step<EW, kSensor, kAdj>(a, kstep, bar, phase);
}

// --- persistent stepping -----------------------------------------------------
// Device-wide barrier between the steps of a persistent launch, on one word
// that the host zeroes before each launch: every CTA adds 1 when it arrives
// (a releasing add), so barrier k is complete when the count reaches
// (k + 1) x gridDim.x, which each CTA then reads with acquiring loads.  Bit 31
// is the abort bit: a CTA whose wait runs out of polls sets it, and every CTA
// leaves at its next barrier instead of waiting (the host reads
// SHM_ERR_TIMEOUT from the flag).  The count stays below bit 31 because the
// host splits runs so that steps x CTAs < 2^30.
struct GridSync {
  unsigned* ctr;
  int spin;  // polls before a wait gives up
};
constexpr unsigned kGridAbort = 0x80000000u;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned atom_add_release_gpu(unsigned* p, unsigned x) {
  unsigned old;
  asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;\n" : "=r"(old) : "l"(p), "r"(x) : "memory");
  return old;
}

// Barrier number k of the launch.  Returns false (in every thread of the
// CTA) when the CTA must stop.
__device__ __forceinline__ bool grid_sync(const GridSync& gs, unsigned k, int* flag) {
  __shared__ int s_go;
  __syncthreads();  // the CTA's stores of this step before its arrival
  if (threadIdx.x == 0) {
    const unsigned target = (k + 1) * gridDim.x;
    const unsigned old = atom_add_release_gpu(gs.ctr, 1u);
    int go = 0;
    if (!(old & kGridAbort)) {
      if (old + 1 == target) {
        go = 1;  // the last CTA to arrive
      } else {
        for (int it = 0; it < gs.spin; ++it) {
          const unsigned v = ld_acquire_gpu(gs.ctr);
          if (v & kGridAbort) break;
          if (v >= target) {
            go = 1;
            break;
          }
        }
        if (!go) {
          atomicOr(gs.ctr, kGridAbort);
          atomicOr(flag, 2);
        }
      }
    }
    s_go = go;
  }
  __syncthreads();
  const bool go = s_go != 0;
  // the next step's bulk copies (async proxy) read other CTAs' stores of
  // this step (generic proxy), which the acquire above made visible
  asm volatile("fence.proxy.async.global;\n" ::: "memory");
  return go;
}

// All `nsteps` steps in one cooperative launch: every CTA is resident, and
// the CTAs meet at a device-wide barrier between steps where consecutive
// launches would meet at the kernel boundary.  The grid may be smaller than
// the task list (each CTA takes every gridDim.x-th task group in each step).
template <int EW, bool kSensor>
__global__ void __launch_bounds__(CTA_THREADS, 2) k_struct_run_f32(F32Args a, int nsteps, GridSync gs) {
  __shared__ __align__(8) unsigned long long bar_mem;
  const unsigned bar = smem_u32(&bar_mem);
  if (threadIdx.x == 0) mbar_init(bar, 1);
  unsigned phase = 0;
  // with at most one task group per CTA, the CTA keeps its group across steps
  const bool single = (a.ntask + F32Geom<EW>::G - 1) / F32Geom<EW>::G <= (int)gridDim.x;
  for (int k = 0; k < nsteps; ++k) {
    struct_f32_step<EW, kSensor, false>(a, k, bar, phase, single && k > 0);
    if (k + 1 < nsteps && !grid_sync(gs, (unsigned)k, a.flag)) break;
  }
}

}  // namespace shm
