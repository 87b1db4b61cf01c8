// Structured fused flat-shell step: one kernel per time step, no scratch.
//
// For plates meshed as an nex x ney grid of equal axis-aligned rectangles
// (the synthetic plates and the structured part of quad2spectral_Fiborek.m)
// the element step, the assembly (12-basket scatter, main_flat_shell.m:724-726)
// and the central-difference update (:742-750) are fused.  A work item
// ("task") is a strip of EW-1 element columns x H element rows of one plate.
// Its CTA lane group owns EW lanes = elements ex = strip*(EW-1)-1 .. +EW-1:
// lane 0 is the left neighbour (halo) so that the strip's left node column
// receives both contributions.  The CTA sweeps the strip's element rows from
// bottom to top (starting one halo row below the block); the element forces of
// a row are summed into a shared-memory band of 6 node rows; node rows
// 5*ey .. 5*ey+4 are then complete and are updated in place, and band row 5 is
// carried to the next element row.  Every node is owned by exactly one task,
// so a step needs no atomics and no global scratch, and the summation order is
// fixed (even lanes, then odd lanes, then the carried row).
#pragma once
#include "shell_element.cuh"

namespace shm {

struct PlateDesc {
  int nex, ney, NX, scen;
  long long node0;   // first global node (0-based)
  long long egrid0;  // first element in grid order (ey*nex + ex)
  double sx, sy, area4;
};

// task: plate, strip, block, rows, first force entry, force count, first
// point-output entry, point-output count (the outputs the task's update owns),
// and the offsets of the forces' and the outputs' node-row pointer tables
// (-1 for a task without them)
struct TaskDesc {
  int plate, strip, block, nrows;
  int f0, fn, o0, on;
  int fr0, or0;
};

template <typename T> struct StructArgs {
  const PlateDesc* __restrict__ plates;
  const TaskDesc* __restrict__ tasks;
  int ntask, H, nn_first, nft;
  int64_t nnode_pad;
  T* UA;
  T* UB;
  T* outp;  // u_{n+1} destination; null = over u_{n-1}
  PressureArgs<T> pr;
  const T* __restrict__ minv;
  T k1[5], k2[5];
  const T* __restrict__ mat;
  const int* __restrict__ emat_g;
  const T* __restrict__ ekeep_g;
  const int* __restrict__ esens_g;
  // forces (per task)
  const int* __restrict__ f_xl;
  const int* __restrict__ f_iy;
  const int* __restrict__ f_field;
  const double* __restrict__ f_val;
  const double* __restrict__ st;
  // outputs
  int nout;
  const int* __restrict__ out_node;
  const int* __restrict__ out_field;
  double* displ;
  double* vsum;
  SensorConst<T> sc;
  FrameSpec fs;
  T* frames;
  T a0, a1, blowup;
  int* flag;
  const int* d_base;
};

template <int EW> struct BandGeom {
  static constexpr int G = 32 / EW;                // lane groups per CTA
  static constexpr int W = 5 * EW + 1;             // node columns of a band
  static constexpr int OWN = 5 * (EW - 1);         // owned node columns per strip
  static constexpr int RAW = 6 * 5 * W;            // words of one group's band
  static constexpr int GSTRIDE = RAW + ((16 - RAW % 32) + 64) % 32;  // = 16 mod 32
};

template <typename T, int EW>
constexpr size_t struct_smem_bytes() {
  return sizeof(T) * (2 * CTA_ELEMS * ELEM_STRIDE + NP * CTA_ELEMS + BandGeom<EW>::G * BandGeom<EW>::GSTRIDE);
}

template <typename T, int EW>
__global__ void __launch_bounds__(CTA_THREADS, sizeof(T) == 4 ? 3 : 1) k_struct_step(StructArgs<T> a, int kstep) {
  using BG = BandGeom<EW>;
  constexpr int G = BG::G;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  T* vred = sm + 2 * CTA_ELEMS * ELEM_STRIDE;
  T* band = vred + NP * CTA_ELEMS;

  const int nn = *a.d_base + kstep;
  const bool odd = ((nn - a.nn_first) & 1);
  const T* __restrict__ cur = odd ? a.UB : a.UA;
  T* prev = odd ? a.UA : a.UB;
  if (blockIdx.x == 0)
    for (int q = threadIdx.x; q < a.nout; q += blockDim.x)
      a.displ[(int64_t)q * a.nft + (nn - 1)] = (double)cur[a.out_field[q] * a.nnode_pad + a.out_node[q]];

  const int j = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int g = lane / EW;  // my lane group
  const int q = lane % EW;  // element within the strip
  T* xs = sm + lane * ELEM_STRIDE;
  T* ys = sm + (CTA_ELEMS + lane) * ELEM_STRIDE;
  const bool frame = a.fs.frm_int > 0 && (nn % a.fs.frm_int) == 0;
  const bool guard = guard_step(a.fs, nn);
  const int ntg = (a.ntask + G - 1) / G;
  bool bad = false;

  for (int tg = blockIdx.x; tg < ntg; tg += gridDim.x) {
    // my group's task
    const int tid = tg * G + g;
    const bool has = tid < a.ntask;
    TaskDesc tk = has ? a.tasks[tid] : TaskDesc{0, 0, 0, 0, 0, 0, 0, 0};
    const PlateDesc pl = a.plates[tk.plate];
    const int eyA = tk.block == 0 ? 0 : tk.block * a.H - 1;
    const int nrows = has ? tk.nrows : 0;
    int maxrows = 0;
#pragma unroll
    for (int gg = 0; gg < G; ++gg) {
      const int t2 = tg * G + gg;
      if (t2 < a.ntask) maxrows = max(maxrows, a.tasks[t2].nrows);
    }
    const int ex = tk.strip * (EW - 1) - 1 + q;
    T* myband = band + g * BG::GSTRIDE;
    const GeoRect<T> geo{(T)pl.sx, (T)pl.sy, (T)pl.area4};

    for (int i = threadIdx.x; i < G * BG::GSTRIDE; i += blockDim.x) band[i] = T(0);
    __syncthreads();

    for (int r = 0; r < maxrows; ++r) {
      const int ey = eyA + r;
      const bool rowact = r < nrows;
      const bool valid = rowact && ex >= 0 && ex < pl.nex;
      const int64_t egrid = pl.egrid0 + (int64_t)ey * pl.nex + ex;
      // phase A
      {
        T u[5][NP];
        if (valid) {
          const int64_t base = pl.node0 + (int64_t)(5 * ey + j) * pl.NX + 5 * ex;
#pragma unroll
          for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int f = 0; f < 5; ++f) u[f][i] = cur[f * a.nnode_pad + base + i];
        } else {
#pragma unroll
          for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int f = 0; f < 5; ++f) u[f][i] = T(0);
        }
        row_deriv_store(u, xs, ys, j);
      }
      __syncthreads();
      // phase B
      if (valid) {
        const int i = j;
        T v[5][NP];
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int k = 0; k < NP; ++k) v[f][k] = xs[f * NPE + i * NP + k];
        const Lam<T> L = load_lam(a.mat + (int64_t)a.emat_g[egrid] * MAT_STRIDE_DEV, a.ekeep_g[egrid]);
        T Fe[5][NP];
        const T vp = shell_column<T, GeoRect<T>, true>(v, ys, xs, i, L, geo, Fe, a.sc);
#pragma unroll
        for (int f = 0; f < 5; ++f)
#pragma unroll
          for (int m = 0; m < NP; ++m) ys[f * NPE + i * NP + m] = Fe[f][m];
        vred[i * CTA_ELEMS + lane] = vp;
      }
      __syncthreads();
      // phase C, then accumulate into the band: even lanes, then odd lanes
      T out[5][NP];
      if (valid) row_transpose_apply(xs, ys, j, out);
#pragma unroll
      for (int parity = 0; parity < 2; ++parity) {
        if (valid && (q & 1) == parity) {
#pragma unroll
          for (int f = 0; f < 5; ++f)
#pragma unroll
            for (int i = 0; i < NP; ++i) myband[(j * 5 + f) * BG::W + 5 * q + i] += out[f][i];
        }
        __syncthreads();
      }
      // PZT sensor partial of owned elements
      const bool owned_row = rowact && (tk.block == 0 || r > 0);
      if (j == 0 && valid && owned_row && q > 0) {
        const int slot = a.esens_g[egrid];
        if (slot >= 0) {
          double s = 0.0;
#pragma unroll
          for (int i = 0; i < NP; ++i) s += (double)vred[i * CTA_ELEMS + lane];
          a.vsum[(int64_t)slot * a.nft + (nn - 1)] = s;
        }
      }
      const bool top = (ey == pl.ney - 1);
      const int nupd = top ? 6 : 5;
      // excitation on owned nodes of this band
      if (owned_row && q == 0 && j == 0) {
        for (int fi = tk.f0; fi < tk.f0 + tk.fn; ++fi) {
          const int rr = a.f_iy[fi] - 5 * ey;
          if (rr >= 0 && rr < nupd) {
            const double sv = a.st[(int64_t)pl.scen * a.nft + (nn - 1)];
            myband[(rr * 5 + a.f_field[fi]) * BG::W + a.f_xl[fi]] -= (T)(a.f_val[fi] * sv);
          }
        }
      }
      __syncthreads();
      // update owned, complete nodes: band rows 0..4 (and 5 at the plate top)
      for (int idx = threadIdx.x; idx < G * 6 * BG::OWN; idx += blockDim.x) {
        const int gg = idx / (6 * BG::OWN);
        const int rem = idx % (6 * BG::OWN);
        const int rr = rem / BG::OWN;
        const int c = rem % BG::OWN;
        const int t2 = tg * G + gg;
        if (t2 >= a.ntask) continue;
        const TaskDesc tk2 = a.tasks[t2];
        if (r >= tk2.nrows || (tk2.block > 0 && r == 0)) continue;
        const PlateDesc pl2 = a.plates[tk2.plate];
        const int ey2 = (tk2.block == 0 ? 0 : tk2.block * a.H - 1) + r;
        const int nup2 = (ey2 == pl2.ney - 1) ? 6 : 5;
        if (rr >= nup2) continue;
        const int ix = 5 * tk2.strip * (EW - 1) + c;
        if (ix >= pl2.NX) continue;
        const int64_t node = pl2.node0 + (int64_t)(5 * ey2 + rr) * pl2.NX + ix;
        const T* bnd = band + gg * BG::GSTRIDE;
        const T mt = a.minv[node], mr = a.minv[a.nnode_pad + node];
        const T fp = a.pr.npf > 0 ? pressure_load(a.pr, nn, a.nnode_pad, node) : T(0);
#pragma unroll
        for (int f = 0; f < 5; ++f) {
          const T F = bnd[(rr * 5 + f) * BG::W + 5 + c] - (f == 4 ? fp : T(0));
          const T u = cur[f * a.nnode_pad + node];
          const T uo = prev[f * a.nnode_pad + node];
          const T im = (f == 1 || f == 3) ? mr : mt;
          const T un = u + a.k1[f] * (u - uo) - a.k2[f] * (im * F);
          (a.outp ? a.outp : prev)[f * a.nnode_pad + node] = un;
          if (frame) store_frame(a.fs, a.frames, a.nnode_pad, node, f, nn, u, uo, un, a.a0, a.a1);
          if (guard && (!isfinite(un) || (f == 4 && u > a.blowup))) bad = true;
        }
      }
      __syncthreads();
      // carry band row 5 to row 0, clear rows 1..5
      for (int idx = threadIdx.x; idx < G * 5 * BG::W; idx += blockDim.x) {
        const int gg = idx / (5 * BG::W);
        const int rem = idx % (5 * BG::W);
        T* bnd = band + gg * BG::GSTRIDE;
        bnd[rem] = bnd[5 * 5 * BG::W + rem];
      }
      __syncthreads();
      for (int idx = threadIdx.x; idx < G * 5 * 5 * BG::W; idx += blockDim.x) {
        const int gg = idx / (5 * 5 * BG::W);
        const int rem = idx % (5 * 5 * BG::W);
        band[gg * BG::GSTRIDE + 5 * BG::W + rem] = T(0);
      }
      __syncthreads();
    }
  }
  if (bad) atomicOr(a.flag, 1);
}

}  // namespace shm
