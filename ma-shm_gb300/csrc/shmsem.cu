// shmsem.cu -- C ABI, plan set-up and the general (unstructured) flat-shell
// step of the GB300 spectral-element engine.
//
// One time step of the reference MAIN LOOP (main_flat_shell.m:651-750) is two
// kernels on the general path:
//   k_elem_general  gather (:655-659) + derivatives (:661-671) + resultants
//                   (:674-681) + transposed operators (:683-689) + PZT voltage
//                   partials (:690-692); element-local forces go to a scratch
//                   array laid out like the reference's F2 (:716-721);
//   k_node_general  deterministic assembly (the 12-basket scatter :724-726,
//                   summed per node in basket order) + the central-difference
//                   update (:742-750) + frames / blow-up guard (:767-804).
// The structured fused path (one kernel per step, no scratch) is in
// shell_structured.cuh.  Both are instantiated for double and float.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "shmsem.h"
#include "shell_element.cuh"
#include "internal.h"

using namespace shm;

// ---------------------------------------------------------------------------
// device kernels: general path
// ---------------------------------------------------------------------------

template <typename T> struct GenArgs {
  // sizes
  int64_t fen_pad, nnode_pad, plane;  // plane: length of one F2 field plane
  int nnode, fen, nn_first, nft;
  // state (two SoA buffers [5][nnode_pad]) and scratch [5][plane]
  T* UA;
  T* UB;
  T* outp;                        // u_{n+1} destination; null = over u_{n-1} (ping-pong)
  const T* __restrict__ grect;    // [3][fen_pad] 2/ax, 2/ay, ax*ay/4 when every element is an
                                  // axis-aligned rectangle (else null: per-node geometry)
  T* F2;
  // mesh
  const int* __restrict__ conn;   // [36][fen_pad], 0-based global nodes
  const T* __restrict__ geo;      // [5][36][fen_pad]
  const int* __restrict__ emat;   // [fen_pad]
  const T* __restrict__ ekeep;    // [fen_pad]
  const T* __restrict__ mat;      // [nmat][24]
  const int* __restrict__ row_ptr;
  const int* __restrict__ slots;
  const T* __restrict__ minv;     // [2][nnode_pad]: 1/M translational, rotational
  T k1[5], k2[5];                 // update coefficients per field
  // excitation: force slots appended after 36*fen_pad in every plane
  int nforce;
  const int* __restrict__ fq_field;
  const int* __restrict__ fq_scen;
  const double* __restrict__ fq_val;
  const double* __restrict__ st;  // [nscen][nft]
  // point outputs
  int nout;
  const int* __restrict__ out_node;
  const int* __restrict__ out_field;
  double* displ;                  // [nout][nft]
  // PZT sensor partial sums
  const int* __restrict__ esens;  // [fen_pad] slot or -1
  double* vsum;                   // [nslot][nft]
  SensorConst<T> sc;
  // frames
  FrameSpec fs;
  T* frames;                      // [nframes][nfields][nnode_pad]
  PressureArgs<T> pr;
  T a0, a1;
  T blowup;                       // 10*h
  int* flag;
  const int* d_base;
  // adjoint (k_elem_adjoint only)
  int nadj;                       // adjoint force slots, one per point output
  const double* __restrict__ asig;  // [nout][nft] misfit residuals in reversed time
  const T* __restrict__ um;       // forward state u_{n-1} paired with this adjoint step
  double* grad;                   // [fen_pad] dJ/dd_e accumulated in FP64
};

template <typename T>
__device__ __forceinline__ void block0_duties(const GenArgs<T>& a, const T* cur, int nn) {
  // excitation samples into the force slots (F2 holds +K*u, so store -f*st)
  const int64_t p36 = (int64_t)NPE * a.fen_pad;
  for (int q = threadIdx.x; q < a.nforce; q += blockDim.x) {
    const double s = a.st[(int64_t)a.fq_scen[q] * a.nft + (nn - 1)];
    const T val = (T)(-a.fq_val[q] * s);
#pragma unroll
    for (int f = 0; f < 5; ++f) a.F2[f * a.plane + p36 + q] = (f == a.fq_field[q]) ? val : T(0);
  }
  // displ(nn,:) = U(outputs): state at the start of the step
  for (int q = threadIdx.x; q < a.nout; q += blockDim.x)
    a.displ[(int64_t)q * a.nft + (nn - 1)] = (double)cur[a.out_field[q] * a.nnode_pad + a.out_node[q]];
}

template <typename T, bool kSensor, bool kRect = false>
__global__ void __launch_bounds__(CTA_THREADS) k_elem_general(GenArgs<T> a, int kstep) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int nn = *a.d_base + kstep;
  const T* __restrict__ cur = ((nn - a.nn_first) & 1) ? a.UB : a.UA;
  if (blockIdx.x == 0) block0_duties(a, cur, nn);

  const int j = threadIdx.x >> 5;   // line (row in phase A/C, column in B)
  const int le = threadIdx.x & 31;  // element within the CTA
  const int e = blockIdx.x * CTA_ELEMS + le;
  T* xs = sm + le * ELEM_STRIDE;
  T* ys = sm + (CTA_ELEMS + le) * ELEM_STRIDE;
  T* vred = sm + 2 * CTA_ELEMS * ELEM_STRIDE;  // [6][32] sensor partials

  // phase A: gather row j of element e (UX=U(Iu) ... :655-659)
  {
    T u[5][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int node = a.conn[(int64_t)(j * NP + i) * a.fen_pad + e];
#pragma unroll
      for (int f = 0; f < 5; ++f) u[f][i] = cur[f * a.nnode_pad + node];
    }
    row_deriv_store(u, xs, ys, j);
  }
  __syncthreads();
  // phase B: column i = j
  {
    const int i = j;
    T v[5][NP];
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int k = 0; k < NP; ++k) v[f][k] = xs[f * NPE + i * NP + k];
    const Lam<T> L = load_lam(a.mat + (int64_t)a.emat[e] * MAT_STRIDE_DEV, a.ekeep[e]);
    T Fe[5][NP];
    T vp;
    if constexpr (kRect) {  // three numbers per element instead of 180 per-node values
      const GeoRect<T> geo{a.grect[e], a.grect[a.fen_pad + e], a.grect[2 * a.fen_pad + e]};
      vp = shell_column<T, GeoRect<T>, kSensor>(v, ys, xs, i, L, geo, Fe, a.sc);
    } else {
      const GeoGeneral<T> geo{a.geo, a.fen_pad, e};
      vp = shell_column<T, GeoGeneral<T>, kSensor>(v, ys, xs, i, L, geo, Fe, a.sc);
    }
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int m = 0; m < NP; ++m) ys[f * NPE + i * NP + m] = Fe[f][m];
    if (kSensor) vred[i * CTA_ELEMS + le] = vp;
  }
  __syncthreads();
  // phase C + write element-local forces F2[f][c][e], c = j*6 + i
  {
    T out[5][NP];
    row_transpose_apply(xs, ys, j, out);
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int i = 0; i < NP; ++i) a.F2[f * a.plane + (int64_t)(j * NP + i) * a.fen_pad + e] = out[f][i];
  }
  if (kSensor && j == 0 && e < a.fen) {
    const int slot = a.esens[e];
    if (slot >= 0) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) s += (double)vred[i * CTA_ELEMS + le];
      a.vsum[(int64_t)slot * a.nft + (nn - 1)] = s;
    }
  }
}

// Adjoint step, element part (general path).  Applies K_e^0 to lambda_{n}
// (current), writes keep_e * K_e^0 lambda to the scratch like the forward
// step, adds the misfit residuals r(n-1) at the point outputs as forces and
// accumulates the damage gradient dJ/dd_e -= lambda_n' K_e^0 u_{n-1} with the
// forward state u_{n-1} of the current checkpoint segment.
template <typename T>
__global__ void __launch_bounds__(CTA_THREADS) k_elem_adjoint(GenArgs<T> a, int kstep) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int nn = *a.d_base + kstep;
  const T* __restrict__ cur = ((nn - a.nn_first) & 1) ? a.UB : a.UA;
  if (blockIdx.x == 0) {
    const int64_t p36 = (int64_t)NPE * a.fen_pad;
    for (int q = threadIdx.x; q < a.nforce; q += blockDim.x)
#pragma unroll
      for (int f = 0; f < 5; ++f) a.F2[f * a.plane + p36 + q] = T(0);
    for (int q = threadIdx.x; q < a.nadj; q += blockDim.x) {
      const T v = (T)a.asig[(int64_t)q * a.nft + (nn - 1)];
#pragma unroll
      for (int f = 0; f < 5; ++f) a.F2[f * a.plane + p36 + a.nforce + q] = (f == a.out_field[q]) ? v : T(0);
    }
  }
  const int j = threadIdx.x >> 5;
  const int le = threadIdx.x & 31;
  const int e = blockIdx.x * CTA_ELEMS + le;
  T* xs = sm + le * ELEM_STRIDE;
  T* ys = sm + (CTA_ELEMS + le) * ELEM_STRIDE;
  T* vred = sm + 2 * CTA_ELEMS * ELEM_STRIDE;
  {
    T u[5][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int node = a.conn[(int64_t)(j * NP + i) * a.fen_pad + e];
#pragma unroll
      for (int f = 0; f < 5; ++f) u[f][i] = cur[f * a.nnode_pad + node];
    }
    row_deriv_store(u, xs, ys, j);
  }
  __syncthreads();
  {
    const int i = j;
    T v[5][NP];
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int k = 0; k < NP; ++k) v[f][k] = xs[f * NPE + i * NP + k];
    const Lam<T> L = load_lam(a.mat + (int64_t)a.emat[e] * MAT_STRIDE_DEV, T(1));  // K_e^0
    GeoGeneral<T> geo{a.geo, a.fen_pad, e};
    T Fe[5][NP];
    shell_column<T, GeoGeneral<T>, false>(v, ys, xs, i, L, geo, Fe, a.sc);
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int m = 0; m < NP; ++m) ys[f * NPE + i * NP + m] = Fe[f][m];
  }
  __syncthreads();
  T out[5][NP];
  row_transpose_apply(xs, ys, j, out);
  // gradient partial: (K_e^0 lambda)' u_{n-1} over the row's nodes
  // (one element line's 30 products in the state precision; the per-element
  // and the across-step sums are FP64)
  const T* __restrict__ um = a.um;
  T dotl = T(0);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    const int node = a.conn[(int64_t)(j * NP + i) * a.fen_pad + e];
#pragma unroll
    for (int f = 0; f < 5; ++f) dotl += out[f][i] * um[f * a.nnode_pad + node];
  }
  const double dot = (double)dotl;
  const T keep = a.ekeep[e];
#pragma unroll
  for (int f = 0; f < 5; ++f)
#pragma unroll
    for (int i = 0; i < NP; ++i) a.F2[f * a.plane + (int64_t)(j * NP + i) * a.fen_pad + e] = keep * out[f][i];
  double* dred = reinterpret_cast<double*>(vred);
  __syncthreads();  // vred region is free (phase B of this kernel does not use it)
  dred[j * CTA_ELEMS + le] = dot;
  __syncthreads();
  if (j == 0 && e < a.fen) {
    double sgr = 0.0;
#pragma unroll
    for (int r = 0; r < NP; ++r) sgr += dred[r * CTA_ELEMS + le];
    a.grad[e] -= sgr;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_node_general(GenArgs<T> a, int kstep) {
  const int nn = *a.d_base + kstep;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.nnode) return;
  const bool odd = ((nn - a.nn_first) & 1);
  const T* __restrict__ cur = odd ? a.UB : a.UA;
  T* prev = odd ? a.UA : a.UB;
  T F[5] = {T(0), T(0), T(0), T(0), T(0)};
  for (int s = a.row_ptr[g]; s < a.row_ptr[g + 1]; ++s) {
    const int64_t slot = a.slots[s];
#pragma unroll
    for (int f = 0; f < 5; ++f) F[f] += a.F2[f * a.plane + slot];
  }
  if (a.pr.npf > 0) F[4] -= pressure_load(a.pr, nn, a.nnode_pad, g);
  T* dst = a.outp ? a.outp : prev;
  const T mt = a.minv[g], mr = a.minv[a.nnode_pad + g];
  const bool frame = a.fs.frm_int > 0 && (nn % a.fs.frm_int) == 0;
  const bool guard = guard_step(a.fs, nn);
  bool bad = false;
#pragma unroll
  for (int f = 0; f < 5; ++f) {
    const T u = cur[f * a.nnode_pad + g];
    const T uo = prev[f * a.nnode_pad + g];
    const T im = (f == 1 || f == 3) ? mr : mt;
    // unew = mg0.*(-F + mg2.*U - mg.*uold + a1*cg.*uold) rewritten as
    // u + k1*(u-uold) - k2*(F/M); F already contains -Fa*st(nn)
    const T un = u + a.k1[f] * (u - uo) - a.k2[f] * (im * F[f]);
    dst[f * a.nnode_pad + g] = un;
    if (frame) store_frame(a.fs, a.frames, a.nnode_pad, g, f, nn, u, uo, un, a.a0, a.a1);
    if (guard && (!isfinite(un) || (f == 4 && u > a.blowup))) bad = true;
  }
  if (bad) atomicOr(a.flag, 1);
}

// assembled K*u only (no update), into out[5][nnode_pad]
template <typename T>
__global__ void k_assemble_only(GenArgs<T> a, T* out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.nnode) return;
  T F[5] = {T(0), T(0), T(0), T(0), T(0)};
  for (int s = a.row_ptr[g]; s < a.row_ptr[g + 1]; ++s) {
    const int64_t slot = a.slots[s];
#pragma unroll
    for (int f = 0; f < 5; ++f) F[f] += a.F2[f * a.plane + slot];
  }
#pragma unroll
  for (int f = 0; f < 5; ++f) out[f * a.nnode_pad + g] = F[f];
}

__global__ void k_advance(int* d_base, int n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *d_base += n;
}

__global__ void k_set(int* d_base, int v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *d_base = v;
}

// voltage(nn,k) = mean over the sensor's local nodes (FP64)
__global__ void k_voltage(const double* vsum, const int* sptr, double* volt, int nsens, int nft) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsens * nft) return;
  const int k = t / nft, n = t % nft;
  double s = 0.0;
  for (int q = sptr[k]; q < sptr[k + 1]; ++q) s += vsum[(int64_t)q * nft + n];
  const int cnt = (sptr[k + 1] - sptr[k]) * NPE;
  volt[(int64_t)k * nft + n] = cnt ? s / cnt : 0.0;
}

// ---------------------------------------------------------------------------
// structured fused path (declared here, defined in shell_structured.cuh)
// ---------------------------------------------------------------------------
#include "shell_structured.cuh"
#include "shell_structured_f32.cuh"
#include "solid_element.cuh"

// laminate coefficient pairs for the packed FP32 kernel (indices into a table row)
static const int kLamPairs[LAMP][2] = {{0, 1},   {1, 3},   {2, 4},   {9, 10},  {10, 12}, {11, 13}, {2, 9},
                                       {4, 10},  {5, 11},  {11, 15}, {13, 16}, {14, 17}, {10, 11}, {12, 13},
                                       {13, 14}, {16, 17}, {18, 19}, {19, 20}, {6, 7},   {7, 8}};

struct StructPlan {
  int tile = 32, H = 16, ntask = 0, grid = 0;
  PlateDesc* plates = nullptr;
  TaskDesc* tasks = nullptr;
  int* emat_g = nullptr;
  void* ekeep_g = nullptr;
  int* esens_g = nullptr;
  int *f_xl = nullptr, *f_iy = nullptr, *f_field = nullptr, *f_rowptr = nullptr;
  double* f_val = nullptr;
  int *o_xl = nullptr, *o_iy = nullptr, *o_field = nullptr, *o_q = nullptr;  // point outputs per task
  int* e_of_g = nullptr;   // grid-order element -> plan element
  float2* matp = nullptr;  // FP32 packed laminate pairs [nmat][LAMP]
  // host copies kept for re-planning the task list (autotuner)
  std::vector<PlateDesc> h_plates;
  std::vector<int> h_fscen, h_fnode, h_ffield;
  std::vector<double> h_fval;
  std::vector<int> h_oscen, h_onode, h_ofield, h_oq;
  std::vector<void*> task_allocs;
};

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct shm_plan {
  std::string err;
  int kind = 0;  // 0 flat shell (5 DOF/node), 1 3D solid (3 DOF/node)
  int nf = 5;    // fields (DOF) per node
  int prec = 64, path = 1, device = 0, steps_per_graph = 0, tile = 0;
  cudaStream_t stream = nullptr;
  int nscen = 0;
  int nft = 0, nn_first = 2, nn = 2;
  double dt = 0, a0 = 0, a1 = 0;
  int64_t nnode = 0, fen = 0, fen_pad = 0, nnode_pad = 0, plane = 0;
  std::vector<int64_t> node_off, elem_off;
  std::vector<int> out_off, sens_off, nout_s, nsens_s;
  int nout = 0, nsens = 0, nslot = 0, nforce = 0;
  int frm_int = 0, nframes = 0, nfields = 0;
  int guard_int = 100;  // blow-up guard every guard_int steps besides the frame steps (0 = frame steps only)
  FrameSpec fspec{};
  std::vector<double> mass;  // [nnode][5] host copy (interleaved)
  // device memory
  std::vector<void*> allocs;
  void *UA = nullptr, *UB = nullptr, *F2 = nullptr, *geo = nullptr, *ekeep = nullptr, *mat = nullptr,
       *minv = nullptr, *frames = nullptr;
  int *conn = nullptr, *emat = nullptr, *row_ptr = nullptr, *slots = nullptr;
  int *fq_field = nullptr, *fq_scen = nullptr, *out_node = nullptr, *out_field = nullptr;
  int *esens = nullptr, *sptr = nullptr, *flag = nullptr, *d_base = nullptr;
  double *fq_val = nullptr, *st = nullptr, *displ = nullptr, *vsum = nullptr, *volt = nullptr;
  double k1[5], k2[5];
  double blowup = 0;
  double sc_k0 = 0, sc_e31 = 0, sc_e32 = 0, sc_hh = 0;
  // structured path
  StructPlan sp;
  bool sp_generic = false;  // FP32 structured: use the generic template instead of the packed kernel
  // adjoint buffers (allocated by the first shm_forward_backward)
  void *LA = nullptr, *LB = nullptr, *seg = nullptr, *ck = nullptr, *F2adj = nullptr;
  void* gbox = nullptr;  // 3D solid plans of axis-aligned box elements: [4][fen_pad]
  void* grect = nullptr; // flat-shell plans of axis-aligned rectangles: [3][fen_pad]
  void *kt_U = nullptr, *kt_out = nullptr;  // shm_apply_stiffness: state in, assembled force out
  int* kt_base = nullptr;
  cudaStream_t aux[2] = {nullptr, nullptr};  // adjoint: recompute and adjoint streams
  // explicit step states (adjoint recompute): cur/prev by parity, u_{n+1} into ov_out
  void *ov_UA = nullptr, *ov_UB = nullptr, *ov_out = nullptr;
  float fb_ms[3] = {0.f, 0.f, 0.f};  // last forward_backward: forward, recompute, adjoint (ms)
  int64_t store_cap = -3;  // bytes for states kept by the forward pass (-1 spare memory, -3 half the free memory)
  // pressure loading: nodal frames [npf][nnode_pad], lumped areas, per-step weights
  int npf = 0;
  void *pf = nullptr, *parea = nullptr;
  double* pcoef = nullptr;
  int last_nstore = 0;
  double *grad = nullptr, *asig = nullptr;
  int* d_base_adj = nullptr;
  int seg_k = 0, nck = 0;
  // graph
  cudaGraphExec_t gexec = nullptr;
  int gsteps = 0;
  bool ran = false;
  // persistent stepping (FP32 structured plans): one cooperative launch per
  // advance, CTAs meeting at a device-wide barrier between steps
  bool persistent = false;
  int spin_limit = 1 << 22;    // barrier polls before a wait gives up
  unsigned* gsync = nullptr;   // barrier word: arrivals, bit 31 = abort
  int coop_max = 0;            // co-resident CTAs of the persistent kernel
  int solid_grid = 0;          // FP32 3D solid: CTAs of the element kernel (resident at once)
  // frames to the caller: two device and two pinned staging buffers of
  // fstage_n values each
  int64_t fstage_n = (int64_t)4 << 20;
  double* fstage = nullptr;
  double* hstage = nullptr;
  cudaEvent_t fev[2] = {nullptr, nullptr};
};

#define CKP(plan, call)                                                               \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      (plan)->err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
      return (e_ == cudaErrorMemoryAllocation) ? SHM_ERR_OOM : SHM_ERR_CUDA;          \
    }                                                                                 \
  } while (0)

static shm_status bad(shm_plan* p, const std::string& m) {
  if (p) p->err = m;
  return SHM_ERR_BAD_ARG;
}

// Frame selection of a run (main_flat_shell.m:765-885, field_variable):
// frame_kind 0 velocity, 1 displacement, 2 acceleration, 3 all three;
// frame_dof 0 = every DOF component, else the one component 1..ndof.
// Fields are ordered kind-major (displacement, velocity, acceleration), then
// by DOF (u, phi_x, v, phi_y, w), the order of the reference's frame files.
static shm_status set_frames(shm_plan* p, const shm_run& r, int ndof) {
  FrameSpec& fs = p->fspec;
  fs = FrameSpec{};
  fs.guard_int = p->guard_int;
  for (int i = 0; i < 15; ++i) fs.slot[i] = -1;
  p->frm_int = r.frm_int > 0 ? r.frm_int : 0;
  p->nframes = p->nfields = 0;
  if (p->frm_int == 0) return SHM_OK;
  if (r.frame_dof < 0 || r.frame_dof > ndof) return bad(p, "frame_dof must be 0 (all) or 1..ndof");
  if (r.frame_kind < 0 || r.frame_kind > 3) return bad(p, "frame_kind must be 0..3");
  static const int kind_of[3] = {1, 0, 2};   // API kind -> displacement/velocity/acceleration slot
  int nf = 0;
  for (int k = 0; k < 3; ++k) {
    if (r.frame_kind != 3 && kind_of[r.frame_kind] != k) continue;
    for (int f = 0; f < ndof; ++f)
      if (r.frame_dof == 0 || r.frame_dof - 1 == f) fs.slot[k * 5 + f] = (signed char)nf++;
  }
  const int nf0 = r.nn_first > 0 ? r.nn_first : 1;
  fs.fc0 = (nf0 + p->frm_int - 1) / p->frm_int;
  p->nfields = nf;
  p->nframes = std::max(0, r.nft / p->frm_int - fs.fc0 + 1);
  fs.frm_int = p->frm_int;
  fs.nframes = p->nframes;
  fs.nfields = nf;
  return SHM_OK;
}

template <typename X>
static shm_status dalloc(shm_plan* p, X** out, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(X);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    p->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return SHM_ERR_OOM;
  }
  cudaMemset(q, 0, bytes);
  p->allocs.push_back(q);
  *out = reinterpret_cast<X*>(q);
  return SHM_OK;
}

template <typename X>
static shm_status upload(shm_plan* p, X** out, const std::vector<X>& v) {
  shm_status s = dalloc(p, out, v.size());
  if (s != SHM_OK) return s;
  if (!v.empty()) CKP(p, cudaMemcpy(*out, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice));
  return SHM_OK;
}

// GLL nodes/weights (Newton on P'_{n-1} from Chebyshev-Lobatto guesses) and
// the Lagrange derivative matrix by barycentric weights.
void shm::gll_setup(int n, std::vector<double>& x, std::vector<double>& w, std::vector<double>& D) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const int N = n - 1;
  auto legendre = [N](double t, double& p, double& dp, double& d2p) {
    double p0 = 1.0, p1 = t;
    if (N == 0) { p = 1; dp = 0; d2p = 0; return; }
    for (int k = 2; k <= N; ++k) {
      double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    p = p1;
    // P' and P'' from the Legendre ODE where |t| < 1
    dp = N * (t * p1 - p0) / (t * t - 1.0);
    d2p = (2.0 * t * dp - N * (N + 1.0) * p) / (1.0 - t * t);
  };
  x[0] = -1.0;
  x[N] = 1.0;
  for (int k = 1; k < N; ++k) {
    double t = -std::cos(M_PI * k / N);
    for (int it = 0; it < 100; ++it) {
      double p, dp, d2p;
      legendre(t, p, dp, d2p);
      double dt = dp / d2p;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[k] = t;
  }
  for (int k = 0; k <= N / 2; ++k) {  // exact symmetry
    double s = 0.5 * (x[N - k] - x[k]);
    x[k] = -s;
    x[N - k] = s;
  }
  if (n % 2 == 1) x[N / 2] = 0.0;
  for (int k = 0; k < n; ++k) {
    double p0 = 1.0, p1 = x[k];
    for (int m = 2; m <= N; ++m) {
      double p2 = ((2.0 * m - 1.0) * x[k] * p1 - (m - 1.0) * p0) / m;
      p0 = p1;
      p1 = p2;
    }
    w[k] = 2.0 / (N * (N + 1.0) * p1 * p1);
  }
  std::vector<double> lam(n, 1.0);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k)
      if (k != j) lam[j] /= (x[j] - x[k]);
  D.assign(n * n, 0.0);
  for (int r = 0; r < n; ++r) {
    double diag = 0.0;
    for (int c = 0; c < n; ++c)
      if (c != r) {
        D[r * n + c] = (lam[c] / lam[r]) / (x[r] - x[c]);
        diag -= D[r * n + c];
      }
    D[r * n + r] = diag;
  }
  // the reference zeroes |entries| < 1e-12 of its derivative operators
  // (shape2D_prim.m:52,54): interior diagonal entries are exactly 0
  for (double& v : D)
    if (std::fabs(v) < 1e-12) v = 0.0;
}

// 12-basket maps (nodesMaps_Fiborek.m): every element copy of a node goes to
// the least-filled basket, ties to the lowest basket number.  Only the
// per-node summation order is taken from it.
static void build_baskets(int fen, int npe, int nnode, const int32_t* nodes_cm,
                          std::vector<int>& IG, std::vector<int>& IL, int& rows) {
  std::vector<int> psi(nnode + 1, 0);
  std::vector<int> start(nnode + 2, 0);
  for (int e = 0; e < fen; ++e)
    for (int c = 0; c < npe; ++c) psi[nodes_cm[(int64_t)c * fen + e]]++;
  for (int k = 1; k <= nnode; ++k) start[k + 1] = start[k] + psi[k];
  std::vector<int> fill(nnode + 2, 0), copyE(start[nnode + 1]), copyL(start[nnode + 1]);
  for (int e = 0; e < fen; ++e)
    for (int c = 0; c < npe; ++c) {
      int k = nodes_cm[(int64_t)c * fen + e];
      int pos = start[k] + fill[k]++;
      copyE[pos] = e + 1;
      copyL[pos] = c + 1;
    }
  rows = (npe * fen + 11) / 12;
  int maxrows = rows + 12;
  IG.assign((size_t)maxrows * 12, 0);
  IL.assign((size_t)maxrows * 12, 0);
  int H[12] = {0};
  for (int k = 1; k <= nnode; ++k) {
    int S[12];
    for (int b = 0; b < 12; ++b) S[b] = b;
    std::stable_sort(S, S + 12, [&](int a, int b) { return H[a] < H[b]; });
    for (int i = 0; i < psi[k] && i < 12; ++i) {
      int b = S[i];
      H[b]++;
      int pos = start[k] + i;
      IG[(size_t)b * maxrows + H[b] - 1] = k;
      IL[(size_t)b * maxrows + H[b] - 1] = (copyE[pos] - 1) * npe + copyL[pos];
    }
  }
  int mr = 0;
  for (int b = 0; b < 12; ++b) mr = std::max(mr, H[b]);
  // compact to column-major [mr x 12]
  std::vector<int> G2((size_t)mr * 12), L2((size_t)mr * 12);
  for (int b = 0; b < 12; ++b)
    for (int r = 0; r < mr; ++r) {
      G2[(size_t)b * mr + r] = IG[(size_t)b * maxrows + r];
      L2[(size_t)b * mr + r] = IL[(size_t)b * maxrows + r];
    }
  IG.swap(G2);
  IL.swap(L2);
  rows = mr;
}

template <typename T> static void fill_sc(shm_plan* p, SensorConst<T>& sc) {
  sc.k0 = (T)p->sc_k0;
  sc.e31 = (T)p->sc_e31;
  sc.e32 = (T)p->sc_e32;
  sc.hh = (T)p->sc_hh;
}

template <typename T> static GenArgs<T> make_args(shm_plan* p) {
  GenArgs<T> a;
  a.fen_pad = p->fen_pad;
  a.nnode_pad = p->nnode_pad;
  a.plane = p->plane;
  a.nnode = (int)p->nnode;
  a.fen = (int)p->fen;
  a.nn_first = p->nn_first;
  a.nft = p->nft;
  a.UA = (T*)(p->ov_UA ? p->ov_UA : p->UA);
  a.UB = (T*)(p->ov_UB ? p->ov_UB : p->UB);
  a.outp = (T*)p->ov_out;
  a.grect = (const T*)p->grect;
  a.F2 = (T*)p->F2;
  a.conn = p->conn;
  a.geo = (const T*)p->geo;
  a.emat = p->emat;
  a.ekeep = (const T*)p->ekeep;
  a.mat = (const T*)p->mat;
  a.row_ptr = p->row_ptr;
  a.slots = p->slots;
  a.minv = (const T*)p->minv;
  for (int f = 0; f < 5; ++f) {
    a.k1[f] = (T)p->k1[f];
    a.k2[f] = (T)p->k2[f];
  }
  a.nforce = p->nforce;
  a.fq_field = p->fq_field;
  a.fq_scen = p->fq_scen;
  a.fq_val = p->fq_val;
  a.st = p->st;
  a.nout = p->nout;
  a.out_node = p->out_node;
  a.out_field = p->out_field;
  a.displ = p->displ;
  a.esens = p->esens;
  a.vsum = p->vsum;
  fill_sc(p, a.sc);
  a.fs = p->fspec;
  a.frames = (T*)p->frames;
  a.pr = PressureArgs<T>{p->npf, (const T*)p->pf, (const T*)p->parea, p->pcoef};
  a.a0 = (T)p->a0;
  a.a1 = (T)p->a1;
  a.blowup = (T)p->blowup;
  a.flag = p->flag;
  a.d_base = p->d_base;
  return a;
}

static size_t elem_smem_bytes(int prec) {
  const size_t ts = prec == 64 ? 8 : 4;
  return ts * (2 * CTA_ELEMS * ELEM_STRIDE + NP * CTA_ELEMS);
}

static size_t adj_smem_bytes(int prec) {
  const size_t ts = prec == 64 ? 8 : 4;
  return ts * (2 * CTA_ELEMS * ELEM_STRIDE) + sizeof(double) * NP * CTA_ELEMS;
}

template <typename T>
static cudaError_t launch_general_step(shm_plan* p, int kstep, cudaStream_t s) {
  GenArgs<T> a = make_args<T>(p);
  const int nblk = (int)(p->fen_pad / CTA_ELEMS);
  const size_t sm = elem_smem_bytes(sizeof(T) == 8 ? 64 : 32);
  if (p->grect) {
    if (p->nslot > 0)
      k_elem_general<T, true, true><<<nblk, CTA_THREADS, sm, s>>>(a, kstep);
    else
      k_elem_general<T, false, true><<<nblk, CTA_THREADS, sm, s>>>(a, kstep);
  } else if (p->nslot > 0) {
    k_elem_general<T, true><<<nblk, CTA_THREADS, sm, s>>>(a, kstep);
  } else {
    k_elem_general<T, false><<<nblk, CTA_THREADS, sm, s>>>(a, kstep);
  }
  k_node_general<T><<<(int)((p->nnode + 255) / 256), 256, 0, s>>>(a, kstep);
  return cudaGetLastError();
}

template <typename T> static cudaError_t launch_struct_step(shm_plan* p, int kstep, cudaStream_t s);

template <typename T> static cudaError_t launch_solid_step(shm_plan* p, int kstep, cudaStream_t s);

static cudaError_t launch_step(shm_plan* p, int kstep, cudaStream_t s) {
  if (p->kind == 1)
    return p->prec == 64 ? launch_solid_step<double>(p, kstep, s) : launch_solid_step<float>(p, kstep, s);
  if (p->path == 2) {
    return p->prec == 64 ? launch_struct_step<double>(p, kstep, s) : launch_struct_step<float>(p, kstep, s);
  }
  return p->prec == 64 ? launch_general_step<double>(p, kstep, s) : launch_general_step<float>(p, kstep, s);
}

static shm_status set_func_attrs(shm_plan* p) {
  const int sm64 = (int)elem_smem_bytes(64), sm32 = (int)elem_smem_bytes(32);
  CKP(p, cudaFuncSetAttribute(k_elem_general<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64));
  CKP(p, cudaFuncSetAttribute(k_elem_general<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64));
  CKP(p, cudaFuncSetAttribute(k_elem_general<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32));
  CKP(p, cudaFuncSetAttribute(k_elem_general<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32));
  CKP(p, cudaFuncSetAttribute(k_elem_general<double, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64));
  CKP(p, cudaFuncSetAttribute(k_elem_general<double, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64));
  CKP(p, cudaFuncSetAttribute(k_elem_general<float, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32));
  CKP(p, cudaFuncSetAttribute(k_elem_general<float, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32));
  CKP(p, cudaFuncSetAttribute(k_elem_adjoint<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)adj_smem_bytes(64)));
  CKP(p, cudaFuncSetAttribute(k_elem_adjoint<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)adj_smem_bytes(32)));
  CKP(p, cudaFuncSetAttribute(k_struct_step<double, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_smem_bytes<double, 32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step<double, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_smem_bytes<double, 16>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step<float, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_smem_bytes<float, 32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step<float, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_smem_bytes<float, 16>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step_f32<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step_f32<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step_f32<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<16>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step_f32<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<16>()));
  CKP(p, cudaFuncSetAttribute(k_struct_run_f32<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_run_f32<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_run_f32<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<16>()));
  CKP(p, cudaFuncSetAttribute(k_struct_run_f32<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<16>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step_f32<32, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<32>()));
  CKP(p, cudaFuncSetAttribute(k_struct_step_f32<16, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)struct_f32_smem_bytes<16>()));
  return SHM_OK;
}


// ---------------------------------------------------------------------------
// structured path: plan build and launch
// ---------------------------------------------------------------------------

// lanes doing useful work for strips of EW lanes (EW-1 owned elements each)
static double lane_utilisation(const shm_mesh* meshes, int nscen, int EW) {
  double used = 0, total = 0;
  for (int s = 0; s < nscen; ++s) {
    const int nex = meshes[s].grid_nex, ney = meshes[s].grid_ney, NX = 5 * nex + 1;
    const int own = 5 * (EW - 1);
    const int ns = (NX + own - 1) / own;
    for (int k = 0; k < ns; ++k) {
      int valid = 0;
      for (int q = 0; q < EW; ++q) {
        const int ex = k * (EW - 1) - 1 + q;
        valid += (ex >= 0 && ex < nex);
      }
      used += (double)valid * ney;
      total += (double)EW * ney;
    }
  }
  return total > 0 ? used / total : 0;
}

// (re)build the structured task list for EW elements per lane group and H
// element rows per task; device arrays of a previous list are released
static shm_status struct_tasks(shm_plan* p, int EW, int H) {
  StructPlan& sp = p->sp;
  const int own = 5 * (EW - 1);
  struct TaskTmp {
    TaskDesc t;
    std::vector<int> fxl, fiy, ffield;
    std::vector<double> fval;
    std::vector<int> oxl, oiy, ofield, oq;
  };
  const int nscen = (int)sp.h_plates.size();
  std::vector<TaskTmp> tasks;
  std::vector<std::vector<int>> task_index(nscen);
  for (int s = 0; s < nscen; ++s) {
    const PlateDesc& pl = sp.h_plates[s];
    const int ns = (pl.NX + own - 1) / own, nb = (pl.ney + H - 1) / H;
    task_index[s].assign((size_t)ns * nb, -1);
    for (int b = 0; b < nb; ++b)
      for (int k = 0; k < ns; ++k) {
        TaskTmp t;
        t.t = TaskDesc{s, k, b, 0, 0, 0, 0, 0, -1, -1};  // rows, forces and outputs set below
        const int last = std::min(H * (b + 1), pl.ney);
        t.t.nrows = b == 0 ? last : last - (H * b - 1);
        task_index[s][(size_t)b * ns + k] = (int)tasks.size();
        tasks.push_back(std::move(t));
      }
  }
  for (size_t q = 0; q < sp.h_fnode.size(); ++q) {
    const int s = sp.h_fscen[q];
    const PlateDesc& pl = sp.h_plates[s];
    const int ns = (pl.NX + own - 1) / own, nb = (pl.ney + H - 1) / H;
    const int node = sp.h_fnode[q];
    const int ix = node % pl.NX, iy = node / pl.NX;
    const int k = ix / own;
    const int b = std::min(iy / (5 * H), nb - 1);
    TaskTmp& t = tasks[task_index[s][(size_t)b * ns + k]];
    t.fxl.push_back(ix - 5 * (k * (EW - 1) - 1));
    t.fiy.push_back(iy);
    t.ffield.push_back(sp.h_ffield[q]);
    t.fval.push_back(sp.h_fval[q]);
  }
  for (size_t q = 0; q < sp.h_onode.size(); ++q) {  // point outputs: the task that updates the node
    const int s = sp.h_oscen[q];
    const PlateDesc& pl = sp.h_plates[s];
    const int ns = (pl.NX + own - 1) / own, nb = (pl.ney + H - 1) / H;
    const int node = sp.h_onode[q];
    const int ix = node % pl.NX, iy = node / pl.NX;
    const int k = ix / own;
    const int b = std::min(iy / (5 * H), nb - 1);
    TaskTmp& t = tasks[task_index[s][(size_t)b * ns + k]];
    t.oxl.push_back(ix - 5 * (k * (EW - 1) - 1));
    t.oiy.push_back(iy);
    t.ofield.push_back(sp.h_ofield[q]);
    t.oq.push_back(sp.h_oq[q]);
  }
  // each task's forces ordered by node row, then column and field, with the
  // entries of one DOF merged (values summed in FP64): a step kernel walks them
  // with one cursor per node row and scatters a row's entries in parallel
  for (TaskTmp& t : tasks) {
    const size_t n = t.fxl.size();
    if (n == 0) continue;
    std::vector<size_t> ord(n);
    for (size_t i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
      if (t.fiy[a] != t.fiy[b]) return t.fiy[a] < t.fiy[b];
      if (t.fxl[a] != t.fxl[b]) return t.fxl[a] < t.fxl[b];
      return t.ffield[a] < t.ffield[b];
    });
    std::vector<int> xl, iy, fld;
    std::vector<double> val;
    for (size_t i : ord) {
      if (!xl.empty() && xl.back() == t.fxl[i] && iy.back() == t.fiy[i] && fld.back() == t.ffield[i]) {
        val.back() += t.fval[i];
        continue;
      }
      xl.push_back(t.fxl[i]);
      iy.push_back(t.fiy[i]);
      fld.push_back(t.ffield[i]);
      val.push_back(t.fval[i]);
    }
    t.fxl.swap(xl);
    t.fiy.swap(iy);
    t.ffield.swap(fld);
    t.fval.swap(val);
  }
  // each task's point outputs ordered by node row, then column (stable: the
  // entries of one DOF keep their order)
  for (TaskTmp& t : tasks) {
    const size_t n = t.oxl.size();
    if (n < 2) continue;
    std::vector<size_t> ord(n);
    for (size_t i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
      return t.oiy[a] != t.oiy[b] ? t.oiy[a] < t.oiy[b] : t.oxl[a] < t.oxl[b];
    });
    std::vector<int> xl(n), iy(n), fld(n), oq(n);
    for (size_t i = 0; i < n; ++i) {
      xl[i] = t.oxl[ord[i]];
      iy[i] = t.oiy[ord[i]];
      fld[i] = t.ofield[ord[i]];
      oq[i] = t.oq[ord[i]];
    }
    t.oxl.swap(xl);
    t.oiy.swap(iy);
    t.ofield.swap(fld);
    t.oq.swap(oq);
  }
  // longest tasks first so that lane groups of a CTA stay in step
  std::stable_sort(tasks.begin(), tasks.end(), [](const TaskTmp& a, const TaskTmp& b) { return a.t.nrows > b.t.nrows; });
  std::vector<TaskDesc> td;
  std::vector<int> fxl, fiy, ffield, oxl, oiy, ofield, oq, frp;
  std::vector<double> fval;
  // node-row pointers of a task's sorted list: the entries of task node row k
  // (node row 5 eyA + k) are [frp[r0 + k], frp[r0 + k + 1]), k = 0 .. 5 nrows
  auto row_pointers = [&](const TaskDesc& td_, const std::vector<int>& iys, int first) {
    const int iy0 = 5 * (td_.block == 0 ? 0 : td_.block * H - 1);
    const int nr = 5 * td_.nrows + 1;
    const int r0 = (int)frp.size();
    size_t k = 0;
    for (int row = 0; row <= nr; ++row) {
      while (k < iys.size() && iys[k] - iy0 < row) ++k;
      frp.push_back(first + (int)k);
    }
    return r0;
  };
  for (TaskTmp& t : tasks) {
    t.t.o0 = (int)oxl.size();
    t.t.on = (int)t.oxl.size();
    if (t.t.on > 0) t.t.or0 = row_pointers(t.t, t.oiy, t.t.o0);
    oxl.insert(oxl.end(), t.oxl.begin(), t.oxl.end());
    oiy.insert(oiy.end(), t.oiy.begin(), t.oiy.end());
    ofield.insert(ofield.end(), t.ofield.begin(), t.ofield.end());
    oq.insert(oq.end(), t.oq.begin(), t.oq.end());
    t.t.f0 = (int)fxl.size();
    t.t.fn = (int)t.fxl.size();
    if (t.t.fn > 0) t.t.fr0 = row_pointers(t.t, t.fiy, t.t.f0);
    fxl.insert(fxl.end(), t.fxl.begin(), t.fxl.end());
    fiy.insert(fiy.end(), t.fiy.begin(), t.fiy.end());
    ffield.insert(ffield.end(), t.ffield.begin(), t.ffield.end());
    fval.insert(fval.end(), t.fval.begin(), t.fval.end());
    td.push_back(t.t);
  }
  // release the previous list
  for (void* q : sp.task_allocs) {
    auto it = std::find(p->allocs.begin(), p->allocs.end(), q);
    if (it != p->allocs.end()) p->allocs.erase(it);
    cudaFree(q);
  }
  sp.task_allocs.clear();
  shm_status st;
  TaskDesc* dt = nullptr;
  if ((st = upload(p, &dt, td)) != SHM_OK) return st;
  if ((st = upload(p, &sp.f_xl, fxl)) != SHM_OK) return st;
  if ((st = upload(p, &sp.f_iy, fiy)) != SHM_OK) return st;
  if ((st = upload(p, &sp.f_field, ffield)) != SHM_OK) return st;
  if ((st = upload(p, &sp.f_val, fval)) != SHM_OK) return st;
  if ((st = upload(p, &sp.f_rowptr, frp)) != SHM_OK) return st;
  if ((st = upload(p, &sp.o_xl, oxl)) != SHM_OK) return st;
  if ((st = upload(p, &sp.o_iy, oiy)) != SHM_OK) return st;
  if ((st = upload(p, &sp.o_field, ofield)) != SHM_OK) return st;
  if ((st = upload(p, &sp.o_q, oq)) != SHM_OK) return st;
  sp.task_allocs = {dt, sp.f_xl, sp.f_iy, sp.f_field, sp.f_val, sp.f_rowptr, sp.o_xl, sp.o_iy, sp.o_field, sp.o_q};
  sp.tasks = dt;
  sp.ntask = (int)td.size();
  sp.tile = EW;
  sp.H = H;
  const int G = 32 / EW;
  sp.grid = (sp.ntask + G - 1) / G;
  return SHM_OK;
}

static shm_status struct_build(shm_plan* p, int nscen, const shm_mesh* meshes, const shm_material* mats,
                               const shm_run* runs, int tile_elems, const std::vector<double>& gw,
                               const std::vector<double>& geo, const std::vector<int>& emat,
                               const std::vector<double>& ekeep, const std::vector<int>& esens,
                               const std::vector<int>& fq_field, const std::vector<double>& fq_val,
                               const std::vector<double>& mat, int rows_per_block, std::string& why) {
  (void)mats;
  (void)fq_field;
  (void)fq_val;
  StructPlan& sp = p->sp;
  const int64_t FP = p->fen_pad;
  std::vector<PlateDesc> plates(nscen);
  int64_t egrid = 0;
  std::vector<int> emat_g(p->fen), esens_g(p->fen, -1), e_of_g(p->fen, 0);
  std::vector<double> ekeep_g(p->fen, 1.0);
  for (int s = 0; s < nscen; ++s) {
    const shm_mesh& m = meshes[s];
    const int nex = m.grid_nex, ney = m.grid_ney;
    if (nex < 1 || ney < 1) { why = "mesh is not declared structured"; return SHM_ERR_UNSUPPORTED; }
    const int NX = 5 * nex + 1, NY = 5 * ney + 1;
    if ((int64_t)m.nnode != (int64_t)NX * NY || m.fen != nex * ney) { why = "grid sizes do not match the mesh"; return SHM_ERR_UNSUPPORTED; }
    std::vector<char> seen((size_t)nex * ney, 0);
    const int64_t e0 = p->elem_off[s];
    double sx = 0, sy = 0, a4 = 0;
    for (int e = 0; e < m.fen; ++e) {
      const int b0 = m.nodes[e] - 1;  // c = 0
      const int ix0 = b0 % NX, iy0 = b0 / NX;
      if (ix0 % 5 || iy0 % 5 || ix0 / 5 >= nex || iy0 / 5 >= ney) { why = "element origin off the grid"; return SHM_ERR_UNSUPPORTED; }
      for (int k = 0; k < NP; ++k)
        for (int i = 0; i < NP; ++i)
          if (m.nodes[(int64_t)(k * NP + i) * m.fen + e] - 1 != (iy0 + k) * NX + ix0 + i) {
            why = "connectivity is not the row-major grid numbering";
            return SHM_ERR_UNSUPPORTED;
          }
      const int ex = ix0 / 5, ey = iy0 / 5;
      if (seen[(size_t)ey * nex + ex]++) { why = "duplicate element"; return SHM_ERR_UNSUPPORTED; }
      const int64_t ge = e0 + e;
      for (int c = 0; c < NPE; ++c) {
        const int64_t base = (int64_t)c * FP + ge;
        const double i11 = geo[0 * NPE * FP + base], i12 = geo[1 * NPE * FP + base];
        const double i21 = geo[2 * NPE * FP + base], i22 = geo[3 * NPE * FP + base];
        const double W = geo[4 * NPE * FP + base] / (gw[c % NP] * gw[c / NP]);
        if (e == 0 && c == 0) { sx = i11; sy = i22; a4 = W; }
        const double tol = 1e-9;
        if (std::fabs(i12) > 1e-12 * std::fabs(i11) || std::fabs(i21) > 1e-12 * std::fabs(i22) ||
            std::fabs(i11 - sx) > tol * std::fabs(sx) || std::fabs(i22 - sy) > tol * std::fabs(sy) ||
            std::fabs(W - a4) > tol * std::fabs(a4)) {
          why = "elements are not equal axis-aligned rectangles";
          return SHM_ERR_UNSUPPORTED;
        }
      }
      emat_g[egrid + (int64_t)ey * nex + ex] = emat[ge];
      ekeep_g[egrid + (int64_t)ey * nex + ex] = ekeep[ge];
      esens_g[egrid + (int64_t)ey * nex + ex] = esens[ge];
      e_of_g[egrid + (int64_t)ey * nex + ex] = (int)ge;
    }
    plates[s] = PlateDesc{nex, ney, NX, s, (long long)p->node_off[s], (long long)egrid, sx, sy, a4};
    egrid += (int64_t)nex * ney;
  }
  sp.h_plates = plates;
  for (int sidx = 0; sidx < nscen; ++sidx)
    for (int q = 0; q < runs[sidx].n_force; ++q) {
      const int d = runs[sidx].force_dof[q];
      sp.h_fscen.push_back(sidx);
      sp.h_fnode.push_back((d - 1) / 5);
      sp.h_ffield.push_back((d - 1) % 5);
      sp.h_fval.push_back(runs[sidx].force_val[q]);
    }
  for (int sidx = 0; sidx < nscen; ++sidx)
    for (int q = 0; q < runs[sidx].n_out; ++q) {
      const int d = runs[sidx].out_dof[q];
      sp.h_oscen.push_back(sidx);
      sp.h_onode.push_back((d - 1) / 5);
      sp.h_ofield.push_back((d - 1) % 5);
      sp.h_oq.push_back(p->out_off[sidx] + q);
    }
  int EW = tile_elems;
  if (EW != 16 && EW != 32) EW = lane_utilisation(meshes, nscen, 32) >= 0.9 * lane_utilisation(meshes, nscen, 16) ? 32 : 16;
  shm_status st;
  {
    PlateDesc* dp = nullptr;
    if ((st = upload(p, &dp, plates)) != SHM_OK) return st;
    sp.plates = dp;
  }
  if ((st = struct_tasks(p, EW, rows_per_block > 0 ? rows_per_block : 16)) != SHM_OK) return st;
  if ((st = upload(p, &sp.emat_g, emat_g)) != SHM_OK) return st;
  if ((st = upload(p, &sp.esens_g, esens_g)) != SHM_OK) return st;
  if ((st = upload(p, &sp.e_of_g, e_of_g)) != SHM_OK) return st;
  if (p->prec == 64) {
    double* k = nullptr;
    if ((st = upload(p, &k, ekeep_g)) != SHM_OK) return st;
    sp.ekeep_g = k;
  } else {
    std::vector<float> k32(ekeep_g.begin(), ekeep_g.end());
    float* k = nullptr;
    if ((st = upload(p, &k, k32)) != SHM_OK) return st;
    sp.ekeep_g = k;
  }
  if (p->prec == 32) {
    const size_t nmat = mat.size() / MAT_STRIDE_DEV;
    std::vector<float2> mp(nmat * LAMP);
    for (size_t m = 0; m < nmat; ++m)
      for (int c = 0; c < LAMP; ++c)
        mp[m * LAMP + c] = make_float2((float)mat[m * MAT_STRIDE_DEV + kLamPairs[c][0]],
                                       (float)mat[m * MAT_STRIDE_DEV + kLamPairs[c][1]]);
    if ((st = upload(p, &sp.matp, mp)) != SHM_OK) return st;
  }
  return SHM_OK;
}

static F32Args struct_f32_args(shm_plan* p) {
  StructPlan& sp = p->sp;
  F32Args a{};
  a.plates = sp.plates;
  a.tasks = sp.tasks;
  a.ntask = sp.ntask;
  a.H = sp.H;
  a.nn_first = p->nn_first;
  a.nft = p->nft;
  a.nnode_pad = p->nnode_pad;
  a.UA = (float*)(p->ov_UA ? p->ov_UA : p->UA);
  a.UB = (float*)(p->ov_UB ? p->ov_UB : p->UB);
  a.outp = (float*)p->ov_out;
  a.minv = (const float*)p->minv;
  for (int f = 0; f < 5; ++f) {
    a.k1[f] = (float)p->k1[f];
    a.k2[f] = (float)p->k2[f];
  }
  a.matp = sp.matp;
  a.emat_g = sp.emat_g;
  a.ekeep_g = (const float*)sp.ekeep_g;
  a.esens_g = sp.esens_g;
  a.f_xl = sp.f_xl;
  a.f_iy = sp.f_iy;
  a.f_rowptr = sp.f_rowptr;
  a.f_field = sp.f_field;
  a.f_val = sp.f_val;
  a.st = p->st;
  a.nout = p->nout;
  a.out_node = p->out_node;
  a.out_field = p->out_field;
  a.displ = p->displ;
  a.vsum = p->vsum;
  fill_sc(p, a.sc);
  a.fs = p->fspec;
  a.frames = (float*)p->frames;
  a.pr = PressureArgs<float>{p->npf, (const float*)p->pf, (const float*)p->parea, p->pcoef};
  a.a0 = (float)p->a0;
  a.a1 = (float)p->a1;
  a.blowup = (float)p->blowup;
  a.flag = p->flag;
  a.d_base = p->d_base;
  a.o_xl = sp.o_xl;
  a.o_iy = sp.o_iy;
  a.o_field = sp.o_field;
  a.o_q = sp.o_q;
  a.e_of_g = sp.e_of_g;
  return a;
}

// Persistent FP32 structured stepping: `nsteps` steps in one cooperative
// launch of at most coop_max CTAs (all resident at once, which the barrier
// between steps needs; the runtime refuses a larger cooperative grid).
static cudaError_t launch_struct_run_f32(shm_plan* p, int nsteps, cudaStream_t s) {
  StructPlan& sp = p->sp;
  F32Args a = struct_f32_args(p);
  const bool sens = p->nslot > 0;
  cudaError_t e = cudaMemsetAsync(p->gsync, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  GridSync gs{p->gsync, p->spin_limit};
  void* args[] = {&a, &nsteps, &gs};
  const int grid = std::max(1, std::min(sp.grid, p->coop_max));
  const void* fn;
  size_t smem;
  if (sp.tile == 32) {
    fn = sens ? (const void*)k_struct_run_f32<32, true> : (const void*)k_struct_run_f32<32, false>;
    smem = struct_f32_smem_bytes<32>();
  } else {
    fn = sens ? (const void*)k_struct_run_f32<16, true> : (const void*)k_struct_run_f32<16, false>;
    smem = struct_f32_smem_bytes<16>();
  }
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(CTA_THREADS), args, smem, s);
}

static cudaError_t launch_struct_step_f32(shm_plan* p, int kstep, cudaStream_t s) {
  StructPlan& sp = p->sp;
  F32Args a = struct_f32_args(p);
  const bool sens = p->nslot > 0;
  if (sp.tile == 32) {
    if (sens)
      k_struct_step_f32<32, true><<<sp.grid, CTA_THREADS, struct_f32_smem_bytes<32>(), s>>>(a, kstep);
    else
      k_struct_step_f32<32, false><<<sp.grid, CTA_THREADS, struct_f32_smem_bytes<32>(), s>>>(a, kstep);
  } else {
    if (sens)
      k_struct_step_f32<16, true><<<sp.grid, CTA_THREADS, struct_f32_smem_bytes<16>(), s>>>(a, kstep);
    else
      k_struct_step_f32<16, false><<<sp.grid, CTA_THREADS, struct_f32_smem_bytes<16>(), s>>>(a, kstep);
  }
  return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_struct_step(shm_plan* p, int kstep, cudaStream_t s) {
  if (sizeof(T) == 4 && !p->sp_generic) return launch_struct_step_f32(p, kstep, s);
  StructPlan& sp = p->sp;
  StructArgs<T> a;
  a.plates = sp.plates;
  a.tasks = sp.tasks;
  a.ntask = sp.ntask;
  a.H = sp.H;
  a.nn_first = p->nn_first;
  a.nft = p->nft;
  a.nnode_pad = p->nnode_pad;
  a.UA = (T*)(p->ov_UA ? p->ov_UA : p->UA);
  a.UB = (T*)(p->ov_UB ? p->ov_UB : p->UB);
  a.outp = (T*)p->ov_out;
  a.minv = (const T*)p->minv;
  for (int f = 0; f < 5; ++f) {
    a.k1[f] = (T)p->k1[f];
    a.k2[f] = (T)p->k2[f];
  }
  a.mat = (const T*)p->mat;
  a.emat_g = sp.emat_g;
  a.ekeep_g = (const T*)sp.ekeep_g;
  a.esens_g = sp.esens_g;
  a.f_xl = sp.f_xl;
  a.f_iy = sp.f_iy;
  a.f_field = sp.f_field;
  a.f_val = sp.f_val;
  a.st = p->st;
  a.nout = p->nout;
  a.out_node = p->out_node;
  a.out_field = p->out_field;
  a.displ = p->displ;
  a.vsum = p->vsum;
  fill_sc(p, a.sc);
  a.fs = p->fspec;
  a.frames = (T*)p->frames;
  a.pr = PressureArgs<T>{p->npf, (const T*)p->pf, (const T*)p->parea, p->pcoef};
  a.a0 = (T)p->a0;
  a.a1 = (T)p->a1;
  a.blowup = (T)p->blowup;
  a.flag = p->flag;
  a.d_base = p->d_base;
  if (sp.tile == 32)
    k_struct_step<T, 32><<<sp.grid, CTA_THREADS, struct_smem_bytes<T, 32>(), s>>>(a, kstep);
  else
    k_struct_step<T, 16><<<sp.grid, CTA_THREADS, struct_smem_bytes<T, 16>(), s>>>(a, kstep);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// plan creation
// ---------------------------------------------------------------------------

// Pressure loading (main_flat_shell_pressure_excit_c.m:64-82,616-632): nodal
// frames and areas on the device, and per step nn = 1..nft the interp1
// ('linear', extrapolation 0) weights of the two frames around t = (nn-1) dt.
template <typename T>
static shm_status pressure_build(shm_plan* p, int nscen, const shm_mesh* meshes, const shm_run* runs,
                                 const std::vector<double>& area) {
  int npf = 0;
  const double* times = nullptr;
  for (int s = 0; s < nscen; ++s) {
    const shm_run& r = runs[s];
    if (r.n_pframes <= 0) continue;
    if (!r.p_times || !r.p_nodal) return bad(p, "run: pressure frames without times or values");
    if (npf == 0) {
      npf = r.n_pframes;
      times = r.p_times;
      for (int k = 1; k < npf; ++k)
        if (!(times[k] > times[k - 1])) return bad(p, "run: pressure frame times must increase");
    } else if (r.n_pframes != npf || !std::equal(times, times + npf, r.p_times)) {
      return bad(p, "run: scenarios with pressure loading must share the frame times");
    }
  }
  p->npf = npf;
  if (npf == 0) return SHM_OK;
  std::vector<T> pf((size_t)npf * p->nnode_pad, T(0)), pa(area.size());
  for (size_t g = 0; g < area.size(); ++g) pa[g] = (T)area[g];
  for (int s = 0; s < nscen; ++s) {
    const shm_run& r = runs[s];
    if (r.n_pframes <= 0) continue;
    const int64_t n0 = p->node_off[s], nn_s = meshes[s].nnode;
    for (int k = 0; k < npf; ++k)
      for (int64_t g = 0; g < nn_s; ++g) pf[(size_t)k * p->nnode_pad + n0 + g] = (T)r.p_nodal[(size_t)k * nn_s + g];
  }
  std::vector<double> coef((size_t)4 * p->nft, 0.0);
  for (int nn = 1; nn <= p->nft; ++nn) {
    const double t = (nn - 1) * p->dt;
    double* c = &coef[(size_t)4 * (nn - 1)];
    if (t < times[0] || t > times[npf - 1]) continue;  // zero outside the frames
    int k = 0;
    while (k + 1 < npf - 1 && t > times[k + 1]) ++k;
    const int k1 = npf > 1 ? k + 1 : k;
    const double al = npf > 1 ? (t - times[k]) / (times[k1] - times[k]) : 0.0;
    c[0] = k;
    c[1] = k1;
    c[2] = 1.0 - al;
    c[3] = al;
  }
  T *dpf = nullptr, *dpa = nullptr;
  shm_status st;
  if ((st = upload(p, &dpf, pf)) != SHM_OK) return st;
  if ((st = upload(p, &dpa, pa)) != SHM_OK) return st;
  if ((st = upload(p, &p->pcoef, coef)) != SHM_OK) return st;
  p->pf = dpf;
  p->parea = dpa;
  return SHM_OK;
}

template <typename T>
static shm_status build_device(shm_plan* p, const std::vector<int>& conn, const std::vector<double>& geo,
                               const std::vector<int>& emat, const std::vector<double>& ekeep,
                               const std::vector<double>& mat, const std::vector<double>& minv) {
  shm_status s;
  auto conv = [](const std::vector<double>& v) {
    std::vector<T> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = (T)v[i];
    return o;
  };
  T *g = nullptr, *k = nullptr, *m = nullptr, *mi = nullptr, *ua = nullptr, *ub = nullptr, *f2 = nullptr,
    *fr = nullptr;
  if ((s = upload(p, &p->conn, conn)) != SHM_OK) return s;
  if ((s = upload(p, &g, conv(geo))) != SHM_OK) return s;
  if ((s = upload(p, &p->emat, emat)) != SHM_OK) return s;
  if ((s = upload(p, &k, conv(ekeep))) != SHM_OK) return s;
  if ((s = upload(p, &m, conv(mat))) != SHM_OK) return s;
  if ((s = upload(p, &mi, conv(minv))) != SHM_OK) return s;
  if ((s = dalloc(p, &ua, (size_t)5 * p->nnode_pad)) != SHM_OK) return s;
  if ((s = dalloc(p, &ub, (size_t)5 * p->nnode_pad)) != SHM_OK) return s;
  if ((s = dalloc(p, &f2, (size_t)5 * p->plane)) != SHM_OK) return s;
  if (p->nframes > 0 && (s = dalloc(p, &fr, (size_t)p->nframes * p->nfields * p->nnode_pad)) != SHM_OK) return s;
  p->geo = g;
  p->ekeep = k;
  p->mat = m;
  p->minv = mi;
  p->UA = ua;
  p->UB = ub;
  p->F2 = f2;
  p->frames = fr;
  return SHM_OK;
}

extern "C" shm_status shm_plan_create(int32_t nscen, const shm_mesh* meshes, const shm_material* mats,
                                      const shm_run* runs, const shm_options* opt, shm_plan** out) {
  if (!out) return SHM_ERR_BAD_ARG;
  *out = nullptr;
  if (nscen < 1 || !meshes || !mats || !runs) return SHM_ERR_BAD_ARG;
  shm_plan* p = new shm_plan();
  *out = p;
  shm_options o{};
  o.precision = 64;
  if (opt) o = *opt;
  if (o.precision != 64 && o.precision != 32) return bad(p, "precision must be 32 or 64");
  p->prec = o.precision;
  p->device = o.device;
  p->steps_per_graph = std::max(0, o.steps_per_graph);
  p->nscen = nscen;
  CKP(p, cudaSetDevice(o.device));
  CKP(p, cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));

  const shm_run& r0 = runs[0];
  if (!(r0.dt > 0) || r0.nft < 1 || (r0.nn_first != 1 && r0.nn_first != 2))
    return bad(p, "run: dt > 0, nft >= 1, nn_first in {1,2} required");
  for (int s = 1; s < nscen; ++s) {
    const shm_run& r = runs[s];
    if (r.dt != r0.dt || r.nft != r0.nft || r.nn_first != r0.nn_first || r.eta_xy != r0.eta_xy ||
        r.eta_z != r0.eta_z || r.frm_int != r0.frm_int || r.frame_dof != r0.frame_dof)
      return bad(p, "all scenarios of a batch must share dt, nft, nn_first, damping and frame settings");
  }
  p->dt = r0.dt;
  p->nft = r0.nft;
  p->nn_first = r0.nn_first;
  p->nn = r0.nn_first;
  // central-difference coefficients (main_flat_shell.m:575-604)
  p->a0 = 1.0 / (r0.dt * r0.dt);
  p->a1 = 1.0 / (2.0 * r0.dt);
  const double eta[5] = {r0.eta_xy, 0.0, r0.eta_xy, 0.0, r0.eta_z};
  for (int f = 0; f < 5; ++f) {
    const double den = p->a0 + p->a1 * eta[f];
    p->k1[f] = (p->a0 - p->a1 * eta[f]) / den;
    p->k2[f] = 1.0 / den;
  }
  if (set_frames(p, r0, 5) != SHM_OK) return SHM_ERR_BAD_ARG;
  p->blowup = 10.0 * r0.h;
  if (!(r0.h > 0)) p->blowup = INFINITY;

  // sizes and offsets
  p->node_off.assign(nscen + 1, 0);
  p->elem_off.assign(nscen + 1, 0);
  for (int s = 0; s < nscen; ++s) {
    const shm_mesh& m = meshes[s];
    if (m.npe != NPE) return bad(p, "npe must be 36 (order-5 elements)");
    if (m.fen < 1 || m.nnode < 1 || !m.nodes || !m.coords) return bad(p, "mesh: empty or NULL arrays");
    p->node_off[s + 1] = p->node_off[s] + m.nnode;
    p->elem_off[s + 1] = p->elem_off[s] + m.fen;
  }
  p->nnode = p->node_off[nscen];
  p->fen = p->elem_off[nscen];
  if (p->nnode > INT32_MAX / 2 || p->fen * NPE > INT32_MAX / 2) return bad(p, "mesh too large for 32-bit slots");
  p->fen_pad = (p->fen + CTA_ELEMS - 1) / CTA_ELEMS * CTA_ELEMS;
  p->nnode_pad = (p->nnode + 4 + 31) / 32 * 32;  // >= 4 spare floats: 16-byte-rounded line copies stay in the field

  // GLL constants
  std::vector<double> gx, gw, D;
  gll_setup(NP, gx, gw, D);
  {
    float D32[36], w32[6];
    for (int i = 0; i < 36; ++i) D32[i] = (float)D[i];
    for (int i = 0; i < 6; ++i) w32[i] = (float)gw[i];
    CKP(p, cudaMemcpyToSymbol(c_D64, D.data(), sizeof(double) * 36));
    CKP(p, cudaMemcpyToSymbol(c_D32, D32, sizeof(float) * 36));
    CKP(p, cudaMemcpyToSymbol(c_w64, gw.data(), sizeof(double) * 6));
    CKP(p, cudaMemcpyToSymbol(c_w32, w32, sizeof(float) * 6));
    float2 dp[6][3], dtp[6][3];
    for (int k = 0; k < 6; ++k)
      for (int q = 0; q < 3; ++q) {
        dp[k][q] = make_float2((float)D[(2 * q) * 6 + k], (float)D[(2 * q + 1) * 6 + k]);
        dtp[k][q] = make_float2((float)D[k * 6 + 2 * q], (float)D[k * 6 + 2 * q + 1]);
      }
    CKP(p, cudaMemcpyToSymbol(c_Dp, dp, sizeof(dp)));
    CKP(p, cudaMemcpyToSymbol(c_DTp, dtp, sizeof(dtp)));
  }

  // connectivity, geometry, materials, slots
  const int64_t FP = p->fen_pad;
  std::vector<int> conn((size_t)NPE * FP, 0);
  std::vector<double> geo((size_t)5 * NPE * FP, 0.0);
  std::vector<int> emat(FP, 0);
  std::vector<double> ekeep(FP, 1.0);
  std::vector<double> mat;
  std::vector<double> elem_m11(p->fen), elem_I11(p->fen);
  std::vector<int> nslot_node(p->nnode + 1, 0);
  std::vector<std::vector<int>> node_slots_tmp;  // filled below via baskets
  std::vector<int> row_ptr(p->nnode + 1, 0), slots;
  int mat_base = 0;
  // per scenario
  std::vector<std::pair<int64_t, int>> dummy;
  std::vector<int> slot_list_sizes;
  // gather basket-ordered slot lists per node
  std::vector<int> node_cnt(p->nnode, 0);
  std::vector<int64_t> node_first(p->nnode + 1, 0);
  std::vector<int> tmp_slots;  // filled in node order later
  std::vector<std::vector<int>> per_node;  // avoided for memory: two-pass below
  // pass 1: count element copies per node
  for (int s = 0; s < nscen; ++s) {
    const shm_mesh& m = meshes[s];
    for (int c = 0; c < NPE; ++c)
      for (int e = 0; e < m.fen; ++e) {
        const int nd = m.nodes[(int64_t)c * m.fen + e];
        if (nd < 1 || nd > m.nnode) return bad(p, "mesh: node number out of range");
        node_cnt[p->node_off[s] + nd - 1]++;
      }
  }
  int nforce_tot = 0, nout_tot = 0;
  for (int s = 0; s < nscen; ++s) {
    if (runs[s].n_force < 0 || (runs[s].n_force > 0 && (!runs[s].force_dof || !runs[s].force_val)))
      return bad(p, "run: bad excitation arrays");
    for (int q = 0; q < runs[s].n_force; ++q) {
      const int d = runs[s].force_dof[q];
      if (d < 1 || d > 5 * meshes[s].nnode) return bad(p, "run: force DOF out of range");
      node_cnt[p->node_off[s] + (d - 1) / 5]++;
    }
    nforce_tot += runs[s].n_force;
    if (runs[s].n_out < 0 || (runs[s].n_out > 0 && !runs[s].out_dof)) return bad(p, "run: bad output arrays");
    for (int q = 0; q < runs[s].n_out; ++q) {
      const int d = runs[s].out_dof[q];
      if (d < 1 || d > 5 * meshes[s].nnode) return bad(p, "run: output DOF out of range");
      node_cnt[p->node_off[s] + (d - 1) / 5]++;  // adjoint force slot of this output
      nout_tot++;
    }
  }
  p->nforce = nforce_tot;
  for (int64_t g = 0; g < p->nnode; ++g) row_ptr[g + 1] = row_ptr[g] + node_cnt[g];
  slots.assign(row_ptr[p->nnode], 0);
  std::vector<int> fillc(p->nnode, 0);
  const int64_t P36 = (int64_t)NPE * FP;
  p->plane = P36 + std::max(nforce_tot + nout_tot, 1);
  p->plane = (p->plane + 31) / 32 * 32;

  std::vector<int> fq_field, fq_scen;
  std::vector<double> fq_val;
  int fq = 0, fo = 0;
  for (int s = 0; s < nscen; ++s) {
    const shm_mesh& m = meshes[s];
    const shm_material& mt = mats[s];
    const int64_t e0 = p->elem_off[s], n0 = p->node_off[s];
    if (mt.nmat < 1 || !mt.table) return bad(p, "material: empty table");
    for (int q = 0; q < mt.nmat; ++q) {
      for (int k = 0; k < SHM_MAT_STRIDE; ++k) mat.push_back(mt.table[(int64_t)q * SHM_MAT_STRIDE + k]);
      mat.push_back(0.0);
    }
    for (int e = 0; e < m.fen; ++e) {
      const int mi = mt.elem_mat ? mt.elem_mat[e] : 0;
      if (mi < 0 || mi >= mt.nmat) return bad(p, "material: elem_mat out of range");
      emat[e0 + e] = mat_base + mi;
      ekeep[e0 + e] = mt.elem_keep ? mt.elem_keep[e] : 1.0;
      elem_m11[e0 + e] = mt.table[(int64_t)mi * SHM_MAT_STRIDE + 21];
      elem_I11[e0 + e] = mt.table[(int64_t)mi * SHM_MAT_STRIDE + 22];
    }
    mat_base += mt.nmat;
    // connectivity and geometry (main_flat_shell.m:309-350, 400-419)
    for (int e = 0; e < m.fen; ++e) {
      double X[NPE], Y[NPE];
      for (int c = 0; c < NPE; ++c) {
        const int nd = m.nodes[(int64_t)c * m.fen + e];
        conn[(int64_t)c * FP + e0 + e] = (int)(n0 + nd - 1);
        X[c] = m.coords[nd - 1];
        Y[c] = m.coords[(int64_t)m.nnode + nd - 1];
      }
      for (int k = 0; k < NP; ++k)
        for (int i = 0; i < NP; ++i) {
          double J11 = 0, J21 = 0, J12 = 0, J22 = 0;
          for (int q = 0; q < NP; ++q) {
            J11 += D[i * NP + q] * X[k * NP + q];
            J21 += D[i * NP + q] * Y[k * NP + q];
            J12 += D[k * NP + q] * X[q * NP + i];
            J22 += D[k * NP + q] * Y[q * NP + i];
          }
          const double det = J11 * J22 - J12 * J21;
          if (!(det > 0)) return bad(p, "mesh: non-positive Jacobian determinant (element " + std::to_string(e + 1) + ")");
          const int c = k * NP + i;
          const int64_t base = (int64_t)c * FP + e0 + e;
          geo[0 * NPE * FP + base] = J22 / det;
          geo[1 * NPE * FP + base] = -J12 / det;
          geo[2 * NPE * FP + base] = -J21 / det;
          geo[3 * NPE * FP + base] = J11 / det;
          geo[4 * NPE * FP + base] = gw[i] * gw[k] * det;
        }
    }
    // assembly order: the 12-basket maps (given or built), basket by basket
    std::vector<int> IG, IL;
    int rows = 0;
    if (m.basket_rows > 0 && m.I_G && m.I_L) {
      rows = m.basket_rows;
      IG.assign(m.I_G, m.I_G + (size_t)rows * 12);
      IL.assign(m.I_L, m.I_L + (size_t)rows * 12);
    } else {
      build_baskets(m.fen, NPE, m.nnode, m.nodes, IG, IL, rows);
    }
    for (int b = 0; b < 12; ++b)
      for (int r = 0; r < rows; ++r) {
        const int kg = IG[(size_t)b * rows + r], kl = IL[(size_t)b * rows + r];
        if (kg == 0) continue;
        if (kg < 1 || kg > m.nnode || kl < 1 || kl > m.fen * NPE) return bad(p, "mesh: basket map out of range");
        const int e = (kl - 1) / NPE, c = (kl - 1) % NPE;
        const int64_t g = n0 + kg - 1;
        if (fillc[g] >= node_cnt[g]) return bad(p, "mesh: basket maps inconsistent with nodes");
        slots[row_ptr[g] + fillc[g]++] = (int)(c * FP + e0 + e);
      }
    // excitation slots after the element slots
    for (int q = 0; q < runs[s].n_force; ++q) {
      const int d = runs[s].force_dof[q];
      const int64_t g = n0 + (d - 1) / 5;
      if (fillc[g] >= node_cnt[g]) return bad(p, "internal: slot overflow");
      slots[row_ptr[g] + fillc[g]++] = (int)(P36 + fq);
      fq_field.push_back((d - 1) % 5);
      fq_scen.push_back(s);
      fq_val.push_back(runs[s].force_val[q]);
      ++fq;
    }
    // adjoint force slots (misfit residuals at the point outputs) after them
    for (int q = 0; q < runs[s].n_out; ++q) {
      const int d = runs[s].out_dof[q];
      const int64_t g = n0 + (d - 1) / 5;
      if (fillc[g] >= node_cnt[g]) return bad(p, "internal: slot overflow");
      slots[row_ptr[g] + fillc[g]++] = (int)(P36 + nforce_tot + fo++);
    }
  }
  for (int64_t g = 0; g < p->nnode; ++g)
    if (fillc[g] != node_cnt[g]) return bad(p, "mesh: basket maps do not cover every element node");

  // axis-aligned rectangles: invJ = diag(2/ax, 2/ay) and det J = ax ay / 4 on
  // every node of every element (then the element kernel reads 3 numbers)
  std::vector<double> grect((size_t)3 * FP, 0.0);
  bool rect = p->fen > 0;
  for (int64_t e = 0; e < p->fen && rect; ++e) {
    auto G = [&](int q, int c) { return geo[(int64_t)q * NPE * FP + (int64_t)c * FP + e]; };
    const double sx = G(0, 0), sy = G(3, 0), a4 = G(4, 0) / (gw[0] * gw[0]);
    for (int c = 0; c < NPE && rect; ++c) {
      if (std::fabs(G(1, c)) > 1e-12 * std::fabs(sx) || std::fabs(G(2, c)) > 1e-12 * std::fabs(sy) ||
          std::fabs(G(0, c) - sx) > 1e-10 * std::fabs(sx) || std::fabs(G(3, c) - sy) > 1e-10 * std::fabs(sy) ||
          std::fabs(G(4, c) / (gw[c % NP] * gw[c / NP]) - a4) > 1e-10 * std::fabs(a4))
        rect = false;
    }
    grect[e] = sx;
    grect[FP + e] = sy;
    grect[2 * FP + e] = a4;
  }

  // diagonal mass (main_flat_shell.m:493-501), summed in basket order
  std::vector<double> minv((size_t)2 * p->nnode_pad, 0.0), area((size_t)p->nnode_pad, 0.0);
  p->mass.assign((size_t)5 * p->nnode, 0.0);
  for (int64_t g = 0; g < p->nnode; ++g) {
    double mt_ = 0, mr_ = 0, ar = 0;
    for (int q = row_ptr[g]; q < row_ptr[g + 1]; ++q) {
      const int64_t sl = slots[q];
      if (sl >= P36) continue;
      const int64_t c = sl / FP, e = sl % FP;
      const double W = geo[4 * NPE * FP + c * FP + e];
      mt_ += W * elem_m11[e];
      mr_ += W * elem_I11[e];
      ar += W;
    }
    area[g] = ar;
    minv[g] = mt_ > 0 ? 1.0 / mt_ : 0.0;
    minv[p->nnode_pad + g] = mr_ > 0 ? 1.0 / mr_ : 0.0;
    p->mass[5 * g + 0] = mt_;
    p->mass[5 * g + 1] = mr_;
    p->mass[5 * g + 2] = mt_;
    p->mass[5 * g + 3] = mr_;
    p->mass[5 * g + 4] = mt_;
  }

  // outputs and sensors
  std::vector<int> out_node, out_field, esens(FP, -1), sptr(1, 0);
  p->out_off.assign(nscen + 1, 0);
  p->sens_off.assign(nscen + 1, 0);
  for (int s = 0; s < nscen; ++s) {
    const shm_run& r = runs[s];
    for (int q = 0; q < r.n_out; ++q) {
      const int d = r.out_dof[q];
      if (d < 1 || d > 5 * meshes[s].nnode) return bad(p, "run: output DOF out of range");
      out_node.push_back((int)(p->node_off[s] + (d - 1) / 5));
      out_field.push_back((d - 1) % 5);
    }
    p->out_off[s + 1] = p->out_off[s] + r.n_out;
    for (int k = 0; k < r.n_sens; ++k) {
      for (int q = r.sens_ptr[k]; q < r.sens_ptr[k + 1]; ++q) {
        const int e = r.sens_el[q];
        if (e < 0 || e >= meshes[s].fen) return bad(p, "run: sensor element out of range");
        if (esens[p->elem_off[s] + e] >= 0) return bad(p, "run: element listed in two sensors");
        esens[p->elem_off[s] + e] = p->nslot++;
      }
      sptr.push_back(p->nslot);
    }
    p->sens_off[s + 1] = p->sens_off[s] + r.n_sens;
    if (r.n_sens > 0) {
      if (!(r.g33 != 0)) return bad(p, "run: g33 must be nonzero with sensors");
      p->sc_k0 = r.pzt_thickness / r.g33;
      p->sc_e31 = r.e31;
      p->sc_e32 = r.e32;
      p->sc_hh = r.h / 2;
    }
  }
  p->nout = p->out_off[nscen];
  p->nsens = p->sens_off[nscen];

  shm_status st;
  if ((st = (p->prec == 64 ? build_device<double>(p, conn, geo, emat, ekeep, mat, minv)
                           : build_device<float>(p, conn, geo, emat, ekeep, mat, minv))) != SHM_OK)
    return st;
  if ((st = upload(p, &p->row_ptr, row_ptr)) != SHM_OK) return st;
  if ((st = upload(p, &p->slots, slots)) != SHM_OK) return st;
  if ((st = upload(p, &p->fq_field, fq_field)) != SHM_OK) return st;
  if ((st = upload(p, &p->fq_scen, fq_scen)) != SHM_OK) return st;
  if ((st = upload(p, &p->fq_val, fq_val)) != SHM_OK) return st;
  if ((st = upload(p, &p->out_node, out_node)) != SHM_OK) return st;
  if ((st = upload(p, &p->out_field, out_field)) != SHM_OK) return st;
  if ((st = upload(p, &p->esens, esens)) != SHM_OK) return st;
  if (rect) {
    if (p->prec == 64) {
      double* gr = nullptr;
      if ((st = upload(p, &gr, grect)) != SHM_OK) return st;
      p->grect = gr;
    } else {
      std::vector<float> g32(grect.begin(), grect.end());
      float* gr = nullptr;
      if ((st = upload(p, &gr, g32)) != SHM_OK) return st;
      p->grect = gr;
    }
  }
  if ((st = upload(p, &p->sptr, sptr)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->st, (size_t)nscen * p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->displ, (size_t)std::max(p->nout, 1) * p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->vsum, (size_t)std::max(p->nslot, 1) * p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->volt, (size_t)std::max(p->nsens, 1) * p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->flag, 4)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->d_base, 4)) != SHM_OK) return st;
  if ((st = set_func_attrs(p)) != SHM_OK) return st;
  if ((st = (p->prec == 64 ? pressure_build<double>(p, nscen, meshes, runs, area)
                           : pressure_build<float>(p, nscen, meshes, runs, area))) != SHM_OK)
    return st;

  // path selection
  p->path = 1;
  p->sp_generic = (o.path == 3);
  if (o.path == 2 || o.path == 0 || o.path == 3) {
    std::string why;
    shm_status ss = struct_build(p, nscen, meshes, mats, runs, o.tile_elems, gw, geo, emat, ekeep, esens, fq_field,
                                 fq_val, mat, o.rows_per_block, why);
    if (ss == SHM_OK) {
      p->path = 2;
    } else if (o.path == 2 || o.path == 3) {
      p->err = "structured path not available: " + why;
      return ss == SHM_ERR_OOM || ss == SHM_ERR_CUDA ? ss : SHM_ERR_UNSUPPORTED;
    }
  }
  CKP(p, cudaDeviceSynchronize());
  return shm_reset(p);
}

extern "C" shm_status shm_plan_destroy(shm_plan* p) {
  if (!p) return SHM_OK;
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  for (void* q : p->allocs) cudaFree(q);
  if (p->hstage) cudaFreeHost(p->hstage);
  for (cudaEvent_t e : p->fev)
    if (e) cudaEventDestroy(e);
  if (p->stream) cudaStreamDestroy(p->stream);
  for (cudaStream_t a : p->aux)
    if (a) cudaStreamDestroy(a);
  delete p;
  return SHM_OK;
}

extern "C" const char* shm_last_error(const shm_plan* p) {
  if (p) return p->err.c_str();
  const char* s = shm::static_last_error();  // calls without a plan (shm_stiffness_static)
  return s ? s : "no plan";
}

static cudaStream_t pick_stream(shm_plan* p, void* stream) {
  return stream ? (cudaStream_t)stream : p->stream;
}

extern "C" shm_status shm_reset(shm_plan* p) {
  if (!p) return SHM_ERR_BAD_ARG;
  cudaStream_t s = p->stream;
  const size_t ts = p->prec == 64 ? 8 : 4;
  CKP(p, cudaMemsetAsync(p->UA, 0, ts * p->nf * p->nnode_pad, s));
  CKP(p, cudaMemsetAsync(p->UB, 0, ts * p->nf * p->nnode_pad, s));
  if (p->frames) CKP(p, cudaMemsetAsync(p->frames, 0, ts * p->nframes * p->nfields * p->nnode_pad, s));
  CKP(p, cudaMemsetAsync(p->displ, 0, sizeof(double) * std::max(p->nout, 1) * p->nft, s));
  CKP(p, cudaMemsetAsync(p->vsum, 0, sizeof(double) * std::max(p->nslot, 1) * p->nft, s));
  CKP(p, cudaMemsetAsync(p->flag, 0, 4, s));
  CKP(p, cudaMemcpyAsync(p->d_base, &p->nn_first, 4, cudaMemcpyHostToDevice, s));
  CKP(p, cudaStreamSynchronize(s));
  p->nn = p->nn_first;
  p->ran = false;
  return SHM_OK;
}

extern "C" shm_status shm_set_signal(shm_plan* p, const double* st, void* stream) {
  if (!p || !st) return SHM_ERR_BAD_ARG;
  cudaStream_t s = pick_stream(p, stream);
  CKP(p, cudaMemcpyAsync(p->st, st, sizeof(double) * p->nscen * p->nft, cudaMemcpyHostToDevice, s));
  return SHM_OK;
}

static shm_status ensure_graph(shm_plan* p, cudaStream_t s) {
  if (p->steps_per_graph <= 0 || p->gexec) return SHM_OK;
  cudaGraph_t g = nullptr;
  CKP(p, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < p->steps_per_graph; ++k) {
    cudaError_t e = launch_step(p, k, s);
    if (e != cudaSuccess) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      p->err = std::string("capture: ") + cudaGetErrorString(e);
      return SHM_ERR_CUDA;
    }
  }
  k_advance<<<1, 1, 0, s>>>(p->d_base, p->steps_per_graph);
  CKP(p, cudaStreamEndCapture(s, &g));
  cudaError_t e = cudaGraphInstantiate(&p->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    p->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e);
    p->gexec = nullptr;
    return SHM_ERR_CUDA;
  }
  p->gsteps = p->steps_per_graph;
  return SHM_OK;
}

static shm_status advance_async(shm_plan* p, int nsteps, cudaStream_t s) {
  if (nsteps < 0) return bad(p, "nsteps < 0");
  if (p->nn + nsteps > p->nft + 1) return bad(p, "advance past nft");
  shm_status st = ensure_graph(p, s);
  if (st != SHM_OK) return st;
  if (p->persistent && p->path == 2 && nsteps > 0) {
    // runs of at most 2^30 / CTAs steps keep the barrier count below its abort bit
    const int grid = std::max(1, std::min(p->sp.grid, p->coop_max));
    const int chunk = std::max(1, (1 << 30) / grid);
    for (int done = 0; done < nsteps;) {
      const int n = std::min(chunk, nsteps - done);
      CKP(p, launch_struct_run_f32(p, n, s));
      k_advance<<<1, 1, 0, s>>>(p->d_base, n);
      CKP(p, cudaGetLastError());
      done += n;
    }
    p->nn += nsteps;
    p->ran = true;
    return SHM_OK;
  }
  int left = nsteps;
  while (p->gexec && left >= p->gsteps) {
    CKP(p, cudaGraphLaunch(p->gexec, s));
    left -= p->gsteps;
  }
  if (left > 0) {
    for (int k = 0; k < left; ++k) CKP(p, launch_step(p, k, s));
    k_advance<<<1, 1, 0, s>>>(p->d_base, left);
    CKP(p, cudaGetLastError());
  }
  p->nn += nsteps;
  p->ran = true;
  return SHM_OK;
}

static shm_status check_flag(shm_plan* p, cudaStream_t s) {
  int flag = 0;
  CKP(p, cudaMemcpyAsync(&flag, p->flag, 4, cudaMemcpyDeviceToHost, s));
  CKP(p, cudaStreamSynchronize(s));
  if (flag & 2) {
    p->err = "a bounded device-side wait gave up (bulk copies or the persistent step barrier)";
    return SHM_ERR_TIMEOUT;
  }
  if (flag) {
    p->err = "integration error: blow-up or non-finite state detected";
    return SHM_ERR_DIVERGED;
  }
  return SHM_OK;
}

extern "C" shm_status shm_advance(shm_plan* p, int32_t nsteps, void* stream) {
  if (!p) return SHM_ERR_BAD_ARG;
  cudaStream_t s = pick_stream(p, stream);
  shm_status st = advance_async(p, nsteps, s);
  if (st != SHM_OK) return st;
  return check_flag(p, s);
}

extern "C" shm_status shm_time_steps(shm_plan* p, int32_t nsteps, float* ms) {
  if (!p || !ms) return SHM_ERR_BAD_ARG;
  cudaStream_t s = p->stream;
  cudaEvent_t e[2] = {nullptr, nullptr};
  auto timed = [&]() -> shm_status {
    CKP(p, cudaEventCreate(&e[0]));
    CKP(p, cudaEventCreate(&e[1]));
    CKP(p, cudaStreamSynchronize(s));
    CKP(p, cudaEventRecord(e[0], s));
    shm_status st = advance_async(p, nsteps, s);
    if (st != SHM_OK) return st;
    CKP(p, cudaEventRecord(e[1], s));
    CKP(p, cudaEventSynchronize(e[1]));
    CKP(p, cudaEventElapsedTime(ms, e[0], e[1]));
    return SHM_OK;
  };
  const shm_status st = timed();
  for (cudaEvent_t ev : e)
    if (ev) cudaEventDestroy(ev);  // released on every return path
  if (st != SHM_OK) return st;
  return check_flag(p, s);
}

// One piece of the frames: rows r = 0 .. nr-1 of `src` (row stride `row`),
// columns 0 .. nc-1, packed ([r][nc]) and widened to FP64
template <typename T>
__global__ void k_pack_frames(const T* __restrict__ src, double* __restrict__ dst, int64_t row, int64_t nc,
                              int64_t nr) {
  const int64_t n = nr * nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / nc;
    dst[i] = (double)src[r * row + (i - r * nc)];
  }
}

// Frames to the caller: device [nframes][nfields][nnode_pad] over all
// scenarios (row = frame x nfields + field) -> host
// [nscen][nframes][nfields][nnode_s] in FP64.  The host array is cut into
// contiguous pieces of at most fstage_n values (default 4 M, 32 MB): runs of whole rows of one
// scenario's node range, or parts of one row when a row alone is larger.
// Each piece is packed and widened on the device into one of two staging
// buffers, moved to pinned host memory by the copy engine, and copied into
// the caller's array by the host while the next piece is in flight
// (pageable destinations never see a DMA).
static shm_status frames_to_host(shm_plan* p, double* frames, cudaStream_t s) {
  const int64_t kStage = p->fstage_n;  // values per staging buffer
  const int64_t row = p->nnode_pad;
  const int64_t rows = (int64_t)p->nframes * p->nfields;
  if (!p->fstage) {
    double* b = nullptr;
    shm_status st = dalloc(p, &b, 2 * (size_t)kStage);
    if (st != SHM_OK) return st;
    p->fstage = b;
  }
  if (!p->hstage) {
    void* h = nullptr;
    CKP(p, cudaMallocHost(&h, 2 * kStage * sizeof(double)));
    p->hstage = static_cast<double*>(h);
  }
  for (int k = 0; k < 2; ++k)
    if (!p->fev[k]) CKP(p, cudaEventCreateWithFlags(&p->fev[k], cudaEventDisableTiming));
  double* pend_dst[2] = {nullptr, nullptr};
  int64_t pend_n[2] = {0, 0};
  auto flush = [&](int b) -> shm_status {
    if (pend_dst[b]) {
      CKP(p, cudaEventSynchronize(p->fev[b]));
      std::memcpy(pend_dst[b], p->hstage + b * kStage, pend_n[b] * sizeof(double));
      pend_dst[b] = nullptr;
    }
    return SHM_OK;
  };
  int b = 0;
  int64_t host_off = 0;
  for (int sc = 0; sc < p->nscen; ++sc) {
    const int64_t n0 = p->node_off[sc], nn = p->node_off[sc + 1] - n0;
    if (nn <= 0) continue;
    const int64_t cw = std::min(nn, kStage);                       // columns per piece
    const int64_t per = nn <= kStage ? std::max<int64_t>(1, kStage / std::max<int64_t>(nn, 1)) : 1;
    for (int64_t r0 = 0; r0 < rows; r0 += per) {
      const int64_t nr = std::min(per, rows - r0);
      for (int64_t c0 = 0; c0 < nn; c0 += cw) {
        const int64_t nc = std::min(cw, nn - c0);
        const int64_t n = nr * nc;
        shm_status st = flush(b);  // buffer b is free once its previous piece is out
        if (st != SHM_OK) return st;
        const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
        const int64_t so = r0 * row + n0 + c0;
        if (p->prec == 32)
          k_pack_frames<float><<<blocks, 256, 0, s>>>((const float*)p->frames + so, p->fstage + b * kStage, row, nc, nr);
        else
          k_pack_frames<double><<<blocks, 256, 0, s>>>((const double*)p->frames + so, p->fstage + b * kStage, row, nc,
                                                       nr);
        CKP(p, cudaGetLastError());
        CKP(p, cudaMemcpyAsync(p->hstage + b * kStage, p->fstage + b * kStage, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
        CKP(p, cudaEventRecord(p->fev[b], s));
        pend_dst[b] = frames + host_off + r0 * nn + c0;  // nr == 1 whenever nc < nn
        pend_n[b] = n;
        b ^= 1;
      }
    }
    host_off += rows * nn;
  }
  for (int k = 0; k < 2; ++k, b ^= 1) {
    shm_status st = flush(b);
    if (st != SHM_OK) return st;
  }
  return SHM_OK;
}

extern "C" shm_status shm_read_outputs(shm_plan* p, double* displ, double* voltage, double* frames,
                                       void* stream) {
  if (!p) return SHM_ERR_BAD_ARG;
  cudaStream_t s = pick_stream(p, stream);
  if (displ && p->nout > 0)
    CKP(p, cudaMemcpyAsync(displ, p->displ, sizeof(double) * p->nout * p->nft, cudaMemcpyDeviceToHost, s));
  if (voltage && p->nsens > 0) {
    const int n = p->nsens * p->nft;
    k_voltage<<<(n + 255) / 256, 256, 0, s>>>(p->vsum, p->sptr, p->volt, p->nsens, p->nft);
    CKP(p, cudaGetLastError());
    CKP(p, cudaMemcpyAsync(voltage, p->volt, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  }
  if (frames && p->nframes > 0) {
    shm_status st = frames_to_host(p, frames, s);
    if (st != SHM_OK) return st;
  }
  CKP(p, cudaStreamSynchronize(s));
  return SHM_OK;
}

extern "C" shm_status shm_forward(shm_plan* p, const double* st, double* displ, double* voltage, double* frames,
                                  void* stream) {
  if (!p || !st) return SHM_ERR_BAD_ARG;
  shm_status r = shm_reset(p);
  if (r != SHM_OK) return r;
  cudaStream_t s = pick_stream(p, stream);
  if ((r = shm_set_signal(p, st, s)) != SHM_OK) return r;
  const int nsteps = p->nft - p->nn_first + 1;
  if ((r = advance_async(p, nsteps, s)) != SHM_OK) return r;
  shm_status div = check_flag(p, s);
  if ((r = shm_read_outputs(p, displ, voltage, frames, s)) != SHM_OK) return r;
  return div;
}

// state transfer in the reference layout [nnode][5]
template <typename T>
static shm_status get_state_t(shm_plan* p, double* U, double* uold) {
  const bool odd = ((p->nn - p->nn_first) & 1);
  const int nf = p->nf;
  std::vector<T> h((size_t)nf * p->nnode_pad);
  for (int which = 0; which < 2; ++which) {
    double* out = which == 0 ? U : uold;
    if (!out) continue;
    const void* src = (which == 0) ? (odd ? p->UB : p->UA) : (odd ? p->UA : p->UB);
    CKP(p, cudaMemcpy(h.data(), src, sizeof(T) * h.size(), cudaMemcpyDeviceToHost));
    for (int64_t g = 0; g < p->nnode; ++g)
      for (int f = 0; f < nf; ++f) out[nf * g + f] = (double)h[(size_t)f * p->nnode_pad + g];
  }
  return SHM_OK;
}

template <typename T>
static shm_status set_state_t(shm_plan* p, const double* U, const double* uold, int nn) {
  p->nn = nn;
  CKP(p, cudaMemcpy(p->d_base, &nn, 4, cudaMemcpyHostToDevice));
  const bool odd = ((nn - p->nn_first) & 1);
  const int nf = p->nf;
  std::vector<T> h((size_t)nf * p->nnode_pad, T(0));
  for (int which = 0; which < 2; ++which) {
    const double* in = which == 0 ? U : uold;
    std::fill(h.begin(), h.end(), T(0));
    if (in)
      for (int64_t g = 0; g < p->nnode; ++g)
        for (int f = 0; f < nf; ++f) h[(size_t)f * p->nnode_pad + g] = (T)in[nf * g + f];
    void* dst = (which == 0) ? (odd ? p->UB : p->UA) : (odd ? p->UA : p->UB);
    CKP(p, cudaMemcpy(dst, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  }
  return SHM_OK;
}

extern "C" shm_status shm_get_state(shm_plan* p, double* U, double* uold) {
  if (!p) return SHM_ERR_BAD_ARG;
  CKP(p, cudaStreamSynchronize(p->stream));
  return p->prec == 64 ? get_state_t<double>(p, U, uold) : get_state_t<float>(p, U, uold);
}

extern "C" shm_status shm_set_state(shm_plan* p, const double* U, const double* uold, int32_t nn) {
  if (!p) return SHM_ERR_BAD_ARG;
  if (nn < p->nn_first || nn > p->nft + 1) return bad(p, "set_state: nn out of range");
  CKP(p, cudaStreamSynchronize(p->stream));
  return p->prec == 64 ? set_state_t<double>(p, U, uold, nn) : set_state_t<float>(p, U, uold, nn);
}

template <typename T>
static shm_status apply_k_t(shm_plan* p, const double* U, double* F) {
  // uses the general element kernel on the plan's own stiffness buffers
  // (allocated by the first call, released with the plan), whatever the path
  std::vector<T> h((size_t)5 * p->nnode_pad, T(0));
  for (int64_t g = 0; g < p->nnode; ++g)
    for (int f = 0; f < 5; ++f) h[(size_t)f * p->nnode_pad + g] = (T)U[5 * g + f];
  shm_status st;
  if (!p->kt_U) {
    T *u = nullptr, *o = nullptr;
    int* b = nullptr;
    if ((st = dalloc(p, &u, h.size())) != SHM_OK) return st;
    if ((st = dalloc(p, &o, h.size())) != SHM_OK) return st;
    if ((st = dalloc(p, &b, 1)) != SHM_OK) return st;
    p->kt_U = u;
    p->kt_out = o;
    p->kt_base = b;
  }
  T* dU = (T*)p->kt_U;
  T* dOut = (T*)p->kt_out;
  CKP(p, cudaMemcpy(dU, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  CKP(p, cudaMemcpy(p->kt_base, &p->nn_first, 4, cudaMemcpyHostToDevice));
  GenArgs<T> a = make_args<T>(p);
  a.UA = dU;
  a.UB = dU;
  a.nforce = 0;
  a.nout = 0;
  a.d_base = p->kt_base;
  const int nblk = (int)(p->fen_pad / CTA_ELEMS);
  k_elem_general<T, false><<<nblk, CTA_THREADS, elem_smem_bytes(sizeof(T) == 8 ? 64 : 32), p->stream>>>(a, 0);
  CKP(p, cudaGetLastError());
  k_assemble_only<T><<<(int)((p->nnode + 255) / 256), 256, 0, p->stream>>>(a, dOut);
  CKP(p, cudaGetLastError());
  CKP(p, cudaMemcpyAsync(h.data(), dOut, sizeof(T) * h.size(), cudaMemcpyDeviceToHost, p->stream));
  CKP(p, cudaStreamSynchronize(p->stream));
  for (int64_t g = 0; g < p->nnode; ++g)
    for (int f = 0; f < 5; ++f) F[5 * g + f] = (double)h[(size_t)f * p->nnode_pad + g];
  return SHM_OK;
}

extern "C" shm_status shm_apply_stiffness(shm_plan* p, const double* U, double* F) {
  if (!p || !U || !F) return SHM_ERR_BAD_ARG;
  if (p->kind != 0) return bad(p, "apply_stiffness: flat-shell plans only");
  CKP(p, cudaStreamSynchronize(p->stream));
  return p->prec == 64 ? apply_k_t<double>(p, U, F) : apply_k_t<float>(p, U, F);
}

extern "C" shm_status shm_plan_info(const shm_plan* p, int64_t* info) {
  if (!p || !info) return SHM_ERR_BAD_ARG;
  info[0] = p->nnode;
  info[1] = p->fen;
  info[2] = (int64_t)p->nf * p->nnode;
  info[3] = p->path;
  info[4] = p->prec;
  info[5] = p->nframes;
  info[6] = p->path == 2 ? (p->persistent ? 0 : 1) : 2;  // 0: one launch per advance
  info[7] = p->path == 2 ? p->sp.tile : 0;
  info[8] = p->path == 2 ? p->sp.H : 0;
  info[9] = p->nfields;
  return SHM_OK;
}

extern "C" shm_status shm_mass(shm_plan* p, double* mg) {
  if (!p || !mg) return SHM_ERR_BAD_ARG;
  std::memcpy(mg, p->mass.data(), sizeof(double) * p->mass.size());
  return SHM_OK;
}

static void drop_graph(shm_plan* p) {
  if (p->gexec) {
    cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
    p->gsteps = 0;
  }
}

extern "C" shm_status shm_set_guard_interval(shm_plan* p, int32_t steps) {
  if (!p) return SHM_ERR_BAD_ARG;
  if (steps < 0) return bad(p, "guard interval must be >= 0");
  p->guard_int = steps;
  p->fspec.guard_int = steps;
  drop_graph(p);  // the step kernels' arguments are captured by value
  return SHM_OK;
}

// whether the plan can step persistently; sets coop_max and allocates the
// barrier words on first use
static shm_status persistent_ready(shm_plan* p) {
  if (p->kind != 0 || p->prec != 32 || p->sp_generic || p->path != 2)
    return bad(p, "persistent stepping needs an FP32 plan on the structured fused kernel");
  if (!p->gsync) {
    int coop = 0, nsm = 0;
    CKP(p, cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, p->device));
    if (!coop) {
      p->err = "the device does not support cooperative launches";
      return SHM_ERR_UNSUPPORTED;
    }
    CKP(p, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
    int per_sm[4] = {0, 0, 0, 0};
    CKP(p, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[0], k_struct_run_f32<32, false>, CTA_THREADS,
                                                         struct_f32_smem_bytes<32>()));
    CKP(p, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[1], k_struct_run_f32<32, true>, CTA_THREADS,
                                                         struct_f32_smem_bytes<32>()));
    CKP(p, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[2], k_struct_run_f32<16, false>, CTA_THREADS,
                                                         struct_f32_smem_bytes<16>()));
    CKP(p, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[3], k_struct_run_f32<16, true>, CTA_THREADS,
                                                         struct_f32_smem_bytes<16>()));
    const int m = *std::min_element(per_sm, per_sm + 4);
    if (m < 1) {
      p->err = "the persistent kernel does not fit on a multiprocessor";
      return SHM_ERR_UNSUPPORTED;
    }
    unsigned* g = nullptr;
    shm_status st = dalloc(p, &g, 4);
    if (st != SHM_OK) return st;
    p->gsync = g;
    p->coop_max = m * nsm;
  }
  return SHM_OK;
}

extern "C" shm_status shm_set_frame_staging(shm_plan* p, int64_t values) {
  if (!p) return SHM_ERR_BAD_ARG;
  if (values < 1) return bad(p, "frame staging needs at least one value");
  if (values != p->fstage_n) {  // the buffers are re-made at the next readback
    if (p->fstage) {
      CKP(p, cudaStreamSynchronize(p->stream));
      p->allocs.erase(std::find(p->allocs.begin(), p->allocs.end(), (void*)p->fstage));
      cudaFree(p->fstage);
      p->fstage = nullptr;
    }
    if (p->hstage) cudaFreeHost(p->hstage);
    p->hstage = nullptr;
    p->fstage_n = values;
  }
  return SHM_OK;
}

extern "C" shm_status shm_set_persistent(shm_plan* p, int32_t enable, int32_t spin_limit) {
  if (!p) return SHM_ERR_BAD_ARG;
  if (enable) {
    shm_status st = persistent_ready(p);
    if (st != SHM_OK) return st;
  }
  p->persistent = enable != 0;
  p->spin_limit = spin_limit < 0 ? (1 << 22) : spin_limit;
  return SHM_OK;
}

extern "C" shm_status shm_autotune(shm_plan* p, int32_t steps, int32_t* tile_out, int32_t* rows_out,
                                   float* ms_out) {
  if (!p) return SHM_ERR_BAD_ARG;
  if (p->path != 2) return bad(p, "autotune: the plan does not use the structured kernel");
  const int avail = p->nft - p->nn_first + 1;
  const int warm = 2;
  steps = std::max(2, std::min(steps, avail - warm));
  if (steps < 2) return bad(p, "autotune: run too short");
  const int tiles[2] = {16, 32};
  // rows per task: fixed candidates, and per tile the fewest rows with which
  // every task of the plan is resident at once (one wave of two CTAs per SM)
  // or in two waves -- a single large plate needs them to fill the GPU
  std::vector<int> cand[2];
  {
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess || nsm < 1) nsm = 1;
    for (int ti = 0; ti < 2; ++ti) {
      cand[ti] = {4, 8, 16, 32, 64};
      const int EW = tiles[ti], own = 5 * (EW - 1), G = 32 / EW;
      auto ntask = [&](int H) {
        long long n = 0;
        for (const PlateDesc& pl : p->sp.h_plates) n += (long long)((pl.NX + own - 1) / own) * ((pl.ney + H - 1) / H);
        return n;
      };
      for (int waves = 1; waves <= 2; ++waves)
        for (int H = 1; H <= 64; ++H)
          if (ntask(H) <= (long long)waves * 2 * nsm * G) {
            if (std::find(cand[ti].begin(), cand[ti].end(), H) == cand[ti].end()) cand[ti].push_back(H);
            break;
          }
    }
  }
  float best = 1e30f;
  int bt = p->sp.tile, bh = p->sp.H;
  bool bp = false;
  // every structured candidate is also timed as a persistent launch when the
  // plan and the device allow it
  const bool can_persist = persistent_ready(p) == SHM_OK;
  if (!can_persist) p->err.clear();
  p->persistent = false;
  // candidate 0: the general element + node kernels
  {
    p->path = 1;
    drop_graph(p);
    shm_status st = shm_reset(p);
    if (st == SHM_OK) st = advance_async(p, warm, p->stream);
    float ms = 0.f;
    if (st == SHM_OK) st = shm_time_steps(p, steps, &ms);
    if (st != SHM_OK) return st;
    best = ms;
    bt = 0;
    p->path = 2;
  }
  for (int ti = 0; ti < 2; ++ti)
    for (int H : cand[ti]) {
      shm_status st = struct_tasks(p, tiles[ti], H);
      if (st != SHM_OK) return st;
      for (int pers = 0; pers <= (can_persist ? 1 : 0); ++pers) {
        p->persistent = pers != 0;
        drop_graph(p);
        if ((st = shm_reset(p)) != SHM_OK) return st;
        if ((st = advance_async(p, warm, p->stream)) != SHM_OK) return st;
        float ms = 0.f;
        if ((st = shm_time_steps(p, steps, &ms)) != SHM_OK) return st;
        if (ms < best) {
          best = ms;
          bt = tiles[ti];
          bh = H;
          bp = pers != 0;
        }
      }
    }
  p->persistent = bt != 0 && bp;
  shm_status st = SHM_OK;
  if (bt == 0) {
    p->path = 1;  // the general kernels were fastest
  } else if ((st = struct_tasks(p, bt, bh)) != SHM_OK) {
    return st;
  }
  drop_graph(p);
  if ((st = shm_reset(p)) != SHM_OK) return st;
  if (tile_out) *tile_out = bt;
  if (rows_out) *rows_out = bh;
  if (ms_out) *ms_out = best / steps;
  return SHM_OK;
}

// ---------------------------------------------------------------------------
// discrete adjoint: misfit gradient with respect to per-element damage
// ---------------------------------------------------------------------------

// Scope guards: device buffers and events released on every return path.
struct DevFree {
  void* p = nullptr;
  ~DevFree() {
    if (p) cudaFree(p);
  }
};
struct EventSet {
  std::vector<cudaEvent_t> ev;
  cudaEvent_t add(unsigned flags = cudaEventDefault) {
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, flags);
    ev.push_back(e);
    return e;
  }
  ~EventSet() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};

template <typename T>
static shm_status fwd_bwd_t(shm_plan* p, const double* st, const double* target, double* misfit, double* grad,
                            int k, cudaStream_t s) {
  const int n0 = p->nn_first, N = p->nft;
  const int nsteps = N - n0 + 1;
  k = std::max(1, std::min(k, nsteps));
  const int nck = (nsteps + k - 1) / k;
  const size_t S = (size_t)5 * p->nnode_pad;
  shm_status st_;
  if (!p->LA) {
    T *la = nullptr, *lb = nullptr;
    if ((st_ = dalloc(p, &la, S)) != SHM_OK) return st_;
    if ((st_ = dalloc(p, &lb, S)) != SHM_OK) return st_;
    if ((st_ = dalloc(p, &p->grad, (size_t)p->fen_pad)) != SHM_OK) return st_;
    if ((st_ = dalloc(p, &p->asig, (size_t)std::max(p->nout, 1) * p->nft)) != SHM_OK) return st_;
    if ((st_ = dalloc(p, &p->d_base_adj, 4)) != SHM_OK) return st_;
    p->LA = la;
    p->LB = lb;
  }
  if (p->seg_k < k) {  // two sets of slots 1..k of a segment's recomputed states (slot 0 = the checkpoint)
    T* sg = nullptr;
    if ((st_ = dalloc(p, &sg, (size_t)2 * (k + 1) * S)) != SHM_OK) return st_;
    p->seg = sg;
    p->seg_k = k;
  }
  if (p->nck < nck) {
    T* c = nullptr;
    if ((st_ = dalloc(p, &c, (size_t)nck * 2 * S)) != SHM_OK) return st_;
    p->ck = c;
    p->nck = nck;
  }
  T* UA = (T*)p->UA;
  T* UB = (T*)p->UB;
  T* ck = (T*)p->ck;
  T* seg = (T*)p->seg;
  const size_t SB = S * sizeof(T);
  EventSet evs;
  cudaEvent_t ev[4];
  for (int i = 0; i < 4; ++i) ev[i] = evs.add();
  float t_rec = 0.f, t_adj = 0.f;
  // the last `nstore` segments keep every state of the forward pass in spare
  // device memory (8 GiB left free), so the backward pass recomputes only the
  // others
  int nstore = 0;
  T* store = nullptr;
  DevFree store_guard;
  {
    size_t fr = 0, tot = 0;
    const size_t per = (size_t)k * SB;
    if (p->store_cap >= 0) {
      nstore = (int)std::min<size_t>((size_t)nck, (size_t)p->store_cap / per);
    } else if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
      // -1: the device's spare memory less 8 GiB (opt-in); -3 (default): half
      // of the free memory, leaving the rest to other users of the device
      const size_t avail = p->store_cap == -1 ? (fr > ((size_t)8 << 30) ? fr - ((size_t)8 << 30) : 0) : fr / 2;
      if (avail >= per) nstore = (int)std::min<size_t>((size_t)nck, avail / per);
    }
    while (nstore > 0 && cudaMalloc(&store, (size_t)nstore * k * SB) != cudaSuccess) {
      cudaGetLastError();
      store = nullptr;
      nstore /= 2;
    }
    store_guard.p = store;
  }
  const int jstore = nck - nstore;  // first stored segment
  p->last_nstore = nstore;
  auto stored = [&](int j, int i) -> T* { return store + ((size_t)(j - jstore) * k + (i - 1)) * S; };
  // 1. forward pass with the plan's own step kernels (the structured fused
  // kernel when the plan uses it), checkpoint (u_n, u_{n-1}) every k steps
  if ((st_ = shm_reset(p)) != SHM_OK) return st_;
  if ((st_ = shm_set_signal(p, st, s)) != SHM_OK) return st_;
  cudaEventRecord(ev[0], s);
  for (int j = 0; j < nck; ++j) {
    const int n = n0 + j * k;
    const int cnt = std::min(k, N - n + 1);
    T* cku = ck + (size_t)j * 2 * S;
    if (j <= jstore) {  // the states are in the ping-pong pair
      const bool odd = ((n - n0) & 1);
      CKP(p, cudaMemcpyAsync(cku, odd ? UB : UA, SB, cudaMemcpyDeviceToDevice, s));
      CKP(p, cudaMemcpyAsync(cku + S, odd ? UA : UB, SB, cudaMemcpyDeviceToDevice, s));
    }
    if (j < jstore) {
      if ((st_ = advance_async(p, cnt, s)) != SHM_OK) return st_;
      continue;
    }
    // stored segment: step i reads state i (and i-1), writes state i+1 into
    // the store; its last step writes the next checkpoint
    k_set<<<1, 1, 0, s>>>(p->d_base, n);
    for (int i = 0; i < cnt; ++i) {
      T* cur = i == 0 ? cku : stored(j, i);
      T* prv = i == 0 ? cku + S : (i == 1 ? cku : stored(j, i - 1));
      T* out = i + 1 < cnt ? stored(j, i + 1) : (j + 1 < nck ? ck + (size_t)(j + 1) * 2 * S : UA);
      const bool odd = ((n + i - n0) & 1);
      p->ov_UA = odd ? prv : cur;
      p->ov_UB = odd ? cur : prv;
      p->ov_out = out;
      cudaError_t e = launch_step(p, i, s);
      p->ov_UA = p->ov_UB = p->ov_out = nullptr;
      if (e != cudaSuccess) {
        p->err = std::string("forward: ") + cudaGetErrorString(e);
        return SHM_ERR_CUDA;
      }
    }
    if (j + 1 < nck)  // u_{n-1} of the next checkpoint
      CKP(p, cudaMemcpyAsync(ck + (size_t)(j + 1) * 2 * S + S, cnt > 1 ? stored(j, cnt - 1) : cku, SB,
                             cudaMemcpyDeviceToDevice, s));
  }
  cudaEventRecord(ev[1], s);
  // 2. misfit (FP64) and the residuals in reversed time
  std::vector<double> disp((size_t)std::max(p->nout, 1) * N);
  CKP(p, cudaMemcpyAsync(disp.data(), p->displ, sizeof(double) * disp.size(), cudaMemcpyDeviceToHost, s));
  CKP(p, cudaStreamSynchronize(s));
  float t_fwd = 0.f;
  cudaEventElapsedTime(&t_fwd, ev[0], ev[1]);
  std::vector<double> asig((size_t)std::max(p->nout, 1) * N, 0.0);
  for (int sc = 0; sc < p->nscen; ++sc) {
    double J = 0.0;
    for (int q = p->out_off[sc]; q < p->out_off[sc + 1]; ++q)
      for (int m = n0; m <= N; ++m) {
        const double r = disp[(size_t)q * N + m - 1] - target[(size_t)q * N + m - 1];
        J += 0.5 * r * r;
        asig[(size_t)q * N + (N + n0 - m) - 1] = r;  // sample read by the adjoint step t' = N + n0 - m
      }
    if (misfit) misfit[sc] = J;
  }
  CKP(p, cudaMemcpyAsync(p->asig, asig.data(), sizeof(double) * asig.size(), cudaMemcpyHostToDevice, s));
  // 3. backward: recompute each segment forward into its state slots with the
  // forward pass's step kernels (bit-identical states, no copies), then step
  // the adjoint back through it.  Segment j-1 is recomputed on one stream
  // while the adjoint steps through segment j on another (two slot sets, a
  // separate element-force scratch for the adjoint); both sweeps are
  // latency-bound, so running them side by side raises the device's use.
  if (!p->F2adj) {
    T* f2a = nullptr;
    if ((st_ = dalloc(p, &f2a, (size_t)5 * p->plane)) != SHM_OK) return st_;
    p->F2adj = f2a;
  }
  for (int i = 0; i < 2; ++i)
    if (!p->aux[i]) CKP(p, cudaStreamCreateWithFlags(&p->aux[i], cudaStreamNonBlocking));
  cudaStream_t sr = p->aux[0], sa = p->aux[1];
  CKP(p, cudaMemsetAsync(p->LA, 0, SB, s));
  CKP(p, cudaMemsetAsync(p->LB, 0, SB, s));
  CKP(p, cudaMemsetAsync(p->F2adj, 0, sizeof(T) * 5 * p->plane, s));
  CKP(p, cudaMemsetAsync(p->grad, 0, sizeof(double) * p->fen_pad, s));
  CKP(p, cudaMemcpyAsync(p->d_base_adj, &n0, 4, cudaMemcpyHostToDevice, s));
  const cudaEvent_t ev_s = evs.add(cudaEventDisableTiming);
  const cudaEvent_t ev_end_r = evs.add(), ev_end_a = evs.add();
  std::vector<cudaEvent_t> evR(nck), evA(nck);
  for (int j = 0; j < nck; ++j) {
    evR[j] = evs.add(cudaEventDisableTiming);
    evA[j] = evs.add(cudaEventDisableTiming);
  }
  CKP(p, cudaEventRecord(ev_s, s));
  CKP(p, cudaStreamWaitEvent(sr, ev_s, 0));
  CKP(p, cudaStreamWaitEvent(sa, ev_s, 0));
  GenArgs<T> a = make_args<T>(p);
  a.UA = (T*)p->LA;
  a.UB = (T*)p->LB;
  a.outp = nullptr;
  a.F2 = (T*)p->F2adj;
  a.d_base = p->d_base_adj;
  a.nadj = p->nout;
  a.asig = p->asig;
  a.grad = p->grad;
  a.fs.frm_int = 0;
  a.pr.npf = 0;  // forward-only loads do not enter the adjoint
  a.nout = 0;
  const int nblk = (int)(p->fen_pad / CTA_ELEMS);
  const size_t smem = adj_smem_bytes(sizeof(T) == 8 ? 64 : 32);
  // plans on the fused FP32 kernel step the adjoint with its adjoint variant
  const bool fused = sizeof(T) == 4 && p->path == 2 && !p->sp_generic;
  F32Args af{};
  if (fused) {
    af = struct_f32_args(p);
    af.UA = (float*)p->LA;
    af.UB = (float*)p->LB;
    af.outp = nullptr;
    af.d_base = p->d_base_adj;
    af.nout = 0;
    af.fs.frm_int = 0;
    af.pr.npf = 0;
    af.asig = p->asig;
    af.grad = p->grad;
  }
  auto seg_state = [&](int j, int i) -> T* {  // u at forward time sj + i of segment j
    T* ck_u = ck + (size_t)j * 2 * S;
    if (i < 0) return ck_u + S;
    if (i == 0) return ck_u;
    if (j >= jstore) return stored(j, i);
    return seg + ((size_t)(j & 1) * (k + 1) + i) * S;
  };
  cudaEventRecord(ev[2], sr);
  auto recompute = [&](int j) -> shm_status {
    if (j >= jstore) {  // states kept by the forward pass
      CKP(p, cudaEventRecord(evR[j], sr));
      return SHM_OK;
    }
    const int sj = n0 + j * k, cnt = std::min(sj + k - 1, N) - sj + 1;
    k_set<<<1, 1, 0, sr>>>(p->d_base, sj);
    for (int i = 0; i + 1 < cnt; ++i) {
      const bool odd = ((sj + i - n0) & 1);
      p->ov_UA = odd ? seg_state(j, i - 1) : seg_state(j, i);
      p->ov_UB = odd ? seg_state(j, i) : seg_state(j, i - 1);
      p->ov_out = seg_state(j, i + 1);
      cudaError_t e = launch_step(p, i, sr);
      p->ov_UA = p->ov_UB = p->ov_out = nullptr;
      if (e != cudaSuccess) {
        p->err = std::string("recompute: ") + cudaGetErrorString(e);
        return SHM_ERR_CUDA;
      }
    }
    CKP(p, cudaEventRecord(evR[j], sr));
    return SHM_OK;
  };
  if ((st_ = recompute(nck - 1)) != SHM_OK) return st_;
  cudaEventRecord(ev[3], sa);
  int nn_adj = n0;  // adjoint loop index of the segment's first adjoint step
  for (int j = nck - 1; j >= 0; --j) {
    const int sj = n0 + j * k, cnt = std::min(sj + k - 1, N) - sj + 1;
    // adjoint through segment j once its states exist
    CKP(p, cudaStreamWaitEvent(sa, evR[j], 0));
    for (int kk = 0; kk < cnt; ++kk) {
      const T* um = seg_state(j, N + n0 - (nn_adj + kk) - sj);  // u at forward time N + n0 - nn
      if (fused) {
        af.um = (const float*)um;
        if (p->sp.tile == 32)
          k_struct_step_f32<32, false, true><<<p->sp.grid, CTA_THREADS, struct_f32_smem_bytes<32>(), sa>>>(af, kk);
        else
          k_struct_step_f32<16, false, true><<<p->sp.grid, CTA_THREADS, struct_f32_smem_bytes<16>(), sa>>>(af, kk);
      } else {
        a.um = um;
        k_elem_adjoint<T><<<nblk, CTA_THREADS, smem, sa>>>(a, kk);
        k_node_general<T><<<(int)((p->nnode + 255) / 256), 256, 0, sa>>>(a, kk);
      }
    }
    k_advance<<<1, 1, 0, sa>>>(p->d_base_adj, cnt);
    CKP(p, cudaGetLastError());
    CKP(p, cudaEventRecord(evA[j], sa));
    nn_adj += cnt;
    // meanwhile recompute segment j-1 into the slot set segment j+1 used
    if (j > 0) {
      if (j + 1 < nck) CKP(p, cudaStreamWaitEvent(sr, evA[j + 1], 0));
      if ((st_ = recompute(j - 1)) != SHM_OK) return st_;
    }
  }
  cudaEventRecord(ev_end_r, sr);
  cudaEventRecord(ev_end_a, sa);
  CKP(p, cudaStreamWaitEvent(s, ev_end_r, 0));
  CKP(p, cudaStreamWaitEvent(s, ev_end_a, 0));
  CKP(p, cudaStreamSynchronize(s));
  cudaEventElapsedTime(&t_rec, ev[2], ev_end_r);
  cudaEventElapsedTime(&t_adj, ev[3], ev_end_a);
  p->fb_ms[0] = t_fwd;
  p->fb_ms[1] = t_rec;
  p->fb_ms[2] = t_adj;
  std::vector<double> g((size_t)p->fen_pad);
  CKP(p, cudaMemcpyAsync(g.data(), p->grad, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, s));
  // leave the adjoint slots zero for later forward runs
  const int64_t p36 = (int64_t)NPE * p->fen_pad;
  for (int f = 0; f < 5; ++f)
    if (p->nout > 0)
      CKP(p, cudaMemsetAsync((T*)p->F2 + f * p->plane + p36 + p->nforce, 0, sizeof(T) * p->nout, s));
  CKP(p, cudaStreamSynchronize(s));
  if (grad) std::memcpy(grad, g.data(), sizeof(double) * p->fen);
  shm_status div = check_flag(p, s);
  st_ = shm_reset(p);
  return div != SHM_OK ? div : st_;
}

extern "C" shm_status shm_forward_backward_timing(const shm_plan* p, float* ms3) {
  if (!p || !ms3) return SHM_ERR_BAD_ARG;
  for (int i = 0; i < 3; ++i) ms3[i] = p->fb_ms[i];
  return SHM_OK;
}

extern "C" shm_status shm_set_adjoint_store(shm_plan* p, int64_t max_bytes, int32_t* last_segments) {
  if (!p) return SHM_ERR_BAD_ARG;
  if (last_segments) *last_segments = p->last_nstore;
  if (max_bytes >= -1 || max_bytes == -3) p->store_cap = max_bytes;
  return SHM_OK;
}

extern "C" shm_status shm_forward_backward(shm_plan* p, const double* st, const double* target, double* misfit,
                                           double* grad, int32_t ckpt_every, void* stream) {
  if (!p || !st || !target) return SHM_ERR_BAD_ARG;
  if (p->kind != 0) return bad(p, "forward_backward: flat-shell plans only");
  if (p->nout < 1) return bad(p, "forward_backward: the misfit needs point outputs");
  cudaStream_t s = pick_stream(p, stream);
  drop_graph(p);
  return p->prec == 64 ? fwd_bwd_t<double>(p, st, target, misfit, grad, ckpt_every, s)
                       : fwd_bwd_t<float>(p, st, target, misfit, grad, ckpt_every, s);
}

// ---------------------------------------------------------------------------
// 3D solid plans (6x6x3 hexahedra, 3 DOF per node)
// ---------------------------------------------------------------------------

template <typename T>
static cudaError_t launch_solid_step(shm_plan* p, int kstep, cudaStream_t s) {
  SolidArgs<T> a;
  a.fen_pad = p->fen_pad;
  a.nnode_pad = p->nnode_pad;
  a.plane = p->plane;
  a.nnode = (int)p->nnode;
  a.fen = (int)p->fen;
  a.nn_first = p->nn_first;
  a.nft = p->nft;
  a.UA = (T*)p->UA;
  a.UB = (T*)p->UB;
  a.F2 = (T*)p->F2;
  a.conn = p->conn;
  a.geo = (const T*)p->geo;
  a.emat = p->emat;
  a.ekeep = (const T*)p->ekeep;
  a.mat = (const T*)p->mat;
  a.row_ptr = p->row_ptr;
  a.slots = p->slots;
  a.minv = (const T*)p->minv;
  for (int f = 0; f < 3; ++f) {
    a.k1[f] = (T)p->k1[f];
    a.k2[f] = (T)p->k2[f];
  }
  a.nforce = p->nforce;
  a.fq_field = p->fq_field;
  a.fq_scen = p->fq_scen;
  a.fq_val = p->fq_val;
  a.st = p->st;
  a.nout = p->nout;
  a.out_node = p->out_node;
  a.out_field = p->out_field;
  a.displ = p->displ;
  a.fs = p->fspec;
  a.frames = (T*)p->frames;
  a.a0 = (T)p->a0;
  a.a1 = (T)p->a1;
  a.blowup = (T)p->blowup;
  a.flag = p->flag;
  a.d_base = p->d_base;
  a.gbox = (const T*)p->gbox;
  if constexpr (sizeof(T) == 4) {  // node lines, on the resident grid
    using SL = SolidLines<T>;
    const int groups = (int)(p->fen_pad / SL::EPB);
    const int grid = p->solid_grid > 0 ? std::min(groups, p->solid_grid) : groups;
    if (p->gbox)
      k_elem_solid<T, true><<<grid, SL::THREADS, SL::SMEM, s>>>(a, kstep);
    else
      k_elem_solid<T, false><<<grid, SL::THREADS, SL::SMEM, s>>>(a, kstep);
  } else {  // a thread per node
    if (p->gbox)
      k_elem_solid_nodes<T, true><<<(int)(p->fen_pad / S_NODE_EPB), S_NODE_THREADS, 0, s>>>(a, kstep);
    else
      k_elem_solid_nodes<T, false><<<(int)(p->fen_pad / S_NODE_EPB), S_NODE_THREADS, 0, s>>>(a, kstep);
  }
  k_node_solid<T><<<(int)((p->nnode + 255) / 256), 256, 0, s>>>(a, kstep);
  return cudaGetLastError();
}

template <typename T>
static shm_status solid_device(shm_plan* p, const std::vector<int>& conn, const std::vector<double>& geo,
                               const std::vector<int>& emat, const std::vector<double>& ekeep,
                               const std::vector<double>& mat, const std::vector<double>& minv,
                               const std::vector<double>* gbox) {
  auto conv = [](const std::vector<double>& v) {
    std::vector<T> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = (T)v[i];
    return o;
  };
  shm_status s;
  T *g = nullptr, *k = nullptr, *m = nullptr, *mi = nullptr, *ua = nullptr, *ub = nullptr, *f2 = nullptr,
    *fr = nullptr;
  if constexpr (sizeof(T) == 4) {
    CKP(p, cudaFuncSetAttribute(k_elem_solid<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SolidLines<T>::SMEM));
    CKP(p, cudaFuncSetAttribute(k_elem_solid<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SolidLines<T>::SMEM));
    // the element kernel loops over element groups on the CTAs that fit at once
    int nsm = 0, per_sm = 0;
    CKP(p, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
    CKP(p, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_elem_solid<T, false>, SolidLines<T>::THREADS,
                                                         SolidLines<T>::SMEM));
    p->solid_grid = std::max(1, per_sm) * nsm;
  }
  if ((s = upload(p, &p->conn, conn)) != SHM_OK) return s;
  if (gbox) {  // box elements: the per-node geometry is not needed on the device
    T* gb = nullptr;
    if ((s = upload(p, &gb, conv(*gbox))) != SHM_OK) return s;
    p->gbox = gb;
  } else if ((s = upload(p, &g, conv(geo))) != SHM_OK) {
    return s;
  }
  if ((s = upload(p, &p->emat, emat)) != SHM_OK) return s;
  if ((s = upload(p, &k, conv(ekeep))) != SHM_OK) return s;
  if ((s = upload(p, &m, conv(mat))) != SHM_OK) return s;
  if ((s = upload(p, &mi, conv(minv))) != SHM_OK) return s;
  if ((s = dalloc(p, &ua, (size_t)3 * p->nnode_pad)) != SHM_OK) return s;
  if ((s = dalloc(p, &ub, (size_t)3 * p->nnode_pad)) != SHM_OK) return s;
  if ((s = dalloc(p, &f2, (size_t)3 * p->plane)) != SHM_OK) return s;
  if (p->nframes > 0 && (s = dalloc(p, &fr, (size_t)p->nframes * p->nfields * p->nnode_pad)) != SHM_OK) return s;
  p->geo = g;
  p->ekeep = k;
  p->mat = m;
  p->minv = mi;
  p->UA = ua;
  p->UB = ub;
  p->F2 = f2;
  p->frames = fr;
  return SHM_OK;
}

extern "C" shm_status shm_solid_plan_create(int32_t nscen, const shm_solid_mesh* meshes,
                                            const shm_solid_material* mats, const shm_run* runs,
                                            const shm_options* opt, shm_plan** out) {
  if (!out) return SHM_ERR_BAD_ARG;
  *out = nullptr;
  if (nscen < 1 || !meshes || !mats || !runs) return SHM_ERR_BAD_ARG;
  shm_plan* p = new shm_plan();
  *out = p;
  p->kind = 1;
  p->nf = 3;
  shm_options o{};
  o.precision = 64;
  if (opt) o = *opt;
  if (o.precision != 64 && o.precision != 32) return bad(p, "precision must be 32 or 64");
  p->prec = o.precision;
  p->device = o.device;
  p->steps_per_graph = std::max(0, o.steps_per_graph);
  p->nscen = nscen;
  p->path = 1;
  CKP(p, cudaSetDevice(o.device));
  CKP(p, cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  const shm_run& r0 = runs[0];
  if (!(r0.dt > 0) || r0.nft < 1 || (r0.nn_first != 1 && r0.nn_first != 2))
    return bad(p, "run: dt > 0, nft >= 1, nn_first in {1,2} required");
  for (int s = 1; s < nscen; ++s)
    if (runs[s].dt != r0.dt || runs[s].nft != r0.nft || runs[s].nn_first != r0.nn_first ||
        runs[s].eta_xy != r0.eta_xy || runs[s].eta_z != r0.eta_z || runs[s].frm_int != r0.frm_int)
      return bad(p, "all scenarios of a batch must share dt, nft, nn_first, damping and frames");
  p->dt = r0.dt;
  p->nft = r0.nft;
  p->nn_first = p->nn = r0.nn_first;
  p->a0 = 1.0 / (r0.dt * r0.dt);
  p->a1 = 1.0 / (2.0 * r0.dt);
  // damping: dv(x,y) = etad_xy, dv(z) = etad_z (main_spec3Dcuda_global_...:864-867)
  const double eta[3] = {r0.eta_xy, r0.eta_xy, r0.eta_z};
  for (int f = 0; f < 3; ++f) {
    const double den = p->a0 + p->a1 * eta[f];
    p->k1[f] = (p->a0 - p->a1 * eta[f]) / den;
    p->k2[f] = 1.0 / den;
  }
  if (set_frames(p, r0, 3) != SHM_OK) return SHM_ERR_BAD_ARG;
  for (int s2 = 0; s2 < nscen; ++s2)
    if (runs[s2].n_pframes > 0) {
      p->err = "pressure loading is built for flat-shell plans";
      return SHM_ERR_UNSUPPORTED;
    }
  p->blowup = INFINITY;
  p->node_off.assign(nscen + 1, 0);
  p->elem_off.assign(nscen + 1, 0);
  for (int s = 0; s < nscen; ++s) {
    const shm_solid_mesh& m = meshes[s];
    if (m.npe != S_NPE) return bad(p, "solid npe must be 108 (6x6x3)");
    if (m.fen < 1 || m.nnode < 1 || !m.nodes || !m.coords) return bad(p, "mesh: empty or NULL arrays");
    p->node_off[s + 1] = p->node_off[s] + m.nnode;
    p->elem_off[s + 1] = p->elem_off[s] + m.fen;
  }
  p->nnode = p->node_off[nscen];
  p->fen = p->elem_off[nscen];
  if (p->nnode > INT32_MAX / 2 || p->fen * (int64_t)S_NPE > INT32_MAX / 2) return bad(p, "mesh too large");
  p->fen_pad = (p->fen + S_EPB - 1) / S_EPB * S_EPB;
  p->nnode_pad = (p->nnode + 31) / 32 * 32;
  std::vector<double> gx, gw, D, gx3, gw3, D3;
  gll_setup(NP, gx, gw, D);
  gll_setup(S_NZ, gx3, gw3, D3);
  {
    float D32[36], D332[9];
    for (int i = 0; i < 36; ++i) D32[i] = (float)D[i];
    for (int i = 0; i < 9; ++i) D332[i] = (float)D3[i];
    CKP(p, cudaMemcpyToSymbol(c_D64, D.data(), sizeof(double) * 36));
    CKP(p, cudaMemcpyToSymbol(c_D32, D32, sizeof(float) * 36));
    CKP(p, cudaMemcpyToSymbol(c_D3_64, D3.data(), sizeof(double) * 9));
    CKP(p, cudaMemcpyToSymbol(c_D3_32, D332, sizeof(float) * 9));
    float w32[NP], w332[S_NZ];
    for (int i = 0; i < NP; ++i) w32[i] = (float)gw[i];
    for (int i = 0; i < S_NZ; ++i) w332[i] = (float)gw3[i];
    CKP(p, cudaMemcpyToSymbol(c_w64, gw.data(), sizeof(double) * NP));
    CKP(p, cudaMemcpyToSymbol(c_w32, w32, sizeof(float) * NP));
    CKP(p, cudaMemcpyToSymbol(c_w3_64, gw3.data(), sizeof(double) * S_NZ));
    CKP(p, cudaMemcpyToSymbol(c_w3_32, w332, sizeof(float) * S_NZ));
  }
  const int64_t FP = p->fen_pad;
  std::vector<int> conn((size_t)S_NPE * FP, 0), emat(FP, 0);
  std::vector<double> geo((size_t)10 * S_NPE * FP, 0.0), ekeep(FP, 1.0), mat, erho(FP, 0.0);
  std::vector<int> node_cnt(p->nnode, 0);
  int mat_base = 0, nforce_tot = 0;
  for (int s = 0; s < nscen; ++s) {
    const shm_solid_mesh& m = meshes[s];
    for (int c = 0; c < S_NPE; ++c)
      for (int e = 0; e < m.fen; ++e) {
        const int nd = m.nodes[(int64_t)c * m.fen + e];
        if (nd < 1 || nd > m.nnode) return bad(p, "mesh: node number out of range");
        node_cnt[p->node_off[s] + nd - 1]++;
      }
    for (int q = 0; q < runs[s].n_force; ++q) {
      const int d = runs[s].force_dof[q];
      if (d < 1 || d > 3 * m.nnode) return bad(p, "run: force DOF out of range");
      node_cnt[p->node_off[s] + (d - 1) / 3]++;
    }
    nforce_tot += runs[s].n_force;
  }
  p->nforce = nforce_tot;
  std::vector<int> row_ptr(p->nnode + 1, 0);
  for (int64_t g = 0; g < p->nnode; ++g) row_ptr[g + 1] = row_ptr[g] + node_cnt[g];
  std::vector<int> slots(row_ptr[p->nnode]), fillc(p->nnode, 0);
  const int64_t P0 = (int64_t)S_NPE * FP;
  p->plane = (P0 + std::max(nforce_tot, 1) + 31) / 32 * 32;
  std::vector<int> fq_field, fq_scen, out_node, out_field;
  std::vector<double> fq_val;
  int fq = 0;
  p->out_off.assign(nscen + 1, 0);
  for (int s = 0; s < nscen; ++s) {
    const shm_solid_mesh& m = meshes[s];
    const shm_solid_material& mt = mats[s];
    const int64_t e0 = p->elem_off[s], n0 = p->node_off[s];
    if (mt.nmat < 1 || !mt.table) return bad(p, "material: empty table");
    for (int q = 0; q < mt.nmat; ++q) {
      for (int k = 0; k < S_MAT; ++k) mat.push_back(mt.table[(int64_t)q * S_MAT + k]);
      mat.push_back(0.0);
      mat.push_back(0.0);
    }
    for (int e = 0; e < m.fen; ++e) {
      const int mi = mt.elem_mat ? mt.elem_mat[e] : 0;
      if (mi < 0 || mi >= mt.nmat) return bad(p, "material: elem_mat out of range");
      emat[e0 + e] = mat_base + mi;
      ekeep[e0 + e] = mt.elem_keep ? mt.elem_keep[e] : 1.0;
      erho[e0 + e] = mt.table[(int64_t)mi * S_MAT + 13];
    }
    mat_base += mt.nmat;
    // geometry at the GLL nodes: J[b][a] = dx_b/dxi_a, invJ = J^-1 (iJ[a][b] = dxi_a/dx_b)
    for (int e = 0; e < m.fen; ++e) {
      double X[S_NPE][3];
      for (int c = 0; c < S_NPE; ++c) {
        const int nd = m.nodes[(int64_t)c * m.fen + e];
        conn[(e0 + e) * S_NPE + c] = (int)(n0 + nd - 1);
        for (int b = 0; b < 3; ++b) X[c][b] = m.coords[(int64_t)b * m.nnode + nd - 1];
      }
      for (int c = 0; c < S_NPE; ++c) {
        const int cx = c % NP, cy = (c / NP) % NP, cz = c / 36;
        double J[3][3] = {{0}};  // J[b][a]
        for (int b = 0; b < 3; ++b) {
          for (int q = 0; q < NP; ++q) {
            J[b][0] += D[cx * NP + q] * X[cz * 36 + cy * NP + q][b];
            J[b][1] += D[cy * NP + q] * X[cz * 36 + q * NP + cx][b];
          }
          for (int q = 0; q < S_NZ; ++q) J[b][2] += D3[cz * S_NZ + q] * X[q * 36 + cy * NP + cx][b];
        }
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        if (!(std::fabs(det) > 0)) return bad(p, "mesh: singular solid element " + std::to_string(e + 1));
        // inverse of J (row b, column a): inv[a][b]
        double inv[3][3];
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        for (int q = 0; q < 9; ++q) geo[((int64_t)q * FP + e0 + e) * S_NPE + c] = inv[q / 3][q % 3];
        geo[((int64_t)9 * FP + e0 + e) * S_NPE + c] = gw[cx] * gw[cy] * gw3[cz] * std::fabs(det);
      }
    }
    std::vector<int> IG, IL;
    int rows = 0;
    if (m.basket_rows > 0 && m.I_G && m.I_L) {
      rows = m.basket_rows;
      IG.assign(m.I_G, m.I_G + (size_t)rows * 12);
      IL.assign(m.I_L, m.I_L + (size_t)rows * 12);
    } else {
      build_baskets(m.fen, S_NPE, m.nnode, m.nodes, IG, IL, rows);
    }
    for (int b = 0; b < 12; ++b)
      for (int r = 0; r < rows; ++r) {
        const int kg = IG[(size_t)b * rows + r], kl = IL[(size_t)b * rows + r];
        if (kg == 0) continue;
        if (kg < 1 || kg > m.nnode || kl < 1 || kl > m.fen * S_NPE) return bad(p, "mesh: basket map out of range");
        const int e = (kl - 1) / S_NPE, c = (kl - 1) % S_NPE;
        const int64_t g = n0 + kg - 1;
        if (fillc[g] >= node_cnt[g]) return bad(p, "mesh: basket maps inconsistent with nodes");
        slots[row_ptr[g] + fillc[g]++] = (int)((e0 + e) * S_NPE + c);
      }
    for (int q = 0; q < runs[s].n_force; ++q) {
      const int d = runs[s].force_dof[q];
      const int64_t g = n0 + (d - 1) / 3;
      slots[row_ptr[g] + fillc[g]++] = (int)(P0 + fq);
      fq_field.push_back((d - 1) % 3);
      fq_scen.push_back(s);
      fq_val.push_back(runs[s].force_val[q]);
      ++fq;
    }
    for (int q = 0; q < runs[s].n_out; ++q) {
      const int d = runs[s].out_dof[q];
      if (d < 1 || d > 3 * m.nnode) return bad(p, "run: output DOF out of range");
      out_node.push_back((int)(n0 + (d - 1) / 3));
      out_field.push_back((d - 1) % 3);
    }
    p->out_off[s + 1] = p->out_off[s] + runs[s].n_out;
  }
  for (int64_t g = 0; g < p->nnode; ++g)
    if (fillc[g] != node_cnt[g]) return bad(p, "mesh: basket maps do not cover every element node");
  p->nout = p->out_off[nscen];
  p->sens_off.assign(nscen + 1, 0);
  // lumped mass rho * w * detJ (mass3D_v2.m), summed in basket order
  std::vector<double> minv((size_t)p->nnode_pad, 0.0);
  p->mass.assign((size_t)3 * p->nnode, 0.0);
  for (int64_t g = 0; g < p->nnode; ++g) {
    double mm = 0.0;
    for (int q = row_ptr[g]; q < row_ptr[g + 1]; ++q) {
      const int64_t sl = slots[q];
      if (sl >= P0) continue;
      const int64_t e = sl / S_NPE;
      mm += geo[(int64_t)9 * FP * S_NPE + sl] * erho[e];
    }
    minv[g] = mm > 0 ? 1.0 / mm : 0.0;
    for (int f = 0; f < 3; ++f) p->mass[3 * g + f] = mm;
  }
  // axis-aligned boxes: diagonal constant inverse Jacobian and constant |det J|
  // per element (4 numbers instead of 1 080 per-node values)
  std::vector<double> gbox((size_t)4 * FP, 0.0);
  bool box = true;
  for (int64_t e = 0; e < p->fen && box; ++e) {
    auto G = [&](int q, int c) { return geo[((int64_t)q * FP + e) * S_NPE + c]; };
    const double s0 = G(0, 0), s1 = G(4, 0), s2 = G(8, 0);
    const double v0 = G(9, 0) / (gw[0] * gw[0] * gw3[0]);
    const double scale = std::fabs(s0) + std::fabs(s1) + std::fabs(s2);
    for (int c = 0; c < S_NPE && box; ++c) {
      const int cx = c % NP, cy = (c / NP) % NP, cz = c / 36;
      for (int q = 0; q < 9; ++q)
        if (q != 0 && q != 4 && q != 8 && std::fabs(G(q, c)) > 1e-12 * scale) box = false;
      if (std::fabs(G(0, c) - s0) > 1e-10 * std::fabs(s0) || std::fabs(G(4, c) - s1) > 1e-10 * std::fabs(s1) ||
          std::fabs(G(8, c) - s2) > 1e-10 * std::fabs(s2))
        box = false;
      const double v = G(9, c) / (gw[cx] * gw[cy] * gw3[cz]);
      if (std::fabs(v - v0) > 1e-10 * std::fabs(v0)) box = false;
    }
    gbox[e] = s0;
    gbox[FP + e] = s1;
    gbox[2 * FP + e] = s2;
    gbox[3 * FP + e] = v0;
  }
  shm_status st = p->prec == 64 ? solid_device<double>(p, conn, geo, emat, ekeep, mat, minv, box ? &gbox : nullptr)
                                : solid_device<float>(p, conn, geo, emat, ekeep, mat, minv, box ? &gbox : nullptr);
  if (st != SHM_OK) return st;
  if ((st = upload(p, &p->row_ptr, row_ptr)) != SHM_OK) return st;
  if ((st = upload(p, &p->slots, slots)) != SHM_OK) return st;
  if ((st = upload(p, &p->fq_field, fq_field)) != SHM_OK) return st;
  if ((st = upload(p, &p->fq_scen, fq_scen)) != SHM_OK) return st;
  if ((st = upload(p, &p->fq_val, fq_val)) != SHM_OK) return st;
  if ((st = upload(p, &p->out_node, out_node)) != SHM_OK) return st;
  if ((st = upload(p, &p->out_field, out_field)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->st, (size_t)nscen * p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->displ, (size_t)std::max(p->nout, 1) * p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->vsum, (size_t)p->nft)) != SHM_OK) return st;  // cleared by shm_reset
  if ((st = dalloc(p, &p->volt, (size_t)p->nft)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->flag, 4)) != SHM_OK) return st;
  if ((st = dalloc(p, &p->d_base, 4)) != SHM_OK) return st;
  CKP(p, cudaDeviceSynchronize());
  return shm_reset(p);
}

shm_status shm::plan_frames_view(shm_plan* p, int scen, FramesView* v) {
  if (!p || !v || scen < 0 || scen >= p->nscen) return SHM_ERR_BAD_ARG;
  v->frames = p->frames;
  v->prec = p->prec;
  v->nnode_pad = p->nnode_pad;
  v->node0 = p->node_off[scen];
  v->nnode = p->node_off[scen + 1] - p->node_off[scen];
  v->nframes = p->nframes;
  v->nfields = p->nfields;
  for (int i = 0; i < 15; ++i) v->slot[i] = p->fspec.slot[i];
  v->device = p->device;
  v->kind = p->kind;
  v->ndof = p->nf;
  v->stream = (void*)p->stream;
  return SHM_OK;
}
