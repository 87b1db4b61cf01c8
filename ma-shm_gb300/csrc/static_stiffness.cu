// static_stiffness.cu -- allocation-free internal-force entry point.
//
// shm_stiffness_static() computes the assembled flat-shell internal force
// F = K*U for a mesh whose arrays already live in device memory, without
// allocating anything: no cudaMalloc, no cudaFree, no library call that
// allocates.  It exists for callers that cannot allocate device memory on
// their own terms:
//   * a MATLAB MEX gateway working on gpuArray data owned by MATLAB's GPU
//     memory manager, which keeps a pool of the device memory and whose
//     accounting a hidden cudaMalloc would bypass (and can fail when MATLAB
//     has reserved most of the memory);
//   * monitoring loops that run for days on a fixed memory budget and forbid
//     any allocation after start-up, so that a run never dies on an
//     out-of-memory error half way.
// The element-local forces (the reference's F2, main_flat_shell.m:716-721)
// are kept in a file-scope device array of SHM_STATIC_MAX_ELEMS elements
// (5 x 36 doubles each, 5.9 MB), which every GPU that loads the library holds
// until the process exits.  The assembly is the reference's 12-basket scatter
// F(I_G(:,b)) += F2(I_L(:,b)), b = 1..12 (main_flat_shell.m:724-726), driven by
// the caller's I_G / I_L maps (nodesMaps_Fiborek.m), so the summation order is
// the reference's.
//
// Set-up: the first call on a device (with that device current) looks up the
// device address of the array with cudaGetSymbolAddress, copies the GLL
// derivative matrix to this file's constant memory and raises the kernel's
// shared-memory limit.  Make that first call before any stream capture.
// Every call uses the same array and leaves its contents behind; calls that
// overlap on the GPU (two streams at once) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "internal.h"
#include "shmsem.h"
#include "shell_element.cuh"

using namespace shm;

namespace {

__device__ __align__(256) double g_static_f2[(size_t)5 * NPE * SHM_STATIC_MAX_ELEMS];

constexpr int kMaxDevices = 64;
double* s_f2_addr[kMaxDevices] = {nullptr};
std::mutex s_setup_mutex;
thread_local std::string t_err;  // text of this thread's last failed call

// records which step failed; the error of a CUDA call made here is cleared so
// that it does not surface in the caller's next error check
shm_status fail(const char* stage, cudaError_t e, bool clear) {
  if (clear) cudaGetLastError();
  t_err = std::string("shm_stiffness_static: ") + stage + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? SHM_ERR_OOM : SHM_ERR_CUDA;
}

constexpr int kGeoStride = 4 * NPE + 1;  // X, Y, dX/dxi, dY/dxi per element (odd stride)

size_t static_smem_bytes() {
  return sizeof(double) * (2 * CTA_ELEMS * ELEM_STRIDE + CTA_ELEMS * kGeoStride);
}

// geometry of the six nodes of one element column, computed in phase B
struct GeoLocal {
  static constexpr bool kAffineRect = false;
  NodeGeo<double> g[NP];
  __device__ __forceinline__ NodeGeo<double> at(int, int k) const { return g[k]; }
};

__global__ void __launch_bounds__(CTA_THREADS) k_static_elem(int fen, int nnode, const int* __restrict__ nodes,
                                                             const double* __restrict__ coords,
                                                             const double* __restrict__ lam,
                                                             const double* __restrict__ U, double* f2) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double* sm = reinterpret_cast<double*>(smraw);
  const int j = threadIdx.x >> 5, le = threadIdx.x & 31;
  const int e = blockIdx.x * CTA_ELEMS + le;
  const bool valid = e < fen;
  double* xs = sm + le * ELEM_STRIDE;
  double* ys = sm + (CTA_ELEMS + le) * ELEM_STRIDE;
  double* gs = sm + 2 * CTA_ELEMS * ELEM_STRIDE + le * kGeoStride;
  // phase A: row j, values and xi-derivatives of the 5 fields and of x, y
  {
    double u[5][NP], X[NP], Y[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      int node = valid ? nodes[(int64_t)(j * NP + i) * fen + e] - 1 : -1;
      if (node < 0 || node >= nnode) node = -1;  // out-of-range entries read as zero
#pragma unroll
      for (int f = 0; f < 5; ++f) u[f][i] = node >= 0 ? U[5 * (int64_t)node + f] : 0.0;
      X[i] = node >= 0 ? coords[node] : 0.0;
      Y[i] = node >= 0 ? coords[(int64_t)nnode + node] : 0.0;
    }
    row_deriv_store(u, xs, ys, j);
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      double jx = 0.0, jy = 0.0;
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        jx = fma(Dm<double>(i, k), X[k], jx);
        jy = fma(Dm<double>(i, k), Y[k], jy);
      }
      gs[0 * NPE + i * NP + j] = X[i];
      gs[1 * NPE + i * NP + j] = Y[i];
      gs[2 * NPE + i * NP + j] = jx;  // J11 = dx/dxi
      gs[3 * NPE + i * NP + j] = jy;  // J21 = dy/dxi
    }
  }
  __syncthreads();
  // phase B: column i = j
  if (valid) {
    const int i = j;
    double v[5][NP];
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int k = 0; k < NP; ++k) v[f][k] = xs[f * NPE + i * NP + k];
    GeoLocal geo;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      double J12 = 0.0, J22 = 0.0;
#pragma unroll
      for (int m = 0; m < NP; ++m) {
        J12 = fma(Dm<double>(k, m), gs[0 * NPE + i * NP + m], J12);  // dx/deta
        J22 = fma(Dm<double>(k, m), gs[1 * NPE + i * NP + m], J22);  // dy/deta
      }
      const double J11 = gs[2 * NPE + i * NP + k], J21 = gs[3 * NPE + i * NP + k];
      const double det = J11 * J22 - J12 * J21;
      const double a = 1.0 / det;
      geo.g[k].i11 = a * J22;
      geo.g[k].i12 = -a * J12;
      geo.g[k].i21 = -a * J21;
      geo.g[k].i22 = a * J11;
      geo.g[k].W = Wg<double>(i) * Wg<double>(k) * det;
    }
    Lam<double> L;
    double* Lp = &L.a11;
#pragma unroll
    for (int q = 0; q < 21; ++q) Lp[q] = lam[(int64_t)q * fen + e];
    double Fe[5][NP];
    SensorConst<double> sc{0.0, 0.0, 0.0, 0.0};
    shell_column<double, GeoLocal, false>(v, ys, xs, i, L, geo, Fe, sc);
#pragma unroll
    for (int f = 0; f < 5; ++f)
#pragma unroll
      for (int m = 0; m < NP; ++m) ys[f * NPE + i * NP + m] = Fe[f][m];
  }
  __syncthreads();
  // phase C: element-local forces in the reference's F2 layout (5 per local node)
  if (valid) {
    double out[5][NP];
    row_transpose_apply(xs, ys, j, out);
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
      for (int f = 0; f < 5; ++f) f2[((int64_t)e * NPE + j * NP + i) * 5 + f] = out[f][i];
  }
}

__global__ void k_static_basket(int rows, int b, int nnode, int nlocal, const int* __restrict__ IG,
                                const int* __restrict__ IL, const double* __restrict__ f2, double* F) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int g = IG[(int64_t)b * rows + r];
  const int l = IL[(int64_t)b * rows + r];
  if (g < 1 || g > nnode || l < 1 || l > nlocal) return;  // empty slot (0) or out of range
#pragma unroll
  for (int f = 0; f < 5; ++f) F[5 * (int64_t)(g - 1) + f] += f2[5 * (int64_t)(l - 1) + f];
}

void gll6(double* D, double* w) {
  // GLL nodes of order 5 (Newton on P5'), weights 2/(30 P5(x)^2), and the
  // Lagrange derivative matrix by barycentric weights; |D| < 1e-12 -> 0
  const int n = NP, N = n - 1;
  double x[NP];
  x[0] = -1.0;
  x[N] = 1.0;
  auto leg = [N](double t, double& p, double& dp) {
    double p0 = 1.0, p1 = t;
    for (int k = 2; k <= N; ++k) {
      const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    p = p1;
    dp = N * (t * p1 - p0) / (t * t - 1.0);
  };
  for (int k = 1; k < N; ++k) {
    double t = -std::cos(M_PI * k / N);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      leg(t, p, dp);
      const double d2p = (2.0 * t * dp - N * (N + 1.0) * p) / (1.0 - t * t);
      const double step = dp / d2p;
      t -= step;
      if (std::fabs(step) < 1e-16) break;
    }
    x[k] = t;
  }
  for (int k = 0; k <= N / 2; ++k) {
    const double s = 0.5 * (x[N - k] - x[k]);
    x[k] = -s;
    x[N - k] = s;
  }
  for (int k = 0; k < n; ++k) {
    double p, dp;
    if (k == 0 || k == N) {
      p = (k == 0) ? -1.0 : 1.0;  // P5(+-1) = +-1
    } else {
      leg(x[k], p, dp);
    }
    w[k] = 2.0 / (N * (N + 1.0) * p * p);
  }
  double lam[NP];
  for (int j = 0; j < n; ++j) {
    lam[j] = 1.0;
    for (int k = 0; k < n; ++k)
      if (k != j) lam[j] /= (x[j] - x[k]);
  }
  for (int r = 0; r < n; ++r) {
    double diag = 0.0;
    for (int c = 0; c < n; ++c)
      if (c != r) {
        D[r * n + c] = (lam[c] / lam[r]) / (x[r] - x[c]);
        diag -= D[r * n + c];
      }
    D[r * n + r] = diag;
  }
  for (int q = 0; q < n * n; ++q)
    if (std::fabs(D[q]) < 1e-12) D[q] = 0.0;
}

// once per device, with the device current
shm_status setup_device(double** f2) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail("cudaGetDevice", e, true);
  if (dev < 0 || dev >= kMaxDevices) {
    t_err = "shm_stiffness_static: device ordinal beyond the library's table";
    return SHM_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(s_setup_mutex);
  if (s_f2_addr[dev] == nullptr) {
    void* ptr = nullptr;
    if ((e = cudaGetSymbolAddress(&ptr, g_static_f2)) != cudaSuccess) return fail("cudaGetSymbolAddress", e, true);
    if (ptr == nullptr) return fail("cudaGetSymbolAddress", cudaErrorInvalidSymbol, false);
    double D[NP * NP], w[NP];
    gll6(D, w);
    if ((e = cudaMemcpyToSymbol(c_D64, D, sizeof(D))) != cudaSuccess) return fail("cudaMemcpyToSymbol", e, true);
    if ((e = cudaMemcpyToSymbol(c_w64, w, sizeof(w))) != cudaSuccess) return fail("cudaMemcpyToSymbol", e, true);
    if ((e = cudaFuncSetAttribute(k_static_elem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)static_smem_bytes())) != cudaSuccess)
      return fail("cudaFuncSetAttribute", e, true);
    s_f2_addr[dev] = static_cast<double*>(ptr);
  }
  *f2 = s_f2_addr[dev];
  return SHM_OK;
}

}  // namespace

extern "C" shm_status shm_stiffness_static(int32_t fen, int32_t nnode, const int32_t* nodes, const double* coords,
                                           const double* lam, int32_t basket_rows, const int32_t* I_G,
                                           const int32_t* I_L, const double* U, double* F, void* stream) {
  if (fen < 1 || fen > SHM_STATIC_MAX_ELEMS || nnode < 1 || basket_rows < 1) {
    t_err = "shm_stiffness_static: fen must be 1..SHM_STATIC_MAX_ELEMS, nnode and basket_rows >= 1";
    return SHM_ERR_BAD_ARG;
  }
  if (!nodes || !coords || !lam || !I_G || !I_L || !U || !F) {
    t_err = "shm_stiffness_static: NULL array";
    return SHM_ERR_BAD_ARG;
  }
  // an error left pending by earlier work of the caller would be read back
  // as a failed launch below: report it before anything is queued (and leave
  // it pending for the caller's own check)
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) return fail("a CUDA error was already pending, nothing queued", e, false);
  double* f2 = nullptr;
  shm_status st = setup_device(&f2);
  if (st != SHM_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((e = cudaMemsetAsync(F, 0, sizeof(double) * 5 * (size_t)nnode, s)) != cudaSuccess)
    return fail("cudaMemsetAsync of F", e, true);
  const int nblk = (fen + CTA_ELEMS - 1) / CTA_ELEMS;
  k_static_elem<<<nblk, CTA_THREADS, static_smem_bytes(), s>>>(fen, nnode, nodes, coords, lam, U, f2);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("k_static_elem launch", e, false);
  const int tb = 256, nb = (basket_rows + tb - 1) / tb;
  for (int b = 0; b < 12; ++b) {
    k_static_basket<<<nb, tb, 0, s>>>(basket_rows, b, nnode, fen * NPE, I_G, I_L, f2, F);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail("k_static_basket launch", e, false);
  }
  t_err.clear();
  return SHM_OK;
}

const char* shm::static_last_error() { return t_err.empty() ? nullptr : t_err.c_str(); }
