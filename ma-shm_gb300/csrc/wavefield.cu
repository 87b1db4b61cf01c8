// Wavefield frames on a uniform grid: the post-processing step
// spec2meshgrid_flat_shell.m (src/models/flat_shell/flat_shell_engine) that
// turns the solver's per-node frames into images Data(Ny, Nx, nFrames).
//
// Set-up (host, FP64, once per mesh and grid), following the reference:
//   grid points   xi = min(x)+Eps : L/(Nx-1) : max(x)-Eps with L = max-min-2 Eps,
//                 Eps = 1e-8, same in y; meshgrid order p = iy + Ny*ix   :56, :101-108
//   owner element candidates = elements whose corner bounding box holds the
//                 point; one candidate -> owner; else the first whose four
//                 edge cross products are all negative, else the first
//                 candidate                                              :140-183
//   local coords  (ksi0, eta0) of the nearest element node plus the inverse
//                 Jacobian of the element's first node times the offset, then
//                 3 Newton steps with the shape-function derivatives at the
//                 current estimate                                        :185-262
// The candidate search walks a uniform bin grid over the element bounding
// boxes instead of testing every element; each bin keeps its elements in
// ascending order, so "first" means the same element as in the reference.
// The reference's clamping of ksi/eta to [-1, 1] (:268-271) runs after the
// shape functions were evaluated and changes nothing; it is not applied.
//
// Per frame (device, k_grid): one thread per grid point, all frames in a loop;
// the owner's 36 node values of the requested motion (1..9, lever +-h/2 for
// the top/bottom surface, :281-510; the motion is a template parameter, the
// arithmetic the frames' precision) are combined with the tensor-product
// Lagrange weights l_i(ksi) l_j(eta), the functions shape2Dp.m evaluates
// through the inverse 2D Vandermonde matrix.  The top-surface rule
// U(nodes_under) = U(nodes_above) (:512-515) is a node remap baked into the
// grid's connectivity.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.h"
#include "shmsem.h"

namespace {

constexpr int NP = 6, NPE = 36;
constexpr double GRID_EPS = 1e-8;  // spec2meshgrid_flat_shell.m:56
constexpr int NEWTON_STEPS = 3;    // nIterations, :226
constexpr int GRID_THREADS = 256;

__constant__ double c_gx[NP];  // GLL nodes
__constant__ double c_lw[NP];  // 1 / prod_{m != i} (x_i - x_m)

struct Lagrange {
  double x[NP], inv[NP];
  void init(const std::vector<double>& gx) {
    for (int i = 0; i < NP; ++i) {
      x[i] = gx[i];
      double p = 1.0;
      for (int m = 0; m < NP; ++m)
        if (m != i) p *= (gx[i] - gx[m]);
      inv[i] = 1.0 / p;
    }
  }
  void eval(double t, double* l, double* dl) const {
    for (int i = 0; i < NP; ++i) {
      double p = 1.0;
      for (int m = 0; m < NP; ++m)
        if (m != i) p *= (t - x[m]);
      l[i] = p * inv[i];
      if (dl) {
        double s = 0.0;
        for (int q = 0; q < NP; ++q) {
          if (q == i) continue;
          double pq = 1.0;
          for (int m = 0; m < NP; ++m)
            if (m != i && m != q) pq *= (t - x[m]);
          s += pq;
        }
        dl[i] = s * inv[i];
      }
    }
  }
};

template <typename TC>
__device__ __forceinline__ void lagrange_dev(double t, TC* l) {
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double p = c_lw[i];
#pragma unroll
    for (int m = 0; m < NP; ++m)
      if (m != i) p *= (t - c_gx[m]);
    l[i] = (TC)p;
  }
}

// value of motion type M (1..9) at one node; o* are offsets of the field
// planes; hs = +h/2 (top) or -h/2 (bottom)
template <int M, typename TF, typename TC>
__device__ __forceinline__ TC motion_value(const TF* __restrict__ fr, int64_t node, int64_t oux, int64_t ofx,
                                           int64_t ouy, int64_t ofy, int64_t ouz, TC hs) {
  if constexpr (M == 1) return (TC)fr[oux + node];
  if constexpr (M == 2) return (TC)fr[ouy + node];
  if constexpr (M == 3) return (TC)fr[ouz + node];
  if constexpr (M == 4) return (TC)fr[ofx + node];
  if constexpr (M == 5) return (TC)fr[ofy + node];
  if constexpr (M == 6) return (TC)fr[oux + node] + hs * (TC)fr[ofx + node];
  if constexpr (M == 7) return (TC)fr[ouy + node] + hs * (TC)fr[ofy + node];
  if constexpr (M == 8) {
    const TC a = (TC)fr[oux + node] + hs * (TC)fr[ofx + node];
    const TC b = (TC)fr[ouy + node] + hs * (TC)fr[ofy + node];
    return sqrt(a * a + b * b);
  }
  if constexpr (M == 9) {
    const TC a = (TC)fr[oux + node] + hs * (TC)fr[ofx + node];
    const TC b = (TC)fr[ouy + node] + hs * (TC)fr[ofy + node];
    const TC c = (TC)fr[ouz + node];
    return sqrt(a * a + b * b + c * c);
  }
  return TC(0);
}

// Data[n][p] = sum_{j,i} l_j(eta_p) l_i(ksi_p) value(node(owner_p, j*6+i)) for
// every frame n; frames fr[n*frame_stride + field_offset + node].  TC is the
// arithmetic type: the frames' own precision (FP32 frames are combined in
// FP32, FP64 frames in FP64).
template <int M, typename TF, typename TC>
__global__ void __launch_bounds__(GRID_THREADS, 2) k_grid(const int* __restrict__ owner,
                                                        const double2* __restrict__ ke,
                                                        const int* __restrict__ conn, int fen_search, int64_t npts,
                                                        const TF* __restrict__ fr, int64_t frame_stride,
                                                        int64_t oux, int64_t ofx, int64_t ouy, int64_t ofy,
                                                        int64_t ouz, double hs, int nframes,
                                                        double* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int e = owner[p];
  const double2 q = ke[p];
  TC lx[NP], ly[NP];
  lagrange_dev(q.x, lx);
  lagrange_dev(q.y, ly);
  int nid[NPE];
#pragma unroll
  for (int k = 0; k < NPE; ++k) nid[k] = conn[(int64_t)k * fen_search + e];
  const TC hsc = (TC)hs;
  for (int n = 0; n < nframes; ++n) {
    const TF* f = fr + (int64_t)n * frame_stride;
    TC acc = TC(0);
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      TC row = TC(0);
#pragma unroll
      for (int i = 0; i < NP; ++i)
        row += lx[i] * motion_value<M, TF, TC>(f, nid[j * NP + i], oux, ofx, ouy, ofy, ouz, hsc);
      acc += ly[j] * row;
    }
    out[(int64_t)n * npts + p] = (double)acc;
  }
}

bool motion_needs(int m, int dof) {
  // dof order u, phi_x, v, phi_y, w
  static const int need[10][5] = {{0, 0, 0, 0, 0}, {1, 0, 0, 0, 0}, {0, 0, 1, 0, 0}, {0, 0, 0, 0, 1},
                                  {0, 1, 0, 0, 0}, {0, 0, 0, 1, 0}, {1, 1, 0, 0, 0}, {0, 0, 1, 1, 0},
                                  {1, 1, 1, 1, 0}, {1, 1, 1, 1, 1}};
  return need[m][dof] != 0;
}

}  // namespace

struct shm_grid {
  std::string err;
  int device = 0, nx = 0, ny = 0, fen_search = 0, nnode = 0;
  int64_t npts = 0;
  std::vector<double> xp, yp, ksi, eta;
  std::vector<int> owner;
  double max_err = 0.0;
  cudaStream_t stream = nullptr;
  int* d_owner = nullptr;
  double2* d_ke = nullptr;
  int* d_conn = nullptr;
};

static shm_status grid_fail(shm_grid* g, const std::string& m, shm_status s = SHM_ERR_BAD_ARG) {
  if (g) g->err = m;
  return s;
}

#define GCK(g, call)                                                                     \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      (g)->err = std::string(#call ": ") + cudaGetErrorString(e_);                       \
      return (e_ == cudaErrorMemoryAllocation) ? SHM_ERR_OOM : SHM_ERR_CUDA;             \
    }                                                                                    \
  } while (0)

static void grid_free(shm_grid* g) {
  if (g->d_owner) cudaFree(g->d_owner);
  if (g->d_ke) cudaFree(g->d_ke);
  if (g->d_conn) cudaFree(g->d_conn);
  if (g->stream) cudaStreamDestroy(g->stream);
  g->d_owner = nullptr;
  g->d_ke = nullptr;
  g->d_conn = nullptr;
  g->stream = nullptr;
}

// Host set-up: grid points, owner elements, local coordinates.
static shm_status grid_setup(shm_grid* g, const shm_mesh& m, const int32_t* remap, std::vector<int>& conn) {
  const int fen = m.fen, fs = g->fen_search, nnode = m.nnode;
  auto X = [&](int node1) { return m.coords[node1 - 1]; };
  auto Y = [&](int node1) { return m.coords[(int64_t)nnode + node1 - 1]; };
  auto NODE = [&](int e, int c) { return m.nodes[(int64_t)c * fen + e]; };
  // grid points (:101-108)
  double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  for (int n = 1; n <= nnode; ++n) {
    xmin = std::min(xmin, X(n));
    xmax = std::max(xmax, X(n));
    ymin = std::min(ymin, Y(n));
    ymax = std::max(ymax, Y(n));
  }
  const double L = xmax - xmin - 2 * GRID_EPS, B = ymax - ymin - 2 * GRID_EPS;
  const double sx = L / (g->nx - 1), sy = B / (g->ny - 1);
  g->npts = (int64_t)g->nx * g->ny;
  g->xp.resize(g->npts);
  g->yp.resize(g->npts);
  for (int ix = 0; ix < g->nx; ++ix)
    for (int iy = 0; iy < g->ny; ++iy) {
      const int64_t p = iy + (int64_t)g->ny * ix;
      g->xp[p] = (xmin + GRID_EPS) + ix * sx;
      g->yp[p] = (ymin + GRID_EPS) + iy * sy;
    }
  // element corners in the order mc = [1, n, n^2, n^2-n+1] (counter-clockwise)
  const int mc[4] = {0, NP - 1, NPE - 1, NPE - NP};
  std::vector<double> cx(4 * (size_t)fs), cy(4 * (size_t)fs), bb(4 * (size_t)fs);
  for (int e = 0; e < fs; ++e) {
    double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    for (int c = 0; c < 4; ++c) {
      const int n1 = NODE(e, mc[c]);
      cx[4 * (size_t)e + c] = X(n1);
      cy[4 * (size_t)e + c] = Y(n1);
      x0 = std::min(x0, X(n1));
      x1 = std::max(x1, X(n1));
      y0 = std::min(y0, Y(n1));
      y1 = std::max(y1, Y(n1));
    }
    bb[4 * (size_t)e + 0] = x0;
    bb[4 * (size_t)e + 1] = x1;
    bb[4 * (size_t)e + 2] = y0;
    bb[4 * (size_t)e + 3] = y1;
  }
  // bins over the element bounding boxes
  const int nb = std::max(1, (int)std::sqrt((double)fs));
  const double bw = (xmax > xmin) ? (xmax - xmin) / nb : 1.0, bh = (ymax > ymin) ? (ymax - ymin) / nb : 1.0;
  auto bin_x = [&](double x) { return std::min(nb - 1, std::max(0, (int)std::floor((x - xmin) / bw))); };
  auto bin_y = [&](double y) { return std::min(nb - 1, std::max(0, (int)std::floor((y - ymin) / bh))); };
  std::vector<int> bptr((size_t)nb * nb + 1, 0), bel;
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int> fill(bptr.begin(), bptr.end() - 1);
    for (int e = 0; e < fs; ++e) {
      const int i0 = bin_x(bb[4 * (size_t)e]), i1 = bin_x(bb[4 * (size_t)e + 1]);
      const int j0 = bin_y(bb[4 * (size_t)e + 2]), j1 = bin_y(bb[4 * (size_t)e + 3]);
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
          const size_t b = (size_t)j * nb + i;
          if (pass == 0)
            ++bptr[b + 1];
          else
            bel[fill[b]++] = e;
        }
    }
    if (pass == 0) {
      for (size_t b = 0; b < (size_t)nb * nb; ++b) bptr[b + 1] += bptr[b];
      bel.assign(bptr.back(), 0);
    }
  }
  // owner elements (:140-183)
  g->owner.assign(g->npts, -1);
  std::vector<int> cand;
  for (int64_t p = 0; p < g->npts; ++p) {
    const double xp = g->xp[p], yp = g->yp[p];
    const size_t b = (size_t)bin_y(yp) * nb + bin_x(xp);
    cand.clear();
    for (int q = bptr[b]; q < bptr[b + 1]; ++q) {
      const int e = bel[q];
      const double* B4 = &bb[4 * (size_t)e];
      if (xp >= B4[0] && xp <= B4[1] && yp >= B4[2] && yp <= B4[3]) cand.push_back(e);
    }
    if (cand.empty()) return grid_fail(g, "grid point outside every element's bounding box");
    if (cand.size() == 1) {
      g->owner[p] = cand[0];
      continue;
    }
    int own = cand[0];
    for (int e : cand) {
      const double* x = &cx[4 * (size_t)e];
      const double* y = &cy[4 * (size_t)e];
      const double x21 = x[1] - x[0], x32 = x[2] - x[1], x43 = x[3] - x[2], x14 = x[0] - x[3];
      const double y21 = y[1] - y[0], y32 = y[2] - y[1], y43 = y[3] - y[2], y14 = y[0] - y[3];
      const double d1 = (xp * y21 - x[0] * y21) - (yp * x21 - y[0] * x21);
      const double d2 = (xp * y32 - x[1] * y32) - (yp * x32 - y[1] * x32);
      const double d3 = (xp * y43 - x[2] * y43) - (yp * x43 - y[2] * x43);
      const double d4 = (xp * y14 - x[3] * y14) - (yp * x14 - y[3] * x14);
      if (d1 < 0 && d2 < 0 && d3 < 0 && d4 < 0) {
        own = e;
        break;
      }
    }
    g->owner[p] = own;
  }
  // local coordinates (:185-262)
  std::vector<double> gx, gw, D;
  shm::gll_setup(NP, gx, gw, D);
  Lagrange lag;
  lag.init(gx);
  g->ksi.resize(g->npts);
  g->eta.resize(g->npts);
  g->max_err = 0.0;
  for (int64_t p = 0; p < g->npts; ++p) {
    const int e = g->owner[p];
    const double xp = g->xp[p], yp = g->yp[p];
    double xe[NPE], ye[NPE];
    for (int k = 0; k < NPE; ++k) {
      xe[k] = X(NODE(e, k));
      ye[k] = Y(NODE(e, k));
    }
    int kmin = 0;
    double dmin = INFINITY;
    for (int k = 0; k < NPE; ++k) {
      const double d = std::sqrt((xe[k] - xp) * (xe[k] - xp) + (ye[k] - yp) * (ye[k] - yp));
      if (d < dmin) {
        dmin = d;
        kmin = k;
      }
    }
    double x0 = xe[kmin], y0 = ye[kmin];
    double ks0 = gx[kmin % NP], et0 = gx[kmin / NP];
    // Jacobian at the element's first local node: xi-derivative along its
    // row (I (x) D), eta-derivative along its column (D (x) I)
    double J11 = 0, J21 = 0, J12 = 0, J22 = 0;
    for (int i = 0; i < NP; ++i) {
      J11 += D[i] * xe[i];
      J21 += D[i] * ye[i];
      J12 += D[i] * xe[i * NP];
      J22 += D[i] * ye[i * NP];
    }
    double a = 1.0 / (J11 * J22 - J12 * J21);
    double ks = ks0 + (a * J22) * (xp - x0) + (a * -J12) * (yp - y0);
    double et = et0 + (a * -J21) * (xp - x0) + (a * J11) * (yp - y0);
    double lx[NP], ly[NP], dlx[NP], dly[NP];
    auto interp = [&](double s, double t, double& xo, double& yo) {
      lag.eval(s, lx, nullptr);
      lag.eval(t, ly, nullptr);
      xo = 0.0;
      yo = 0.0;
      for (int j = 0; j < NP; ++j)
        for (int i = 0; i < NP; ++i) {
          const double N = lx[i] * ly[j];
          xo += N * xe[j * NP + i];
          yo += N * ye[j * NP + i];
        }
    };
    double x1, y1;
    interp(ks, et, x1, y1);
    for (int it = 0; it < NEWTON_STEPS; ++it) {
      ks0 = ks;
      et0 = et;
      x0 = x1;
      y0 = y1;
      lag.eval(ks0, lx, dlx);
      lag.eval(et0, ly, dly);
      J11 = J12 = J21 = J22 = 0.0;
      for (int j = 0; j < NP; ++j)
        for (int i = 0; i < NP; ++i) {
          const double Nx = dlx[i] * ly[j], Ny = lx[i] * dly[j];
          J11 += Nx * xe[j * NP + i];
          J12 += Ny * xe[j * NP + i];
          J21 += Nx * ye[j * NP + i];
          J22 += Ny * ye[j * NP + i];
        }
      a = 1.0 / (J11 * J22 - J12 * J21);
      ks = ks0 + (a * J22) * (xp - x0) + (a * -J12) * (yp - y0);
      et = et0 + (a * -J21) * (xp - x0) + (a * J11) * (yp - y0);
      interp(ks, et, x1, y1);
    }
    g->ksi[p] = ks;
    g->eta[p] = et;
    g->max_err = std::max(g->max_err, std::sqrt((xp - x1) * (xp - x1) + (yp - y1) * (yp - y1)));
  }
  // connectivity of the searched elements, [36][fen_search], 0-based, remapped
  conn.resize((size_t)NPE * fs);
  for (int k = 0; k < NPE; ++k)
    for (int e = 0; e < fs; ++e) {
      int n1 = NODE(e, k);
      if (remap) n1 = remap[n1 - 1];
      conn[(size_t)k * fs + e] = n1 - 1;
    }
  return SHM_OK;
}

extern "C" shm_status shm_grid_create(const shm_mesh* mesh, int32_t fen_search, const int32_t* remap, int32_t nx,
                                      int32_t ny, int32_t device, shm_grid** out) {
  if (!out) return SHM_ERR_BAD_ARG;
  *out = nullptr;
  if (!mesh || !mesh->nodes || !mesh->coords || mesh->npe != NPE || mesh->fen < 1 || mesh->nnode < 1 || nx < 2 ||
      ny < 2 || fen_search < 1 || fen_search > mesh->fen)
    return SHM_ERR_BAD_ARG;
  for (int64_t i = 0; i < (int64_t)mesh->fen * NPE; ++i)
    if (mesh->nodes[i] < 1 || mesh->nodes[i] > mesh->nnode) return SHM_ERR_BAD_ARG;
  if (remap)
    for (int i = 0; i < mesh->nnode; ++i)
      if (remap[i] < 1 || remap[i] > mesh->nnode) return SHM_ERR_BAD_ARG;
  shm_grid* g = new shm_grid();
  *out = g;
  g->device = device;
  g->nx = nx;
  g->ny = ny;
  g->fen_search = fen_search;
  g->nnode = mesh->nnode;
  std::vector<int> conn;
  shm_status s = grid_setup(g, *mesh, remap, conn);
  if (s != SHM_OK) return s;
  if (device < 0) return SHM_OK;  // set-up only (no device copy; interpolation refused)
  GCK(g, cudaSetDevice(device));
  std::vector<double> gx, gw, D;
  shm::gll_setup(NP, gx, gw, D);
  Lagrange lag;
  lag.init(gx);
  GCK(g, cudaMemcpyToSymbol(c_gx, gx.data(), sizeof(double) * NP));
  GCK(g, cudaMemcpyToSymbol(c_lw, lag.inv, sizeof(double) * NP));
  GCK(g, cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  GCK(g, cudaMalloc(&g->d_owner, sizeof(int) * g->npts));
  GCK(g, cudaMalloc(&g->d_ke, sizeof(double2) * g->npts));
  GCK(g, cudaMalloc(&g->d_conn, sizeof(int) * conn.size()));
  std::vector<double2> ke(g->npts);
  for (int64_t p = 0; p < g->npts; ++p) ke[p] = make_double2(g->ksi[p], g->eta[p]);
  GCK(g, cudaMemcpy(g->d_owner, g->owner.data(), sizeof(int) * g->npts, cudaMemcpyHostToDevice));
  GCK(g, cudaMemcpy(g->d_ke, ke.data(), sizeof(double2) * g->npts, cudaMemcpyHostToDevice));
  GCK(g, cudaMemcpy(g->d_conn, conn.data(), sizeof(int) * conn.size(), cudaMemcpyHostToDevice));
  return SHM_OK;
}

extern "C" shm_status shm_grid_destroy(shm_grid* g) {
  if (!g) return SHM_OK;
  grid_free(g);
  delete g;
  return SHM_OK;
}

extern "C" const char* shm_grid_last_error(const shm_grid* g) { return g ? g->err.c_str() : "null grid"; }

extern "C" shm_status shm_grid_points(const shm_grid* g, double* xp, double* yp, int32_t* owner, double* ksi,
                                      double* eta, double* max_err) {
  if (!g) return SHM_ERR_BAD_ARG;
  for (int64_t p = 0; p < g->npts; ++p) {
    if (xp) xp[p] = g->xp[p];
    if (yp) yp[p] = g->yp[p];
    if (owner) owner[p] = g->owner[p];
    if (ksi) ksi[p] = g->ksi[p];
    if (eta) eta[p] = g->eta[p];
  }
  if (max_err) *max_err = g->max_err;
  return SHM_OK;
}

template <int M, typename TF>
static void launch_grid_m(shm_grid* g, const TF* fr, int64_t frame_stride, const int64_t off[5], double hs,
                          int nframes, double* d_out, cudaStream_t s) {
  const int64_t nblk = (g->npts + GRID_THREADS - 1) / GRID_THREADS;
  k_grid<M, TF, TF><<<(unsigned)nblk, GRID_THREADS, 0, s>>>(g->d_owner, g->d_ke, g->d_conn, g->fen_search,
                                                            g->npts, fr, frame_stride, off[0], off[1], off[2],
                                                            off[3], off[4], hs, nframes, d_out);
}

template <typename TF>
static shm_status launch_grid(shm_grid* g, const TF* fr, int64_t frame_stride, const int64_t off[5], int motion,
                              double hs, int nframes, double* d_out, cudaStream_t s) {
  if (nframes <= 0) return SHM_OK;
  switch (motion) {
    case 1: launch_grid_m<1>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 2: launch_grid_m<2>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 3: launch_grid_m<3>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 4: launch_grid_m<4>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 5: launch_grid_m<5>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 6: launch_grid_m<6>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 7: launch_grid_m<7>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    case 8: launch_grid_m<8>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
    default: launch_grid_m<9>(g, fr, frame_stride, off, hs, nframes, d_out, s); break;
  }
  GCK(g, cudaGetLastError());
  return SHM_OK;
}

static shm_status check_motion(shm_grid* g, int motion, int surface, const int32_t* dof_field, int nfields) {
  if (!g->d_owner) return grid_fail(g, "grid was created without a device", SHM_ERR_STATE);
  if (motion < 1 || motion > 9) return grid_fail(g, "motion must be 1..9");
  if (surface != 0 && surface != 1) return grid_fail(g, "surface must be 0 (top) or 1 (bottom)");
  for (int d = 0; d < 5; ++d)
    if (motion_needs(motion, d) && (dof_field[d] < 0 || dof_field[d] >= nfields))
      return grid_fail(g, "a DOF component the motion needs is not among the frame fields");
  return SHM_OK;
}

extern "C" shm_status shm_grid_interpolate(shm_grid* g, const double* frames, int32_t nframes, int32_t nfields,
                                           const int32_t* dof_field, int32_t motion, int32_t surface, double h,
                                           double* data, void* stream) {
  if (!g || !frames || !dof_field || !data || nframes < 0 || nfields < 1) return SHM_ERR_BAD_ARG;
  shm_status st = check_motion(g, motion, surface, dof_field, nfields);
  if (st != SHM_OK) return st;
  GCK(g, cudaSetDevice(g->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
  const int64_t fsz = (int64_t)nfields * g->nnode;  // doubles per frame
  // frames in chunks of at most ~1 GiB of input
  const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(nframes, (int64_t(1) << 27) / std::max<int64_t>(fsz, 1)));
  double *d_in = nullptr, *d_out = nullptr;
  GCK(g, cudaMalloc(&d_in, sizeof(double) * fsz * std::max(chunk, 1)));
  cudaError_t ea = cudaMalloc(&d_out, sizeof(double) * g->npts * std::max(chunk, 1));
  if (ea != cudaSuccess) {
    cudaFree(d_in);
    return grid_fail(g, "cudaMalloc failed", SHM_ERR_OOM);
  }
  int64_t off[5];
  for (int d = 0; d < 5; ++d) off[d] = (int64_t)std::max(dof_field[d], 0) * g->nnode;
  const double hs = (surface == 0 ? 0.5 : -0.5) * h;
  for (int n0 = 0; n0 < nframes && st == SHM_OK; n0 += chunk) {
    const int nc = std::min(chunk, nframes - n0);
    cudaError_t e = cudaMemcpyAsync(d_in, frames + (int64_t)n0 * fsz, sizeof(double) * fsz * nc,
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) st = grid_fail(g, cudaGetErrorString(e), SHM_ERR_CUDA);
    if (st == SHM_OK) st = launch_grid<double>(g, d_in, fsz, off, motion, hs, nc, d_out, s);
    if (st == SHM_OK) {
      e = cudaMemcpyAsync(data + (int64_t)n0 * g->npts, d_out, sizeof(double) * g->npts * nc,
                          cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) st = grid_fail(g, cudaGetErrorString(e), SHM_ERR_CUDA);
    }
  }
  cudaFree(d_in);
  cudaFree(d_out);
  return st;
}

extern "C" shm_status shm_grid_interpolate_plan(shm_grid* g, shm_plan* plan, int32_t scen, int32_t kind,
                                                int32_t motion, int32_t surface, double h, double* data,
                                                void* stream) {
  if (!g || !plan || !data) return SHM_ERR_BAD_ARG;
  shm::FramesView v;
  if (shm::plan_frames_view(plan, scen, &v) != SHM_OK) return grid_fail(g, "no such scenario in the plan");
  if (v.kind != 0) return grid_fail(g, "wavefield grids are for flat-shell plans", SHM_ERR_UNSUPPORTED);
  if (v.nnode != g->nnode) return grid_fail(g, "the grid's mesh and the scenario's differ in node count");
  if (v.nframes <= 0 || !v.frames) return grid_fail(g, "the plan records no frames", SHM_ERR_STATE);
  if (kind < 0 || kind > 2) return grid_fail(g, "kind must be 0 (velocity), 1 (displacement) or 2 (acceleration)");
  static const int kind_of[3] = {1, 0, 2};
  int32_t dof_field[5];
  for (int d = 0; d < 5; ++d) dof_field[d] = v.slot[kind_of[kind] * 5 + d];
  shm_status st = check_motion(g, motion, surface, dof_field, v.nfields);
  if (st != SHM_OK) return st;
  GCK(g, cudaSetDevice(g->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : (cudaStream_t)v.stream;
  double* d_out = nullptr;
  GCK(g, cudaMalloc(&d_out, sizeof(double) * g->npts * v.nframes));
  int64_t off[5];
  for (int d = 0; d < 5; ++d) off[d] = (int64_t)std::max(dof_field[d], 0) * v.nnode_pad + v.node0;
  const double hs = (surface == 0 ? 0.5 : -0.5) * h;
  const int64_t fstride = (int64_t)v.nfields * v.nnode_pad;
  if (v.prec == 64)
    st = launch_grid<double>(g, (const double*)v.frames, fstride, off, motion, hs, v.nframes, d_out, s);
  else
    st = launch_grid<float>(g, (const float*)v.frames, fstride, off, motion, hs, v.nframes, d_out, s);
  if (st == SHM_OK) {
    cudaError_t e = cudaMemcpyAsync(data, d_out, sizeof(double) * g->npts * v.nframes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = grid_fail(g, cudaGetErrorString(e), SHM_ERR_CUDA);
  }
  cudaFree(d_out);
  return st;
}

extern "C" shm_status shm_grid_time(shm_grid* g, shm_plan* plan, int32_t scen, int32_t kind, int32_t motion,
                                    int32_t surface, double h, int32_t reps, float* ms) {
  // device time of `reps` interpolations of all the plan's frames (CUDA events
  // on the plan's stream, output kept on the device)
  if (!g || !plan || !ms || reps < 1) return SHM_ERR_BAD_ARG;
  shm::FramesView v;
  if (shm::plan_frames_view(plan, scen, &v) != SHM_OK || v.kind != 0 || v.nnode != g->nnode || v.nframes <= 0)
    return grid_fail(g, "plan frames unusable for this grid");
  static const int kind_of[3] = {1, 0, 2};
  if (kind < 0 || kind > 2) return SHM_ERR_BAD_ARG;
  int32_t dof_field[5];
  for (int d = 0; d < 5; ++d) dof_field[d] = v.slot[kind_of[kind] * 5 + d];
  shm_status st = check_motion(g, motion, surface, dof_field, v.nfields);
  if (st != SHM_OK) return st;
  GCK(g, cudaSetDevice(g->device));
  cudaStream_t s = (cudaStream_t)v.stream;
  double* d_out = nullptr;
  GCK(g, cudaMalloc(&d_out, sizeof(double) * g->npts * v.nframes));
  int64_t off[5];
  for (int d = 0; d < 5; ++d) off[d] = (int64_t)std::max(dof_field[d], 0) * v.nnode_pad + v.node0;
  const double hs = (surface == 0 ? 0.5 : -0.5) * h;
  const int64_t fstride = (int64_t)v.nfields * v.nnode_pad;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int r = 0; r <= reps && st == SHM_OK; ++r) {
    if (r == 1) cudaEventRecord(e0, s);
    st = v.prec == 64 ? launch_grid<double>(g, (const double*)v.frames, fstride, off, motion, hs, v.nframes, d_out, s)
                      : launch_grid<float>(g, (const float*)v.frames, fstride, off, motion, hs, v.nframes, d_out, s);
  }
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  *ms = t / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_out);
  return st;
}
