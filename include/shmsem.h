/*
 * shmsem.h -- C ABI of the GB300 spectral-element guided-wave engine.
 *
 * The engine replaces the explicit central-difference loop of ma-shm's
 * MATLAB solvers (src/models/flat_shell/flat_shell_engine/main_flat_shell*.m,
 * MAIN LOOP main_flat_shell.m:651-920) behind a plain C interface: plain
 * pointers and sizes, MATLAB (column-major, 1-based) layouts at the boundary,
 * integer status codes, no exceptions, no CUDA or torch types.  A MEX gateway
 * (mexFunction) or a ctypes/cffi binding maps the solver's arguments onto
 * these calls.
 *
 * Ownership: the caller owns every host array it passes; the plan copies what
 * it needs at creation and owns all device memory.  One plan is not
 * re-entrant (one stream at a time); distinct plans may run concurrently.
 */
#ifndef SHMSEM_H
#define SHMSEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SHM_OK = 0,
  SHM_ERR_BAD_ARG = 1,     /* invalid argument (size, index, NULL pointer) */
  SHM_ERR_CUDA = 2,        /* a CUDA call failed; shm_last_error() has the text */
  SHM_ERR_DIVERGED = 3,    /* blow-up / non-finite guard (main_flat_shell.m:786-804) */
  SHM_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  SHM_ERR_OOM = 5,         /* device allocation failed */
  SHM_ERR_STATE = 6,       /* call out of order (e.g. outputs before a run) */
  SHM_ERR_UNSUPPORTED = 7  /* option combination not built */
} shm_status;

typedef struct shm_plan shm_plan;

/* Mesh of one scenario.  Replaces `load(meshfile)` (main_flat_shell.m:39):
 * nodes(fen, npe), coords(nnode, 3), and optionally the 12-basket maps I_G,
 * I_L produced by nodesMaps_Fiborek.m (when absent the library builds its
 * own).  grid_nex/grid_ney > 0 declare a structured rectangular plate whose
 * global nodes are numbered row by row (x fastest, see mesh.py); the library
 * verifies that before it uses its structured fused kernel. */
typedef struct {
  int32_t fen;             /* number of elements */
  int32_t npe;             /* nodes per element: 36 (order 5, 6x6 GLL) */
  int32_t nnode;           /* number of nodes */
  const int32_t *nodes;    /* [fen x npe] column-major, 1-based */
  const double *coords;    /* [nnode x 3] column-major (x, y, z) */
  int32_t basket_rows;     /* rows of I_G / I_L, 0 when not given */
  const int32_t *I_G;      /* [basket_rows x 12] column-major, 1-based, 0 = empty */
  const int32_t *I_L;      /* [basket_rows x 12] column-major, 1-based, 0 = empty */
  int32_t grid_nex;        /* structured plate: elements along x (0 = unstructured) */
  int32_t grid_ney;        /* structured plate: elements along y */
} shm_mesh;

/* Laminate of one scenario.  Replaces the outputs of composite_plate*.m
 * (m11, I11, a11..d66), which the reference expands per local node; here one
 * row per material plus a material index and a stiffness factor per element. */
#define SHM_MAT_STRIDE 23
typedef struct {
  int32_t nmat;
  const double *table;     /* [nmat x 23] row-major: a11 a12 a16 a22 a26 a66 a44 a45 a55
                              b11 b12 b16 b22 b26 b66 d11 d12 d16 d22 d26 d66 m11 I11 */
  const int32_t *elem_mat; /* [fen] 0-based material of each element, NULL = 0 */
  const double *elem_keep; /* [fen] stiffness factor 1 - d_e of each element, NULL = 1 */
} shm_material;

/* Run parameters of one scenario (input*.m fields and the solver's derived
 * vectors).  All scenarios of a batch must share dt, nft, nn_first, eta_*. */
typedef struct {
  double dt;               /* time step [s] (main_flat_shell.m:116) */
  int32_t nft;             /* number of signal samples */
  int32_t nn_first;        /* first loop index: 2 (main_flat_shell.m:651) or 1 (_multi_pzt_c.m:579) */
  double eta_xy;           /* in-plane mass-proportional damping (etad_xy) */
  double eta_z;            /* out-of-plane damping (etad_z) */
  int32_t n_force;         /* nonzeros of the excitation vector Fi / Fa */
  const int32_t *force_dof;  /* [n_force] 1-based global DOF, 5*(node-1)+{1..5} */
  const double *force_val;   /* [n_force] value multiplying st(nn) */
  int32_t n_out;           /* point outputs (main_flat_shell.m:752-764) */
  const int32_t *out_dof;  /* [n_out] 1-based global DOF */
  int32_t n_sens;          /* PZT sensors (main_flat_shell_multi_pzt_c.m:619-623) */
  const int32_t *sens_ptr; /* [n_sens+1] CSR offsets into sens_el */
  const int32_t *sens_el;  /* 0-based element numbers of each sensor */
  double pzt_thickness;    /* sensor constants: Volt = t/g33*(e31*(..)+e32*(..)) */
  double g33, e31, e32;
  double h;                /* laminate thickness h (voltage lever arm, blow-up guard 10*h) */
  int32_t frm_int;         /* frame interval in steps, 0 = no frames */
  int32_t frame_dof;       /* 0 = all DOF components, 1..5: one component (5 = w) */
  int32_t frame_kind;      /* field_variable: 0 velocity, 1 displacement, 2 acceleration,
                              3 all three (main_flat_shell.m:765-885) */
  /* Pressure loading (main_flat_shell_pressure_excit_c.m:64-82,616-632,705-730): nodal
   * pressure frames p(node, t_k), linear in time between the frames and 0 outside
   * (interp1 'linear', 0) at t(nn) = (nn-1)*dt, applied to w as the lumped load
   * p * sum of w_i w_j detJ over the node's element copies.  All scenarios of a
   * batch that carry pressure share the frame times. */
  int32_t n_pframes;       /* 0 = no pressure loading */
  const double *p_times;   /* [n_pframes] s, increasing */
  const double *p_nodal;   /* [n_pframes x nnode] row-major (frame after frame), Pa */
} shm_run;

typedef struct {
  int32_t precision;       /* 64 or 32 (state and element arithmetic) */
  int32_t path;            /* 0 auto, 1 general (element + node kernels), 2 structured fused,
                              3 structured fused with the generic (unpacked) FP32 kernel */
  int32_t steps_per_graph; /* CUDA-graph chunk length, 0 = plain launches */
  int32_t tile_elems;      /* structured path: elements per lane group (16/32), 0 = by lane use */
  int32_t device;          /* CUDA device ordinal */
  int32_t rows_per_block;  /* structured path: element rows per task, 0 = 16 */
} shm_options;

/* Creates a plan for `nscen` scenarios advanced together (one launch per
 * kernel per step covers all of them).  Replaces the set-up part of
 * main_flat_shell*.m (:35-650): geometry, mass, maps, device upload. */
shm_status shm_plan_create(int32_t nscen, const shm_mesh *meshes, const shm_material *mats,
                           const shm_run *runs, const shm_options *opt, shm_plan **out);
shm_status shm_plan_destroy(shm_plan *plan);
/* Text of the plan's last error.  With plan == NULL: the text of the calling
 * thread's last failed shm_stiffness_static call ("no plan" if none). */
const char *shm_last_error(const shm_plan *plan);

/* Whole forward solve, the MAIN LOOP (main_flat_shell.m:651-917).
 *   st      [nscen][nft]            excitation samples st(nn) (Hanning_signal.m)
 *   displ   [nscen][nft x n_out]    column-major per scenario (displ, :926)
 *   voltage [nscen][nft x n_sens]   column-major per scenario (voltage, :925)
 *   frames  [nscen][nframes][nfields][nnode] frame fields ({U,V,A}{x,Fix,y,Fiy,z}_frame<c>):
 *           kind-major (displacement, velocity, acceleration) then DOF order
 * Any output pointer may be NULL.  `stream` is a cudaStream_t or NULL. */
shm_status shm_forward(shm_plan *plan, const double *st, double *displ, double *voltage,
                       double *frames, void *stream);

/* Blow-up guard interval.  The reference checks for a non-finite state or
 * w > 10 h only at frame steps (main_flat_shell.m:786-804), so a run without
 * frames is never checked; the engine also checks every `steps` time steps
 * (default 100; 0 = at frame steps only).  A detected blow-up makes
 * shm_advance / shm_forward return SHM_ERR_DIVERGED. */
shm_status shm_set_guard_interval(shm_plan *plan, int32_t steps);

/* Frames are handed to the caller through two device and two pinned host
 * staging buffers of `values` FP64 values each (default 4 M = 32 MB each):
 * runs of frame rows (or parts of a row longer than a buffer) are packed and
 * widened on the device, copied to pinned memory and from there into the
 * caller's array while the next run is in flight.  Smaller buffers save
 * memory at the cost of more copies. */
shm_status shm_set_frame_staging(shm_plan *plan, int64_t values);

/* Fine-grained stepping used by forward/adjoint drivers and benchmarks. */
shm_status shm_reset(shm_plan *plan);                        /* zero state, nn = nn_first */
shm_status shm_set_signal(shm_plan *plan, const double *st, void *stream);
shm_status shm_advance(shm_plan *plan, int32_t nsteps, void *stream);
shm_status shm_read_outputs(shm_plan *plan, double *displ, double *voltage, double *frames,
                            void *stream);
/* Device time of `nsteps` steps (CUDA events on the plan's stream). */
shm_status shm_time_steps(shm_plan *plan, int32_t nsteps, float *ms);

/* State in the reference's DOF layout: [total_nodes x 5] interleaved
 * (u, phi_x, v, phi_y, w per node), scenarios concatenated. */
shm_status shm_get_state(shm_plan *plan, double *U, double *uold);
shm_status shm_set_state(shm_plan *plan, const double *U, const double *uold, int32_t nn);

/* Assembled internal force K*U for a given state (same layout), no update. */
shm_status shm_apply_stiffness(shm_plan *plan, const double *U, double *F);

/* Plan facts: [0] total nodes, [1] total elements, [2] total DOF, [3] path
 * used (1 general, 2 structured), [4] precision, [5] frames per scenario,
 * [6] kernel launches per step (0: persistent, one launch per advance), [7] tile
 * elements (structured), [8] rows per task,
 * [9] fields per frame. */
shm_status shm_plan_info(const shm_plan *plan, int64_t *info10);

/* 3D solid (src/models/solid3D/main_spec3Dcuda_global_cpu_gpu3_wave_sens_opt_single_PCT_mat.m):
 * hexahedral spectral elements of 6 x 6 x 3 nodes, 3 DOF per node (u, v, w;
 * DOF 3*(node-1)+{1,2,3}).  nodes [fen x 108] column-major, 1-based, local
 * order x fastest, then y, then z (shape3D_prim_v2.m, extrude_mesh.m). */
typedef struct {
  int32_t fen, npe, nnode;
  const int32_t *nodes;    /* [fen x 108] column-major, 1-based */
  const double *coords;    /* [nnode x 3] column-major */
  int32_t basket_rows;
  const int32_t *I_G, *I_L;
} shm_solid_mesh;

/* material rows: D11 D12 D13 D14 D22 D23 D24 D33 D34 D44 D55 D56 D66 rho
 * (stresses_spec_p.m, Voigt order xx yy zz xy yz xz). */
#define SHM_SOLID_MAT_STRIDE 14
typedef struct {
  int32_t nmat;
  const double *table;     /* [nmat x 14] row-major */
  const int32_t *elem_mat; /* [fen] 0-based, NULL = 0 */
  const double *elem_keep; /* [fen] stiffness factor, NULL = 1 */
} shm_solid_material;

/* Creates a 3D-solid plan; shm_forward, shm_reset, shm_set_signal,
 * shm_advance, shm_read_outputs, shm_time_steps, shm_get_state (3 values per
 * node), shm_set_state, shm_mass and shm_plan_destroy accept it.  shm_run's
 * force_dof/out_dof use the 3-DOF numbering, frame_dof is 0 (all) or 1..3, PZT sensor
 * fields are ignored. */
shm_status shm_solid_plan_create(int32_t nscen, const shm_solid_mesh *meshes, const shm_solid_material *mats,
                                 const shm_run *runs, const shm_options *opt, shm_plan **out);

/* Discrete adjoint of the whole forward solve (no counterpart in the
 * reference, which has no gradients).  Misfit per scenario
 *   J = 1/2 sum_q sum_{nn=nn_first..nft} (displ(nn,q) - target(nn,q))^2
 * with displ as in shm_forward; grad[e] = dJ/dd_e for every element of every
 * scenario (concatenated), where the element stiffness is (1 - d_e) K_e^0, i.e.
 * d_e = 1 - elem_keep.  The forward pass keeps (u_n, u_{n-1}) every
 * `ckpt_every` steps, each segment is recomputed forward and the adjoint
 * lambda is stepped back through it with the same element operator; misfit
 * and gradient are accumulated in FP64.  Runs the plan's own kernels: the
 * fused structured adjoint step on structured FP32 plans, the general element
 * and node kernels otherwise.
 *   target [nscen][nft x n_out] column-major per scenario, like displ;
 *   misfit [nscen]; grad [total elements]. */
shm_status shm_forward_backward(shm_plan *plan, const double *st, const double *target, double *misfit,
                                double *grad, int32_t ckpt_every, void *stream);
/* Device time (ms, CUDA events) of the last shm_forward_backward's phases:
 * [0] forward pass with checkpoints, [1] segment recomputes, [2] adjoint steps. */
shm_status shm_forward_backward_timing(const shm_plan *plan, float *ms3);
/* Device memory that shm_forward_backward may use to keep every state of the
 * last checkpoint segments of the forward pass (those segments are not
 * recomputed): max_bytes > 0 = at most that many bytes, 0 = recompute every
 * segment, -3 = half of the device's free memory at the call (default),
 * -1 = the device's free memory less 8 GiB (opt-in: leaves little to other
 * users of the GPU, e.g. a MATLAB gpuArray pool); other negative values
 * leave the setting unchanged.  last_segments (may be NULL) receives the
 * number of segments the last call kept. */
shm_status shm_set_adjoint_store(shm_plan *plan, int64_t max_bytes, int32_t *last_segments);

/* Autotuner for plans on the structured path: times `steps` steps of the
 * general kernels and of every (elements per lane group, element rows per
 * task) candidate of the structured kernel -- {16, 32} x {4, 8, 16, 32, 64,
 * and per width the fewest rows that keep all tasks within one and within
 * two waves of two CTAs per SM} -- re-planning the task list each time, keeps
 * the fastest and resets the state.  On FP32 plans each structured candidate
 * is timed both as graph-chunked launches and as a persistent launch
 * (shm_set_persistent); the faster mode is kept (shm_plan_info [6] = 0 when
 * persistent).  Returns the choice (tile_elems = 0: general kernels) and its
 * ms per step. */
shm_status shm_autotune(shm_plan *plan, int32_t steps, int32_t *tile_elems, int32_t *rows_per_block,
                        float *ms_per_step);

/* Persistent stepping.  The reference launches its gpuArray operations one
 * by one for every step (main_flat_shell.m:651-917); by default the engine
 * launches one fused kernel per step, chunked into CUDA graphs.  With
 * enable = 1 an FP32 plan on the structured fused kernel advances all the
 * steps of an shm_advance / shm_forward call in ONE cooperative launch whose
 * CTAs stay resident and meet at a device-wide barrier between steps (the
 * grid is at most the number of co-resident CTAs; each CTA takes the same
 * task groups every step).  This removes the per-step launch gap that
 * dominates small plates.  Results are bit-identical to the per-step
 * launches.  spin_limit bounds each barrier wait (polls of ~32 ns; < 0 =
 * default 2^22): a wait that runs out makes every CTA leave at its next
 * barrier and the call return SHM_ERR_TIMEOUT.  Returns SHM_ERR_BAD_ARG for a
 * plan that is not FP32 structured, SHM_ERR_UNSUPPORTED when the device has
 * no cooperative launch.  enable = 0 restores per-step launches. */
shm_status shm_set_persistent(shm_plan *plan, int32_t enable, int32_t spin_limit);

/* Diagonal mass vector of the plan (reference mg before scaling, :493-501),
 * [total_nodes x 5] interleaved. */
shm_status shm_mass(shm_plan *plan, double *mg);

/* Allocation-free internal force.  No counterpart in the reference: it is the
 * element step (gather, K_e*u_e) plus the reference's 12-basket assembly,
 * exposed for callers that must not allocate device memory -- a MEX gateway
 * whose gpuArray memory belongs to MATLAB's GPU memory manager, or a
 * long-running monitoring loop on a fixed memory budget.  Every pointer is a
 * DEVICE pointer owned by the caller:
 *   nodes  [fen x 36] column-major, 1-based (mesh `nodes`)
 *   coords [nnode x 3] column-major (mesh `coords`, z unused)
 *   lam    [21 x fen]: coefficient q of element e at lam[q*fen + e], order
 *          a11 a12 a16 a22 a26 a66 a44 a45 a55 b11 b12 b16 b22 b26 b66 d11 d12 d16 d22 d26 d66
 *   I_G, I_L [basket_rows x 12] column-major, 1-based, 0 = empty (nodesMaps_Fiborek.m)
 *   U, F   [5*nnode] in the reference DOF order (u, phi_x, v, phi_y, w per node)
 * The element-local forces live in a fixed device array inside the library
 * (SHM_STATIC_MAX_ELEMS elements, 5.9 MB, held by every GPU that loads the
 * library until exit); larger meshes return SHM_ERR_BAD_ARG.  The first call
 * on a device sets up that device (symbol address, constants): make it before
 * any stream capture.  The set-up is cached per device for the life of the
 * process: a caller that resets the device (cudaDeviceReset) invalidates it,
 * and the next call would use a stale address -- do not reset a device that
 * this entry point has run on.  All calls share the array, so calls that
 * overlap on the GPU race; calls ordered on one stream are safe (each call
 * clears F and writes every element slot it reads).  Errors: SHM_ERR_BAD_ARG
 * for sizes or NULL arrays, SHM_ERR_CUDA when a CUDA error was already pending
 * (nothing is queued then) or a set-up step or launch fails;
 * shm_last_error(NULL) names the step.  FP64. */
#define SHM_STATIC_MAX_ELEMS 4096
shm_status shm_stiffness_static(int32_t fen, int32_t nnode, const int32_t *nodes, const double *coords,
                                const double *lam, int32_t basket_rows, const int32_t *I_G, const int32_t *I_L,
                                const double *U, double *F, void *stream);

/* Wavefield frames on a uniform grid, spec2meshgrid_flat_shell.m:55-583.
 * A grid holds, for nx x ny points spanning the mesh's bounding box inset by
 * 1e-8 m (point p = iy + ny*ix, meshgrid order), the owner element among
 * elements 0..fen_search-1 and the local coordinates (ksi, eta) after the
 * reference's three Newton steps.  fen_search = fen minus the elements
 * appended above a delamination (the reference searches 1..fen-|den_above|).
 * remap [nnode] (1-based, or NULL) names the node whose value is read in
 * place of each node: shell_surface 'top' over a delamination reads the
 * den_above copy for every den_under node (U(nodes_under) = U(nodes_above)).
 * device < 0 builds the set-up on the host only (shm_grid_points works, the
 * interpolation calls return SHM_ERR_STATE). */
typedef struct shm_grid shm_grid;
shm_status shm_grid_create(const shm_mesh *mesh, int32_t fen_search, const int32_t *remap, int32_t nx,
                           int32_t ny, int32_t device, shm_grid **out);
shm_status shm_grid_destroy(shm_grid *grid);
const char *shm_grid_last_error(const shm_grid *grid);
/* Set-up results, each [nx*ny] (any pointer may be NULL); owner is 0-based;
 * max_err = max distance between a point and its mapped (ksi, eta) (:264-266). */
shm_status shm_grid_points(const shm_grid *grid, double *xp, double *yp, int32_t *owner, double *ksi,
                           double *eta, double *max_err);
/* Data [nframes][nx*ny] of motion 1..9 (flat_shell_variable_names.m:8-17:
 * 1 x, 2 y, 3 z, 4 phi_x, 5 phi_y, 6 x + s phi_x, 7 y + s phi_y,
 * 8 |in-plane|, 9 |total|, s = +h/2 surface 0 'top', -h/2 surface 1 'bottom')
 * from host frames [nframes][nfields][nnode]; dof_field[5] gives the field
 * index of u, phi_x, v, phi_y, w (-1 = absent). */
shm_status shm_grid_interpolate(shm_grid *grid, const double *frames, int32_t nframes, int32_t nfields,
                                const int32_t *dof_field, int32_t motion, int32_t surface, double h,
                                double *data, void *stream);
/* The same from the device-resident frames of scenario `scen` of a plan
 * (field_variable kind: 0 velocity, 1 displacement, 2 acceleration), with no
 * host round trip of the frames; data [nframes][nx*ny] on the host. */
shm_status shm_grid_interpolate_plan(shm_grid *grid, shm_plan *plan, int32_t scen, int32_t kind,
                                     int32_t motion, int32_t surface, double h, double *data, void *stream);
/* Device time (ms, CUDA events) of one interpolation of all the plan's frames. */
shm_status shm_grid_time(shm_grid *grid, shm_plan *plan, int32_t scen, int32_t kind, int32_t motion,
                         int32_t surface, double h, int32_t reps, float *ms);

#ifdef __cplusplus
}
#endif
#endif /* SHMSEM_H */
