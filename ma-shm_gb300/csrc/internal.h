// Library-internal interfaces shared between translation units of
// libshmsem.so (not part of the C ABI).
#pragma once
#include <stdint.h>

#include <vector>

#include "shmsem.h"

namespace shm {

// GLL nodes x, weights w and Lagrange derivative matrix D[r*n + c] = l_c'(x_r)
// (gll.m, shape2D_prim.m; entries below 1e-12 in magnitude set to zero).
void gll_setup(int n, std::vector<double>& x, std::vector<double>& w, std::vector<double>& D);

// Read-only view of a plan's device-resident wavefield frames for one scenario.
struct FramesView {
  const void* frames;      // device [nframes][nfields][nnode_pad]
  int prec;                // 64: double, 32: float
  int64_t nnode_pad;       // field stride (elements)
  int64_t node0, nnode;    // the scenario's node range
  int nframes, nfields;
  signed char slot[15];    // slot[kind*5 + dof]: field index (kind 0 U, 1 V, 2 A) or -1
  int device, kind, ndof;  // kind 0 flat shell, 1 solid
  void* stream;            // the plan's cudaStream_t
};
shm_status plan_frames_view(shm_plan* p, int scen, FramesView* v);

// Text of the calling thread's last failed shm_stiffness_static call (NULL
// when its last call succeeded or it made none).
const char* static_last_error();

}  // namespace shm
