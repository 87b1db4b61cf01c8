/*
 * Oracle, time-loop half: FP64 CPU restatement of ma-shm's flat-shell
 * explicit central-difference loop.
 *
 * TEST INFRASTRUCTURE ONLY.  The product never links, loads or calls this
 * file.  Parity unpinned: the reference has no golden outputs for this loop
 * (only its set-up constants are pinned, see tests/golden/).  tests/ compare
 * the GPU results with it; bench.py's --impl reference arm and cpu_baseline
 * leg time it as the reference's CPU path (the MATLAB original cannot run
 * without MATLAB).
 *
 * It follows src/models/flat_shell/flat_shell_engine/main_flat_shell.m,
 * MAIN LOOP (:651-920), literally, one element at a time:
 *   gather           UX=U(Iu) ... FIY=U(Ifiy)                    :655-659
 *   derivatives      Npx*UX ... Npy*UZ  (sparse element blocks)   :661-671
 *   resultants       Sxx Sxxz Sxy Sxyz Syy Syyz Syz Sxz           :674-681
 *   internal forces  fu fv mx my fw (transposed blocks)           :683-689
 *   PZT voltage      Volt, mean over the sensor's nodes           :690-694
 *                    (main_flat_shell_multi_pzt_c.m:619-623 for several sensors)
 *   12-basket scatter F(I_G_dofs(:,b)) += F2(I_L_dofs(:,b))       :716-726
 *   update           F=-F+mg2.*U+Fa*st(nn)-mg.*uold+a1*cg.*uold;
 *                    unew=mg0.*F                                  :742-750
 *   outputs          displ(nn,:)=U(outputs)                       :752-764
 *   frames           Uc=U, v=a1*(-uold+unew), a=a0*(uold-2*U+unew)
 *                    every frm_int steps                          :765-885
 *   blow-up guard    max(UZ)>10*h or isnan(unew(3))               :786-804
 * Expression order inside each formula is the reference's (MATLAB evaluates
 * left to right).  Element work runs in parallel with OpenMP; every basket
 * is conflict free by construction (nodesMaps_Fiborek.m:19-27), so rows of
 * one basket are also added in parallel with no change to the result.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NPE 36

typedef struct {
  /* mesh */
  int32_t fen, nnode;
  const int32_t *nodes; /* [fen*36] element-major, 1-based: nodes(ne,c) */
  /* sparse element blocks of Npx / Npy in MATLAB find() order (0-based) */
  int32_t nnzx, nnzy;
  const int32_t *nx_row, *nx_col;
  const double *nx_val;
  const int32_t *ny_row, *ny_col;
  const double *ny_val;
  /* per local node (fen*36): inverse Jacobian and weights*detJ */
  const double *invJ11, *invJ12, *invJ21, *invJ22, *WWDetJ;
  /* per local node laminate coefficients: 21 stiffness arrays, order
     a11 a12 a16 a22 a26 a66 a44 a45 a55 b11 b12 b16 b22 b26 b66
     d11 d12 d16 d22 d26 d66, each fen*36 long (coef[k*L + l]) */
  const double *coef;
  /* basket maps I_G_dofs / I_L_dofs: [rows5 * 12] column-major, 1-based */
  int32_t rows5;
  const int64_t *IGd, *ILd;
  /* diagonal matrices (already scaled as in :592-604): length 5*nnode */
  const double *mg, *mg2, *mg0, *cg;
  double a0, a1;
  /* signal and loop range (1-based nn = nn_first..nft) */
  int32_t nn_first, nft;
  const double *st; /* [nft] */
  /* excitation vector (dense, 5*nnode) */
  const double *Fa;
  /* point outputs (1-based DOF numbers) */
  int32_t nout;
  const int32_t *out_dof;
  double *displ; /* [nft * nout] row-major: displ[(nn-1)*nout + k] */
  /* PZT sensors: CSR over elements (0-based element numbers) */
  int32_t nsens;
  const int32_t *sens_ptr, *sens_el;
  double pzt_thickness, g33, e31, e32, h;
  double *voltage; /* [nft * nsens] */
  /* frames (:765-885): every frm_int steps, field_variable frame_kind
     (0 velocity, 1 displacement, 2 acceleration, 3 all three) of component
     frame_dof (0 = all five, else 1..5) of every node, stored as
     frames[(c*nfields + field)*nnode + node]; fields kind-major
     (displacement, velocity, acceleration), then DOF order */
  int32_t frm_int, frame_dof, frame_kind, nframes_max;
  double *frames;
  double *t_frames_step; /* nn of each frame (for t_frames) */
  int32_t nthreads;
  /* in/out: initial and final state (5*nnode each) */
  double *U, *uold;
  /* result */
  int32_t frames_written;
  int32_t diverged_at; /* 0 if fine, else nn */
  /* pressure loading (main_flat_shell_pressure_excit_c.m:64-82,616-632,
     705-730): nodal frames p_nodal[k*nnode + node] at times p_t1[k];
     t_sem = (nn-1)*p_dt; 0 = none */
  int32_t n_pf;
  const double *p_t1, *p_nodal;
  double p_dt;
} oracle_args;

static inline void spmv_block(int nnz, const int32_t *row, const int32_t *col, const double *val,
                              const double *x, double *y) {
  /* y = N*x for one element block; nonzeros in column-major order */
  for (int c = 0; c < NPE; ++c) y[c] = 0.0;
  for (int k = 0; k < nnz; ++k) y[row[k]] += val[k] * x[col[k]];
}

static inline void spmv_block_t(int nnz, const int32_t *row, const int32_t *col, const double *val,
                                const double *x, double *y) {
  /* y = N'*x (N' built explicitly in the reference: Npxt=Npx') */
  for (int c = 0; c < NPE; ++c) y[c] = 0.0;
  for (int k = 0; k < nnz; ++k) y[col[k]] += val[k] * x[row[k]];
}

int oracle_flat_shell_run(oracle_args *A) {
  const int fen = A->fen;
  const int L = fen * NPE;
  const int ndof = 5 * A->nnode;
#ifdef _OPENMP
  if (A->nthreads > 0) omp_set_num_threads(A->nthreads);
#endif
  double *F2 = (double *)calloc((size_t)5 * L, sizeof(double));
  double *F = (double *)calloc((size_t)ndof, sizeof(double));
  double *unew = (double *)calloc((size_t)ndof, sizeof(double));
  double *Vsum = (double *)calloc((size_t)(fen > 0 ? fen : 1), sizeof(double));
  double *Fpl = NULL, *Fpr = NULL, *pt = NULL;
  if (A->n_pf > 0) {
    Fpl = (double *)calloc((size_t)5 * L, sizeof(double));
    Fpr = (double *)calloc((size_t)ndof, sizeof(double));
    pt = (double *)calloc((size_t)A->nnode, sizeof(double));
    if (!Fpl || !Fpr || !pt) return -1;
  }
  if (!F2 || !F || !unew || !Vsum) return -1;
  double *U = A->U, *uold = A->uold;
  int frame_c = 0;
  A->diverged_at = 0;
  const double *cf = A->coef;

  for (int nn = A->nn_first; nn <= A->nft; ++nn) {
    double maxUZ = -INFINITY;
#pragma omp parallel for schedule(static) reduction(max : maxUZ)
    for (int e = 0; e < fen; ++e) {
      double UX[NPE], UY[NPE], UZ[NPE], FIX[NPE], FIY[NPE];
      double NpxUX[NPE], NpxUY[NPE], NpxFIX[NPE], NpxFIY[NPE];
      double NpyUX[NPE], NpyUY[NPE], NpyFIX[NPE], NpyFIY[NPE];
      double NpxUZ[NPE], NpyUZ[NPE];
      double Sxx[NPE], Sxxz[NPE], Sxy[NPE], Sxyz[NPE], Syy[NPE], Syyz[NPE], Syz[NPE], Sxz[NPE];
      double tmp[NPE], acc[NPE];
      const int32_t *nd = A->nodes + (size_t)e * NPE;
      for (int c = 0; c < NPE; ++c) {
        const int g = nd[c];
        UX[c] = U[5 * g - 5];  /* Iu   = 5*nodes-4 */
        FIX[c] = U[5 * g - 4]; /* Ifix = 5*nodes-3 */
        UY[c] = U[5 * g - 3];  /* Iv   = 5*nodes-2 */
        FIY[c] = U[5 * g - 2]; /* Ifiy = 5*nodes-1 */
        UZ[c] = U[5 * g - 1];  /* Iw   = 5*nodes   */
        if (UZ[c] > maxUZ) maxUZ = UZ[c];
      }
      spmv_block(A->nnzx, A->nx_row, A->nx_col, A->nx_val, UX, NpxUX);
      spmv_block(A->nnzx, A->nx_row, A->nx_col, A->nx_val, UY, NpxUY);
      spmv_block(A->nnzx, A->nx_row, A->nx_col, A->nx_val, FIX, NpxFIX);
      spmv_block(A->nnzx, A->nx_row, A->nx_col, A->nx_val, FIY, NpxFIY);
      spmv_block(A->nnzy, A->ny_row, A->ny_col, A->ny_val, UX, NpyUX);
      spmv_block(A->nnzy, A->ny_row, A->ny_col, A->ny_val, UY, NpyUY);
      spmv_block(A->nnzy, A->ny_row, A->ny_col, A->ny_val, FIX, NpyFIX);
      spmv_block(A->nnzy, A->ny_row, A->ny_col, A->ny_val, FIY, NpyFIY);
      spmv_block(A->nnzx, A->nx_row, A->nx_col, A->nx_val, UZ, NpxUZ);
      spmv_block(A->nnzy, A->ny_row, A->ny_col, A->ny_val, UZ, NpyUZ);
      const size_t l0 = (size_t)e * NPE;
      const double *iJ11 = A->invJ11 + l0, *iJ12 = A->invJ12 + l0;
      const double *iJ21 = A->invJ21 + l0, *iJ22 = A->invJ22 + l0;
      const double *W = A->WWDetJ + l0;
#define C(k) (cf[(size_t)(k) * L + l0 + c])
      for (int c = 0; c < NPE; ++c) {
        const double a11 = C(0), a12 = C(1), a16 = C(2), a22 = C(3), a26 = C(4), a66 = C(5);
        const double a44 = C(6), a45 = C(7), a55 = C(8);
        const double b11 = C(9), b12 = C(10), b16 = C(11), b22 = C(12), b26 = C(13), b66 = C(14);
        const double d11 = C(15), d12 = C(16), d16 = C(17), d22 = C(18), d26 = C(19), d66 = C(20);
        const double i11 = iJ11[c], i12 = iJ12[c], i21 = iJ21[c], i22 = iJ22[c];
        /* main_flat_shell.m:674-681, term by term */
        Sxx[c] = ((NpxUX[c]) * i11 + (NpyUX[c]) * i21) * a11 + ((NpxFIX[c]) * i11 + (NpyFIX[c]) * i21) * b11 +
                 ((NpxUY[c]) * i12 + (NpyUY[c]) * i22) * a12 + ((NpxFIY[c]) * i12 + (NpyFIY[c]) * i22) * b12 +
                 ((NpxUX[c]) * i12 + (NpyUX[c]) * i22) * a16 + ((NpxFIX[c]) * i12 + (NpyFIX[c]) * i22) * b16 +
                 ((NpxUY[c]) * i11 + (NpyUY[c]) * i21) * a16 + ((NpxFIY[c]) * i11 + (NpyFIY[c]) * i21) * b16;
        Sxxz[c] = ((NpxUX[c]) * i11 + (NpyUX[c]) * i21) * b11 + ((NpxFIX[c]) * i11 + (NpyFIX[c]) * i21) * d11 +
                  ((NpxUY[c]) * i12 + (NpyUY[c]) * i22) * b12 + ((NpxFIY[c]) * i12 + (NpyFIY[c]) * i22) * d12 +
                  ((NpxUX[c]) * i12 + (NpyUX[c]) * i22) * b16 + ((NpxFIX[c]) * i12 + (NpyFIX[c]) * i22) * d16 +
                  ((NpxUY[c]) * i11 + (NpyUY[c]) * i21) * b16 + ((NpxFIY[c]) * i11 + (NpyFIY[c]) * i21) * d16;
        Sxy[c] = ((NpxUX[c]) * i11 + (NpyUX[c]) * i21) * a16 + ((NpxFIX[c]) * i11 + (NpyFIX[c]) * i21) * b16 +
                 ((NpxUY[c]) * i12 + (NpyUY[c]) * i22) * a26 + ((NpxFIY[c]) * i12 + (NpyFIY[c]) * i22) * b26 +
                 ((NpxUX[c]) * i12 + (NpyUX[c]) * i22) * a66 + ((NpxFIX[c]) * i12 + (NpyFIX[c]) * i22) * b66 +
                 ((NpxUY[c]) * i11 + (NpyUY[c]) * i21) * a66 + ((NpxFIY[c]) * i11 + (NpyFIY[c]) * i21) * b66;
        Sxyz[c] = ((NpxUX[c]) * i11 + (NpyUX[c]) * i21) * b16 + ((NpxFIX[c]) * i11 + (NpyFIX[c]) * i21) * d16 +
                  ((NpxUY[c]) * i12 + (NpyUY[c]) * i22) * b26 + ((NpxFIY[c]) * i12 + (NpyFIY[c]) * i22) * d26 +
                  ((NpxUX[c]) * i12 + (NpyUX[c]) * i22) * b66 + ((NpxFIX[c]) * i12 + (NpyFIX[c]) * i22) * d66 +
                  ((NpxUY[c]) * i11 + (NpyUY[c]) * i21) * b66 + ((NpxFIY[c]) * i11 + (NpyFIY[c]) * i21) * d66;
        Syy[c] = ((NpxUX[c]) * i11 + (NpyUX[c]) * i21) * a12 + ((NpxFIX[c]) * i11 + (NpyFIX[c]) * i21) * b12 +
                 ((NpxUY[c]) * i12 + (NpyUY[c]) * i22) * a22 + ((NpxFIY[c]) * i12 + (NpyFIY[c]) * i22) * b22 +
                 ((NpxUX[c]) * i12 + (NpyUX[c]) * i22) * a26 + ((NpxFIX[c]) * i12 + (NpyFIX[c]) * i22) * b26 +
                 ((NpxUY[c]) * i11 + (NpyUY[c]) * i21) * a26 + ((NpxFIY[c]) * i11 + (NpyFIY[c]) * i21) * b26;
        Syyz[c] = ((NpxUX[c]) * i11 + (NpyUX[c]) * i21) * b12 + ((NpxFIX[c]) * i11 + (NpyFIX[c]) * i21) * d12 +
                  ((NpxUY[c]) * i12 + (NpyUY[c]) * i22) * b22 + ((NpxFIY[c]) * i12 + (NpyFIY[c]) * i22) * d22 +
                  ((NpxUX[c]) * i12 + (NpyUX[c]) * i22) * b26 + ((NpxFIX[c]) * i12 + (NpyFIX[c]) * i22) * d26 +
                  ((NpxUY[c]) * i11 + (NpyUY[c]) * i21) * b26 + ((NpxFIY[c]) * i11 + (NpyFIY[c]) * i21) * d26;
        Syz[c] = (FIY[c] + (NpxUZ[c]) * i12 + (NpyUZ[c]) * i22) * a44 + (FIX[c] + (NpxUZ[c]) * i11 + (NpyUZ[c]) * i21) * a45;
        Sxz[c] = (FIY[c] + (NpxUZ[c]) * i12 + (NpyUZ[c]) * i22) * a45 + (FIX[c] + (NpxUZ[c]) * i11 + (NpyUZ[c]) * i21) * a55;
      }
#undef C
      /* main_flat_shell.m:683-689: each force is a left-to-right sum of
         transposed products of weighted resultants */
#define TERM(first, S, IJ, NPT)                                                           \
  do {                                                                                    \
    double v_[NPE];                                                                       \
    for (int c = 0; c < NPE; ++c) v_[c] = S[c] * IJ[c] * W[c];                            \
    if (NPT) spmv_block_t(A->nnzx, A->nx_row, A->nx_col, A->nx_val, v_, tmp);             \
    else spmv_block_t(A->nnzy, A->ny_row, A->ny_col, A->ny_val, v_, tmp);                 \
    if (first) for (int c = 0; c < NPE; ++c) acc[c] = tmp[c];                             \
    else for (int c = 0; c < NPE; ++c) acc[c] = acc[c] + tmp[c];                          \
  } while (0)
      double *f2 = F2 + (size_t)5 * l0;
      /* fu */
      TERM(1, Sxx, iJ11, 1); TERM(0, Sxx, iJ21, 0); TERM(0, Sxy, iJ12, 1); TERM(0, Sxy, iJ22, 0);
      for (int c = 0; c < NPE; ++c) f2[5 * c + 0] = acc[c];
      /* fv */
      TERM(1, Syy, iJ12, 1); TERM(0, Syy, iJ22, 0); TERM(0, Sxy, iJ11, 1); TERM(0, Sxy, iJ21, 0);
      for (int c = 0; c < NPE; ++c) f2[5 * c + 2] = acc[c];
      /* mx */
      TERM(1, Sxxz, iJ11, 1); TERM(0, Sxxz, iJ21, 0); TERM(0, Sxyz, iJ12, 1); TERM(0, Sxyz, iJ22, 0);
      for (int c = 0; c < NPE; ++c) f2[5 * c + 1] = acc[c] + Sxz[c] * W[c];
      /* my */
      TERM(1, Syyz, iJ12, 1); TERM(0, Syyz, iJ22, 0); TERM(0, Sxyz, iJ11, 1); TERM(0, Sxyz, iJ21, 0);
      for (int c = 0; c < NPE; ++c) f2[5 * c + 3] = acc[c] + Syz[c] * W[c];
      /* fw */
      TERM(1, Syz, iJ12, 1); TERM(0, Syz, iJ22, 0); TERM(0, Sxz, iJ11, 1); TERM(0, Sxz, iJ21, 0);
      for (int c = 0; c < NPE; ++c) f2[5 * c + 4] = acc[c];
#undef TERM
      /* PZT voltage partial sum (main_flat_shell.m:690-692; note invJ12 and
         invJ21 enter the x and y derivatives here, as in the reference) */
      if (A->nsens > 0) {
        double s = 0.0;
        const double k0 = A->pzt_thickness / A->g33, hh = A->h / 2;
        for (int c = 0; c < NPE; ++c) {
          const double v = k0 * (A->e31 * (NpxUX[c] * iJ11[c] + NpyUX[c] * iJ12[c] + hh * NpxFIX[c] * iJ11[c] +
                                           hh * NpyFIX[c] * iJ12[c]) +
                                 A->e32 * (NpxUY[c] * iJ21[c] + NpyUY[c] * iJ22[c] + hh * NpxFIY[c] * iJ21[c] +
                                           hh * NpyFIY[c] * iJ22[c]));
          s += v;
        }
        Vsum[e] = s;
      }
    }
    /* sensor voltages: mean over all local nodes of the sensor's elements */
    for (int k = 0; k < A->nsens; ++k) {
      double s = 0.0;
      int cnt = 0;
      for (int q = A->sens_ptr[k]; q < A->sens_ptr[k + 1]; ++q) {
        s += Vsum[A->sens_el[q]];
        cnt += NPE;
      }
      A->voltage[(size_t)(nn - 1) * A->nsens + k] = cnt ? s / cnt : 0.0;
    }
    /* 12-basket scatter */
    memset(F, 0, sizeof(double) * ndof);
    for (int b = 0; b < 12; ++b) {
      const int64_t *g = A->IGd + (size_t)b * A->rows5;
      const int64_t *l = A->ILd + (size_t)b * A->rows5;
#pragma omp parallel for schedule(static)
      for (int r = 0; r < A->rows5; ++r)
        if (g[r] > 0) F[g[r] - 1] = F[g[r] - 1] + F2[l[r] - 1];
    }
    /* pressure: pt = interp1(t1, p', t_sem, 'linear', 0); Fi(5:5:end) = pt';
       fl = Fi(Iw).*WWDetJ; Fp(5:5:end) = fl; baskets into F_pressure */
    if (A->n_pf > 0) {
      const double ts = (nn - 1) * A->p_dt;
      const int np = A->n_pf;
      int k = -1;
      if (ts >= A->p_t1[0] && ts <= A->p_t1[np - 1]) {
        k = 0;
        while (k + 1 < np - 1 && ts > A->p_t1[k + 1]) ++k;
      }
      for (int q = 0; q < A->nnode; ++q) {
        if (k < 0) {
          pt[q] = 0.0;
        } else if (np == 1) {
          pt[q] = A->p_nodal[q];
        } else {
          const double y0 = A->p_nodal[(size_t)k * A->nnode + q], y1 = A->p_nodal[(size_t)(k + 1) * A->nnode + q];
          pt[q] = y0 + (y1 - y0) * ((ts - A->p_t1[k]) / (A->p_t1[k + 1] - A->p_t1[k]));
        }
      }
      for (int l = 0; l < L; ++l) Fpl[5 * (size_t)l + 4] = pt[A->nodes[l] - 1] * A->WWDetJ[l];
      memset(Fpr, 0, sizeof(double) * ndof);
      for (int b = 0; b < 12; ++b) {
        const int64_t *g = A->IGd + (size_t)b * A->rows5;
        const int64_t *l = A->ILd + (size_t)b * A->rows5;
        for (int r = 0; r < A->rows5; ++r)
          if (g[r] > 0) Fpr[g[r] - 1] = Fpr[g[r] - 1] + Fpl[l[r] - 1];
      }
    }
    /* time integration, main_flat_shell.m:742-750 (+ F_pressure,
       main_flat_shell_pressure_excit_c.m:730) */
    const double s_nn = A->st[nn - 1];
#pragma omp parallel for schedule(static)
    for (int d = 0; d < ndof; ++d) {
      double f = -F[d] + A->mg2[d] * U[d] + A->Fa[d] * s_nn;
      if (Fpr) f = f + Fpr[d];
      f = f - A->mg[d] * uold[d] + A->a1 * A->cg[d] * uold[d];
      unew[d] = A->mg0[d] * f;
    }
    /* outputs: displacement before the update (:752-764) */
    for (int k = 0; k < A->nout; ++k) A->displ[(size_t)(nn - 1) * A->nout + k] = U[A->out_dof[k] - 1];
    /* frames and blow-up guard */
    if (A->frm_int > 0 && nn % A->frm_int == 0) {
      if (A->frames && frame_c < A->nframes_max) {
        /* API kind -> 0 displacement, 1 velocity, 2 acceleration */
        static const int kind_slot[3] = {1, 0, 2};
        const int nkind = A->frame_kind == 3 ? 3 : 1;
        const int ncomp = A->frame_dof == 0 ? 5 : 1;
        int fld = 0;
        for (int k = 0; k < 3; ++k) {
          if (A->frame_kind != 3 && kind_slot[A->frame_kind] != k) continue;
          for (int comp = 0; comp < 5; ++comp) {
            if (A->frame_dof != 0 && A->frame_dof - 1 != comp) continue;
            double *fr = A->frames + ((size_t)frame_c * nkind * ncomp + fld) * A->nnode;
            for (int q = 0; q < A->nnode; ++q) {
              const size_t d = 5 * (size_t)q + comp;
              if (k == 0)
                fr[q] = U[d];
              else if (k == 1)
                fr[q] = A->a1 * (-uold[d] + unew[d]);
              else
                fr[q] = A->a0 * (uold[d] - 2 * U[d] + unew[d]);
            }
            ++fld;
          }
        }
        if (A->t_frames_step) A->t_frames_step[frame_c] = nn;
        ++frame_c;
      }
      if (maxUZ > 10 * A->h || isnan(unew[2])) {
        A->diverged_at = nn;
        break;
      }
    }
    /* uold = U; U = unew */
    memcpy(uold, U, sizeof(double) * ndof);
    memcpy(U, unew, sizeof(double) * ndof);
  }
  A->frames_written = frame_c;
  free(F2);
  free(F);
  free(unew);
  free(Vsum);
  free(Fpl);
  free(Fpr);
  free(pt);
  return 0;
}

/* Element force only (one application of K to U, no update): used by the
   tests to compare element operators.  Fout = assembled K*U (5*nnode). */
int oracle_flat_shell_apply_k(oracle_args *A, double *Fout) {
  oracle_args B = *A;
  /* run one "step" with mg2=mg=cg=Fa=0, mg0=-1 so that unew = F */
  const int ndof = 5 * A->nnode;
  double *zero = (double *)calloc((size_t)ndof, sizeof(double));
  double *minus1 = (double *)malloc(sizeof(double) * ndof);
  double *U = (double *)malloc(sizeof(double) * ndof);
  double *uo = (double *)calloc((size_t)ndof, sizeof(double));
  double st1[1] = {0.0};
  if (!zero || !minus1 || !U || !uo) return -1;
  for (int d = 0; d < ndof; ++d) minus1[d] = -1.0;
  memcpy(U, A->U, sizeof(double) * ndof);
  B.mg = zero; B.mg2 = zero; B.cg = zero; B.Fa = zero; B.mg0 = minus1;
  B.nn_first = 1; B.nft = 1; B.st = st1; B.nout = 0; B.nsens = 0; B.frm_int = 0;
  B.U = U; B.uold = uo;
  int rc = oracle_flat_shell_run(&B);
  memcpy(Fout, U, sizeof(double) * ndof);
  free(zero); free(minus1); free(U); free(uo);
  return rc;
}

/* ------------------------------------------------------------------------
 * 3D solid loop: src/models/solid3D/main_spec3Dcuda_global_cpu_gpu3_wave_sens_opt_single_PCT_mat.m:922-1040
 * strains_spec_p.m, stresses_spec_p.m, forces :944-954, 12-basket scatter,
 * update :1032-1037, outputs U(outputs).  Element blocks of Npx, Npy, Npz
 * (108 x 108) as nonzero lists in MATLAB find() order.
 * ------------------------------------------------------------------------ */
#define SNPE 108

typedef struct {
  int32_t fen, nnode;
  const int32_t *nodes; /* [fen*108] element-major, 1-based */
  int32_t nnz[3];
  const int32_t *row[3], *col[3];
  const double *val[3];
  const double *invJ;   /* [9][fen*108]: invJ11 invJ12 invJ13 invJ21 ... invJ33 */
  const double *W;      /* [fen*108] WWWDetJ */
  const double *D;      /* [13][fen*108]: D11 D12 D13 D14 D22 D23 D24 D33 D34 D44 D55 D56 D66 */
  int32_t rows3;
  const int64_t *IGd, *ILd; /* [rows3*12] column-major, 1-based, 3-dof numbering */
  const double *mg, *mg2, *mg0, *cg;
  double a0, a1;
  int32_t nn_first, nft;
  const double *st;
  const double *Fa;
  int32_t nout;
  const int32_t *out_dof;
  double *displ;
  int32_t nthreads;
  double *U, *uold;
} oracle_solid_args;

static inline void sp3(int nnz, const int32_t *row, const int32_t *col, const double *val, const double *x, double *y) {
  for (int c = 0; c < SNPE; ++c) y[c] = 0.0;
  for (int k = 0; k < nnz; ++k) y[row[k]] += val[k] * x[col[k]];
}
static inline void sp3t(int nnz, const int32_t *row, const int32_t *col, const double *val, const double *x, double *y) {
  for (int c = 0; c < SNPE; ++c) y[c] = 0.0;
  for (int k = 0; k < nnz; ++k) y[col[k]] += val[k] * x[row[k]];
}

int oracle_solid_run(oracle_solid_args *A) {
  const int fen = A->fen;
  const int L = fen * SNPE;
  const int ndof = 3 * A->nnode;
#ifdef _OPENMP
  if (A->nthreads > 0) omp_set_num_threads(A->nthreads);
#endif
  double *F2 = (double *)calloc((size_t)3 * L, sizeof(double));
  double *F = (double *)calloc((size_t)ndof, sizeof(double));
  double *unew = (double *)calloc((size_t)ndof, sizeof(double));
  if (!F2 || !F || !unew) return -1;
  double *U = A->U, *uold = A->uold;
  for (int nn = A->nn_first; nn <= A->nft; ++nn) {
#pragma omp parallel for schedule(static)
    for (int e = 0; e < fen; ++e) {
      double UX[SNPE], UY[SNPE], UZ[SNPE], d[9][SNPE];
      const int32_t *nd = A->nodes + (size_t)e * SNPE;
      for (int c = 0; c < SNPE; ++c) {
        UX[c] = U[3 * nd[c] - 3];
        UY[c] = U[3 * nd[c] - 2];
        UZ[c] = U[3 * nd[c] - 1];
      }
      /* d[3*k + f]: Np{x,y,z}[k] * U{X,Y,Z}[f] */
      const double *Uf[3] = {UX, UY, UZ};
      for (int k = 0; k < 3; ++k)
        for (int f = 0; f < 3; ++f) sp3(A->nnz[k], A->row[k], A->col[k], A->val[k], Uf[f], d[3 * k + f]);
      const size_t l0 = (size_t)e * SNPE;
#define IJ(a, b) A->invJ[(size_t)(3 * (a) + (b)) * L + l0 + c]
#define DD(k) A->D[(size_t)(k) * L + l0 + c]
      double Sxx[SNPE], Syy[SNPE], Szz[SNPE], Sxy[SNPE], Syz[SNPE], Sxz[SNPE];
      for (int c = 0; c < SNPE; ++c) {
        /* strains_spec_p.m:8-27 (NpxU = d[0..2], NpyU = d[3..5], NpzU = d[6..8]) */
        const double Exx = (d[0][c]) * IJ(0, 0) + (d[3][c]) * IJ(1, 0) + (d[6][c]) * IJ(2, 0);
        const double Eyy = (d[1][c]) * IJ(0, 1) + (d[4][c]) * IJ(1, 1) + (d[7][c]) * IJ(2, 1);
        const double Ezz = (d[2][c]) * IJ(0, 2) + (d[5][c]) * IJ(1, 2) + (d[8][c]) * IJ(2, 2);
        const double B41UX = (d[0][c]) * IJ(0, 1) + (d[3][c]) * IJ(1, 1) + (d[6][c]) * IJ(2, 1);
        const double B42UY = (d[1][c]) * IJ(0, 0) + (d[4][c]) * IJ(1, 0) + (d[7][c]) * IJ(2, 0);
        const double Exy = B41UX + B42UY;
        const double B52UY = (d[1][c]) * IJ(0, 2) + (d[4][c]) * IJ(1, 2) + (d[7][c]) * IJ(2, 2);
        const double B53UZ = (d[2][c]) * IJ(0, 1) + (d[5][c]) * IJ(1, 1) + (d[8][c]) * IJ(2, 1);
        const double Eyz = B52UY + B53UZ;
        const double B61UX = (d[0][c]) * IJ(0, 2) + (d[3][c]) * IJ(1, 2) + (d[6][c]) * IJ(2, 2);
        const double B63UZ = (d[2][c]) * IJ(0, 0) + (d[5][c]) * IJ(1, 0) + (d[8][c]) * IJ(2, 0);
        const double Exz = B61UX + B63UZ;
        /* stresses_spec_p.m:5-10 */
        Sxx[c] = Exx * DD(0) + Eyy * DD(1) + Ezz * DD(2) + Exy * DD(3);
        Syy[c] = Exx * DD(1) + Eyy * DD(4) + Ezz * DD(5) + Exy * DD(6);
        Szz[c] = Exx * DD(2) + Eyy * DD(5) + Ezz * DD(7) + Exy * DD(8);
        Sxy[c] = Exx * DD(3) + Eyy * DD(6) + Ezz * DD(8) + Exy * DD(9);
        Syz[c] = Eyz * DD(10) + Exz * DD(11);
        Sxz[c] = Eyz * DD(11) + Exz * DD(12);
      }
      /* forces, :944-954: f = sum over terms left to right */
      const double *W = A->W + l0;
      double acc[SNPE], tmp[SNPE], v_[SNPE];
#define T3(first, S, a, b, k)                                                     \
  do {                                                                            \
    for (int c = 0; c < SNPE; ++c) v_[c] = S[c] * IJ(a, b) * W[c];                \
    sp3t(A->nnz[k], A->row[k], A->col[k], A->val[k], v_, tmp);                    \
    if (first) for (int c = 0; c < SNPE; ++c) acc[c] = tmp[c];                    \
    else for (int c = 0; c < SNPE; ++c) acc[c] = acc[c] + tmp[c];                 \
  } while (0)
      double *f2 = F2 + 3 * l0;
      /* fu: Sxx (invJ11,21,31), Sxy (invJ12,22,32), Sxz (invJ13,23,33) */
      T3(1, Sxx, 0, 0, 0); T3(0, Sxx, 1, 0, 1); T3(0, Sxx, 2, 0, 2);
      T3(0, Sxy, 0, 1, 0); T3(0, Sxy, 1, 1, 1); T3(0, Sxy, 2, 1, 2);
      T3(0, Sxz, 0, 2, 0); T3(0, Sxz, 1, 2, 1); T3(0, Sxz, 2, 2, 2);
      for (int c = 0; c < SNPE; ++c) f2[3 * c + 0] = acc[c];
      /* fv: Syy (12,22,32), Sxy (11,21,31), Syz (13,23,33) */
      T3(1, Syy, 0, 1, 0); T3(0, Syy, 1, 1, 1); T3(0, Syy, 2, 1, 2);
      T3(0, Sxy, 0, 0, 0); T3(0, Sxy, 1, 0, 1); T3(0, Sxy, 2, 0, 2);
      T3(0, Syz, 0, 2, 0); T3(0, Syz, 1, 2, 1); T3(0, Syz, 2, 2, 2);
      for (int c = 0; c < SNPE; ++c) f2[3 * c + 1] = acc[c];
      /* fw: Szz (13,23,33), Syz (12,22,32), Sxz (11,21,31) */
      T3(1, Szz, 0, 2, 0); T3(0, Szz, 1, 2, 1); T3(0, Szz, 2, 2, 2);
      T3(0, Syz, 0, 1, 0); T3(0, Syz, 1, 1, 1); T3(0, Syz, 2, 1, 2);
      T3(0, Sxz, 0, 0, 0); T3(0, Sxz, 1, 0, 1); T3(0, Sxz, 2, 0, 2);
      for (int c = 0; c < SNPE; ++c) f2[3 * c + 2] = acc[c];
#undef T3
#undef IJ
#undef DD
    }
    memset(F, 0, sizeof(double) * ndof);
    for (int b = 0; b < 12; ++b) {
      const int64_t *g = A->IGd + (size_t)b * A->rows3;
      const int64_t *l = A->ILd + (size_t)b * A->rows3;
#pragma omp parallel for schedule(static)
      for (int r = 0; r < A->rows3; ++r)
        if (g[r] > 0) F[g[r] - 1] = F[g[r] - 1] + F2[l[r] - 1];
    }
    const double s_nn = A->st[nn - 1];
#pragma omp parallel for schedule(static)
    for (int dd = 0; dd < ndof; ++dd) {
      double f = -F[dd] + A->mg2[dd] * U[dd] + A->Fa[dd] * s_nn - A->mg[dd] * uold[dd] + A->a1 * A->cg[dd] * uold[dd];
      unew[dd] = A->mg0[dd] * f;
    }
    for (int k = 0; k < A->nout; ++k) A->displ[(size_t)(nn - 1) * A->nout + k] = U[A->out_dof[k] - 1];
    memcpy(uold, U, sizeof(double) * ndof);
    memcpy(U, unew, sizeof(double) * ndof);
  }
  free(F2);
  free(F);
  free(unew);
  return 0;
}
