/*
 * w3o.h -- the oracle: a CPU restatement of WARP3D's element-block hot
 * path (tangent stiffness, strain/stress recovery with mm01, internal
 * forces). TEST INFRASTRUCTURE ONLY: it is the parity checker for the
 * CUDA path and the timed CPU baseline; the product never calls it.
 *
 * Same data layouts and argument meaning as include/w3g.h.
 */
#ifndef W3O_H
#define W3O_H
#include "../include/w3g.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Threads for the OpenMP block loops (0 = OpenMP default). */
void w3o_set_threads(int nthreads);
/* 1 = assemble ifv serially in block order (reproducible fixtures),
   0 = OpenMP ATOMIC scatter as in src/addifv.f:93-98. */
void w3o_set_deterministic(int on);

int w3o_tanstf(const w3g_model_desc* m, const w3g_block_state* s,
               int step, int iter, const double* c, const double* u,
               const double* du, double* const* estiff);

int w3o_recover(const w3g_model_desc* m, const w3g_block_state* s,
                int step, int iter, int extrapolated_du, const double* c,
                const double* u, const double* du, double* ifv,
                w3g_recover_info* info);

int w3o_update(const w3g_model_desc* m, const w3g_block_state* s);

/* Element library probes used by the tests: Gauss point (xi, eta, zeta,
   weight) and shape-function derivatives of element type etype. */
int w3o_gauss_point(int etype, int order, int gpn, double* xyzw);
int w3o_shape_derivs(int etype, double xi, double eta, double zeta,
                     double* nxi, double* neta, double* nzeta);

/* Hooks for the single-point material tests: one mm01 update of `span`
   points followed by cnst1 (src/mm01.f:24, :1196). Arrays use the
   oracle's (span, k) column-major layout of the reference. */
int w3o_mm01_point(int span, int step, const double* e, const double* nu,
                   const double* beta, const double* hprime,
                   const double* yld, const double* cgn, double* cgn1,
                   const double* deps, double* history, double* history1,
                   double* cep /* (span,6,6) */);

/* Hook for the single-point crystal tests: one mm10 update of one Gauss
   point (one crystal) as drive_10_update calls it. hist_n, hist_n1: 158
   values; urcs_n, urcs_n1: 9; uddt: 6; rot_n1: 9 (column-major). */
/* one point of the UMAT path (drive_umat_update + the example UMAT) */
int w3o_umat_point(const double* props, int step, int iter, int extrapolated_du, const double* urcs_n,
                   const double* eps_n, const double* uddt, const double* hist, double* urcs_n1,
                   double* hist1, double* cep21);
int w3o_mm10_point(const w3g_crystal* crystal, const double* angles, int step, int iter,
                   int extrapolated_du, double dt, double* hist_n, double* hist_n1,
                   const double* urcs_n, double* urcs_n1, const double* uddt,
                   const double* rot_n1);

#ifdef __cplusplus
}
#endif
#endif
