/*
 * w3g.h -- C-ABI of the GB300 element-block engine for WARP3D's
 * tangent-stiffness and strain/stress/internal-force block loops.
 *
 * The entry points replace, one for one, the two OpenMP block loops that
 * WARP3D's Newton driver calls once per iteration phase:
 *
 *   w3g_tanstf   <- subroutine tanstf              (src/tanstf.f:17, block
 *                   loop at :80-88, per-block work do_nlek_block :119)
 *   w3g_recover  <- subroutine drive_eps_sig_internal_forces
 *                   (src/drive_eps_sig_internal_forces.f:20, block loop
 *                   :160-180, ifv scatter :287-305)
 *   w3g_update   <- subroutine update, block-state copy n+1 -> n
 *                   (src/update.f:73-94)
 *
 * Every array keeps the layout of WARP3D's module elem_block_data
 * (src/mod_eleblocks.f:17-150) and of the element property tables
 * props/iprops/lprops (src/mod_main.f:47-52):
 *
 *   estiff   (utsz, span)        upper triangle, column packed:
 *                                pos = j(j-1)/2 + i for row i <= col j
 *                                (src/setup.f:265-275, :407-417)
 *   cep      (21, span, ngp)     lower triangle of [D], row-wise
 *                                (src/rstgp1.f:5360-5397)
 *   history  (hist, ngp, span)   per-Gauss-point material history
 *   urcs     (9, ngp, span)      unrotated Cauchy stress + U, Wp, ebarp
 *   eps      (6, ngp, span)      strains
 *   rot_n1   (9, ngp, span)      [R,n+1] column-major 3x3
 *   einfvec  (span, totdof)      element internal forces
 *   elem_vol (span)              element volumes at n+1
 *   edest/cdest (totdof, span)   int32, 1-based global dof / coordinate
 *                                index, ordered u1..un, v1..vn, w1..wn
 *   props/iprops/lprops (43, noelem)  float32 / int32 / logical(int32)
 *   elblks   (0:2, nelblk)       span, first element (1-based), owner
 *
 * Per-block arrays are passed as arrays of nelblk host pointers, exactly
 * as a Fortran caller obtains them with c_loc(x_blocks(blk)%ptr).
 *
 * All functions return an int status:
 *     0  ok
 *     1  step cut requested: det[F] <= 0 at some Gauss point
 *        (src/gtmat1.f:649-664 -> material_cut_step)
 *     2  local material solve failed (material_cut_step)
 *    <0  fatal: bad argument, unsupported element/material, CUDA error
 *        (replaces die_abort). w3g_last_error() gives the message.
 *
 * Nothing in this header uses torch or CUDA types; device pointers and
 * streams travel as void*.
 */
#ifndef W3G_H
#define W3G_H

#ifdef __cplusplus
extern "C" {
#endif

#define W3G_MXELPR 43
#define W3G_MXVL 128

/* Element types (iprops(1,elem)), src/elprp.f */
#define W3G_ETYPE_Q3DISOP 1   /* 20-node hexahedron */
#define W3G_ETYPE_L3DISOP 2   /* 8-node hexahedron  */
#define W3G_ETYPE_TET10 6     /* 10-node tetrahedron */

/* Material models (iprops(25,elem)) */
#define W3G_MAT_BILINEAR 1    /* mm01: bilinear Mises, mixed hardening */
#define W3G_MAT_UMAT 8        /* Abaqus UMAT interface (drive_umat_update) */
#define W3G_MAT_CRYSTAL 10    /* mm10: crystal plasticity */
#define W3G_UMAT_NPROPS 50    /* UMAT properties per element (dmatprp(151:200)) */

/* Status codes */
#define W3G_OK 0
#define W3G_STEP_CUT 1
#define W3G_LOCAL_FAIL 2
#define W3G_EARG -1
#define W3G_EUNSUPPORTED -2
#define W3G_ECUDA -3
#define W3G_ENOMEM -4
#define W3G_EFATAL -5

/* Precision of the tangent contraction (w3g_set_tangent_precision). */
#define W3G_TANGENT_FP64 0    /* plain form: everything FP64            */
#define W3G_TANGENT_FP32 1    /* Ke in FP32 (CUDA-core FP32 FMA)        */
#define W3G_TANGENT_TF32 2    /* B^T D B on the tensor cores, TF32 operands,
                                 FP32 accumulation, Ke stored FP32 (8- and
                                 20-node bricks; tetrahedra as
                                 W3G_TANGENT_FP32)                       */
#define W3G_TANGENT_BF16 3    /* the same with BF16 operands             */
#define W3G_TANGENT_TF32X3 4  /* TF32 with split operands (x = hi + lo,
                                 three MMAs): near-FP32 Ke accuracy       */
#define W3G_TANGENT_BF16X3 5  /* BF16 with split operands                */

/*
 * One crystal definition of mm10 crystal plasticity: c_array(cnum) of
 * module crystal_data (src/mod_crystals.f:140-230) as the crystal input
 * sets it (src/incrystal.f). Supported: slip_type 1 (fcc) and 2 (bcc,
 * the 12 {110}<111> systems), elastic_type 1 (isotropic), h_type 1 (Voce,
 * one hardening variable), one crystal per Gauss point, the default
 * Newton solver.
 */
typedef struct w3g_crystal {
  int slip_type;                /* 1 = fcc, 2 = bcc (12 systems)         */
  int elastic_type;             /* 1 = isotropic                         */
  int h_type;                   /* 1 = Voce                              */
  int miter;                    /* local Newton iteration limit (30)     */
  double e, nu;                 /* elastic constants                     */
  double harden_n;              /* slip-rate exponent n                  */
  double tau_y, tau_v;          /* Voce initial and saturation strength  */
  double theta_o;               /* Voce hardening modulus theta_0        */
  double voche_m;               /* Voce exponent m (1)                   */
  double iD_v;                  /* diffusion rate coefficient (0)        */
  double k_o, b;                /* geometric hardening k_0 and Burgers   */
  double atol, atol1, rtol, rtol1;  /* local tolerances (1e-5, 1e-5, 5e-5, 1e-5) */
} w3g_crystal;

/*
 * Model description: what WARP3D holds in elblks, props/iprops/lprops,
 * edest_blocks and cdest_blocks after input processing.
 */
typedef struct w3g_model_desc {
  int nelblk;
  const int* elblks;            /* 3*nelblk: span, felem, owner          */
  int noelem;
  const float* props;           /* 43*noelem                             */
  const int* iprops;            /* 43*noelem                             */
  const int* lprops;            /* 43*noelem, nonzero = .true.           */
  const int* const* edest;      /* nelblk pointers to (totdof, span)     */
  const int* const* cdest;      /* nelblk pointers to (totdof, span)     */
  int nodof;                    /* length of u, du, ifv                  */
  int ncoord;                   /* length of c                           */
  int qbar_flag;                /* consistent Q-bar term, default 1      */
  double beta_fact;             /* plane-strain thickness factor, 1 in 3-D */
  /* mm10 elements (iprops(25) = 10) only; NULL/0 otherwise */
  const w3g_crystal* crystals;  /* crystal definitions                   */
  int ncrystals;
  const int* elem_crystal;      /* noelem: 0-based crystal of the element */
  const double* elem_angles;    /* 3*noelem: Euler angles, degrees, Kocks */
  double dt;                    /* time increment of the load step       */
  double eps_bbar;              /* b-bar stabilization factor (0), the
                                   global eps_bbar, src/initst.f:537      */
  int asymmetric_assembly;      /* "assembly asymmetric on" (main_data):
                                   full (totdof*totdof, span) element
                                   matrices, column-major per element
                                   (gptns1.f bdbt_asym, tanstf.f:223-225),
                                   mm10 tangents not symmetrized
                                   (mm10_a.f:1165-1166); FP64 and FP32
                                   tangent forms */
  /* UMAT elements (iprops(25) = 8) only; NULL otherwise */
  const double* umat_props;     /* W3G_UMAT_NPROPS*noelem: the element's
                                   material umat values as rknstr loads
                                   them (local_work%umat_props,
                                   src/rknstr.f:1528) */
} w3g_model_desc;

/*
 * Host copies of the blocked element state (module elem_block_data).
 * Any member may be NULL when a call does not move that array.
 */
typedef struct w3g_block_state {
  double* const* history;       /* (hist, ngp, span), state n            */
  double* const* history1;      /* (hist, ngp, span), state n+1          */
  double* const* urcs_n;        /* (9, ngp, span)                        */
  double* const* urcs_n1;       /* (9, ngp, span)                        */
  double* const* eps_n;         /* (6, ngp, span)                        */
  double* const* eps_n1;        /* (6, ngp, span)                        */
  double* const* rot_n1;        /* (9, ngp, span)                        */
  double* const* cep;           /* (21, span, ngp)                       */
  double* const* einfvec;       /* (span, totdof)                        */
  double* const* element_vol;   /* (span)                                */
} w3g_block_state;

/* Scalars drive_eps_sig_internal_forces returns to the Newton driver
   (src/drive_eps_sig_internal_forces.f:210-226, :276-319). */
typedef struct w3g_recover_info {
  double internal_energy;
  double plastic_work;
  double sum_ifv;               /* sum |eleifv|, addifv.f:101-106        */
  long long num_term_ifv;       /* totdof*span summed over blocks        */
  int material_cut_step;
  int first_bad_element;        /* 1-based element of a det[F]<=0 GP, or 0 */
} w3g_recover_info;

typedef struct w3g_context w3g_context;

/* ---- context and model -------------------------------------------- */

/* Creates a context on CUDA device `device` and copies the model tables
   to the device. Replaces the per-run setup that WARP3D does in
   src/reopen.f cdest_init/edest_init and the block allocations in
   src/mod_eleblocks.f. The state arrays start as WARP3D initialises
   them: zeros, with rot_n1 = identity (src/reopen.f:1912-1915). */
int w3g_create(int device, const w3g_model_desc* model, w3g_context** out);
int w3g_destroy(w3g_context* ctx);
const char* w3g_last_error(void);

/* Selects the precision form of the tangent (W3G_TANGENT_*). Every form
   but FP64 writes Ke as float into a separate device array; w3g_tanstf then
   widens to double only when host estiff pointers are given. The tensor-
   core forms (TF32, BF16, and their split X3 variants) cover 8-node and
   20-node bricks, each element matrix with the rigid translations
   projected out after the accumulation; tetrahedra take the FP32 kernel
   in the same call. w3g_tanstf returns W3G_EFATAL if a tensor-core tile's
   bounded wait for its MMAs gave up (that tile's Ke is then NaN). */
int w3g_set_tangent_precision(w3g_context* ctx, int precision);

/* The UMAT compiled into the library describes itself as WARP3D's
   umat_set_features does (src/user_routines_umat.f:35-66): info[0] =
   state variables per material point (the history words of W3G_MAT_UMAT
   blocks), info[1] = 21 symmetric [D] terms, info[2] = 0 when it returns
   unrotated Cauchy stresses (1: Cauchy), info[3] = output states. The
   device UMAT is an Abaqus-style routine (warp3d_gb300/csrc/w3g_umat.cuh);
   a user UMAT replaces it there and the library is rebuilt, as WARP3D
   links user_routines_umat.f into its executable. */
int w3g_umat_features(int* info);

/* Bounded waits of the tensor-core tangent kernels (no WARP3D
   counterpart). Every wait of a kernel for its own copies or MMAs gives up
   after `polls` polls (default W3G_WAIT_LIMIT_DEFAULT; a negative value
   restores it). A wait that gives up ends that CTA's work: no further MMA
   is issued, its copies and MMAs still in flight are waited out (bounded)
   before tensor memory is freed, the element matrices it did not finish
   are NaN and w3g_tanstf returns W3G_EFATAL. With 0 every such wait gives
   up at once, before the first MMA: a driver can exercise its handling of
   that status without any fault on the GPU. */
#define W3G_WAIT_LIMIT_DEFAULT (1ll << 22)
int w3g_set_wait_limit(w3g_context* ctx, long long polls);

/* ---- state transfer (restart, fixtures, output) -------------------- */
int w3g_state_upload(w3g_context* ctx, const w3g_block_state* host);
int w3g_state_download(w3g_context* ctx, const w3g_block_state* host);

/*
 * The element-block section of a WARP3D restart file (replaces, for a
 * driver without WARP3D's own restart code, store_blocks as called by
 * store, src/store.f:329-341, :915-1010; and its readers in src/reopen.f):
 * Fortran sequential unformatted records (4-byte little-endian lengths) of
 * history (state n) and cep per block, then urcs_n, rot_n1 of the geonl
 * blocks, eps_n and element volumes, each array followed by the check
 * record 2147483647 and each section after the first by one more.
 * w3g_store_blocks writes the resident state (append = 1: at the end of an
 * existing file); w3g_reopen_blocks reads it starting at byte `offset`,
 * checks every record length and check record (W3G_EARG otherwise),
 * uploads it with the n+1 arrays equal to the n arrays, as reopen does,
 * and returns the offset after the section in *end_offset (may be NULL).
 */
int w3g_store_blocks(w3g_context* ctx, const char* path, int append);
int w3g_reopen_blocks(w3g_context* ctx, const char* path, long long offset, long long* end_offset);

/* ---- the hot path, host arrays ------------------------------------- */

/* tanstf (src/tanstf.f:17): element tangent stiffnesses for all blocks.
   c, u, du: global coordinate / displacement / increment vectors.
   estiff: nelblk host pointers to (utsz, span) doubles, or NULL to keep
   the matrices resident on the device only. */
int w3g_tanstf(w3g_context* ctx, int step, int iter,
               const double* c, const double* u, const double* du,
               double* const* estiff);

/* drive_eps_sig_internal_forces (src/drive_eps_sig_internal_forces.f:20):
   strains, stresses, material update, [D] storage, element internal
   forces and their assembly into ifv (length nodof, overwritten).
   extrapolated_du follows main_data::extrapolated_du (mnralg.f:255-285). */
int w3g_recover(w3g_context* ctx, int step, int iter, int extrapolated_du,
                const double* c, const double* u, const double* du,
                double* ifv, w3g_recover_info* info);

/* update (src/update.f:73-94): history, strains, stresses n+1 -> n. */
int w3g_update(w3g_context* ctx);

/* How w3g_update moves the converged state to n. W3G_UPDATE_COPY (the
   default) copies n+1 into n, as WARP3D's update does, so both hold the
   same values afterwards. W3G_UPDATE_SWAP exchanges the n and n+1 arrays
   instead (no copy): n then holds the converged state and n+1 the state
   of the step before, until the next recovery overwrites it -- except the
   history of crystal-plasticity (mm10) blocks, which is copied back into
   n+1 because their local solve starts from it. Every array the recovery
   and tangent read is the same in both modes, so results are bitwise
   identical; only a download of the n+1 arrays between an update and the
   next recovery differs. */
#define W3G_UPDATE_COPY 0
#define W3G_UPDATE_SWAP 1
int w3g_set_update_mode(w3g_context* ctx, int mode);

/* ---- the hot path, device-resident arrays --------------------------
   Same work as above on device pointers (c, u, du, ifv of type double*
   on ctx's device) enqueued on `stream` (a cudaStream_t, or NULL for the
   legacy default stream). The call returns after enqueueing; info is
   written to a device buffer and read back by w3g_recover_info_get. */
int w3g_tanstf_dev(w3g_context* ctx, int step, int iter,
                   const void* d_c, const void* d_u, const void* d_du,
                   void* stream);
int w3g_recover_dev(w3g_context* ctx, int step, int iter,
                    int extrapolated_du, const void* d_c, const void* d_u,
                    const void* d_du, void* d_ifv, void* stream);
int w3g_recover_info_get(w3g_context* ctx, w3g_recover_info* info);

/* Device pointer of the resident element stiffnesses: FP64 (utsz, span)
   blocks back to back for W3G_TANGENT_FP64, FP32 for the other forms.
   *count receives the number of values. */
int w3g_estiff_device(w3g_context* ctx, void** d_estiff, long long* count);

/* Number of kernels the last w3g_tanstf/w3g_recover(_dev)/w3g_iteration_dev
   call launched (kernels inside a replayed graph included). */
int w3g_last_launch_count(w3g_context* ctx);

/* ---- batching form (no single WARP3D counterpart) ------------------
   WARP3D runs one element block per OpenMP thread (tanstf.f:80-88,
   drive_eps_sig_internal_forces.f:160-180). Here the work items of all
   blocks, of every element type and size, are either launched per element
   type (W3G_SCHED_PER_TYPE) or taken from a device work queue by one
   persistent launch per phase (W3G_SCHED_PERSISTENT): CTAs resident on
   every SM pull the next items with an atomic counter, heaviest element
   type first (W3G_ORDER_HEAVY_FIRST) or in block order. The schedule
   changes only the order in which element results are produced, never
   their values. */
#define W3G_SCHED_PER_TYPE 0
#define W3G_SCHED_PERSISTENT 1
#define W3G_ORDER_BLOCKS 0
#define W3G_ORDER_HEAVY_FIRST 1

typedef struct w3g_schedule {
  int mode;                  /* W3G_SCHED_*                                */
  int recover_ctas_per_sm;   /* persistent recovery CTAs per SM, 0 = max  */
  int tangent_ctas_per_sm;   /* persistent tangent CTAs per SM, 0 = max   */
  int recover_grain;         /* queue entries taken per fetch (>= 1)       */
  int tangent_grain;
  int order;                 /* W3G_ORDER_*                                */
} w3g_schedule;

int w3g_set_schedule(w3g_context* ctx, const w3g_schedule* sched);
int w3g_get_schedule(w3g_context* ctx, w3g_schedule* sched);

/* One Newton iteration's element work on device pointers: recovery
   (what & W3G_ITER_RECOVER, as w3g_recover_dev) then the tangent
   (what & W3G_ITER_TANGENT, as w3g_tanstf_dev), replayed as one CUDA
   graph. The graph is captured on the first call and again whenever the
   pointers, `what`, the precision or the schedule change; afterwards a
   call costs one small launch (the step/iteration scalars) plus one
   graph launch. */
#define W3G_ITER_RECOVER 1
#define W3G_ITER_TANGENT 2
int w3g_iteration_dev(w3g_context* ctx, int step, int iter, int extrapolated_du, int what,
                      const void* d_c, const void* d_u, const void* d_du, void* d_ifv,
                      void* stream);

/* mm10 Gauss points: local Newton iterations of the last recovery, in
   block / element / Gauss-point order (n = number of mm10 Gauss points).
   The persistent mm10 kernel orders its work queue by these counts
   (W3G_ORDER_HEAVY_FIRST) so that a warp's lanes get similar counts. */
int w3g_local_iterations(w3g_context* ctx, int* counts, int n);

/* Autotuner: times candidate schedules (launch mode, persistent CTAs per
   SM, queue grain, item order) on this model with the given inputs,
   recovery and tangent separately, `reps` timed runs each, and keeps the
   fastest. Runs the iteration's element work several times; afterwards
   the element state is that of one w3g_iteration_dev call with these
   arguments. *best (may be NULL) receives the chosen schedule,
   *best_ms (may be NULL) its recovery + tangent time. */
int w3g_autotune(w3g_context* ctx, int step, int iter, int extrapolated_du,
                 const void* d_c, const void* d_u, const void* d_du, void* d_ifv,
                 void* stream, int reps, w3g_schedule* best, double* best_ms);

/* ---- global stiffness on the device and its solve -------------------
   The step after the element path in WARP3D's Newton iteration:
   drive_assemble_solve (src/drive_assemble_solve.f:11) builds the
   sparsity of the equilibrium equations once (ds_setup_sparsity_local,
   :358), assembles the element stiffnesses row by row (assem_by_row,
   src/assemble_code.f:659; a thread builds a whole equation row) and
   calls a sparse solver (direct, or hypre's PCG, :990). Here the pattern
   and an (element, local pair) gather map are built once per context; the
   assembly reads the resident element stiffnesses (FP64, or the FP32 of
   the precision forms) on the device, summing every coefficient's
   contributions in a fixed order (bitwise reproducible), into a CSR
   matrix over all nodof dofs (full rows, both triangles, 0-based).
   The solve is a Jacobi-preconditioned conjugate gradient restricted to
   the free dofs (fixed_mask[dof] != 0: constrained, solution 0 there),
   with deterministic reductions; its iterations replay as CUDA graphs. */
typedef struct w3g_csr w3g_csr;

int w3g_csr_create(w3g_context* ctx, w3g_csr** out);
int w3g_csr_destroy(w3g_csr* csr);
/* sizes and device pointers: rowptr (n+1, int32), colind (nnz, int32),
   values (nnz, double); any output may be NULL */
int w3g_csr_info(w3g_csr* csr, int* n, long long* nnz, void** d_rowptr,
                 void** d_colind, void** d_values);
/* The matrix product and preconditioner use the node blocks (a warp
   reads a node's three rows with one set of column indices; inverse 3x3
   diagonal blocks) when the three dofs of every node share their column
   pattern, the default; enable = 0 selects the row kernels and the
   diagonal preconditioner. Returns 1 when the node kernels are in use. */
int w3g_csr_set_node_blocks(w3g_csr* csr, int enable);
/* assembles the values from ctx's current element stiffnesses */
int w3g_csr_assemble_dev(w3g_csr* csr, void* stream);
/* host copies of the pattern and values (arrays of n+1, nnz, nnz) */
int w3g_csr_download(w3g_csr* csr, int* rowptr, int* colind, double* values);

/* Solves K_ff x_f = b_scale * b_f (device vectors of nodof doubles; the
   mask is nodof bytes) to ||r|| <= rtol ||b_f|| in at most maxit
   iterations; x = 0 on constrained dofs. Returns 0 when converged,
   W3G_PCG_MAXIT when not within maxit, W3G_PCG_BREAKDOWN when p.Kp <= 0
   (the matrix is not positive definite on the free dofs); *iters and
   *relres (either may be NULL) receive the iterations and ||r|| / ||b_f||.
   Blocks until the solve ends; ordered after prior work on `stream`. */
#define W3G_PCG_MAXIT 1
#define W3G_PCG_BREAKDOWN 2
int w3g_pcg_dev(w3g_csr* csr, const void* d_fixed_mask, const void* d_b,
                double b_scale, void* d_x, double rtol, int maxit,
                void* stream, int* iters, double* relres);

/* Newton convergence norms as one device reduction (the residual-force
   norm of cvtest, src/cvtest.f:20-60): d_out[0] = ||v_f||^2 over the free
   dofs, d_out[1] = ||v||^2 over all dofs (device doubles). */
int w3g_residual_norms_dev(w3g_csr* csr, const void* d_v, const void* d_fixed_mask,
                           void* d_out, void* stream);

/* d_out[0] = sum over the free dofs of a_i b_i (device doubles), one
   deterministic device reduction: the s-value of the line search
   (mnralg_ls_get_s, src/mnralg.f:1135-1158, s = -sum res idu over the
   unconstrained dofs) with a = -res (the internal forces under
   displacement control) and b = the Newton correction idu. */
int w3g_free_dot_dev(w3g_csr* csr, const void* d_a, const void* d_b, const void* d_fixed_mask,
                     void* d_out, void* stream);

/* One Newton iteration of a device-resident driver as ONE CUDA graph (the
   body of mnralg's iteration loop, src/mnralg.f:435-569, with the solve of
   drive_assemble_solve): the solve of K_ff d = -ifv_f by Jacobi-PCG as a
   device-side loop (a conditional graph node over batches of 16 CG
   iterations: no host round trip inside the solve), d_d = d, du += d, the
   element work at the new du (recovery for (step, iter), then the tangent
   for the next iteration; the context's precision and schedule), the
   assembly of K and cvtest's two norms of the new ifv into d_norms (2
   device doubles). The host waits once, for the scalars returned here:
   the PCG's iteration count and relative residual, the recovery's status
   (0, or 1/2 = step cut as w3g_recover) and the norms (norms[0] = ||ifv_f||^2,
   norms[1] = ||ifv||^2, host). The graph is built on the first call and
   rebuilt when a pointer, the precision, the schedule or the wait limit
   changes. Returns 0, W3G_PCG_MAXIT or W3G_PCG_BREAKDOWN as w3g_pcg_dev. */
int w3g_newton_iteration_dev(w3g_csr* csr, int step, int iter, int extrapolated_du, const void* d_c,
                             const void* d_u, void* d_du, void* d_ifv, const void* d_fixed_mask, void* d_d,
                             double rtol, int maxit, void* d_norms, void* stream, int* pcg_iters,
                             double* pcg_relres, int* recover_status, double* norms);

/* ---- internal-force assembly without device allocation --------------
   No counterpart in the reference. For callers that cannot allocate
   device memory -- a Fortran code whose device arrays come from a pool or
   a framework that owns the allocator, or a run where allocation is
   forbidden after start-up -- and so cannot create a w3g_context: given
   element internal forces d_einfvec (all blocks back to back, each
   (span, totdof)) and d_edest (each (totdof, span), 1-based) on the
   current device, writes the nodal vector d_ifv (nodof, zeroed first)
   and *d_sum_ifv = sum |einfvec| (addifv, src/addifv.f:86-124).
   elblks (3*nelblk) and totdof (nelblk) are host arrays.
   Allocates nothing: its scratch is a fixed static device array for at
   most W3G_NOALLOC_MAX_BLOCKS element blocks (larger models: W3G_EARG).
   The first call on a device looks up the array's address and caches it
   for the device's primary context (stale after cudaDeviceReset: do not
   call again on that device afterwards). Every call copies the host
   tables and waits for its work, so no call may be made while `stream`
   is being captured (W3G_EARG). Calls share the array: calls that
   overlap on the GPU race and must be serialised. edest entries outside
   1..nodof are skipped and reported as W3G_EARG with the first block that
   holds one. Returns after the work ends. */
#define W3G_NOALLOC_MAX_BLOCKS 65536
int w3g_assemble_ifv_noalloc(int nelblk, const int* elblks, const int* totdof,
                             int nodof, const double* d_einfvec,
                             const int* d_edest, double* d_ifv,
                             double* d_sum_ifv, void* stream);

/* ---- timing and output checks --------------------------------------
   Host wall time of the entry points, accumulated per context under
   WARP3D's own timing categories (thyme calc 2 "tangent stiffness" and
   calc 6 "sig-eps & internal force", src/thyme.f:15-35, printed by
   src/outime.f); for the *_dev entry points this is the enqueue time. Each
   call is also an NVTX range named after its entry point. */
typedef struct w3g_timers {
  double tangent_s;            /* w3g_tanstf, w3g_tanstf_dev              */
  double recover_s;            /* w3g_recover, w3g_recover_dev            */
  double update_s;             /* w3g_update                              */
  long long tangent_calls, recover_calls, update_calls;
} w3g_timers;
int w3g_timers_get(w3g_context* ctx, w3g_timers* t);
int w3g_timers_reset(w3g_context* ctx);

/* Number of non-finite values (NaN, Inf) in the resident outputs:
   urcs_n1, eps_n1, history1, einfvec and the element stiffnesses of the
   current precision. WARP3D has no such scan (a NaN input travels through
   its element routines without a step cut, as it does here); a driver can
   call this after a recovery or a tangent. */
int w3g_check_finite(w3g_context* ctx, long long* bad);

/* Name of CUDA device `device` (NUL-terminated, truncated to len), e.g.
   for keying an autotuning cache. */
int w3g_device_name(int device, char* name, int len);

/* ---- measurement helper (no WARP3D counterpart) ---------------------
   Sustained FP64 FMA throughput of `device` in TFLOP/s (2 flops per FMA),
   the roofline denominator of the FP64-bound element kernels. */
int w3g_measure_fp64_peak(int device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* W3G_H */
