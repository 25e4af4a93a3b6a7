/*
 * euler2d.h - C ABI of the GB300 (sm_103a) 2D Euler MUSCL finite-volume solver.
 *
 * This is the drop-in boundary for pyHype's hot path: the per-block residual
 * (FiniteVolumeMethod.dUdt), the explicit Runge-Kutta driver
 * (ExplicitRungeKutta.integrate), the ghost/halo + boundary-condition fill
 * (Blocks.apply_boundary_condition) and the CFL time step (Solver.get_dt).
 * Everything is plain C: integers, doubles, pointers and sizes.  No torch or CUDA
 * runtime types appear in the signatures (streams are passed as void*).
 *
 * Memory model.  e2d_create copies the block table and the geometry planes from
 * host memory into device memory owned by the handle; all blocks of a problem live
 * in one GPU's HBM.  States cross the boundary either as host buffers
 * (e2d_set_state / e2d_get_state) or as device buffers owned by the caller
 * (the *_device variants).  A state is structure-of-arrays: 4 planes (rho, rho*u,
 * rho*v, E) of `ncells` doubles each, block b occupying
 * [cell_offset[b], cell_offset[b] + nx*ny) of every plane in row-major (y, x) order.
 *
 * Threading.  One host thread drives one handle; calls on a handle are
 * stream-ordered on the handle's stream.  Handles are independent.
 *
 * Errors.  Every call returns 0 on success or a negative E2D_ERR_* code;
 * e2d_last_error() returns a thread-local message for the last failure.
 */
#ifndef EULER2D_H
#define EULER2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define E2D_API __attribute__((visibility("default")))
#else
#define E2D_API
#endif

#define E2D_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------- */
#define E2D_OK 0
#define E2D_ERR_INVALID (-1)      /* bad argument / inconsistent block table      */
#define E2D_ERR_CUDA (-2)         /* CUDA runtime error (message in last_error)   */
#define E2D_ERR_UNREALIZABLE (-3) /* rho <= 0 or E <= 0 after a step              */
#define E2D_ERR_TIMEOUT (-4)      /* a bounded device wait gave up                */
#define E2D_ERR_UNSUPPORTED (-5)  /* option not built into this library           */
#define E2D_ERR_NOMEM (-6)        /* device allocation failed                     */

/* ---- scheme choices (string keys of pyhype/solver_config.py:64-92) ----------- */
enum e2d_flux { E2D_FLUX_ROE = 0, E2D_FLUX_HLLL = 1, E2D_FLUX_HLLE = 2 };
enum e2d_limiter {
  E2D_LIM_VENKATAKRISHNAN = 0,
  E2D_LIM_BARTH_JESPERSEN = 1,
  E2D_LIM_VAN_ALBADA = 2,
  E2D_LIM_VAN_LEER = 3
};
enum e2d_recon { E2D_RECON_CONSERVATIVE = 0, E2D_RECON_PRIMITIVE = 1 };
enum e2d_precision { E2D_FP64 = 0, E2D_FP32 = 1 };

/* ---- block sides: how the ghost cells and the outside flux state are formed --- */
enum e2d_side_kind {
  /* inter-block side (BC None + neighbour): ghost = the neighbour's adjacent cells;
     the outside state of the boundary flux is that ghost cell average
     (pyhype/blocks/ghost.py:187-216, pyhype/fvm/base.py:305-325)                  */
  E2D_SIDE_NEIGHBOR = 0,
  /* BC None and no neighbour: ghost = copy of the block's own boundary cells,
     outside state = that copy (first order)                                        */
  E2D_SIDE_COPY = 1,
  /* "Reflection" / "Slipwall": normal velocity flipped in the wall frame, applied to
     the ghost (conservative) and to the block's own limited boundary-face state
     (pyhype/boundary_conditions/funcs.py:28-43)                                    */
  E2D_SIDE_REFLECT = 2,
  /* "OutletDirichlet": no-op BC; ghost = own boundary cells, outside state = own
     limited boundary-face state (pyhype/blocks/ghost.py:250-254)                   */
  E2D_SIDE_OUTLET = 3,
  /* fixed state (PrimitiveDirichletBC with a uniform state): ghost and outside
     state are constants given per side in E2DBlock.dirichlet_*                      */
  E2D_SIDE_DIRICHLET = 4,
  /* per-cell mix of REFLECT and DIRICHLET along one side, with an optional moving
     switch point (double-Mach-reflection walls, inflow and the exact-shock top
     boundary); parameters in E2DBlock.mixed                                         */
  E2D_SIDE_MIXED = 5
};
enum e2d_side { E2D_E = 0, E2D_W = 1, E2D_N = 2, E2D_S = 3 };

/* Per-cell switch along a MIXED side: cells whose centroid coordinate along the side
   (x for N/S sides, y for E/W sides) is below  x0 + speed * t  use kind_below, the
   others kind_above (each E2D_SIDE_REFLECT or E2D_SIDE_DIRICHLET).  t is the
   solver time at the start of the step (the reference passes no stage time to its
   boundary conditions).                                                            */
typedef struct {
  double x0;
  double speed;
  int32_t kind_below;
  int32_t kind_above;
  double ghost_below[4];   /* conservative ghost state for a DIRICHLET cell   */
  double face_below[4];    /* reconstruction-variable outside state           */
  double ghost_above[4];
  double face_above[4];
} E2DMixedSide;

typedef struct {
  int32_t nx, ny;
  int32_t is_cartesian;      /* pyhype/blocks/quad_block.py:96-113               */
  int32_t side_kind[4];      /* e2d_side_kind per E, W, N, S                     */
  int32_t neighbor[4];       /* block index for E2D_SIDE_NEIGHBOR, else -1       */
  int32_t instance;          /* independent-problem id (batched runs), else 0    */
  int64_t cell_offset;       /* start of this block in every cell plane          */
  int64_t vface_offset;      /* start in the vertical-face planes, ny*(nx+1)      */
  int64_t hface_offset;      /* start in the horizontal-face planes, (ny+1)*nx    */
  double dirichlet_ghost[4][4]; /* per side: conservative ghost state (DIRICHLET) */
  double dirichlet_face[4][4];  /* per side: outside state in recon variables    */
  E2DMixedSide mixed[4];
  /* centroid coordinate along each side for MIXED sides, host pointer to
     ny (E/W) or nx (N/S) doubles; ignored otherwise                              */
  const double* side_coord[4];
} E2DBlock;

typedef struct {
  int32_t nblocks;
  int32_t flux;              /* e2d_flux     */
  int32_t limiter;           /* e2d_limiter  */
  int32_t recon;             /* e2d_recon    */
  int32_t precision;         /* e2d_precision */
  int32_t ninstances;        /* >= 1; per-instance dt when > 1 */
  double gamma;              /* 1.4                                     */
  double gm1;                /* gamma - 1 as formed by the host (1.4-1) */
  double cfl;
  int32_t nqp;               /* face quadrature points per face: 1 (0 = 1), 2, 3
                                (SolverConfig.fvm_num_quadrature_points)          */
  int32_t reserved;
} E2DConfig;

/* Geometry planes (host pointers), each the concatenation over blocks.
   Cell planes hold sum(nx*ny) doubles, vertical-face planes sum(ny*(nx+1)),
   horizontal-face planes sum((ny+1)*nx).                                          */
enum e2d_cell_plane {
  E2D_G_A = 0,      /* cell area                                               */
  E2D_G_INV_A,      /* 1.0 / A                                                 */
  E2D_G_HX_E,       /* quadrature point - centroid, x, east side               */
  E2D_G_HX_W,
  E2D_G_HX_N,
  E2D_G_HX_S,
  E2D_G_HY_E,       /* quadrature point - centroid, y                          */
  E2D_G_HY_W,
  E2D_G_HY_N,
  E2D_G_HY_S,
  E2D_G_CFL_DX,     /* east-west face-midpoint distance                        */
  E2D_G_CFL_DY,     /* north-south face-midpoint distance                      */
  E2D_G_NCELL
};
enum e2d_face_plane {
  E2D_F_L = 0,      /* face length                                              */
  E2D_F_LC,         /* L * cos(theta)                                          */
  E2D_F_LS,         /* L * sin(theta)                                          */
  E2D_F_COS,        /* cos(theta)                                              */
  E2D_F_SIN,        /* sin(theta)                                              */
  E2D_F_NFACE
};
#define E2D_MAX_QP 3
typedef struct {
  const double* cell[E2D_G_NCELL];
  const double* vface[E2D_F_NFACE];
  const double* hface[E2D_F_NFACE];
  /* With nqp > 1: quadrature point - centroid of point q (in the order of
     pyhype/mesh/quadratures.py:33-37) per side, [q][0..3] = x for E, W, N, S and
     [q][4..7] = y, cell planes; unused (NULL) with one point, whose offsets are the
     E2D_G_HX_* / E2D_G_HY_* planes.                                                */
  const double* qp[E2D_MAX_QP][8];
} E2DGeometry;

/* Result of the positivity check (pyhype/solvers/Euler2D.py:144-152). */
typedef struct {
  int32_t ok;           /* 1 if every cell has rho > 0 and E > 0              */
  int32_t block;        /* first offending block, -1 if ok                    */
  int64_t cell;         /* first offending cell index within that block       */
  int64_t nbad;         /* number of offending cells                          */
} E2DRealizability;

/* Optional per-operator outputs of one residual evaluation (device pointers, NULL to
   skip).  Cell quantities are 4 cell planes (reconstruction variables); face
   quantities are 4 planes over all vertical (ny*(nx+1) per block) or horizontal
   ((ny+1)*nx per block) faces.                                                     */
typedef struct {
  double* gx;           /* Green-Gauss gradient (greengauss.py:110-155)            */
  double* gy;
  double* phi;          /* limiter value (limiters/base.py:147-187)                */
  double* vL;           /* left/right primitive states fed to the x-sweep flux,     */
  double* vR;           /*   rotated into the face frame (fvm/base.py:327-390)      */
  double* hL;           /* same for the y-sweep (fvm/base.py:392-486)               */
  double* hR;
  double* vflux_raw;    /* flux function output in the face frame                   */
  double* hflux_raw;
  double* vflux;        /* flux rotated back to the x/y frame                        */
  double* hflux;
} E2DDebug;

typedef struct E2DSolver* E2DHandle;

E2D_API int e2d_abi_version(void);
E2D_API const char* e2d_last_error(void);

/* ---- lifecycle ---------------------------------------------------------------- */
/* Replaces Blocks.build + QuadBlock construction (pyhype/blocks/base.py:515-572). */
E2D_API int e2d_create(const E2DConfig* cfg, const E2DBlock* blocks, const E2DGeometry* geo,
               E2DHandle* out);
E2D_API int e2d_destroy(E2DHandle h);
/* Use a caller stream (cudaStream_t as void*); NULL selects the handle's own. */
E2D_API int e2d_set_stream(E2DHandle h, void* stream);
E2D_API int64_t e2d_num_cells(E2DHandle h);

/* ---- state transfer ------------------------------------------------------------- */
E2D_API int e2d_set_state(E2DHandle h, const double* host_soa);
E2D_API int e2d_get_state(E2DHandle h, double* host_soa);
E2D_API int e2d_set_state_device(E2DHandle h, const double* dev_soa);
E2D_API int e2d_get_state_device(E2DHandle h, double* dev_soa);

/* ---- time integration ---------------------------------------------------------- */
/* Butcher rows of ExplicitRungeKutta (pyhype/time_marching/explicit_runge_kutta.py:
   91-274): nstages rows, row s holds a[s][0..s]; row-major nstages x nstages.     */
E2D_API int e2d_set_tableau(E2DHandle h, int32_t nstages, const double* a);
/* Solver.get_dt without the t_final clamp: CFL * min over all cells of all blocks
   (pyhype/solvers/base.py:114-136, pyhype/blocks/quad_block.py:423-436).
   Batched problems write one value per instance.                                  */
E2D_API int e2d_compute_dt(E2DHandle h, double* dt_host);
/* One ExplicitRungeKutta.integrate(dt) including the ghost/BC refresh after every
   stage; t is the solver time at the start of the step (moving BCs).              */
E2D_API int e2d_step(E2DHandle h, double dt, double t);
/* The Euler2D._solve loop (pyhype/solvers/Euler2D.py:175-216): dt -> clamp to
   t_final - t -> step -> realizability, until t >= t_final or max_steps.  Time is
   non-dimensional (t_final already multiplied by a_inf).  *t_inout is updated.
   With several instances, *t_inout is ignored on entry (every instance continues
   from its own time, 0 after e2d_create) and receives instance 0's time; max_steps
   counts the steps of this call per instance.
   Returns E2D_ERR_UNREALIZABLE (with *real filled) if a step produced rho<=0 or
   E<=0.                                                                            */
E2D_API int e2d_run(E2DHandle h, double* t_inout, double t_final, int32_t max_steps,
            int32_t* steps_done, E2DRealizability* real);
E2D_API int e2d_check_realizable(E2DHandle h, E2DRealizability* out);
/* Solver time and steps taken of every instance (batched problems advance each
   instance with its own CFL dt); arrays of E2DConfig.ninstances entries.        */
E2D_API int e2d_instance_times(E2DHandle h, double* t_out, int32_t* steps_out);
/* Conserved totals of the current state: totals[4 q + v] = sum over the cells of
   instance q of A * U_v (mass, x and y momentum, energy), accumulated in FP64 on
   either path in a fixed order (reproducible run to run).  No counterpart in the
   reference; the FP32 form's conservation drift is stated against these.        */
E2D_API int e2d_totals(E2DHandle h, double* totals);

/* ---- per-operator entry points (parity testing) ---------------------------------- */
/* dUdt of the current state (FiniteVolumeMethod.dUdt, pyhype/fvm/base.py:108-139)
   at solver time t (time-dependent sides) into a caller device buffer of 4 cell
   planes; optional intermediates in dbg.                                           */
E2D_API int e2d_residual(E2DHandle h, double t, double* dudt_dev, const E2DDebug* dbg);
/* Ghost layer of every block at solver time t, in the reconstruction variables
   (Blocks.apply_boundary_condition followed by the ghost conversion of
   ReconstructionBlock.from_block: pyhype/blocks/base.py:448-471,
   pyhype/blocks/ghost.py:149-216, pyhype/blocks/quad_block.py:120-134).  ghosts_dev
   is a caller device buffer of 4 planes of nghost = sum over blocks of 2 (nx + ny)
   doubles; block b's layer starts at the sum of the earlier blocks' lengths and
   holds E (ny cells, south to north), W (ny), N (nx, west to east), S (nx).  The
   kernels form these values on the fly; this entry point writes them out.          */
E2D_API int e2d_ghost_layer(E2DHandle h, double t, double* ghosts_dev);

/* ---- adjoint (reverse mode) -------------------------------------------------------
   No counterpart in the reference (it has no differentiation); the forward steps are
   the functions above.  Roe, HLLL or HLLE flux, one instance, one face quadrature
   point; FP64 or FP32 path, any limiter, reconstruction type, side kind and explicit
   tableau.  Subgradients: min/max take the operand the forward selects (the wave-speed
   bounds of HLLL/HLLE included), Harten's fix and the HLL branches the branch taken,
   HLLL's alpha = max(0, 1 - |r|/k) nothing where it is 0, a norm nothing at a zero
   vector, the slope's davg == 0 branch is constant, a clipped negative limiter value
   passes nothing back.                                                             */

/* Objective J = sum over steps n of dt_n * P(U^{n+1}), where P(U) sums, over the cells
   along side `side` (e2d_side) of block `block`, the cell pressure times the length
   of the cell's boundary face.                                                      */
typedef struct {
  int32_t block;
  int32_t side;
} E2DPressureObjective;

/* out_dev = (dR/dU)^T lam_dev at the current state and solver time t, R the residual
   of e2d_residual; both 4 cell planes on the device.                               */
E2D_API int e2d_residual_vjp(E2DHandle h, double t, const double* lam_dev, double* out_dev);
/* Recorded forward pass: nsteps RK steps from the current state at time t0, keeping
   the state every ckpt_every steps.  dts_in == NULL takes each step's CFL dt (no
   t_final clamp) and writes the schedule to dts_out (nsteps entries, may be NULL);
   otherwise the given schedule is replayed (finite differences at a frozen dt).
   *J_out receives J.  Device memory: ceil(nsteps/ckpt_every) states plus, for
   ckpt_every steps x stages, one state and one set of face states.               */
E2D_API int e2d_adjoint_forward(E2DHandle h, double t0, int32_t nsteps, int32_t ckpt_every,
                                const E2DPressureObjective* obj, const double* dts_in, double* dts_out,
                                double* J_out);
/* Reverse pass of the last recorded forward pass at its dt schedule: grad_dev (4 cell
   planes, device) = dJ/dU^0.  Segments between checkpoints are recomputed.  The
   current state is U^N afterwards.                                                  */
E2D_API int e2d_adjoint_backward(E2DHandle h, double* grad_dev);

/* ---- allocation-free CFL time step ----------------------------------------------
   No counterpart in the reference.  For callers that may not allocate device
   memory: an application that hands all of its GPU memory to its own pool
   allocator and forbids cudaMalloc/cudaFree once it is running (an allocation
   synchronizes the device and fragments the pool), so it cannot create a handle.
   From caller-owned device buffers - the SoA state (4 planes of ncell doubles) and
   the CFL_DX / CFL_DY geometry planes - it computes what e2d_compute_dt computes
   for a single-instance problem: *dt_host = cfl * min over cells of
   min(dx/(|u|+a), dy/(|v|+a)), bit for bit.  Its scratch is a file-scope device
   array of E2D_NOALLOC_MAX_CELLS/256 + 1 eight-byte words (512 KiB) that every GPU
   loading the library keeps until the process exits; ncell above
   E2D_NOALLOC_MAX_CELLS returns E2D_ERR_INVALID.  The first call on a device looks
   up that array's device address (a one-time set-up); make that first call before
   any stream capture begins.  All calls share the array and each overwrites the part
   it uses: calls that overlap on the GPU (different streams or threads) race.  Runs
   on `stream` (NULL = legacy default stream); every call is a blocking host call: it
   copies the result into host memory and synchronizes `stream` before it returns.
   A CUDA error already pending on the calling thread is reported (E2D_ERR_CUDA, its
   text in e2d_last_error) and left in place; nothing is launched then.            */
#define E2D_NOALLOC_MAX_CELLS 16777216
E2D_API int e2d_compute_dt_noalloc(const double* dev_state, int64_t ncell, const double* dev_cfl_dx,
                                   const double* dev_cfl_dy, double gamma, double gm1, double cfl,
                                   void* stream, double* dt_host);

#ifdef __cplusplus
}
#endif
#endif /* EULER2D_H */
