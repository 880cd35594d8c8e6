/*
 * rkdg_gpu.h — C ABI of the GB300 (sm_103a) RKDG hot path.
 *
 * This is the drop-in boundary for the reference's explicit DG right-hand
 * side, limiter and Runge-Kutta stage loop.  Every entry point takes plain
 * pointers and sizes; state vectors are DEVICE pointers unless a name says
 * "host".  State layout is the reference's (MFEM Ordering::byNODES, main.cpp:
 * 119-141): x[k*NDofs + e*nd + i] for equation k, element e, node i, i.e.
 * structure-of-arrays by variable, element-contiguous inside a variable.
 *
 * Every call returns an rkdg_status.  A context owns one CUDA stream, all
 * device tables and all scratch buffers.  A context is not thread-safe;
 * distinct contexts are independent.  There are no process globals: the
 * physics constants the reference keeps in globals (main.cpp:39-56) live in
 * the context.
 */
#ifndef RKDG_GPU_H
#define RKDG_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rkdg_ctx rkdg_ctx;

typedef enum {
  RKDG_OK = 0,
  RKDG_ERR_INVALID = 1,      /* bad argument or call order */
  RKDG_ERR_UNPHYSICAL = 2,   /* a Riemann solver saw a non-physical state; the
                                reference exits here (face_integrator.cpp:214-218) */
  RKDG_ERR_CUDA = 3,         /* a CUDA runtime call failed */
  RKDG_ERR_NOMESH = 4,       /* no mesh uploaded */
  RKDG_ERR_TIMEOUT = 5,      /* a bounded device wait gave up */
  RKDG_ERR_UNSUPPORTED = 6,  /* element type / order / geometry not supported */
  RKDG_ERR_ALLOC = 7,        /* device allocation failed */
  RKDG_ERR_NOT_FOUND = 8     /* the CUDA extension or a device is missing */
} rkdg_status;

/* Geometry codes follow MFEM's Geometry::Type numbering. */
enum { RKDG_GEOM_TRIANGLE = 2, RKDG_GEOM_SQUARE = 3, RKDG_GEOM_CUBE = 5 };
enum { RKDG_RS_RUSANOV = 0, RKDG_RS_LLF = 1, RKDG_RS_HLL = 2, RKDG_RS_HLLC = 3 };
enum { RKDG_AVG_TRRS = 0, RKDG_AVG_EINFELDT = 1 };
enum {
  RKDG_BC_SLIP = 0,             /* boundary_integrator_slip.cpp:7-17 */
  RKDG_BC_OPEN = 1,             /* "outlet", boundary_integrator_open.cpp:9-12 */
  RKDG_BC_FIXED_ROTATED = 2,    /* BoundaryIntegratorConstant, boundary_integrator_constant.cpp:8-20 */
  RKDG_BC_SUPERSONIC_INLET = 3, /* boundary_integrator_supersonic_inlet.cpp:8-19 */
  RKDG_BC_WALL = 4,             /* boundary_integrator_wall.cpp:7-17 (same as slip) */
  RKDG_BC_SUBSONIC_INLET = 5,   /* boundary_integrator_subsonic_inlet.cpp:10-19:
                                   2 * fixed - own in the rotated frame */
  /* perfect-gas ghost states; state = {pTot, TTot} / {pFix, TTot} / {pFix} /
   * {pTot, TFix} in its first entries (an array of neq values): */
  RKDG_BC_SUBSONIC_INLET_TOTAL_PRESSURE = 6, /* ..._subsonic_inlet_total_pressure.cpp:10-40 */
  RKDG_BC_SUBSONIC_INLET_FIXED_PRESSURE = 7, /* ..._subsonic_inlet_fixed_pressure.cpp:10-36 */
  RKDG_BC_FIXED_PRESSURE_OUTLET = 8,         /* boundary_integrator_open_fixed_pressure.cpp:10-30 */
  RKDG_BC_TOTAL_PRESSURE_OUTLET = 9,         /* boundary_integrator_open_total_pressure.cpp:10-40;
                                                m.n uses the normal's own components */
  /* boundary_integrator_char_outlet.cpp:14-57; state = the outer
   * conservative state.  The reference's ghost vector enters its
   * computeRightState unassigned (the previous boundary point's ghost state,
   * uninitialised memory at the first); here it enters as the interior
   * state at every point. */
  RKDG_BC_CHAR_OUTLET = 10
};
enum { RKDG_LIM_FINDIFF = 0, RKDG_LIM_MULTI = 1 };
/* RKDG_IND_SHU: IndicatorShu (indicator_shu.cpp:13-74) with the extrapolated
 * stencil averages of averager.cpp:154-273; FinDiff limiter only (with Multi
 * the reference multiplies by a per-cell factor the Shu indicator never
 * writes: RKDG_ERR_UNSUPPORTED). */
enum { RKDG_IND_NOWHERE = 0, RKDG_IND_EVERYWHERE = 1, RKDG_IND_BJ = 2, RKDG_IND_SHU = 3 };
enum { RKDG_FUN_BJ = 0, RKDG_FUN_VENKATAKRISHNAN = 1, RKDG_FUN_MICHALAK = 2 };
/* flags of rkdg_set_limiter: 0 reproduces the shipped reference.
 * RKDG_QUIRK_MULTIPLIER_ONCE applies the multiplier once instead of nd times;
 * RKDG_LIMITER_LINEARIZE is the reference's "linearize" option of the Multi
 * limiter (limiter_multiplier.cpp:101-178, case_manager.cpp:551-554): quads
 * and hexes of order 1 (its point rule has fewer points than nodes above
 * order 1: RKDG_ERR_UNSUPPORTED), a no-op on triangles. */
enum { RKDG_QUIRK_MULTIPLIER_ONCE = 1, RKDG_LIMITER_LINEARIZE = 2 };
enum { RKDG_FP64 = 0, RKDG_FP32_BULK = 1 };

/* Mesh as the host (MFEM) sees it after every adapt.  elem_vertices are
 * topological vertex ids in MFEM local order (periodic meshes share ids
 * across the periodic seam); elem_coords are each element's own corner
 * coordinates in the same order; boundary faces carry 1-based attributes. */
typedef struct {
  int dim;                   /* 2 or 3 */
  int geom;                  /* RKDG_GEOM_* */
  int order;                 /* polynomial order p of DG_FECollection(p, dim) */
  int num_elements;
  const int* elem_vertices;  /* [num_elements][verts per element] */
  const double* elem_coords; /* [num_elements][verts per element][dim] */
  int num_bdr;
  const int* bdr_vertices;   /* [num_bdr][verts per face] */
  const int* bdr_attr;       /* [num_bdr] */
} rkdg_mesh_desc;

/* ---- context ---------------------------------------------------------- */
int rkdg_create(rkdg_ctx** out, int device);
int rkdg_destroy(rkdg_ctx* ctx);
/* Message and offending element / face id of the last error. */
const char* rkdg_last_error(rkdg_ctx* ctx, long long* where);
/* Use an external cudaStream_t (NULL = the context's own stream). */
int rkdg_set_stream(rkdg_ctx* ctx, void* cuda_stream);
int rkdg_synchronize(rkdg_ctx* ctx);

/* ---- setup -------------------------------------------------------------
 * Replaces the RiemannSolver factory (case_manager.cpp:523-543) and the
 * physics globals (case_manager.cpp:84-101). */
int rkdg_set_physics(rkdg_ctx* ctx, int rsolver, int averaging, double gamma,
                     double covolume, double gas_constant);
/* Replaces FE_Evolution::UpdateInverseMassMatrix / UpdateAfluxPointer
 * (fe_evolution.hpp:78-81) and the integrator set-up of main.cpp:148-164:
 * builds every device face / element / stencil table.  Idempotent; call it
 * after every AMR adapt (main.cpp:610-611).  Nonconforming meshes (hanging
 * vertices left by the reference's NC refinement, any number of levels):
 * a face that no second element shares and no boundary face lists is
 * integrated as MFEM does -- each slave face from its fine element against
 * the coarse element across, the master face not at all.  Such a face must
 * lie inside a face of the element across it, or be covered by such faces,
 * else RKDG_ERR_INVALID (a hole; also a hanging face across a periodic seam).
 * Elements: affine triangles, parallelograms and parallelepipeds, and
 * general (bilinear) quadrilaterals; non-affine hexahedra return
 * RKDG_ERR_UNSUPPORTED, as do the Shu indicator and hanging faces on
 * non-parallelogram quadrilaterals.
 * Limiters see the elements across hanging faces as stencil cells and
 * evaluate indicator points on the element's own slave and master faces
 * (limiter.cpp:95-245); the adjoint covers them too.  Batched problems on
 * such meshes return RKDG_ERR_UNSUPPORTED. */
int rkdg_upload_mesh(rkdg_ctx* ctx, const rkdg_mesh_desc* mesh);
/* Deviations from the shipped reference, off by default.
 * RKDG_QUIRK_HLLC_NEGATIVE_SPEED_OK: the reference treats any negative face
 * wave speed as a non-physical state and exits (face_integrator.cpp:214-218),
 * which also fires on HLLC's signed max(SL, SR) (rs_hllc.cpp:98) in
 * supersonic flow against the face normal; with this flag only the -1 of a
 * non-physical state is an error. */
/* RKDG_QUIRK_NO_INITIAL_LIMIT: rkdg_run and rkdg_batch_run step the state as
 * given.  By default they first limit it once, as the reference limits the
 * projected initial solution before its time loop (main.cpp:264-265); set the
 * flag to continue a run from a state that was already limited. */
enum { RKDG_QUIRK_HLLC_NEGATIVE_SPEED_OK = 1, RKDG_QUIRK_NO_INITIAL_LIMIT = 2 };
int rkdg_set_solver_quirks(rkdg_ctx* ctx, int flags);
/* Replaces CaseManager::addBoundaryIntegrators (case_manager.cpp:614-820)
 * for one boundary attribute.  state: conservative variables or NULL. */
int rkdg_set_bc(rkdg_ctx* ctx, int attr, int type, const double* state);
/* Replaces CaseManager::loadLimiter (case_manager.cpp:545-612). */
int rkdg_set_limiter(rkdg_ctx* ctx, int limiter, int indicator, int function,
                     int last_hope, int quirk_flags);
/* Replaces the ExplicitRKLimitedSolver constructor arguments
 * (rk_explicit_limited.hpp:46-48, tableaux case_manager.cpp:822-895):
 * MFEM lower-triangular packing a[s*(s-1)/2], b[s], c[s-1].  1 <= s <= 4. */
int rkdg_set_tableau(rkdg_ctx* ctx, int s, const double* a, const double* b,
                     const double* c);
int rkdg_set_precision(rkdg_ctx* ctx, int precision);
/* Kernel tuning knobs (no counterpart in the reference; set by hand or by
 * rkdg_autotune).  RKDG_TUNE_HEX_KERNEL: 0 default, 1 warp per element,
 * 2 five-lane team per element, 3 five-lane team face pass (each face once,
 * into per-element flux slots the context allocates) + element pass,
 * 4 five-lane team over Morton-ordered groups of 24 elements whose faces
 * inside the group are evaluated once (order <= 2 hexahedra; the plain team
 * kernel when the mesh's face graph needs more than 8 rounds), 5 face-once
 * tiles of 32 Morton-ordered elements (order <= 2; the FP32 Q2 default),
 * 6 the tile kernel with the collocated volume contraction on the tensor
 * cores (tcgen05 TF32 MMAs, operands split into TF32 hi + lo; FP32-bulk Q2
 * only, else the default).
 * RKDG_TUNE_GENERIC_BLOCK /
 * RKDG_TUNE_LIMITER_BLOCK: elements (threads) per CTA of the triangle/quad
 * right-hand-side kernel and of the limiter, 0 (default 128) or a multiple of
 * 32 up to 256. */
enum { RKDG_TUNE_HEX_KERNEL = 1, RKDG_TUNE_GENERIC_BLOCK = 2, RKDG_TUNE_LIMITER_BLOCK = 3 };
int rkdg_set_tuning(rkdg_ctx* ctx, int key, int value);
/* Autotuner (no counterpart in the reference): times each candidate launch
 * shape of the stage kernel, and of the limiter when one is set, on the state
 * x_dev and keeps the fastest for this context (mesh, order and precision as
 * set now).  Outputs (each may be NULL) receive the chosen
 * RKDG_TUNE_HEX_KERNEL, RKDG_TUNE_GENERIC_BLOCK and RKDG_TUNE_LIMITER_BLOCK.
 * Results do not depend on the choice beyond rounding of the hexahedral
 * kernels' summation order. */
int rkdg_autotune(rkdg_ctx* ctx, const double* x_dev, int* hex_kernel, int* generic_block,
                  int* limiter_block);

/* ---- queries ------------------------------------------------------------ */
/* NDofs (scalar nodes), nodes per element, number of equations. */
int rkdg_sizes(rkdg_ctx* ctx, long long* ndofs, int* nd, int* neq);
/* Physical node coordinates (host buffer [dim][NDofs]) for nodal projection
 * of initial conditions (GridFunction::ProjectCoefficient on nodal L2). */
int rkdg_node_coords_host(rkdg_ctx* ctx, double* out);
/* h_min = min over elements of Mesh::GetElementSize(i, 1) (main.cpp:191-201) */
int rkdg_hmin(rkdg_ctx* ctx, double* hmin);

/* ---- hot path ----------------------------------------------------------- */
/* FE_Evolution::Mult (fe_evolution.hpp:75, fe_evolution.cpp:102-216):
 * y = M^-1 [(F(u), grad phi) - <Fhat.n, phi>], x and y device arrays of
 * length NDofs*neq.  *max_char_speed_out (host) receives the global
 * max_char_speed the reference leaves in main.cpp:50. */
int rkdg_rhs(rkdg_ctx* ctx, const double* x_dev, double* y_dev,
             double* max_char_speed_out);
/* A.Mult only (face and boundary terms), the initial-dt evaluation of
 * main.cpp:473-483: returns the face-only max characteristic speed. */
int rkdg_face_speed(rkdg_ctx* ctx, const double* x_dev, double* max_char_speed_out);
/* Limiter::update (limiter.hpp:111, limiter.cpp:22-94), in place. */
int rkdg_limit(rkdg_ctx* ctx, double* x_dev);
/* Averager::computeMeanValues (averager.cpp:84-109): means[k*NE + e]. */
int rkdg_cell_means(rkdg_ctx* ctx, const double* x_dev, double* means_dev);
/* ExplicitRKLimitedSolver::Step (rk_explicit_limited.cpp:30-82): all stages,
 * limiter after every stage and after the combination.  Does not advance t
 * (as the reference).  *next_mcs (host, may be NULL) = max_char_speed of the
 * last stage, which the reference turns into the next dt (main.cpp:538-547). */
int rkdg_step(rkdg_ctx* ctx, double* x_dev, double dt, double* next_mcs);
/* The time loop of main.cpp:467-553,701-733, preceded by the limit of the
 * initial state (main.cpp:264-265) unless RKDG_QUIRK_NO_INITIAL_LIMIT is set.
 * dt_mode 0: dynamic CFL dt; 1: dt from CFL once at t=0, then constant;
 * 2: constant dt0.  max_steps > 0 stops early.  Outputs (host, may be NULL):
 * steps taken, t as the reference books it (t += new dt), last dt, and the
 * physical time actually integrated (sum of dt_real). */
int rkdg_run(rkdg_ctx* ctx, double* x_dev, double t_end, double cfl, double dt0,
             int dt_mode, int max_steps, int* steps_out, double* t_out,
             double* dt_out, double* sum_dt_out);
/* The same time loop continued from time t0 with the next step's dt already
 * known: no limit of the state and no initial dt (the reference's restart,
 * main.cpp:461-490: t and dt from the restart frame), or the next chunk of a
 * run split into pieces (t0 = *t_out and dt = *dt_out of the previous piece:
 * the pieces together step exactly as one rkdg_run).  dt_mode 0 forms the
 * following dts from CFL, 1 and 2 keep dt. */
int rkdg_run_continue(rkdg_ctx* ctx, double* x_dev, double t0, double dt, double t_end,
                      double cfl, int dt_mode, int max_steps, int* steps_out, double* t_out,
                      double* dt_out, double* sum_dt_out);
/* Discretely conserved totals sum_e sum_j (int phi_j) u_j per equation
 * (host output [neq]); the device form of check_total_energy.cpp:3-62. */
int rkdg_totals(rkdg_ctx* ctx, const double* x_dev, double* totals_host);
/* Pointwise Riemann solver (test hook for RiemannSolver::Eval,
 * rs_basic.hpp:49-50): device arrays u1,u2 [n][neq], nor [n][dim] (unit),
 * flux [n][neq], speed [n] (-1 where the reference returns -1). */
int rkdg_riemann_batch(rkdg_ctx* ctx, int n, const double* u1, const double* u2,
                       const double* nor, double* flux, double* speed);
/* ---- batched independent problems ----------------------------------------
 * Many independent solves (different meshes, states and EoS constants) in one
 * context: the mesh passed to rkdg_upload_mesh is the disjoint union of the
 * problems' meshes, problem p owning elements [elem_offsets[p],
 * elem_offsets[p+1]).  Riemann solver, limiter, tableau and boundary
 * conditions are shared; gamma and covolume are per problem.  There is no
 * counterpart in the reference, which runs one problem per process; each
 * problem follows the reference's single-problem semantics (main.cpp:467-733)
 * with its own h_min, CFL dt and time.  Adapted (nonconforming) problems are
 * allowed; since rkdg_upload_mesh pairs hanging faces by position, such
 * problems must occupy disjoint regions of space, and offsets that put the
 * two sides of a face or hanging face into different problems return
 * RKDG_ERR_INVALID.  Quadrilaterals and triangles. */
int rkdg_batch_setup(rkdg_ctx* ctx, int nprob, const int* elem_offsets,
                     const double* gamma, const double* covolume);
/* Advance every problem to t_end (dt_mode as rkdg_run, per problem; the
 * initial limit as rkdg_run).  With
 * use_graph != 0 the whole multi-step solve is one CUDA-graph launch: the RK
 * step is captured once as the body of a device-controlled while node and the
 * loop ends on the device when the last problem finishes.  Host outputs
 * (arrays of nprob, may be NULL): steps, booked t, integrated time.  A
 * problem that meets a non-physical state stops there (where the reference
 * would exit) while the others continue; its steps entry is then negative
 * (-steps taken). */
int rkdg_batch_run(rkdg_ctx* ctx, double* x_dev, double t_end, double cfl, double dt0,
                   int dt_mode, int max_steps, int use_graph, int* steps_out,
                   double* t_out, double* sum_dt_out);
/* ---- discrete adjoint (FP64 path) ------------------------------------------
 * Vector-Jacobian products of the hot path (no counterpart in the reference,
 * which has no adjoint).  Supported: every element type and order of the forward path (triangles
 * P1/P2, quads Q1-Q3, hexes Q1/Q2).
 * xbar = (d FE_Evolution::Mult / dx)^T kbar: */
int rkdg_rhs_vjp(rkdg_ctx* ctx, const double* x_dev, const double* kbar_dev, double* xbar_dev);
/* zbar = (d Limiter::update / dz)^T ybar (active branch of min/max and of the
 * indicator thresholds; Venkatakrishnan is differentiated exactly): */
int rkdg_limit_vjp(rkdg_ctx* ctx, const double* z_dev, const double* ybar_dev, double* zbar_dev);
/* Reverse of one ExplicitRKLimitedSolver::Step at x_n with step dt: xbar holds
 * the adjoint of x_{n+1} on entry and the adjoint of x_n on return. */
int rkdg_step_vjp(rkdg_ctx* ctx, const double* x_dev, double dt, double* xbar_dev);
/* Gradient through nsteps fixed-dt steps from x0: xbar holds dJ/dx(T) on entry
 * and dJ/dx0 on return; states are checkpointed every `checkpoint_every`
 * steps and recomputed between checkpoints.  xT_dev (may be NULL) receives
 * x(T). */
int rkdg_adjoint_run(rkdg_ctx* ctx, const double* x0_dev, int nsteps, double dt,
                     int checkpoint_every, double* xbar_dev, double* xT_dev);
/* Number of kernels this context launched since creation (instrumentation). */
long long rkdg_kernel_launches(rkdg_ctx* ctx);

/* ---- allocation-free limiter ----------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory while they step -- a host code whose device memory is owned by its
 * own memory manager or a framework's caching pool, or a time loop that must
 * not stall the GPU (cudaMalloc / cudaFree can synchronise the device).  Same
 * result as rkdg_limit (bit for bit), but the cell means it needs go to a
 * fixed device array of RKDG_LIMIT_STATIC_MAX_VALUES doubles (16 MiB) built
 * into the library instead of context memory; the call allocates nothing.
 * Meshes with neq * NE > RKDG_LIMIT_STATIC_MAX_VALUES are rejected with
 * RKDG_ERR_INVALID and x is left untouched.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress), so make that first
 * call before any stream capture; the address stays cached for the life of
 * the process, so a device reset (cudaDeviceReset) ends the use of this entry
 * point in that process.  The call returns once the limiter has finished on
 * the context's stream (it synchronises that stream, so it is never called
 * while the stream is being captured into a graph).  The array is shared by every context on a device:
 * calls that overlap in time on one device (other host threads, other
 * streams) race on it and must be serialised by the caller. */
#define RKDG_LIMIT_STATIC_MAX_VALUES (1u << 21)
int rkdg_limit_static(rkdg_ctx* ctx, double* x_dev);

#ifdef __cplusplus
}
#endif
#endif
