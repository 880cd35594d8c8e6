/*
 * refcpu — CPU FP64 oracle for the RKDG3D explicit DG hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker and the timed
 * CPU baseline; it is never linked into, loaded by, or called from the product
 * path (rkdg3d_gb300).  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference leg may load it.
 *
 * It restates, line by line, the reference's CPU algorithm:
 *   src/physics/physics.cpp, src/riemannsolvers/rs_{basic,rusanov,llf,hll,hllc}.cpp,
 *   src/eq_terms/face_integrator.cpp, src/eq_terms/domain_integrator.cpp,
 *   src/bc/boundary_integrator{,_slip,_open,_constant,_supersonic_inlet,_wall}.cpp,
 *   src/fe_evolution/fe_evolution.cpp, src/averager/averager.cpp:84-119,
 *   src/limiter/limiter{,_multiplier,_findiff}.cpp,
 *   src/indicator/indicator_bj.cpp, src/ode_solver/rk_explicit_limited.cpp,
 *   main.cpp:191-201,467-553,701-733
 * together with the MFEM behaviours those files rely on (nodal Gauss-Legendre
 * L2 bases, Gauss-Legendre / tensor quadrature orders, face geometry, mass and
 * average rules), which are restated from MFEM's documented semantics because
 * MFEM is not present.
 *
 * PARITY UNPINNED: the reference ships no tests or golden vectors and cannot
 * be built here (MFEM, MPI, rapidyaml are absent), so this oracle is pinned
 * only by its own known-answer tests (consistency, rotation invariance,
 * free-stream preservation, discrete conservation, Sod vs. an exact Riemann
 * solution) and by regression fixtures it generated itself.
 */
#ifndef RKDG_REFCPU_H
#define RKDG_REFCPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry codes follow MFEM's Geometry::Type numbering. */
#define REF_GEOM_TRIANGLE 2
#define REF_GEOM_SQUARE 3
#define REF_GEOM_CUBE 5

#define REF_OK 0
#define REF_ERR_INVALID 1
#define REF_ERR_UNPHYSICAL 2

typedef struct ref_ctx ref_ctx;

/* Mesh: topological vertices (for face matching), per-element vertex
 * coordinates in MFEM local vertex order (periodic meshes give the physical
 * coordinates of each element's own corners), boundary faces with 1-based
 * attributes. */
ref_ctx* ref_create(int dim, int geom, int order, int num_elements,
                    const int* elem_vertices, const double* elem_coords,
                    int num_bdr, const int* bdr_vertices, const int* bdr_attr);
void ref_destroy(ref_ctx* c);

/* rsolver: 0 Rusanov, 1 LLF, 2 HLL, 3 HLLC; averaging: 0 TRRS, 1 Einfeldt */
int ref_set_physics(ref_ctx* c, int rsolver, int averaging, double gamma,
                    double covolume, double gas_constant);
/* bc type: 0 slip, 1 open (outlet), 2 fixed state in the rotated frame
 * (BoundaryIntegratorConstant), 3 supersonic inlet (global-frame state),
 * 4 wall (same as slip), 5 subsonic inlet (fixed rotated-frame state),
 * 6 subsonicInletTotalPressure {pTot, TTot}, 7 subsonicInletFixedPressure
 * {pFix, TTot}, 8 fixedPressureOutlet {pFix}, 9
 * totalPressureFixedTemperatureOutlet {pTot, TFix}, 10 charOutlet (outer
 * conservative state; the ghost vector, which the reference reads before it
 * assigns it, enters as the interior state).  state (neq values) =
 * conservative variables (types 2, 3, 5, 10), the listed parameters in its
 * first entries (6-9), or NULL. */
int ref_set_bc(ref_ctx* c, int attr, int type, const double* state);
/* computeRightState of attribute attr's boundary condition for the state s1
 * and the unit outward normal nor (test hook). */
int ref_right_state(ref_ctx* c, int attr, const double* s1, const double* nor, double* s2);
/* limiter: 0 FinDiff, 1 Multi; indicator: 0 Nowhere, 1 Everywhere, 2 BJ family,
 * 3 Shu (FinDiff only: with Multi the reference reads a factor Shu never sets);
 * function: 0 BJ, 1 Venkatakrishnan, 2 Michalak; quirks bit0: apply the
 * multiplier once instead of nd times; bit1: the "linearize" option of the
 * Multi limiter (quads and hexes of order 1; a no-op on triangles). */
int ref_set_limiter(ref_ctx* c, int limiter, int indicator, int function,
                    int last_hope, int quirks);
int ref_set_tableau(ref_ctx* c, int s, const double* a, const double* b,
                    const double* cc);
/* bit 0: a negative HLLC wave speed (signed max(SL,SR)) is not treated as a
 * non-physical state (the reference exits on it); bit 1: ref_run does not
 * limit the initial state (the reference limits the projected state once
 * before its time loop, main.cpp:264-265). */
int ref_set_solver_quirks(ref_ctx* c, int flags);
void ref_set_threads(int n);

long long ref_ndofs(ref_ctx* c);   /* scalar nodes (NDofs) */
int ref_nd(ref_ctx* c);            /* nodes per element */
int ref_neq(ref_ctx* c);
int ref_nfaces(ref_ctx* c, int* interior, int* boundary);
int ref_node_coords(ref_ctx* c, double* out);      /* [dim][NDofs] */
double ref_hmin(ref_ctx* c);

/* FE_Evolution::Mult: y = M^-1 [(F(u),grad phi) - <Fhat.n, phi>] */
int ref_rhs(ref_ctx* c, const double* x, double* y, double* max_char_speed);
/* A.Mult only (faces), as used for the initial dt (main.cpp:473-483) */
int ref_face_speed(ref_ctx* c, const double* x, double* max_char_speed);
int ref_means(ref_ctx* c, const double* x, double* means);   /* [neq][NE] */
int ref_limit(ref_ctx* c, double* x);
int ref_step(ref_ctx* c, double* x, double dt, double* next_mcs);
/* Time loop of main.cpp:467-553,701-733.
 * dt_mode 0: dynamic CFL dt (time.type: dynamic);
 * dt_mode 1: dt computed once from cfl at t=0, then kept constant;
 * dt_mode 2: constant dt = dt0 (time.type: constant).
 * max_steps > 0 stops after that many steps.  Unless solver quirk bit 1 is
 * set, x is limited once first (main.cpp:264-265). */
int ref_run(ref_ctx* c, double* x, double t_end, double cfl, double dt0,
            int dt_mode, int max_steps, int* steps_out, double* t_out,
            double* dt_out, double* sum_dt_out);
/* The same loop continued at time t0 with the next dt known (no initial
 * limit, no initial dt): the reference's restart, main.cpp:461-490. */
int ref_run_continue(ref_ctx* c, double* x, double t0, double dt, double t_end, double cfl,
                     int dt_mode, int max_steps, int* steps_out, double* t_out,
                     double* dt_out, double* sum_dt_out);
int ref_totals(ref_ctx* c, const double* x, double* totals); /* [neq] */
double ref_total_energy(ref_ctx* c, const double* x); /* check_total_energy.cpp */
/* pointwise Riemann solver on n states: u1,u2 [n][neq], nor [n][dim] (unit) */
int ref_riemann(ref_ctx* c, int n, const double* u1, const double* u2,
                const double* nor, double* flux, double* speed);
/* pointwise physics (test hook): what 0 = EoS of u1, out[n][4] = pressure,
 * sound speed, max characteristic speed, StateIsPhysical; 1 = physical flux
 * of u1, out[n][neq][dim]; 2 / 3 = TRRS / Einfeldt wave speeds of u1, u2
 * rotated into nor's frame, out[n][neq]. */
int ref_pointwise(ref_ctx* c, int what, int n, const double* u1, const double* u2,
                  const double* nor, double* out);
const char* ref_last_error(ref_ctx* c);

#ifdef __cplusplus
}
#endif
#endif
