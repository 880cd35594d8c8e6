// Test-only C entry points around the reference's own pointwise sources,
// compiled unmodified against the MFEM stand-in in this folder (recipe:
// oracle/Makefile, target `ref`, output oracle/_ref/librefpin.so).  The CPU
// tests call these to produce golden vectors from the reference's arithmetic
// and to pin the oracle (and, through the committed vectors, the GPU kernels)
// to it.  Nothing in the library or the benchmark links this.
//
// Covered reference code:
//   physics/physics.cpp            EoS, fluxes, TRRS / Einfeldt wave speeds
//   riemannsolvers/rs_basic.cpp    Rotate / InverseRotate
//   riemannsolvers/rs_{rusanov,llf,hll,hllc}.cpp   RiemannSolver*::Eval
//   bc/boundary_integrator_{slip,wall,open,constant,supersonic_inlet,
//      subsonic_inlet,subsonic_inlet_total_pressure,
//      subsonic_inlet_fixed_pressure,open_fixed_pressure,
//      open_total_pressure,char_outlet}.cpp        computeRightState
#include <vector>

#include "physics.hpp"
#include "rs_basic.hpp"
#include "rs_hll.hpp"
#include "rs_hllc.hpp"
#include "rs_llf.hpp"
#include "rs_rusanov.hpp"
#include "boundary_integrator.hpp"
#include "boundary_integrator_char_outlet.hpp"
#include "boundary_integrator_constant.hpp"
#include "boundary_integrator_open.hpp"
#include "boundary_integrator_open_fixed_pressure.hpp"
#include "boundary_integrator_open_total_pressure.hpp"
#include "boundary_integrator_slip.hpp"
#include "boundary_integrator_subsonic_inlet.hpp"
#include "boundary_integrator_subsonic_inlet_fixed_pressure.hpp"
#include "boundary_integrator_subsonic_inlet_total_pressure.hpp"
#include "boundary_integrator_supersonic_inlet.hpp"
#include "boundary_integrator_wall.hpp"

// The reference's process globals (main.cpp:39-56).
double specific_heat_ratio = 1.4;
double covolume_constant = 0.0;
double gas_constant = 1.0;
int num_equation = 4;
int myRank = 0;
double max_char_speed = 0.0;

// The base-class pieces live in bc/boundary_integrator.cpp next to the face
// assembly, which needs the rest of MFEM; the harness only needs the
// constructor (same member initialisation) and an inert assembly.
BoundaryIntegrator::BoundaryIntegrator(RiemannSolver& rsolver_, const int dim_)
    : rsolver(rsolver_), funval1(num_equation), funval2(num_equation), nor(dim_),
      fluxN(num_equation), dim(dim_) {}
void BoundaryIntegrator::AssembleFaceVector(const FiniteElement&, const FiniteElement&,
                                            FaceElementTransformations&, const Vector&,
                                            Vector&) {}

namespace {

RiemannSolver* make_solver(int rs) {
  switch (rs) {
    case 0: return new RiemannSolverRusanov();
    case 1: return new RiemannSolverLLF();
    case 2: return new RiemannSolverHLL();
    case 3: return new RiemannSolverHLLC();
  }
  return nullptr;
}

}  // namespace

extern "C" {

// Physics globals; neq = dim + 2.
void pin_set_physics(double gamma, double covolume, double R, int neq) {
  specific_heat_ratio = gamma;
  covolume_constant = covolume;
  gas_constant = R;
  num_equation = neq;
}

// Pointwise EoS on n states u[n][neq]: out[n][6] = pressure, sound speed,
// max characteristic speed, Mach number, StateIsPhysical, temperature.
void pin_eos(int n, int dim, const double* u, double* out) {
  const int neq = dim + 2;
  for (int i = 0; i < n; ++i) {
    Vector s(neq);
    for (int k = 0; k < neq; ++k) s(k) = u[(size_t)i * neq + k];
    double* o = out + (size_t)i * 6;
    o[0] = ComputePressure(s, dim);
    o[1] = ComputeSoundSpeed(s, dim);
    o[2] = ComputeMaxCharSpeed(s, dim);
    o[3] = ComputeM(s, dim);
    o[4] = StateIsPhysical(s, dim) ? 1.0 : 0.0;
    o[5] = ComputeTemperature(s, dim);
  }
}

// Physical flux F(u) (ComputeFlux): f[n][neq][dim].
void pin_flux(int n, int dim, const double* u, double* f) {
  const int neq = dim + 2;
  for (int i = 0; i < n; ++i) {
    Vector s(neq);
    for (int k = 0; k < neq; ++k) s(k) = u[(size_t)i * neq + k];
    DenseMatrix F(neq, dim);
    ComputeFlux(s, dim, F);
    for (int k = 0; k < neq; ++k)
      for (int d = 0; d < dim; ++d) f[((size_t)i * neq + k) * dim + d] = F(k, d);
  }
}

// Wave speeds of two states, kind 0 ComputeToroCharSpeeds (TRRS), 1
// ComputeEinfeldtCharSpeeds: lam[n][neq].  The states are rotated into the
// normal's frame first, as the solvers do before they call them.
void pin_speeds(int kind, int n, int dim, const double* u1, const double* u2, const double* nor,
                double* lam) {
  const int neq = dim + 2;
  RiemannSolverHLL rot;  // Rotate is a member of every solver
  for (int i = 0; i < n; ++i) {
    Vector s1(neq), s2(neq), l(neq), nv(dim);
    for (int k = 0; k < neq; ++k) {
      s1(k) = u1[(size_t)i * neq + k];
      s2(k) = u2[(size_t)i * neq + k];
    }
    for (int d = 0; d < dim; ++d) nv(d) = nor[(size_t)i * dim + d];
    rot.Rotate(s1, nv, dim);
    rot.Rotate(s2, nv, dim);
    if (kind == 0)
      ComputeToroCharSpeeds(s1, s2, l, dim);
    else
      ComputeEinfeldtCharSpeeds(s1, s2, l, dim);
    for (int k = 0; k < neq; ++k) lam[(size_t)i * neq + k] = l(k);
  }
}

// RiemannSolver::Eval for rs = 0 Rusanov, 1 LLF, 2 HLL, 3 HLLC on n point
// pairs: flux[n][neq], speed[n] (-1 for a non-physical state, as returned).
// Eval rotates its inputs in place (const_cast), so each call gets copies.
int pin_riemann(int rs, int n, int dim, const double* u1, const double* u2, const double* nor,
                double* flux, double* speed) {
  const int neq = dim + 2;
  RiemannSolver* solver = make_solver(rs);
  if (!solver) return 1;
  for (int i = 0; i < n; ++i) {
    Vector s1(neq), s2(neq), f(neq), nv(dim);
    for (int k = 0; k < neq; ++k) {
      s1(k) = u1[(size_t)i * neq + k];
      s2(k) = u2[(size_t)i * neq + k];
      f(k) = 0.0;
    }
    for (int d = 0; d < dim; ++d) nv(d) = nor[(size_t)i * dim + d];
    speed[i] = solver->Eval(s1, s2, nv, f);
    for (int k = 0; k < neq; ++k) flux[(size_t)i * neq + k] = f(k);
  }
  delete solver;
  return 0;
}

// computeRightState of one boundary condition on n points.
// bc: 0 slip, 1 open, 2 constant (rotated frame), 3 supersonic inlet, 4 wall,
// 5 subsonic inlet, 6 subsonic inlet total pressure {pTot, TTot}, 7 subsonic
// inlet fixed pressure {pFix, TTot}, 8 fixed-pressure outlet {pFix}, 9 total-
// pressure outlet {pTot, TFix}, 10 characteristic outlet (state = outer
// conservative state).  prm: the fixed state (neq values) or the parameters.
// nor_pad: the value stored right after the normal's dim components (the
// total-pressure outlet reads nor[1..dim], one past the end).
// s2_in (may be NULL): what state2 holds on entry; the characteristic outlet
// reads it before writing it.  s2_out[n][neq].
int pin_right_state(int bc, int rs, int n, int dim, const double* s1, const double* nor,
                    double nor_pad, const double* prm, const double* s2_in, double* s2_out) {
  const int neq = dim + 2;
  RiemannSolver* solver = make_solver(rs);
  if (!solver) return 1;
  Vector fixed(neq);
  for (int k = 0; k < neq; ++k) fixed(k) = prm ? prm[k] : 0.0;
  BoundaryIntegrator* b = nullptr;
  switch (bc) {
    case 0: b = new BoundaryIntegratorSlip(*solver, dim); break;
    case 1: b = new BoundaryIntegratorOpen(*solver, dim); break;
    case 2: b = new BoundaryIntegratorConstant(*solver, dim, fixed); break;
    case 3: b = new BoundaryIntegratorSupersonicInlet(*solver, dim, fixed); break;
    case 4: b = new BoundaryIntegratorWall(*solver, dim); break;
    case 5: b = new BoundaryIntegratorSubsonicInlet(*solver, dim, fixed); break;
    case 6: b = new BoundaryIntegratorSubsonicInletTotalPressure(*solver, dim, prm[0], prm[1]); break;
    case 7: b = new BoundaryIntegratorSubsonicInletFixedPressure(*solver, dim, prm[0], prm[1]); break;
    case 8: b = new BoundaryIntegratorOpenFixedPressure(*solver, dim, prm[0]); break;
    case 9: b = new BoundaryIntegratorOpenTotalPressure(*solver, dim, prm[0], prm[1]); break;
    case 10: b = new BoundaryIntegratorCharOutlet(*solver, dim, fixed); break;
    default: delete solver; return 1;
  }
  std::vector<double> nbuf(dim + 1);
  for (int i = 0; i < n; ++i) {
    Vector a(neq), g(neq);
    for (int k = 0; k < neq; ++k) {
      a(k) = s1[(size_t)i * neq + k];
      g(k) = s2_in ? s2_in[(size_t)i * neq + k] : 0.0;
    }
    for (int d = 0; d < dim; ++d) nbuf[d] = nor[(size_t)i * dim + d];
    nbuf[dim] = nor_pad;
    Vector nv(nbuf.data(), dim);
    b->computeRightState(a, g, nv);
    for (int k = 0; k < neq; ++k) s2_out[(size_t)i * neq + k] = g(k);
  }
  delete b;
  delete solver;
  return 0;
}

}  // extern "C"
