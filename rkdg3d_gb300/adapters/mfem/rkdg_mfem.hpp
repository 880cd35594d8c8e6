// MFEM adapter of the GB300 RKDG library: drop-in replacements for the
// reference's FE_Evolution (src/fe_evolution/fe_evolution.hpp:27-82),
// ExplicitRKLimitedSolver (src/ode_solver/rk_explicit_limited.hpp:24-60) and
// Limiter::update (src/limiter/limiter.hpp:102-111), plus the mesh upload the
// reference's set-up and AMR path call where it rebuilds its operators
// (main.cpp:148-164, 610-611).
//
// Compiled in the user's MFEM build (with CUDA): it uses MFEM's public mesh,
// vector and operator interfaces and the library's C ABI (include/rkdg_gpu.h);
// link with -lrkdg_gb300 -lcudart.  State vectors keep MFEM's byNODES layout,
// so the reference's `sol` is passed through unchanged.
//
// Vectors: with `device_memory` set, the adapter takes device pointers from
// MFEM's memory manager (Vector::Read / Write / ReadWrite, MFEM configured
// with a CUDA device); otherwise it stages the vectors' host data through
// device buffers it owns (one host <-> device copy per call).
#pragma once

#include <vector>

#include "mfem.hpp"
#include "rkdg_gpu.h"

namespace rkdg_mfem {

// Mesh description of an MFEM mesh for rkdg_upload_mesh: topological vertex
// ids, each element's own corner coordinates (through its transformation, so
// periodic meshes with a nodal grid function are handled) and the boundary
// elements with their attributes.  Call it at set-up and after every adapt
// (the place of UpdateInverseMassMatrix / UpdateAfluxPointer).
int UploadMesh(rkdg_ctx* ctx, mfem::Mesh& mesh, int order);

// Device staging of MFEM vectors (see above).
class VectorBridge {
 public:
  VectorBridge(rkdg_ctx* ctx, bool device_memory) : ctx_(ctx), device_memory_(device_memory) {}
  ~VectorBridge();
  VectorBridge(const VectorBridge&) = delete;
  VectorBridge& operator=(const VectorBridge&) = delete;
  // device pointers for reading x / writing y / updating x in place
  const double* In(const mfem::Vector& x, int slot);
  double* Out(mfem::Vector& y, int slot);
  double* InOut(mfem::Vector& x, int slot);
  // copy a staged output back to the host vector (no-op with device memory)
  void Back(mfem::Vector& y, int slot);

 private:
  double* Buffer(int slot, int n);
  rkdg_ctx* ctx_;
  bool device_memory_;
  double* buf_[2] = {nullptr, nullptr};
  int cap_[2] = {0, 0};
};

// Replaces FE_Evolution: Mult(x, y) = rkdg_rhs; the maximum characteristic
// speed the reference leaves in its global (main.cpp:50) goes to
// *max_char_speed when the pointer is given.
class GpuEvolution : public mfem::TimeDependentOperator {
 public:
  GpuEvolution(rkdg_ctx* ctx, int size, double* max_char_speed = nullptr,
               bool device_memory = false);
  void Mult(const mfem::Vector& x, mfem::Vector& y) const override;
  // A.Mult for the initial dt (main.cpp:473-483): the face-only speed
  double FaceSpeed(const mfem::Vector& x) const;
  rkdg_ctx* Context() const { return ctx_; }

 private:
  rkdg_ctx* ctx_;
  double* mcs_;
  mutable VectorBridge io_;
};

// Replaces ExplicitRKLimitedSolver(s, a, b, c, limiter): the reference's
// tableau arrays verbatim; Step runs every stage, the limiter after each
// stage and after the combination, on the device; t is not advanced (as the
// reference's Step); the last stage's speed goes to *max_char_speed.
class GpuRKLimited : public mfem::ODESolver {
 public:
  GpuRKLimited(rkdg_ctx* ctx, int s, const double* a, const double* b, const double* c,
               double* max_char_speed = nullptr, bool device_memory = false);
  void Init(mfem::TimeDependentOperator& f) override;
  void Step(mfem::Vector& x, double& t, double& dt) override;

 private:
  rkdg_ctx* ctx_;
  double* mcs_;
  VectorBridge io_;
};

// Replaces Limiter::update(x) (the initial limit of main.cpp:264-265 and any
// standalone use); the limiter set with rkdg_set_limiter.
class GpuLimiter {
 public:
  GpuLimiter(rkdg_ctx* ctx, bool device_memory = false) : ctx_(ctx), io_(ctx, device_memory) {}
  void update(mfem::Vector& x);

 private:
  rkdg_ctx* ctx_;
  VectorBridge io_;
};

}  // namespace rkdg_mfem
