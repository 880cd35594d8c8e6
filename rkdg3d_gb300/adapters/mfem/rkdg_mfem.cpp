// MFEM adapter of the GB300 RKDG library (see rkdg_mfem.hpp).
#include "rkdg_mfem.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <string>

namespace rkdg_mfem {

namespace {

// The reference prints and exits where a Riemann solver meets a non-physical
// state (face_integrator.cpp:214-218); the adapter stops the same way on any
// failed call.
void check(rkdg_ctx* ctx, int status, const char* what) {
  if (status == RKDG_OK) return;
  long long where = -1;
  const char* msg = rkdg_last_error(ctx, &where);
  std::string s = std::string(what) + ": " + (msg ? msg : "error") +
                  (where >= 0 ? " (element " + std::to_string(where) + ")" : std::string());
  mfem::mfem_error(s.c_str());
}

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) mfem::mfem_error((std::string(what) + ": " + cudaGetErrorString(e)).c_str());
}

}  // namespace

int UploadMesh(rkdg_ctx* ctx, mfem::Mesh& mesh, int order) {
  const int dim = mesh.Dimension(), ne = mesh.GetNE();
  if (ne <= 0) return RKDG_ERR_INVALID;
  const int geom = mesh.GetElementBaseGeometry(0);  // MFEM Geometry::Type: 2, 3, 5
  const int nv = mfem::Geometry::NumVerts[geom];
  const mfem::IntegrationRule* corners = mfem::Geometries.GetVertices(geom);
  std::vector<int> ev((size_t)ne * nv);
  std::vector<double> ec((size_t)ne * nv * dim);
  mfem::Array<int> v;
  mfem::Vector x(dim);
  for (int e = 0; e < ne; ++e) {
    mesh.GetElementVertices(e, v);
    mfem::ElementTransformation* T = mesh.GetElementTransformation(e);
    for (int k = 0; k < nv; ++k) {
      ev[(size_t)e * nv + k] = v[k];
      T->Transform(corners->IntPoint(k), x);
      for (int d = 0; d < dim; ++d) ec[((size_t)e * nv + k) * dim + d] = x(d);
    }
  }
  const int nb = mesh.GetNBE(), nvf = dim == 2 ? 2 : (geom == 5 ? 4 : 3);
  std::vector<int> bv((size_t)nb * nvf), ba(nb);
  for (int b = 0; b < nb; ++b) {
    mesh.GetBdrElementVertices(b, v);
    for (int k = 0; k < nvf; ++k) bv[(size_t)b * nvf + k] = v[k];
    ba[b] = mesh.GetBdrAttribute(b);
  }
  rkdg_mesh_desc d;
  d.dim = dim;
  d.geom = geom;
  d.order = order;
  d.num_elements = ne;
  d.elem_vertices = ev.data();
  d.elem_coords = ec.data();
  d.num_bdr = nb;
  d.bdr_vertices = bv.data();
  d.bdr_attr = ba.data();
  return rkdg_upload_mesh(ctx, &d);
}

// ---- VectorBridge -------------------------------------------------------------
VectorBridge::~VectorBridge() {
  for (double* p : buf_)
    if (p) cudaFree(p);
}

double* VectorBridge::Buffer(int slot, int n) {
  if (cap_[slot] < n) {
    if (buf_[slot]) cudaFree(buf_[slot]);
    buf_[slot] = nullptr;
    check_cuda(cudaMalloc(&buf_[slot], sizeof(double) * (size_t)n), "device buffer");
    cap_[slot] = n;
  }
  return buf_[slot];
}

const double* VectorBridge::In(const mfem::Vector& x, int slot) {
  if (device_memory_) return x.Read();
  double* d = Buffer(slot, x.Size());
  check_cuda(cudaMemcpy(d, x.GetData(), sizeof(double) * (size_t)x.Size(), cudaMemcpyHostToDevice),
             "host to device");
  return d;
}

double* VectorBridge::Out(mfem::Vector& y, int slot) {
  if (device_memory_) return y.Write();
  return Buffer(slot, y.Size());
}

double* VectorBridge::InOut(mfem::Vector& x, int slot) {
  if (device_memory_) return x.ReadWrite();
  return const_cast<double*>(In(x, slot));
}

void VectorBridge::Back(mfem::Vector& y, int slot) {
  if (device_memory_) return;
  check(ctx_, rkdg_synchronize(ctx_), "synchronize");
  check_cuda(cudaMemcpy(y.GetData(), buf_[slot], sizeof(double) * (size_t)y.Size(),
                        cudaMemcpyDeviceToHost),
             "device to host");
}

// ---- GpuEvolution -----------------------------------------------------------
GpuEvolution::GpuEvolution(rkdg_ctx* ctx, int size, double* max_char_speed, bool device_memory)
    : mfem::TimeDependentOperator(size), ctx_(ctx), mcs_(max_char_speed), io_(ctx, device_memory) {}

void GpuEvolution::Mult(const mfem::Vector& x, mfem::Vector& y) const {
  double mcs = 0.0;
  const double* xd = io_.In(x, 0);
  double* yd = io_.Out(y, 1);
  check(ctx_, rkdg_rhs(ctx_, xd, yd, &mcs), "rkdg_rhs");
  io_.Back(y, 1);
  if (mcs_) *mcs_ = mcs;
}

double GpuEvolution::FaceSpeed(const mfem::Vector& x) const {
  double mcs = 0.0;
  check(ctx_, rkdg_face_speed(ctx_, io_.In(x, 0), &mcs), "rkdg_face_speed");
  return mcs;
}

// ---- GpuRKLimited -----------------------------------------------------------
GpuRKLimited::GpuRKLimited(rkdg_ctx* ctx, int s, const double* a, const double* b, const double* c,
                           double* max_char_speed, bool device_memory)
    : ctx_(ctx), mcs_(max_char_speed), io_(ctx, device_memory) {
  check(ctx_, rkdg_set_tableau(ctx_, s, a, b, c), "rkdg_set_tableau");
}

void GpuRKLimited::Init(mfem::TimeDependentOperator& f) { mfem::ODESolver::Init(f); }

void GpuRKLimited::Step(mfem::Vector& x, double& t, double& dt) {
  (void)t;  // ExplicitRKLimitedSolver::Step does not advance t either
  double mcs = 0.0;
  double* xd = io_.InOut(x, 0);
  check(ctx_, rkdg_step(ctx_, xd, dt, &mcs), "rkdg_step");
  io_.Back(x, 0);
  if (mcs_) *mcs_ = mcs;
}

// ---- GpuLimiter -------------------------------------------------------------
void GpuLimiter::update(mfem::Vector& x) {
  double* xd = io_.InOut(x, 0);
  check(ctx_, rkdg_limit(ctx_, xd), "rkdg_limit");
  io_.Back(x, 0);
}

}  // namespace rkdg_mfem
