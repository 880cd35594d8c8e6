// Test-only stand-in for the few pieces of MFEM's interface that the
// reference's pointwise physics, Riemann-solver and boundary-state sources
// use (physics/physics.cpp, riemannsolvers/rs_*.cpp, bc/boundary_integrator_*.cpp).
//
// It exists so that those reference files compile UNMODIFIED into
// oracle/_ref/librefpin.so (recipe: oracle/Makefile, target `ref`), which the
// CPU tests use to pin the oracle and the GPU kernels to the reference's own
// arithmetic.  MFEM itself is not installed here.
//
// Semantics kept from MFEM's documented interface:
//  * Vector(int n) allocates n doubles (left uninitialised by MFEM; filled
//    with NaN here so that reading a value before writing it is visible);
//  * Vector(double* p, int n) is a non-owning view;
//  * operator= (Vector) resizes to the source size, then copies;
//  * operator() and operator[] are unchecked element access;
//  * DenseMatrix is column-major, A(i, j) = data[i + j * height].
// Everything below "assembly-only types" is declared so that files which also
// hold face-assembly code compile; none of it is ever called by the harness.
#ifndef RKDG_TEST_MFEM_SHIM_HPP
#define RKDG_TEST_MFEM_SHIM_HPP

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>

#define MFEM_ASSERT(cond, msg) ((void)0)

namespace mfem {

inline void mfem_error(const char* msg = nullptr) {
  std::cerr << "mfem_error: " << (msg ? msg : "") << std::endl;
  std::abort();
}

class Vector {
 public:
  Vector() = default;
  explicit Vector(int n) { SetSize(n); }
  Vector(double* p, int n) : data_(p), size_(n), cap_(n), owns_(false) {}
  Vector(const Vector& v) { *this = v; }
  ~Vector() { release(); }

  void SetSize(int n) {
    if (n <= cap_) {
      size_ = n;
      return;
    }
    release();
    data_ = new double[n];
    for (int i = 0; i < n; ++i) data_[i] = std::numeric_limits<double>::quiet_NaN();
    size_ = cap_ = n;
    owns_ = true;
  }
  int Size() const { return size_; }
  double* GetData() const { return data_; }

  double& operator()(int i) { return data_[i]; }
  const double& operator()(int i) const { return data_[i]; }
  double& operator[](int i) { return data_[i]; }
  const double& operator[](int i) const { return data_[i]; }

  Vector& operator=(double v) {
    for (int i = 0; i < size_; ++i) data_[i] = v;
    return *this;
  }
  Vector& operator=(const Vector& v) {
    if (this == &v) return *this;
    SetSize(v.size_);
    if (size_) std::memmove(data_, v.data_, sizeof(double) * size_);
    return *this;
  }
  Vector& operator*=(double a) {
    for (int i = 0; i < size_; ++i) data_[i] *= a;
    return *this;
  }
  double Norml2() const {
    double s = 0;
    for (int i = 0; i < size_; ++i) s += data_[i] * data_[i];
    return std::sqrt(s);
  }
  void Print(std::ostream& os = std::cout) const {
    for (int i = 0; i < size_; ++i) os << data_[i] << (i + 1 < size_ ? " " : "\n");
  }

 private:
  void release() {
    if (owns_) delete[] data_;
    data_ = nullptr;
    size_ = cap_ = 0;
    owns_ = false;
  }
  double* data_ = nullptr;
  int size_ = 0;
  int cap_ = 0;
  bool owns_ = false;
};

class DenseMatrix {
 public:
  DenseMatrix() = default;
  DenseMatrix(int h, int w) { SetSize(h, w); }
  DenseMatrix(double* p, int h, int w) : data_(p), h_(h), w_(w), owns_(false) {}
  ~DenseMatrix() {
    if (owns_) delete[] data_;
  }
  DenseMatrix(const DenseMatrix&) = delete;
  DenseMatrix& operator=(const DenseMatrix&) = delete;

  void SetSize(int h, int w) {
    if (owns_) delete[] data_;
    data_ = new double[(size_t)h * w];
    for (int i = 0; i < h * w; ++i) data_[i] = std::numeric_limits<double>::quiet_NaN();
    h_ = h;
    w_ = w;
    owns_ = true;
  }
  int Height() const { return h_; }
  int Width() const { return w_; }
  double* Data() const { return data_; }
  double& operator()(int i, int j) { return data_[i + (size_t)j * h_]; }
  const double& operator()(int i, int j) const { return data_[i + (size_t)j * h_]; }
  void MultTranspose(const Vector& x, Vector& y) const {
    y.SetSize(w_);
    for (int j = 0; j < w_; ++j) {
      double s = 0;
      for (int i = 0; i < h_; ++i) s += (*this)(i, j) * x(i);
      y(j) = s;
    }
  }

 private:
  double* data_ = nullptr;
  int h_ = 0, w_ = 0;
  bool owns_ = false;
};

// ---- assembly-only types (declared for compilation, never called) ----------
struct IntegrationPoint {
  double x = 0, y = 0, z = 0, weight = 0;
};

class IntegrationRule {
 public:
  int GetNPoints() const { return 0; }
  const IntegrationPoint& IntPoint(int) const { return ip_; }

 private:
  IntegrationPoint ip_;
};

struct IntegrationRules {
  const IntegrationRule& Get(int, int) const { return r_; }
  IntegrationRule r_;
};
static IntegrationRules IntRules;

struct FunctionSpace {
  enum { Pk = 0, Qk = 1 };
};

class FiniteElement {
 public:
  int GetDof() const { return 0; }
  int GetOrder() const { return 0; }
  int Space() const { return FunctionSpace::Qk; }
  void CalcShape(const IntegrationPoint&, Vector&) const {}
};

struct ElementTransformation {
  int OrderW() const { return 0; }
  const DenseMatrix& Jacobian() { return J_; }
  void SetIntPoint(const IntegrationPoint*) {}
  DenseMatrix J_;
};

struct IntegrationPointTransformation {
  void Transform(const IntegrationPoint&, IntegrationPoint&) const {}
};

struct FaceElementTransformations {
  int Elem1No = 0, Elem2No = -1, FaceGeom = 0;
  ElementTransformation* Elem1 = nullptr;
  ElementTransformation* Elem2 = nullptr;
  ElementTransformation* Face = nullptr;
  IntegrationPointTransformation Loc1, Loc2;
};

inline void CalcOrtho(const DenseMatrix&, Vector&) {}

class NonlinearFormIntegrator {
 public:
  virtual ~NonlinearFormIntegrator() = default;
};

}  // namespace mfem

#endif
