// Test-only stand-in for the few pieces of MFEM's interface that the
// reference's pointwise physics, Riemann-solver and boundary-state sources
// use (physics/physics.cpp, riemannsolvers/rs_*.cpp, bc/boundary_integrator_*.cpp),
// and that the library's MFEM adapter (rkdg3d_gb300/adapters/mfem) uses:
// the adapter is compile-checked against it (tests/test_mfem_adapter.py).
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
#include <vector>

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
  // MFEM's memory-manager accessors (here: the host data)
  const double* Read(bool on_dev = true) const { (void)on_dev; return data_; }
  double* Write(bool on_dev = true) { (void)on_dev; return data_; }
  double* ReadWrite(bool on_dev = true) { (void)on_dev; return data_; }
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
  void Transform(const IntegrationPoint&, Vector& x) { x = 0.0; }
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

// ---- what the adapter uses (declared for compilation) -------------------------
template <class T>
class Array {
 public:
  int Size() const { return (int)v_.size(); }
  void SetSize(int n) { v_.resize(n); }
  T& operator[](int i) { return v_[i]; }
  const T& operator[](int i) const { return v_[i]; }
  T* GetData() { return v_.data(); }

 private:
  std::vector<T> v_;
};

class Geometry {
 public:
  enum Type { INVALID = -1, POINT = 0, SEGMENT, TRIANGLE, SQUARE, TETRAHEDRON, CUBE };
  static constexpr int NumVerts[8] = {1, 2, 3, 4, 4, 8, 6, 5};
  const IntegrationRule* GetVertices(int) const { return &r_; }

 private:
  IntegrationRule r_;
};
inline Geometry Geometries;

class Mesh {
 public:
  int Dimension() const { return 0; }
  int GetNE() const { return 0; }
  Geometry::Type GetElementBaseGeometry(int) const { return Geometry::SQUARE; }
  void GetElementVertices(int, Array<int>& v) const { v.SetSize(0); }
  ElementTransformation* GetElementTransformation(int) { return &T_; }
  int GetNBE() const { return 0; }
  void GetBdrElementVertices(int, Array<int>& v) const { v.SetSize(0); }
  int GetBdrAttribute(int) const { return 1; }

 private:
  ElementTransformation T_;
};

class Operator {
 public:
  explicit Operator(int s = 0) : height(s), width(s) {}
  virtual ~Operator() = default;
  int Height() const { return height; }
  int Width() const { return width; }
  virtual void Mult(const Vector& x, Vector& y) const = 0;

 protected:
  int height, width;
};

class TimeDependentOperator : public Operator {
 public:
  explicit TimeDependentOperator(int n = 0, double t_ = 0.0) : Operator(n), t(t_) {}
  virtual void SetTime(double t_) { t = t_; }
  double GetTime() const { return t; }

 protected:
  double t;
};

class ODESolver {
 public:
  virtual ~ODESolver() = default;
  virtual void Init(TimeDependentOperator& f_) { f = &f_; }
  virtual void Step(Vector& x, double& t, double& dt) = 0;

 protected:
  TimeDependentOperator* f = nullptr;
};

}  // namespace mfem

#endif
