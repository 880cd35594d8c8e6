// Dispatch of the generic kernels plus small utility kernels: pointwise
// Riemann batch, FP64 <-> float-pair conversion and conserved totals.
#include "rkdg_generic.cuh"
#include "rkdg_launch.h"

namespace rkdg {

bool generic_supported(int geom, int p) {
  if (geom == 2) return p == 1 || p == 2;
  if (geom == 3) return p >= 1 && p <= 3;
  if (geom == 5) return p == 1 || p == 2;
  return false;
}

#define RKDG_DISPATCH(CALL)                        \
  switch (geom * 10 + p) {                         \
    case 21: return CALL(2, 1);                    \
    case 22: return CALL(2, 2);                    \
    case 31: return CALL(3, 1);                    \
    case 32: return CALL(3, 2);                    \
    case 33: return CALL(3, 3);                    \
    case 51: return CALL(5, 1);                    \
    case 52: return CALL(5, 2);                    \
    default: return cudaErrorInvalidValue;         \
  }

cudaError_t launch_rhs(int geom, int p, int prec, const RhsParams& prm, const void* u,
                       const void* ep, cudaStream_t st) {
#define CALL_RHS(G, P) launch_rhs_t<G, P>(prec, prm, u, ep, st)
  RKDG_DISPATCH(CALL_RHS)
#undef CALL_RHS
}

cudaError_t launch_rhs_v(int variant, int geom, int p, int prec, const RhsParams& prm,
                         const void* u, const void* ep, cudaStream_t st) {
  if (geom == 5 && variant != 0) return launch_hex_variant(variant, p, prec, prm, u, ep, st);
  return launch_rhs(geom, p, prec, prm, u, ep, st);
}

cudaError_t launch_limit(int geom, int p, int mode, const LimParams& prm, void* u, float* ulo,
                         cudaStream_t st) {
#define CALL_LIM(G, P) launch_limit_t<G, P>(mode, prm, u, ulo, st)
  RKDG_DISPATCH(CALL_LIM)
#undef CALL_LIM
}

cudaError_t launch_means(int geom, int p, int mode, int ne, long long ndofs,
                         const RefTables* tab, const void* u, const float* ulo, double* means,
                         cudaStream_t st) {
#define CALL_MEANS(G, P) launch_means_t<G, P>(mode, ne, ndofs, tab, u, ulo, means, st)
  RKDG_DISPATCH(CALL_MEANS)
#undef CALL_MEANS
}

template <int DIM, typename R>
__global__ void k_riemann_batch(int n, const double* u1, const double* u2, const double* nor,
                                double* flux, double* speed, double gamma, double cov, int rs,
                                int avg) {
  constexpr int NEQ = DIM + 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  R s1[NEQ], s2[NEQ], nn[DIM], F[NEQ];
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    s1[k] = (R)u1[(long long)i * NEQ + k];
    s2[k] = (R)u2[(long long)i * NEQ + k];
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) nn[d] = (R)nor[(long long)i * DIM + d];
  const R sp = riemann<DIM>(s1, s2, nn, F, (R)gamma, (R)cov, rs, avg);
  speed[i] = (double)sp;
  // -1 flags a non-physical state; HLLC's signed max(SL, SR) may be negative
  // with a valid flux
#pragma unroll
  for (int k = 0; k < NEQ; ++k) flux[(long long)i * NEQ + k] = sp == R(-1) ? 0.0 : (double)F[k];
}

cudaError_t launch_riemann_batch(int dim, int prec, int n, const double* u1, const double* u2,
                                 const double* nor, double* flux, double* speed, double gamma,
                                 double cov, int rs, int avg, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int bs = 128, grid = (n + bs - 1) / bs;
  if (dim == 2) {
    if (prec == 0)
      k_riemann_batch<2, double><<<grid, bs, 0, st>>>(n, u1, u2, nor, flux, speed, gamma, cov, rs, avg);
    else
      k_riemann_batch<2, float><<<grid, bs, 0, st>>>(n, u1, u2, nor, flux, speed, gamma, cov, rs, avg);
  } else {
    if (prec == 0)
      k_riemann_batch<3, double><<<grid, bs, 0, st>>>(n, u1, u2, nor, flux, speed, gamma, cov, rs, avg);
    else
      k_riemann_batch<3, float><<<grid, bs, 0, st>>>(n, u1, u2, nor, flux, speed, gamma, cov, rs, avg);
  }
  return cudaGetLastError();
}

__global__ void k_split(long long n, const double* __restrict__ x, float* __restrict__ hi,
                        float* __restrict__ lo) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = (float)v;
    hi[i] = h;
    lo[i] = (float)(v - (double)h);
  }
}
__global__ void k_join(long long n, const float* __restrict__ hi, const float* __restrict__ lo,
                       double* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = (double)hi[i] + (double)lo[i];
}
__global__ void k_to_float(long long n, const double* __restrict__ x, float* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void k_copy_f(long long n, const float* __restrict__ x, float* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = x[i];
}

static int grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  if (g < 1) g = 1;
  return (int)g;
}

cudaError_t launch_split(long long n, const double* x, float* hi, float* lo, cudaStream_t st) {
  k_split<<<grid_for(n), 256, 0, st>>>(n, x, hi, lo);
  return cudaGetLastError();
}
cudaError_t launch_join(long long n, const float* hi, const float* lo, double* x,
                        cudaStream_t st) {
  k_join<<<grid_for(n), 256, 0, st>>>(n, hi, lo, x);
  return cudaGetLastError();
}
cudaError_t launch_to_float(long long n, const double* x, float* y, cudaStream_t st) {
  k_to_float<<<grid_for(n), 256, 0, st>>>(n, x, y);
  return cudaGetLastError();
}
cudaError_t launch_copy_f(long long n, const float* x, float* y, cudaStream_t st) {
  k_copy_f<<<grid_for(n), 256, 0, st>>>(n, x, y);
  return cudaGetLastError();
}

// Discretely conserved totals: sum over elements of det J_e * sum_j m_j u_j,
// m_j = reference integral of phi_j (wmean * |ref element|).  One partial sum
// per block and equation; the host adds the partials.
__global__ void k_totals(int nd, int neq, int ne, long long ndofs, const RefTables* tab,
                         const double* __restrict__ wdet, const double* __restrict__ u,
                         double* __restrict__ partial) {
  __shared__ double red[256];
  for (int k = 0; k < neq; ++k) {
    double s = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
      double v = 0.0;
      for (int j = 0; j < nd; ++j)
        v += (tab->wmn_e ? tab->wmn_e[(long long)e * nd + j] : tab->wmean[j]) *
             u[k * ndofs + (long long)e * nd + j];
      s += wdet[e] * v;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[k * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}

// ---- batched problems: device-side time control ------------------------------
__device__ __forceinline__ double bits_to_double(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

// Initial dt per problem from its face-only max speed (main.cpp:467-484) or
// the given constant, and the first step's dt_real.
// Map of the active work for the stage kernels: the active problems in order
// and the exclusive prefix sums of their element counts, by the first warp of
// a single CTA (a warp scan over runs of 32 problems).
__device__ void build_active_map(const BatchState& bs) {
  if (!bs.act_cum || threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  int run = 0, na = 0;
  for (int base = 0; base < bs.nprob; base += 32) {
    const int p = base + lane;
    const bool a = p < bs.nprob && bs.active[p];
    const int sz = a ? bs.poff[p + 1] - bs.poff[p] : 0;
    int cs = sz, cf = a ? 1 : 0;  // inclusive scans of sizes and of active flags
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int ts = __shfl_up_sync(0xffffffffu, cs, o);
      const int tf = __shfl_up_sync(0xffffffffu, cf, o);
      if (lane >= o) {
        cs += ts;
        cf += tf;
      }
    }
    if (a) {
      bs.act_pid[na + cf - 1] = p;
      bs.act_cum[na + cf - 1] = run + cs - sz;
    }
    run += __shfl_sync(0xffffffffu, cs, 31);
    na += __shfl_sync(0xffffffffu, cf, 31);
  }
  if (lane == 0) {
    bs.act_cum[na] = run;
    bs.act_n[0] = na;
  }
}

__global__ void k_batch_map(BatchState bs) { build_active_map(bs); }

// dt_real of problem p as a float pair for the FP32 stage kernels
__device__ __forceinline__ void store_dtr2(const BatchState& bs, int p) {
  if (!bs.dtr2) return;
  const double d = bs.dtr[p];
  const float h = (float)d;
  bs.dtr2[p] = make_float2(h, (float)(d - (double)h));
}

__global__ void k_batch_init(BatchState bs, double dt0) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < bs.nprob; p += gridDim.x * blockDim.x) {
    double dt = dt0;
    if (bs.dt_mode != 2) dt = bs.cfl * bs.hmin[p] / bits_to_double(bs.mcs_last[p]) / bs.denom;
    bs.dt[p] = dt;
    bs.t[p] = 0.0;
    bs.sum_dt[p] = 0.0;
    bs.steps[p] = 0;
    const bool ok = isfinite(dt) && dt > 0.0;
    bs.active[p] = ok ? 1 : 0;
    bs.dtr[p] = fmin(dt, bs.t_end);
    store_dtr2(bs, p);
  }
}

// After a step: per-problem bookkeeping of main.cpp:512-553,701-733 (dt from
// the last stage's max speed, t += new dt, done test), the count of problems
// still running, and the while-condition of the graph that drives the loop.
__global__ void k_batch_control(BatchState bs, cudaGraphConditionalHandle handle, int use_handle) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int local = 0;
  for (int p = threadIdx.x; p < bs.nprob; p += blockDim.x) {
    if (!bs.active[p]) continue;
    bs.steps[p] += 1;
    if (bs.fail[p]) {  // the reference would exit here; this problem stops
      bs.active[p] = 0;
      continue;
    }
    bs.sum_dt[p] += bs.dtr[p];
    double dt = bs.dt[p];
    if (bs.dt_mode == 0) dt = bs.cfl * bs.hmin[p] / bits_to_double(bs.mcs_last[p]) / bs.denom;
    const double t = bs.t[p] + dt;
    bs.dt[p] = dt;
    bs.t[p] = t;
    bool done = t >= bs.t_end - 1e-8 * dt;
    if (bs.max_steps > 0 && bs.steps[p] >= bs.max_steps) done = true;
    if (!isfinite(dt) || !(dt > 0.0)) done = true;
    if (done) {
      bs.active[p] = 0;
    } else {
      bs.dtr[p] = fmin(dt, bs.t_end - t);
      store_dtr2(bs, p);
      ++local;
    }
  }
  if (local) atomicAdd(&cnt, local);
  __syncthreads();
  if (threadIdx.x == 0) {
    bs.nactive[0] = cnt;
    if (use_handle) cudaGraphSetConditional(handle, cnt > 0 ? 1u : 0u);
  }
  build_active_map(bs);
}

cudaError_t launch_batch_init(const BatchState& bs, double dt0, cudaStream_t st) {
  k_batch_init<<<(bs.nprob + 127) / 128, 128, 0, st>>>(bs, dt0);
  if (bs.act_cum) k_batch_map<<<1, 32, 0, st>>>(bs);
  return cudaGetLastError();
}
cudaError_t launch_batch_map(const BatchState& bs, cudaStream_t st) {
  k_batch_map<<<1, 32, 0, st>>>(bs);
  return cudaGetLastError();
}
cudaError_t launch_batch_control(const BatchState& bs, cudaGraphConditionalHandle h, int use_handle,
                                 cudaStream_t st) {
  k_batch_control<<<1, 1024, 0, st>>>(bs, h, use_handle);
  return cudaGetLastError();
}

cudaError_t launch_totals(int nd, int neq, int ne, long long ndofs, const RefTables* tab,
                          const double* wdet, const double* u, double* partial, int nblocks,
                          cudaStream_t st) {
  k_totals<<<nblocks, 256, 0, st>>>(nd, neq, ne, ndofs, tab, wdet, u, partial);
  return cudaGetLastError();
}

}  // namespace rkdg
