// sph_device.cuh -- device-side SPH arithmetic and per-particle kernels of
// the Plume-SPH particle step.
//
// Every pair formula restates the reference (paths inside the Plume-SPH
// source tree) with the reference's operation order, so that the FP64 path
// agrees with it to rounding:
//   weight / d_weight          src/plume/sph_lib.cc:210-253
//   compute_F                  src/plume/sph_lib.cc:257-281
//   art_vis                    src/plume/sph_lib.cc:402-424
//   SPH_epsilon_mom            src/plume/sph_lib.cc:1331-1338
//   SPH_epsilon_heat_cond.     src/plume/sph_lib.cc:1399-1440
//   update_second_var (EOS)    src/datstr/particle.cc:528-604
//   predicates                 src/datstr/particle.h:555-615
// The mixed path evaluates the same formulas in FP32 on bucket-relative
// coordinates with compensated (Kahan) FP32 sums.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

namespace plume {

constexpr double T1_INV_SQRT_PI = 0.564189583547756;  // sph_lib.cc:206
constexpr double KCUTOFF = 3.0;                       // CUTOFF, constant.h
constexpr double EPS_HALF = 0.4;                      // EPSILON_HALF
constexpr double PRANDTL = 0.85;                      // PRANDTL_NUM
constexpr double E_SMOOTH = 4.0;                      // E_SMOOTH_RATIO
constexpr double MSFRC_TH = 1.0e-6;                   // MSFRC_THRESH
constexpr double TINY_D = 1.0e-8;                     // TINY
constexpr double M4_S1 = 0.66666666666666663;         // cubic spline, 1D
constexpr double M4_S3 = 0.31830988618379069;         // cubic spline, 3D
constexpr uint8_t BC_DEAD = 255;                      // deleted this step

struct Opt {
  int dim, prec, kernel, lans, esmooth, pgc, adaptive, interval, num_loop;
  double thresh, c_smooth, eta, alpha, beta, ata, cfl, cutoff2, list_factor, g;
  double ng0, cvs, cvg, cva, rg, ra, vent_z, sml2;
  double max_time, timeoutput, stat_erupt, end_erupt;
  double ksupport;  // kernel support in units of h (3 Gaussian box, 2 M4)
  int max_steps;
  // GSPH (USE_GSPH 1): RIEMANN_SOLVER, MINI_DERIVATIVE_COND,
  // GSPH_SPECIFIC_VOL_APP, GSPH_MODIFIED_MONOTONICITY
  int method, gsph_solver, gsph_recon, gsph_vol, gsph_mono;
  int gsph_wave;  // HLL_WAVE_SPEED_EVA of the HLLC_RP_Solver_my solver
};

struct Geo {
  double mind[3];
  double del;
  double cw;  // fine cell edge = del / s
  double idel, icw;  // 1/del, 1/cw (multiplies instead of FP64 divisions)
  float icwf;        // 1/cw in FP32 (fine-cell index within a bucket)
  int nb[3];
  int s;
  int G[3];   // fine cells per axis = nb * s
  int dim;
  double lo[3], hi[3];  // original domain (escape planes)
  // place of the member's grid in the context's tables: its fine cells are
  // [cell_base, cell_base + G0*G1*G2) of the cell-start table, its buckets
  // [bucket_base, bucket_base + nbk) of the per-bucket tables
  uint32_t cell_base;
  int bucket_base, nbk;
};

struct Dev {  // particle arrays (one buffer set)
  uint64_t* key;
  double *x, *y, *z, *vx, *vy, *vz, *vsx, *vsy, *vsz, *mass, *h, *rho, *e, *p, *Y, *gam, *c, *T, *cp;
  uint8_t *phase, *bc, *inv;
  int32_t* bkt;   // member-local linear bucket id at the last search
  uint16_t* mem;  // ensemble member of the particle (0 for a single run)
};

struct Work {  // per-step scratch arrays (sorted order)
  double* hlist;  // h at the last search (list radius base, neighs.cc:84)
  double *nv0, *nv1, *nv2, *ne, *nrho, *nY, *nE;
  float *xr, *yr, *zr;  // bucket-relative coordinates (mixed path)
  // recorded for the adjoint (null otherwise): the energy-smoothing and LANS
  // normalisations sum_j (m_j / rho_j) W of the density and velocity sweeps
  double *wnd, *wnv;
};

struct TimeState {  // TimeProps on the device, properties.h:17-83
  double time, dtime, ndtimeoutput;
  int step, ioutput;
  unsigned long long dtmin_bits;  // min h/c of the step (positive doubles)
  int status;                     // first PLUME_E_* of the step
  int erupt;                      // iferupt() after incrtime
  unsigned long long n_lost;
  unsigned long long n_real;
  int active;  // the member steps (false once it reached TimeProps::ifend when frozen)
  int freeze;  // stop the member at ifend (ensembles); single runs step on
};

__device__ __forceinline__ void set_status(TimeState* ts, int code) { atomicCAS(&ts->status, 0, code); }

__device__ __forceinline__ bool need_neigh(uint8_t bc) { return bc == 100 || bc == 99; }
__device__ __forceinline__ bool is_real(uint8_t bc) { return bc == 100 || bc == 99; }
__device__ __forceinline__ bool contr_dens(uint8_t bc, int mode) {
  if (mode == 1) return bc == 100 || bc == 99 || bc == 1;
  if (mode == 2) return bc == 100 || bc == 99 || bc == 1 || bc == 0;
  return bc == 100 || bc == 99;
}
__device__ __forceinline__ bool contr_vel_smooth(uint8_t bc) { return bc == 100 || bc == 99 || bc == 2; }

// ---------------------------------------------------------------- kernels W
// Gaussian weight (sph_lib.cc:210-230).  Returns W; zero if any |s_k| > 3.
template <int D, typename T>
__device__ __forceinline__ T w_gauss(const T* s, T h) {
#pragma unroll
  for (int i = 0; i < D; i++)
    if (fabs(s[i]) > T(KCUTOFF)) return T(0);
  T norm = 1, expt = 0;
#pragma unroll
  for (int i = 0; i < D; i++) {
    norm *= T(T1_INV_SQRT_PI) / h;
    expt += s[i] * s[i];
  }
  return norm * exp(-expt);
}
template <>
__device__ __forceinline__ float w_gauss<3, float>(const float* s, float h) {
#pragma unroll
  for (int i = 0; i < 3; i++)
    if (fabsf(s[i]) > 3.0f) return 0.0f;
  float r = float(T1_INV_SQRT_PI) * __fdividef(1.0f, h);
  float expt = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
  return r * r * r * __expf(-expt);
}
// 1D: accurate expf and division.  The 1D sweeps are cheap, and the
// particles next to the tube-end ghosts amplify per-step errors by orders of
// magnitude, so the fast exponential's error (up to ~1e-6 relative at
// |s| = 3) is not worth its saving there.
template <>
__device__ __forceinline__ float w_gauss<1, float>(const float* s, float h) {
  if (fabsf(s[0]) > 3.0f) return 0.0f;
  return (float(T1_INV_SQRT_PI) / h) * expf(-s[0] * s[0]);
}
// cubic B-spline, radial support 2h
template <int D, typename T>
__device__ __forceinline__ T w_m4(const T* s, T h) {
  T r2 = 0;
#pragma unroll
  for (int i = 0; i < D; i++) r2 += s[i] * s[i];
  T q = sqrt(r2);
  if (q >= T(2)) return T(0);
  T norm = (D == 1) ? T(M4_S1) : T(M4_S3);
#pragma unroll
  for (int i = 0; i < D; i++) norm = norm / h;
  T w;
  if (q < T(1)) {
    w = T(1.0) - T(1.5) * q * q + T(0.75) * q * q * q;
  } else {
    T t = T(2.0) - q;
    w = T(0.25) * t * t * t;
  }
  return norm * w;
}
template <int D, typename T>
__device__ __forceinline__ T kw(int kernel, const T* s, T h) {
  return kernel == 1 ? w_m4<D, T>(s, h) : w_gauss<D, T>(s, h);
}
// gradient: dwdx[k] = d_weight(s, h, k) (sph_lib.cc:240-253) for all k
template <int D, typename T>
__device__ __forceinline__ void kdw(int kernel, const T* s, T h, T* dwdx) {
  if (kernel == 1) {
    T r2 = 0;
#pragma unroll
    for (int i = 0; i < D; i++) r2 += s[i] * s[i];
    T q = sqrt(r2);
    if (q >= T(2) || q == T(0)) {
#pragma unroll
      for (int k = 0; k < D; k++) dwdx[k] = T(0);
      return;
    }
    T norm = (D == 1) ? T(M4_S1) : T(M4_S3);
#pragma unroll
    for (int i = 0; i < D; i++) norm = norm / h;
    T dw;
    if (q < T(1)) {
      dw = T(-3.0) * q + T(2.25) * q * q;
    } else {
      T t = T(2.0) - q;
      dw = T(-0.75) * t * t;
    }
#pragma unroll
    for (int k = 0; k < D; k++) dwdx[k] = norm * dw * s[k] / (q * h);
  } else {
    T w = w_gauss<D, T>(s, h);
#pragma unroll
    for (int k = 0; k < D; k++) {
      T tmp = T(-2) * s[k] / h;
      dwdx[k] = tmp * w;
    }
  }
}

// compensated accumulator (plain for double)
template <typename T>
struct Acc {
  T s;
  __device__ __forceinline__ Acc() : s(0) {}
  __device__ __forceinline__ void add(T v) { s += v; }
  __device__ __forceinline__ void sub(T v) { s -= v; }
  __device__ __forceinline__ T get() const { return s; }
};
template <>
struct Acc<float> {
  float s, c;
  __device__ __forceinline__ Acc() : s(0.f), c(0.f) {}
  __device__ __forceinline__ void add(float v) {  // Kahan
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ void sub(float v) { add(-v); }
  __device__ __forceinline__ float get() const { return s; }
};

// Cascaded compensated accumulator of the list sweeps: terms are summed in
// plain arithmetic into a partial (the few pairs of one list window or row
// segment), and each partial is added to a compensated (Kahan) sum by
// flush().  FP64: plain.
template <typename T>
struct CAcc {
  T s;
  __device__ __forceinline__ CAcc() : s(0) {}
  __device__ __forceinline__ void add(T v) { s += v; }
  __device__ __forceinline__ void sub(T v) { s -= v; }
  __device__ __forceinline__ void flush() {}
  __device__ __forceinline__ T get() { return s; }
};
#ifndef PLUME_CASCADE
#define PLUME_CASCADE 0  // 1: plain partial sums per window, compensated across windows (measured slower)
#endif
#if PLUME_CASCADE
template <>
struct CAcc<float> {
  Acc<float> k;
  float w;
  __device__ __forceinline__ CAcc() : w(0.f) {}
  __device__ __forceinline__ void add(float v) { w += v; }
  __device__ __forceinline__ void sub(float v) { w -= v; }
  __device__ __forceinline__ void flush() {
    k.add(w);
    w = 0.f;
  }
  __device__ __forceinline__ float get() {
    flush();
    return k.get();
  }
};
#else
template <>
struct CAcc<float> {
  Acc<float> k;
  __device__ __forceinline__ void add(float v) { k.add(v); }
  __device__ __forceinline__ void sub(float v) { k.add(-v); }
  __device__ __forceinline__ void flush() {}
  __device__ __forceinline__ float get() { return k.get(); }
};
#endif

// Particle::update_second_var (particle.cc:528-604), ideal-gas mixture
__device__ __forceinline__ void eos(const Opt& o, double rho, double Y, double e, double& gam, double& p,
                                    double& c, double& T, double& cp, bool lans) {
  double na = 1 - Y;
  double ng = o.ng0 * Y;
  double ns = Y - ng;
  double Cvm = ns * o.cvs + ng * o.cvg + na * o.cva;
  double Rm = ng * o.rg + na * o.ra;
  double Rmg = Rm / (ng + na);
  gam = 1 + Rm / Cvm;
  double desmg = rho * (na + ng);
  p = Rmg * desmg * e / Cvm;
  c = sqrt(gam * p / desmg);
  T = e / Cvm;
  if (lans) cp = Cvm;
}

// ---------------------------------------------------------------- grid
// bucket index per axis with the comparisons of Bucket::contains
// (bucket.h:238-245) against mind + b*del; clamped into [0, nb-1]
__device__ __forceinline__ int bucket_axis(double x, double mind, double del, double idel, int nb,
                                           bool* outside) {
  // first guess by a multiply (the FP64 pipe of sm_103a is narrow), then the
  // exact comparisons of Bucket::contains decide
  double f = floor((x - mind) * idel);
  int b;
  if (!(f > -1.0)) {
    b = 0;
  } else if (!(f < (double)nb)) {
    b = nb - 1;
  } else {
    b = (int)f;
  }
  while (b > 0 && x < mind + b * del) b--;
  while (b < nb - 1 && x >= mind + (b + 1) * del) b++;
  if (outside) *outside = (x < mind + b * del) || (x >= mind + (b + 1) * del) || (x != x);
  return b;
}
// fine cell per axis: bucket * s + clamped sub-cell (monotone in x)
// binary64 -> binary32 rounding toward zero on the integer pipe (the
// exponent rebiased, the top 23 fraction bits kept): the FP64 pipe, which
// executes F2F, is narrow on this part.  Below the binary32 normal range the
// result is a signed zero, above it a signed infinity; NaN stays NaN.
__device__ __forceinline__ float f32_rz(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned sign = hi & 0x80000000u;
  const int ex = (int)((hi >> 20) & 0x7ffu);
  const int e = ex - 1023 + 127;
  unsigned r = sign | ((unsigned)e << 23) | ((unsigned)(b >> 29) & 0x7fffffu);
  if (e <= 0) r = sign;
  if (e >= 255) r = sign | 0x7f800000u;
  if (ex == 0x7ff && (b & 0xfffffffffffffull)) r = 0x7fc00000u;
  return __uint_as_float(r);
}

// Fine cell of x on axis a: the bucket exactly (Bucket::contains), the cell
// inside it from the FP32 offset (a monotone function of x, which is all the
// cell walks need: every user of cells calls this one function)
__device__ __forceinline__ int cell_axis(const Geo& g, int a, double x, int* bucket, bool* outside) {
  int b = bucket_axis(x, g.mind[a], g.del, g.idel, g.nb[a], outside);
  if (bucket) *bucket = b;
  const double off = x - (g.mind[a] + b * g.del);
  const float f = floorf(f32_rz(off) * g.icwf);
  int sub = (f > 0.f) ? (int)fminf(f, (float)(g.s - 1)) : 0;
  return b * g.s + sub;
}

}  // namespace plume
