// sph_warp.cuh -- warp-per-particle 3D pair sweeps with ballot compaction.
//
// One warp owns one particle i at a time.  Its lanes walk i's candidate
// rows (the search box clipped to the 27 buckets around i's bucket,
// search_neighs_consth, neighs.cc:37-211) 32 candidates at a time and apply
// a cheap, conservative filter: the reference's list rule (own bucket or
// inside list_factor * h_i, neighs.cc:84-131), the sweep's particle
// predicate and box, and the kernel support |dx_k| <= ksupport * h_ij.
// Survivors are compacted (ballot + popc) into a per-warp buffer; every
// time 32 have gathered, each lane evaluates one pair with the exact
// arithmetic of the sweep (pairs beyond the kernel support contribute
// exactly zero in the reference, so dropping them changes no sum).  The
// lanes' partial sums are reduced in FP64 at the end of the particle.
//
// The FP64 path reads the particle arrays directly; the mixed path reads
// per-sweep packed FP32 records (float4) written by k_pack_* with
// bucket-relative coordinates.
#pragma once
#include "sph_kernels.cuh"

namespace plume {

constexpr unsigned WFULL = 0xffffffffu;
constexpr int WP_WARPS = 4;  // warps per block (128 threads)

// Grid of a particle's member.  A single run (MULTI = false) reads its one
// grid from the kernel parameters (constant bank, no registers held across
// the pair loops); an ensemble (MULTI = true) reads the member's entry of
// the per-member table.
template <bool MULTI>
struct Geos {
  Geo g0;
  const Geo* __restrict__ tab;
  __device__ __forceinline__ int member(const Dev& A, int i) const { return MULTI ? (int)A.mem[i] : 0; }
  __device__ __forceinline__ const Geo& of(int m) const { return MULTI ? tab[m] : g0; }
};

// packed FP32 records of the mixed path (one set, rewritten per sweep)
struct Packed {
  float4* P;  // (xr, yr, zr, h or -h when the particle does not contribute)
  float4* Q;
  float4* R;
  float4* S;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(WFULL, v, o);
  return v;
}

// per-warp compaction buffer
template <typename T>
struct WBuf {
  int j[64];
  T dx[4][64];  // dx and h_j of the compacted pairs
};

// fast reciprocal for the mixed path, exact division for FP64
template <typename T>
__device__ __forceinline__ T rcp(T x) { return T(1) / x; }
template <>
__device__ __forceinline__ float rcp<float>(float x) { return __fdividef(1.0f, x); }

// Walks the candidates of particle i (warp-uniform arguments) and calls
// s.math(j, dx) for every survivor of s.filter(j, own, ox, oy, oz, dx).
template <typename T, class S>
__device__ __forceinline__ void wp_walk(const Geo& g, const uint32_t* __restrict__ cs, const double* xi,
                                        const int* bi, double R, WBuf<T>& B, S& s) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  int count = 0;
  int lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    int l = cell_axis(g, a, xi[a] - R, nullptr, nullptr);
    int h = cell_axis(g, a, xi[a] + R, nullptr, nullptr);
    lo[a] = max(l, max((bi[a] - 1) * g.s, 0));
    hi[a] = min(h, min((bi[a] + 2) * g.s - 1, g.G[a] - 1));
  }
  constexpr bool REL = sizeof(T) == 4;
  const T delT = T(g.del);
  for (int cz = lo[2]; cz <= hi[2]; cz++) {
    const int bz = cz / g.s;
    const T oz = REL ? T(bi[2] - bz) * delT : T(0);
    for (int cy = lo[1]; cy <= hi[1]; cy++) {
      const int by = cy / g.s;
      const T oy = REL ? T(bi[1] - by) * delT : T(0);
      const size_t rowbase = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      int cx = lo[0];
      while (cx <= hi[0]) {
        const int bx = cx / g.s;
        const int e = min(hi[0], bx * g.s + g.s - 1);
        const uint32_t j0 = cs[rowbase + cx];
        const uint32_t j1 = cs[rowbase + e + 1];
        const bool own = (bx == bi[0]) && (by == bi[1]) && (bz == bi[2]);
        const T ox = REL ? T(bi[0] - bx) * delT : T(0);
        for (uint32_t jb = j0; jb < j1; jb += 32) {
          const uint32_t j = jb + lane;
          T dx[3], hj;
          const bool take = (j < j1) && s.filter(j, own, ox, oy, oz, dx, hj);
          const unsigned m = __ballot_sync(WFULL, take);
          if (take) {
            const int slot = count + __popc(m & lt);
            B.j[slot] = (int)j;
            B.dx[0][slot] = dx[0];
            B.dx[1][slot] = dx[1];
            B.dx[2][slot] = dx[2];
            B.dx[3][slot] = hj;
          }
          count += __popc(m);
          __syncwarp();
          if (count >= 32) {
            T d[3] = {B.dx[0][lane], B.dx[1][lane], B.dx[2][lane]};
            s.math(B.j[lane], d, B.dx[3][lane]);
            if constexpr (sizeof(T) == 4) s.flush();
            __syncwarp();
            const int rest = count - 32;
            if (lane < rest) {
              B.j[lane] = B.j[lane + 32];
              B.dx[0][lane] = B.dx[0][lane + 32];
              B.dx[1][lane] = B.dx[1][lane + 32];
              B.dx[2][lane] = B.dx[2][lane + 32];
              B.dx[3][lane] = B.dx[3][lane + 32];
            }
            count = rest;
            __syncwarp();
          }
        }
        cx = e + 1;
      }
    }
  }
  if (lane < count) {
    T d[3] = {B.dx[0][lane], B.dx[1][lane], B.dx[2][lane]};
    s.math(B.j[lane], d, B.dx[3][lane]);
  }
  __syncwarp();
}

// ------------------------------------------------------------ particle data
// FP64 path: SoA loads; mixed path: packed records
template <typename T>
struct JPos;
template <>
struct JPos<double> {
  __device__ __forceinline__ static void get(const Dev& A, const Packed&, uint32_t j, double* x, double& h) {
    x[0] = A.x[j]; x[1] = A.y[j]; x[2] = A.z[j];
    h = A.h[j];
  }
};
// list sweeps that load the next window's list entry one window ahead
// (S::kListAhead): on the 134^3 plume at h ~ 1.5 dx the momentum sweep 13.44
// -> 12.87 ms and the LANS filter 8.02 -> 7.72 ms, while the density sweep
// went 7.35 -> 7.79 ms and keeps the plain load (all measured with the
// earlier register caps, 6, 8 and 8 blocks per SM).  0 turns it off
// everywhere.
#ifndef PLUME_LIST_AHEAD
#define PLUME_LIST_AHEAD 1
#endif

template <>
struct JPos<float> {
  __device__ __forceinline__ static void get(const Dev&, const Packed& K, uint32_t j, float* x, float& h) {
    const float4 p = K.P[j];
    x[0] = p.x; x[1] = p.y; x[2] = p.z;
    h = p.w;
  }
};

// ------------------------------------------------------------ momentum
// FP32 momentum record and pair: 1 stores h, rho, c, cp halved and m V (the
// same pair values with fewer operations), 2 also forms |s|^2 as |dx|^2/h^2
// and folds 1/Pr into the heat term's constant (rounding differs)
#ifndef PLUME_MOM_FOLD
#define PLUME_MOM_FOLD 2
#endif
constexpr bool kMomHalf = PLUME_MOM_FOLD >= 1;
constexpr bool kMomFold = PLUME_MOM_FOLD >= 2;
template <typename T>
struct WMom {
  const Dev& A;
  const Packed& K;
  const Opt& o;
  bool lans;
  uint32_t i;
  T xs[3], hi, supp, Lb, rhoi, Vi, pvsqi, ci, tempi, Cp_i, veli[3];
  __device__ __forceinline__ const T* xpos() const { return xs; }
  T ks_half, ata, alpha, beta;  // option constants in the sweep's type
  CAcc<T> rv[3], re;
  __device__ __forceinline__ void flush() {
    rv[0].flush(); rv[1].flush(); rv[2].flush(); re.flush();
  }
  static constexpr bool kListAhead = true;  // the list walk's entry look-ahead
  static constexpr bool kSkipDecode = false;  // the list walk keeps a repeated bucket's offsets
  __device__ WMom(const Dev& A_, const Packed& K_, const Opt& o_) : A(A_), K(K_), o(o_) {}
  // i-side set-up; returns false (with the status set) when i is skipped
  __device__ __forceinline__ bool setup(int ii, const Geo& g, const Work& W, const double* hmax, TimeState* ts,
                                        double* xi, int* bi, double& R) {
    const double rho_i = A.rho[ii];
    if (!(rho_i > 0)) {
      set_status(ts, 4);
      return false;
    }
    lans = o.lans != 0;
    i = (uint32_t)ii;
    xi[0] = A.x[ii]; xi[1] = A.y[ii]; xi[2] = A.z[ii];
    const int b = A.bkt[ii];
    bucket_coords<3>(g, b, bi);
    Pos<3, T>::load(A, W, ii, xs);
    const double hi_d = A.h[ii];
    hi = T(hi_d);
    supp = T(o.cutoff2) * hi;
    Lb = T(o.list_factor * W.hlist[ii]);
    rhoi = T(rho_i);
    Vi = T(1.0) / rhoi;
    pvsqi = T(A.p[ii]) * Vi * Vi;
    ci = T(A.c[ii]);
    tempi = T(A.T[ii]);
    Cp_i = T(A.cp[ii]);
    if (lans) {
      veli[0] = T(A.vsx[ii]); veli[1] = T(A.vsy[ii]); veli[2] = T(A.vsz[ii]);
    } else {
      veli[0] = T(A.vx[ii]); veli[1] = T(A.vy[ii]); veli[2] = T(A.vz[ii]);
    }
    R = fmin(o.cutoff2 * hi_d, o.ksupport * 0.5 * (hi_d + hmax[b])) * (1.0 + 1e-10);
    ks_half = T(o.ksupport * 0.5 * (1.0 + 1e-6));
    ata = T(o.ata);
    alpha = T(o.alpha);
    beta = T(o.beta);
    return true;
  }
  template <bool WARP>
  __device__ __forceinline__ void finish(int ii, Work& W, TimeState* ts) {
    double r0 = (double)rv[0].get(), r1 = (double)rv[1].get(), r2 = (double)rv[2].get();
    double e = (double)re.get();
    if (WARP) {
      r0 = warp_sum(r0); r1 = warp_sum(r1); r2 = warp_sum(r2); e = warp_sum(e);
      if ((threadIdx.x & 31) != 0) return;
    }
    const double dt = ts->dtime;
    const double grav = -o.g;
    double unew2 = A.vz[ii] + dt * r2;
    unew2 += dt * grav;
    W.nv0[ii] = A.vx[ii] + dt * r0;
    W.nv1[ii] = A.vy[ii] + dt * r1;
    W.nv2[ii] = unew2;
    W.ne[ii] = A.e[ii] + dt * (e + (double)veli[2] * grav);
  }
  // LISTED: j comes from the stored list, which already passed the list
  // box and the CUTOFF2 box (k_build_lists)
  template <bool LISTED = false>
  __device__ __forceinline__ bool filter(uint32_t j, bool own, T ox, T oy, T oz, T* dx, T& hj) const {
    if (j == i) return false;
    T xj[3];
    JPos<T>::get(A, K, j, xj, hj);
    // listed: ox, oy, oz are i's position shifted into j's bucket
    dx[0] = (LISTED ? ox : xs[0] + ox) - xj[0];
    dx[1] = (LISTED ? oy : xs[1] + oy) - xj[1];
    dx[2] = (LISTED ? oz : xs[2] + oz) - xj[2];
    if (!LISTED) {
      if (!own && !in_box<3, T>(dx, Lb)) return false;
      if (!in_box<3, T>(dx, supp)) return false;
    }
    if constexpr (sizeof(T) == 4 && kMomHalf) hj *= 2.0f;  // the record holds h_j / 2
    const T ks = ks_half * (hi + fabs(hj));
    return in_box<3, T>(dx, ks);
  }
  // j-side fields; pVVj = p_j V_j V_j, the reference's pressj * Vj * Vj
  __device__ __forceinline__ void load_j(uint32_t j, T& mj, T& rhoj, T& Vj, T& pVVj, T& cj, T& Tj, T& cpj,
                                         T* vj) const;
  // A listed candidate of the mixed Gaussian path, in one piece: the four
  // records of j are loaded together, then the pair arithmetic of math()
  // runs without branches; a candidate outside the kernel support (or j ==
  // i) contributes exactly zero through f = 0.  o[] is i's position shifted
  // into j's bucket.  W = pi^-3/2 ih^3 e^-|s|^2, f = -2 ih W.
  __device__ __forceinline__ void listed(uint32_t j, float ox, float oy, float oz) {
    if (lans)
      listed_l<true>(j, ox, oy, oz);
    else
      listed_l<false>(j, ox, oy, oz);
  }
  // LANS: the LANS terms (o.lans), a compile-time choice in the list loop
  template <bool LANS>
  __device__ __forceinline__ void listed_l(uint32_t j, float ox, float oy, float oz) {
    const float4 pj = K.P[j], qj = K.Q[j], rj = K.R[j], sj = K.S[j];
    const float d0 = ox - pj.x, d1 = oy - pj.y, d2 = oz - pj.z;
    // kMomHalf: the record holds h_j/2, rho_j/2, c_j/2, cp_j/2 and m_j V_j,
    // so each mean is one FMA (the same values: halving is exact)
    const float h = kMomHalf ? fmaf(0.5f, hi, pj.w) : 0.5f * (hi + pj.w);
    const float ih = rcp<float>(h);
    const float s0 = d0 * ih, s1 = d1 * ih, s2 = d2 * ih;
    const float dist_sq = d0 * d0 + d1 * d1 + d2 * d2;
    const float v0 = veli[0] - rj.w, v1 = veli[1] - sj.x, v2 = veli[2] - sj.y;
    const float sndspdab = kMomHalf ? fmaf(0.5f, ci, rj.x) : 0.5f * (ci + rj.x);
    const float vrab = d0 * v0 + d1 * v1 + d2 * v2;
    const float miuab = h * vrab * rcp<float>(dist_sq + ata * h * h);
    const float rhoab = kMomHalf ? fmaf(0.5f, rhoi, qj.y) : 0.5f * (rhoi + qj.y);
    float vis = (vrab < 0.0f) ? (beta * miuab - alpha * sndspdab) * miuab * rcp<float>(rhoab) : 0.0f;
    const float dotv = v0 * v0 + v1 * v1 + v2 * v2;
    if constexpr (LANS) vis -= float(EPS_HALF) * dotv * qj.z;
    const float mpvsqij = qj.x * (qj.w + pvsqi + vis);
    const bool in = (j != i) && fabsf(s0) <= 3.0f && fabsf(s1) <= 3.0f && fabsf(s2) <= 3.0f;
    const float ih2 = ih * ih;
    const float qq = kMomFold ? dist_sq * ih2 : s0 * s0 + s1 * s1 + s2 * s2;
    const float f = in ? KF * (ih2 * ih2) * __expf(-qq) : 0.0f;
    const float gm = mpvsqij * f;
    rv[0].sub(gm * s0);
    rv[1].sub(gm * s1);
    rv[2].sub(gm * s2);
    float heat_tran = 0.0f;
    if constexpr (LANS) {
      // m_j V_j V_i k_ij (T_i - T_j) f/h with k_ij = 10 eps Cp_ij |dx|^2
      // |v_ij|^2 / (Pr dotvr h c_ab)
      const float Cp_ij = kMomHalf ? fmaf(0.5f, Cp_i, rj.z) : 0.5f * (rj.z + Cp_i);
      const float dotvr = fabsf(v0 * d0) + fabsf(v1 * d1) + fabsf(v2 * d2);
      const float kij = kMomFold ? float(10.0 * EPS_HALF / PRANDTL) * Cp_ij * dist_sq * dotv *
                                       rcp<float>(dotvr * h * sndspdab)
                                 : 10.0f * float(EPS_HALF) * Cp_ij * dist_sq * dotv *
                                       rcp<float>(float(PRANDTL) * dotvr * h * sndspdab);
      const float mVj = kMomHalf ? sj.z : qj.x * qj.z;
      heat_tran = (dotvr != 0.0f) ? mVj * Vi * kij * (tempi - rj.y) * (f * ih) : 0.0f;
    }
    re.add(0.5f * gm * ih * vrab + heat_tran);
  }
  static constexpr float KF = float(-2.0 * T1_INV_SQRT_PI * T1_INV_SQRT_PI * T1_INV_SQRT_PI);
  __device__ __forceinline__ void math(uint32_t j, const T* dx, T hj) {
    T mj, rhoj, Vj, pVVj, cj, Tj, cpj, vj[3];
    load_j(j, mj, rhoj, Vj, pVVj, cj, Tj, cpj, vj);
    const T h = T(0.5) * (hi + hj);
    const T ih = rcp<T>(h);
    T si[3], dist_sq = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      si[k] = (sizeof(T) == 8) ? dx[k] / h : dx[k] * ih;
      dist_sq += dx[k] * dx[k];
    }
    T velij[3] = {veli[0] - vj[0], veli[1] - vj[1], veli[2] - vj[2]};
    const T rhoab = T(0.5) * (rhoi + rhoj);
    const T sndspdab = T(0.5) * (ci + cj);
    T vrab = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) vrab += dx[k] * velij[k];
    const T miuab = (sizeof(T) == 8) ? h * vrab / (dist_sq + ata * h * h)
                                     : h * vrab * rcp<T>(dist_sq + ata * h * h);
    T vis = 0;
    if (vrab < 0)
      vis = (sizeof(T) == 8) ? (beta * miuab - alpha * sndspdab) * miuab / rhoab
                             : (beta * miuab - alpha * sndspdab) * miuab * rcp<T>(rhoab);
    T dotv = 0;
    if (lans) {
#pragma unroll
      for (int k = 0; k < 3; k++) dotv += velij[k] * velij[k];
      vis -= T(EPS_HALF) * dotv * Vj;
    }
    const T mpvsqij = mj * (pVVj + pvsqi + vis);
    if constexpr (sizeof(T) == 4) {
      if (o.kernel != 1) {
        // Gaussian, mixed: dW/dx_k = f s_k with f = -2 W / h; the reference's
        // sums regrouped with s = dx / h: dW . v_ij = f vrab / h,
        // dW . dx = f |dx|^2 / h, so F_ij = dW . dx / |dx|^2 = f / h
        const T w = (fabs(si[0]) > T(3) || fabs(si[1]) > T(3) || fabs(si[2]) > T(3))
                        ? T(0)
                        : (T(T1_INV_SQRT_PI) * ih) * (T(T1_INV_SQRT_PI) * ih) * (T(T1_INV_SQRT_PI) * ih) *
                              __expf(-(si[0] * si[0] + si[1] * si[1] + si[2] * si[2]));
        const T f = T(-2) * ih * w;
        const T gm = mpvsqij * f;
#pragma unroll
        for (int k = 0; k < 3; k++) rv[k].sub(gm * si[k]);
        T heat_tran = 0;
        if (lans && f != T(0)) {
          const T Cp_ij = T(0.5) * (cpj + Cp_i);
          T dotvr = 0;
#pragma unroll
          for (int k = 0; k < 3; k++) dotvr += fabs(velij[k] * dx[k]);
          if (dotvr != T(0)) {
            // k_ij = 10 eps Cp_ij |dx|^2 |v_ij|^2 / (Pr dotvr h c_ab), one reciprocal
            const T kij = T(10.0) * T(EPS_HALF) * Cp_ij * dist_sq * dotv *
                          rcp<T>(T(PRANDTL) * dotvr * h * sndspdab);
            heat_tran = mj * Vj * Vi * kij * (tempi - Tj) * (f * ih);
          }
        }
        re.add(T(0.5) * gm * ih * vrab + heat_tran);
        return;
      }
    }
    T dwdx[3];
    kdw<3, T>(o.kernel, si, h, dwdx);
    T heat_tran = 0;
    if (lans) {
      const T Cp_ij = T(0.5) * (cpj + Cp_i);
      T dotvr = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) dotvr += fabs(velij[k] * dx[k]);
      T kij = 0;
      if (dotvr != T(0)) {
        const T kab = (sizeof(T) == 8)
                          ? T(10.0) * T(EPS_HALF) * Cp_ij * dist_sq * dotv / (T(PRANDTL) * dotvr)
                          : T(10.0) * T(EPS_HALF) * Cp_ij * dist_sq * dotv * rcp<T>(T(PRANDTL) * dotvr);
        kij = (sizeof(T) == 8) ? kab / (h * sndspdab) : kab * rcp<T>(h * sndspdab);
      }
      T W_r = 0, Fij = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) W_r += dwdx[k] * dx[k];
      if (W_r != T(0)) Fij = (sizeof(T) == 8) ? W_r / dist_sq : W_r * rcp<T>(dist_sq);
      heat_tran = mj * Vj * Vi * kij * (tempi - Tj) * Fij;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) rv[k].sub(mpvsqij * dwdx[k]);
    T deltae = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) deltae += T(0.5) * (mpvsqij * dwdx[k]) * velij[k];
    re.add(deltae + heat_tran);
  }
};
template <>
__device__ __forceinline__ void WMom<double>::load_j(uint32_t j, double& mj, double& rhoj, double& Vj,
                                                     double& pVVj, double& cj, double& Tj, double& cpj,
                                                     double* vj) const {
  mj = A.mass[j]; rhoj = A.rho[j]; cj = A.c[j]; Tj = A.T[j]; cpj = A.cp[j];
  Vj = 1.0 / rhoj;
  pVVj = A.p[j] * Vj * Vj;
  if (lans) {
    vj[0] = A.vsx[j]; vj[1] = A.vsy[j]; vj[2] = A.vsz[j];
  } else {
    vj[0] = A.vx[j]; vj[1] = A.vy[j]; vj[2] = A.vz[j];
  }
}
template <>
__device__ __forceinline__ void WMom<float>::load_j(uint32_t j, float& mj, float& rhoj, float& Vj, float& pVVj,
                                                    float& cj, float& Tj, float& cpj, float* vj) const {
  const float4 q = K.Q[j], r = K.R[j], s = K.S[j];
  const float u = kMomHalf ? 2.0f : 1.0f;  // halved means in the record
  mj = q.x; rhoj = u * q.y; Vj = q.z; pVVj = q.w;
  cj = u * r.x; Tj = r.y; cpj = u * r.z; vj[0] = r.w;
  vj[1] = s.x; vj[2] = s.y;
}

// momentum record: P (xr,yr,zr,h), Q (m, rho, 1/rho, p/rho^2), R (c,T,cp,vx),
// S (vy,vz, m/rho); with kMomHalf h, rho, c and cp are stored halved (the
// pair forms their means with one FMA)
__global__ void k_pack_mom(Dev A, Packed K, Work W, int lans, const int* __restrict__ d_count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *d_count) return;
  // fields narrowed on the integer pipe, V and p V^2 formed in FP32
  const float rho = f32_rz(A.rho[j]), V = 1.0f / rho;
  const float u = kMomHalf ? 0.5f : 1.0f;
  const float m = f32_rz(A.mass[j]);
  K.P[j] = make_float4(W.xr[j], W.yr[j], W.zr[j], u * f32_rz(A.h[j]));
  K.Q[j] = make_float4(m, u * rho, V, f32_rz(A.p[j]) * V * V);
  const double vx = lans ? A.vsx[j] : A.vx[j];
  const double vy = lans ? A.vsy[j] : A.vy[j];
  const double vz = lans ? A.vsz[j] : A.vz[j];
  K.R[j] = make_float4(u * f32_rz(A.c[j]), f32_rz(A.T[j]), u * f32_rz(A.cp[j]), f32_rz(vx));
  K.S[j] = make_float4(f32_rz(vy), f32_rz(vz), m * V, 0.f);
}

// ------------------------------------------------------------ density
template <typename T>
struct WDens {
  const Dev& A;
  const Packed& K;
  const Opt& o;
  int pgc;
  T xs[3], hi, supp, Lb, ks_half;
  __device__ __forceinline__ const T* xpos() const { return xs; }
  CAcc<T> rho1, rho2, wnorm_e, engr;
  bool esm;
  __device__ __forceinline__ void flush() {
    rho1.flush(); rho2.flush(); wnorm_e.flush(); engr.flush();
  }
  static constexpr bool kListAhead = false;  // the list walk's entry look-ahead
  static constexpr bool kSkipDecode = false;  // the list walk keeps a repeated bucket's offsets
  __device__ WDens(const Dev& A_, const Packed& K_, const Opt& o_) : A(A_), K(K_), o(o_) {}
  __device__ __forceinline__ bool setup(int ii, const Geo& g, const Work& W, const double* hmax, TimeState*,
                                        double* xi, int* bi, double& R) {
    pgc = o.pgc;
    esm = o.esmooth != 0;
    xi[0] = A.x[ii]; xi[1] = A.y[ii]; xi[2] = A.z[ii];
    const int b = A.bkt[ii];
    bucket_coords<3>(g, b, bi);
    Pos<3, T>::load(A, W, ii, xs);
    const double hi_d = A.h[ii];
    hi = T(hi_d);
    supp = T(o.cutoff2) * hi;
    Lb = T(o.list_factor * W.hlist[ii]);
    R = fmin(o.cutoff2 * hi_d, o.ksupport * 0.5 * (hi_d + hmax[b])) * (1.0 + 1e-10);
    ks_half = T(o.ksupport * 0.5 * (1.0 + 1e-6));
    return true;
  }
  template <bool WARP>
  __device__ __forceinline__ void finish(int ii, Work& W, TimeState* ts) {
    double r1 = (double)rho1.get(), r2 = (double)rho2.get();
    double wn = (double)wnorm_e.get(), en = (double)engr.get();
    if (WARP) {
      r1 = warp_sum(r1); r2 = warp_sum(r2); wn = warp_sum(wn); en = warp_sum(en);
      if ((threadIdx.x & 31) != 0) return;
    }
    if (esm) {
      if (!(wn > 0)) {
        set_status(ts, 4);
        return;
      }
      W.nE[ii] = en / wn;
      if (W.wnd) W.wnd[ii] = wn;
    }
    double density = 0.0;
    density += r1;
    density += r2;
    if (!(density > 0)) {
      set_status(ts, (density != density) ? 3 : 4);
      return;
    }
    W.nrho[ii] = density;
    W.nY[ii] = r2 / density;
  }
  template <bool LISTED = false>
  __device__ __forceinline__ bool filter(uint32_t j, bool own, T ox, T oy, T oz, T* dx, T& hj) const {
    T xj[3];
    JPos<T>::get(A, K, j, xj, hj);
    if (sizeof(T) == 8) {
      const uint8_t ph = A.phase[j];
      if (!contr_dens(A.bc[j], pgc) || (ph != 1 && ph != 2)) return false;
    } else if (hj < T(0)) {
      return false;
    }
    // listed: ox, oy, oz are i's position shifted into j's bucket
    dx[0] = (LISTED ? ox : xs[0] + ox) - xj[0];
    dx[1] = (LISTED ? oy : xs[1] + oy) - xj[1];
    dx[2] = (LISTED ? oz : xs[2] + oz) - xj[2];
    if (!LISTED) {
      if (!own && !in_box<3, T>(dx, Lb)) return false;
      if (!in_box<3, T>(dx, supp)) return false;
    }
    const T ks = ks_half * (hi + fabs(hj));
    return in_box<3, T>(dx, ks);
  }
  // the mixed Gaussian pair of math() with j's density record q = (m, m/rho,
  // m e/rho, phase) already loaded: W(s, h) = r^3 exp(-s.s), r = 1/(sqrt(pi)
  // h); the energy-smoothing kernel at h/4 is 64 r^3 exp(-16 s.s), zero once
  // any |s_k| > 3/4
  __device__ __forceinline__ void math_q(const float4 q, float d0, float d1, float d2, float hj) {
    const float hh = 0.5f * (float(hi) + hj);
    const float ih = rcp<float>(hh);
    const float s0 = d0 * ih, s1 = d1 * ih, s2 = d2 * ih;
    const float ax = fabsf(s0), ay = fabsf(s1), az = fabsf(s2);
    const float qq = s0 * s0 + s1 * s1 + s2 * s2;
    const float r = float(T1_INV_SQRT_PI) * ih;
    const float r3 = r * r * r;
    const float amax = fmaxf(ax, fmaxf(ay, az));
    if (esm && amax <= 0.75f) {
      const float w_e = 64.0f * r3 * __expf(-16.0f * qq);
      wnorm_e.add(w_e * q.y);
      engr.add(w_e * q.z);
    }
    if (amax > 3.0f) return;
    const float wm = r3 * __expf(-qq) * q.x;
    if (q.w == 1.0f)
      rho1.add(wm);
    else
      rho2.add(wm);
  }
  __device__ __forceinline__ void math(uint32_t j, const T* ds, T hj) {
    if constexpr (sizeof(T) == 4) {
      if (o.kernel != 1) {
        math_q(K.Q[j], ds[0], ds[1], ds[2], fabsf(hj));
        return;
      }
    }
    // FP64: the reference's fields; mixed: (m, m/rho, m e/rho, phase)
    T mj, rhoj = 0, ej = 0, mvr = 0, mer = 0, ph;
    if constexpr (sizeof(T) == 8) {
      mj = A.mass[j]; rhoj = A.rho[j]; ej = A.e[j]; ph = T(A.phase[j]);
    } else {
      const float4 q = K.Q[j];
      mj = q.x; mvr = q.y; mer = q.z; ph = q.w;
      hj = fabsf(hj);
    }
    const T hh = T(0.5) * (hi + hj);
    T sv[3];
    const T ih = rcp<T>(hh);
#pragma unroll
    for (int k = 0; k < 3; k++) sv[k] = (sizeof(T) == 8) ? ds[k] / hh : ds[k] * ih;
    if (esm) {
      T s_e[3];
#pragma unroll
      for (int k = 0; k < 3; k++) s_e[k] = (sizeof(T) == 8) ? T(E_SMOOTH) * ds[k] / hh : T(E_SMOOTH) * ds[k] * ih;
      if constexpr (sizeof(T) == 8) {
        const T wm_e = kw<3, T>(o.kernel, s_e, hh / T(E_SMOOTH)) * mj;
        wnorm_e.add(wm_e / rhoj);
        engr.add(wm_e * ej / rhoj);
      } else {
        const T w_e = kw<3, T>(o.kernel, s_e, hh * T(0.25));
        wnorm_e.add(w_e * mvr);
        engr.add(w_e * mer);
      }
    }
    const T wm = kw<3, T>(o.kernel, sv, hh) * mj;
    if (ph == T(1))
      rho1.add(wm);
    else
      rho2.add(wm);
  }
};

template <typename T>
__device__ __forceinline__ void dens_listed(WDens<T>& s, uint32_t j, float ox, float oy, float oz) {
  // a listed candidate of the mixed Gaussian path: both records loaded
  // together, then math() (which drops pairs outside the support)
  const float4 pj = s.K.P[j], qj = s.K.Q[j];
  if (pj.w < 0.0f) return;  // not contributing
  s.math_q(qj, ox - pj.x, oy - pj.y, oz - pj.z, pj.w);
}

// density record: P (xr,yr,zr,+-h: - when not contributing),
// Q (m, m/rho, m e/rho, phase)
__global__ void k_pack_dens(Dev A, Packed K, Work W, int pgc, const int* __restrict__ d_count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *d_count) return;
  const uint8_t ph = A.phase[j];
  const bool c = contr_dens(A.bc[j], pgc) && (ph == 1 || ph == 2);
  const float h = f32_rz(A.h[j]);
  const float m = f32_rz(A.mass[j]), mr = m / f32_rz(A.rho[j]);
  K.P[j] = make_float4(W.xr[j], W.yr[j], W.zr[j], c ? h : -h);
  K.Q[j] = make_float4(m, mr, mr * f32_rz(A.e[j]), (float)ph);
}

// ------------------------------------------------------------ velocity
template <typename T>
struct WVel {
  const Dev& A;
  const Packed& K;
  const Opt& o;
  T xs[3], hi, supp, ks, Lb, vi[3];
  __device__ __forceinline__ const T* xpos() const { return xs; }
  T ihi, r3;  // 1/h_i and (1/(sqrt(pi) h_i))^3 (mixed Gaussian)
  CAcc<T> dv[3], wnorm;
  __device__ __forceinline__ void flush() {
    dv[0].flush(); dv[1].flush(); dv[2].flush(); wnorm.flush();
  }
  static constexpr bool kListAhead = true;  // the list walk's entry look-ahead
  static constexpr bool kSkipDecode = true;  // the list walk keeps a repeated bucket's offsets
  __device__ WVel(const Dev& A_, const Packed& K_, const Opt& o_) : A(A_), K(K_), o(o_) {}
  double vi_d[3];
  __device__ __forceinline__ bool setup(int ii, const Geo& g, const Work& W, const double*, TimeState*,
                                        double* xi, int* bi, double& R) {
    xi[0] = A.x[ii]; xi[1] = A.y[ii]; xi[2] = A.z[ii];
    bucket_coords<3>(g, A.bkt[ii], bi);
    Pos<3, T>::load(A, W, ii, xs);
    const double hi_d = A.h[ii];
    hi = T(hi_d);
    supp = T(o.cutoff2) * hi;
    ks = T(o.ksupport * (1.0 + 1e-6)) * hi;
    Lb = T(o.list_factor * W.hlist[ii]);
    ihi = rcp<T>(hi);
    r3 = (T(T1_INV_SQRT_PI) * ihi) * (T(T1_INV_SQRT_PI) * ihi) * (T(T1_INV_SQRT_PI) * ihi);
    vi_d[0] = A.vx[ii]; vi_d[1] = A.vy[ii]; vi_d[2] = A.vz[ii];
    vi[0] = T(vi_d[0]); vi[1] = T(vi_d[1]); vi[2] = T(vi_d[2]);
    R = fmin(o.cutoff2, o.ksupport) * hi_d * (1.0 + 1e-10);
    return true;
  }
  template <bool WARP>
  __device__ __forceinline__ void finish(int ii, Work& W, TimeState* ts) {
    double d0 = (double)dv[0].get(), d1 = (double)dv[1].get(), d2 = (double)dv[2].get();
    double wn = (double)wnorm.get();
    if (WARP) {
      d0 = warp_sum(d0); d1 = warp_sum(d1); d2 = warp_sum(d2); wn = warp_sum(wn);
      if ((threadIdx.x & 31) != 0) return;
    }
    if (!(wn > 0)) {
      set_status(ts, 4);
      return;
    }
    if (W.wnv) W.wnv[ii] = wn;
    A.vsx[ii] = vi_d[0] + d0 / wn;
    A.vsy[ii] = vi_d[1] + d1 / wn;
    A.vsz[ii] = vi_d[2] + d2 / wn;
  }
  template <bool LISTED = false>
  __device__ __forceinline__ bool filter(uint32_t j, bool own, T ox, T oy, T oz, T* dx, T& flag) const {
    T xj[3];
    JPos<T>::get(A, K, j, xj, flag);
    if (sizeof(T) == 8) {
      if (!contr_vel_smooth(A.bc[j])) return false;
    } else if (flag < T(0)) {
      return false;
    }
    // listed: ox, oy, oz are i's position shifted into j's bucket
    dx[0] = (LISTED ? ox : xs[0] + ox) - xj[0];
    dx[1] = (LISTED ? oy : xs[1] + oy) - xj[1];
    dx[2] = (LISTED ? oz : xs[2] + oz) - xj[2];
    if (!LISTED) {
      if (!own && !in_box<3, T>(dx, Lb)) return false;
      if (!in_box<3, T>(dx, supp)) return false;
    }
    return in_box<3, T>(dx, ks);
  }
  // a listed candidate of the mixed Gaussian path: both records loaded
  // together; outside the support (|s_k| > 3) the weight is zero
  __device__ __forceinline__ void listed(uint32_t j, float ox, float oy, float oz) {
    const float4 pj = K.P[j], qj = K.Q[j];
    if (pj.w < 0.0f) return;  // not contributing
    const float s0 = (ox - pj.x) * ihi, s1 = (oy - pj.y) * ihi, s2 = (oz - pj.z) * ihi;
    const bool in = fabsf(s0) <= 3.0f && fabsf(s1) <= 3.0f && fabsf(s2) <= 3.0f;
    const float mvw = in ? r3 * __expf(-(s0 * s0 + s1 * s1 + s2 * s2)) * qj.x : 0.0f;
    dv[0].add(mvw * (qj.y - vi[0]));
    dv[1].add(mvw * (qj.z - vi[1]));
    dv[2].add(mvw * (qj.w - vi[2]));
    wnorm.add(mvw);
  }
  __device__ __forceinline__ void math(uint32_t j, const T* ds, T) {
    // FP64: the reference's fields; mixed: (m/rho, vx, vy, vz)
    T mj = 0, rhoj = 0, mvr = 0, vj[3];
    if constexpr (sizeof(T) == 8) {
      mj = A.mass[j]; rhoj = A.rho[j];
      vj[0] = A.vx[j]; vj[1] = A.vy[j]; vj[2] = A.vz[j];
    } else {
      const float4 q = K.Q[j];
      mvr = q.x; vj[0] = q.y; vj[1] = q.z; vj[2] = q.w;
    }
    T sv[3];
#pragma unroll
    for (int k = 0; k < 3; k++) sv[k] = (sizeof(T) == 8) ? ds[k] / hi : ds[k] * ihi;
    T wght;
    if (sizeof(T) == 4 && o.kernel != 1) {
      // Gaussian, mixed: the normalisation of h_i formed once per particle
      const T q = sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2];
      wght = (fabs(sv[0]) > T(3) || fabs(sv[1]) > T(3) || fabs(sv[2]) > T(3)) ? T(0) : r3 * __expf(-q);
    } else {
      wght = kw<3, T>(o.kernel, sv, hi);
    }
    const T mvw = (sizeof(T) == 8) ? wght * mj / rhoj : wght * mvr;
#pragma unroll
    for (int k = 0; k < 3; k++) dv[k].add(mvw * (vj[k] - vi[k]));
    wnorm.add(mvw);
  }
};

// velocity record: P (xr,yr,zr,+-1: - when not contributing),
// Q (m/rho, vx, vy, vz)
__global__ void k_pack_vel(Dev A, Packed K, Work W, const int* __restrict__ d_count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *d_count) return;
  K.P[j] = make_float4(W.xr[j], W.yr[j], W.zr[j], contr_vel_smooth(A.bc[j]) ? 1.f : -1.f);
  K.Q[j] = make_float4(f32_rz(A.mass[j]) / f32_rz(A.rho[j]), f32_rz(A.vx[j]), f32_rz(A.vy[j]), f32_rz(A.vz[j]));
}


// ------------------------------------------------------------ driver kernel
// WARP = true: one warp per particle with ballot compaction (wp_walk);
// WARP = false: one thread per particle walking its own rows.
template <typename T, template <typename> class SW, bool WARP, bool MULTI>
__global__ void __launch_bounds__(128) k_sweep3(Opt o, Geos<MULTI> geo, Dev A, Work W, Packed K,
                                                const uint32_t* __restrict__ cs_all,
                                                const double* __restrict__ hmax_all,
                                                const int* __restrict__ d_count, TimeState* ts_all) {
  const int n = *d_count;
  if (WARP) {
    __shared__ WBuf<T> bufs[WP_WARPS];
    WBuf<T>& B = bufs[threadIdx.x >> 5];
    const int nw = gridDim.x * WP_WARPS;
    for (int i = blockIdx.x * WP_WARPS + (threadIdx.x >> 5); i < n; i += nw) {
      if (!need_neigh(A.bc[i])) continue;
      const int m = geo.member(A, i);
      TimeState* ts = ts_all + m;
      if (!ts->active) continue;
      const Geo& g = geo.of(m);
      const uint32_t* cs = MULTI ? cs_all + g.cell_base : cs_all;
      const double* hmax = MULTI ? hmax_all + g.bucket_base : hmax_all;
      SW<T> s(A, K, o);
      double xi[3], R;
      int bi[3];
      if (!s.setup(i, g, W, hmax, ts, xi, bi, R)) continue;
      wp_walk<T>(g, cs, xi, bi, R, B, s);
      s.template finish<true>(i, W, ts);
    }
  } else {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !need_neigh(A.bc[i])) return;
    const int m = geo.member(A, i);
    TimeState* ts = ts_all + m;
    if (!ts->active) return;
    const Geo& g = geo.of(m);
    const uint32_t* cs = MULTI ? cs_all + g.cell_base : cs_all;
    const double* hmax = MULTI ? hmax_all + g.bucket_base : hmax_all;
    SW<T> s(A, K, o);
    double xi[3], R;
    int bi[3];
    if (!s.setup(i, g, W, hmax, ts, xi, bi, R)) return;
    for_segments<3, T>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
      for (uint32_t j = j0; j < j1; j++) {
        T dx[3], hj;
        if (s.filter(j, own, ox, oy, oz, dx, hj)) s.math(j, dx, hj);
      }
      if constexpr (sizeof(T) == 4) s.flush();
    });
    s.template finish<false>(i, W, ts);
  }
}


// ------------------------------------------------------------ neighbour lists
// Per-step masked neighbour lists.  One walk per step (after the adaptive
// smoothing length, when positions and h are final for the step) records,
// for every need_neigh particle, the windows of at most 32 consecutive
// candidates of one row segment that hold at least one pair of the union
// of the three sweeps' supports, as (window start | bucket-offset code << 26,
// 32-bit mask).  The momentum, density and velocity sweeps then visit the
// set bits in order (row, segment, index: the walk's order) and apply their
// own exact tests, so the sums are those of the walk; the divergent
// candidate filtering is paid once per step instead of once per sweep.
constexpr int LCAP = 160;                 // windows per particle
#ifndef PLUME_LIST_STREAM
#define PLUME_LIST_STREAM 0  // 1: list entries stored and loaded evict-first (measured slower)
#endif
__device__ __forceinline__ uint2 list_load(const uint2* p) {
#if PLUME_LIST_STREAM
  return __ldcs(p);
#else
  return *p;
#endif
}
__device__ __forceinline__ void list_store(uint2* p, uint2 v) {
#if PLUME_LIST_STREAM
  __stcs(p, v);
#else
  *p = v;
#endif
}
constexpr uint16_t NL_OVERFLOW = 0xFFFF;  // particle walks instead
constexpr uint32_t NL_JMASK = (1u << 26) - 1u;

struct NList {
  uint2* e;        // capacity * LCAP entries
  uint16_t* cnt;   // windows per particle, or NL_OVERFLOW
};

// like for_segments, with the bucket offset of the segment as a code of
// three 2-bit fields, (dbx+1) | (dby+1) << 2 | (dbz+1) << 4, db = segment
// bucket - own bucket (OWN_CODE: the own bucket)
template <typename T, class F>
__device__ __forceinline__ void for_segments_code(const Geo& g, const uint32_t* __restrict__ cs,
                                                  const float* xr, const int* bi, double R, F&& f) {
  int lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; a++) cell_range(g, a, bi[a], xr[a], R, lo[a], hi[a]);
  for (int cz = lo[2]; cz <= hi[2]; cz++) {
    const int bz = cz / g.s;
    for (int cy = lo[1]; cy <= hi[1]; cy++) {
      const int by = cy / g.s;
      const size_t rowbase = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      int cx = lo[0];
      while (cx <= hi[0]) {
        const int bx = cx / g.s;
        const int e = min(hi[0], bx * g.s + g.s - 1);
        const int code = (bx - bi[0] + 1) | (by - bi[1] + 1) << 2 | (bz - bi[2] + 1) << 4;
        f(cs[rowbase + cx], cs[rowbase + e + 1], code);
        cx = e + 1;
      }
    }
  }
}

// delT: the bucket edge in the sweep's type, formed once per particle (the
// FP64 pipe of sm_103a is narrow: no double arithmetic per window)
constexpr int OWN_CODE = 1 | 1 << 2 | 1 << 4;
template <typename T>
__device__ __forceinline__ void decode_offsets(T delT, int code, bool& own, T& ox, T& oy, T& oz) {
  own = (code == OWN_CODE);
  constexpr bool REL = sizeof(T) == 4;
  const int dbx = (code & 3) - 1, dby = ((code >> 2) & 3) - 1, dbz = (code >> 4) - 1;
  ox = REL ? T(-dbx) * delT : T(0);
  oy = REL ? T(-dby) * delT : T(0);
  oz = REL ? T(-dbz) * delT : T(0);
}

// FP32 list test of the nb <= 32 candidates from wb on (P records): bit q
// set when max_k |xsh_k - x_k| <= min(Ti, max(kB |h_j| + kA, kC)) -- one
// threshold per candidate, min(list and CUTOFF2 boxes, support box), the
// first exactly as the sweeps assume, the support term (which the sweeps
// test again) with a wider margin.  Branch-free, loads issued 4 at a time.
__device__ __forceinline__ uint32_t window_mask(const Packed& K, uint32_t wb, int nb, const float* xsh, float Ti,
                                                float kA, float kB, float kC) {
  uint32_t mask = 0;
  for (int q = 0; q < nb; q += 4) {
    float4 pr[4];
#pragma unroll
    for (int u = 0; u < 4; u++) pr[u] = (q + u < nb) ? K.P[wb + q + u] : make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f);
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const float dx0 = fabsf(xsh[0] - pr[u].x), dx1 = fabsf(xsh[1] - pr[u].y), dx2 = fabsf(xsh[2] - pr[u].z);
      const float m = fmaxf(dx0, fmaxf(dx1, dx2));
      const float thr = fminf(Ti, fmaxf(fmaf(kB, fabsf(pr[u].w), kA), kC));
      mask |= (uint32_t)(m <= thr) << (q + u);
    }
  }
  return mask & ((nb == 32) ? 0xffffffffu : ((1u << nb) - 1u));
}

// union filter of the momentum, density and velocity sweeps
template <typename T, bool MULTI>
// (over the compacted need_neigh particles of the stepping members: only
// their lists are read)
__global__ void __launch_bounds__(128) k_build_lists(Opt o, Geos<MULTI> geo, Dev A, Work W, Packed K,
                                                     const uint32_t* __restrict__ cs_all,
                                                     const double* __restrict__ hmax_all,
                                                     const int* __restrict__ d_real,
                                                     const uint32_t* __restrict__ real_idx,
                                                     const TimeState* __restrict__ ts_all, NList L) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *d_real) return;
  const int i = (int)real_idx[r];
  const int m = geo.member(A, i);
  const Geo& g = geo.of(m);
  const uint32_t* cs = MULTI ? cs_all + g.cell_base : cs_all;
  const double* hmax = MULTI ? hmax_all + g.bucket_base : hmax_all;
  const int b = A.bkt[i];
  int bi[3];
  bucket_coords<3>(g, b, bi);
  T xs[3];
  Pos<3, T>::load(A, W, i, xs);
  const double hi_d = A.h[i];
  const T hi = T(hi_d);
  const T supp = T(o.cutoff2) * hi;
  const T Lb = T(o.list_factor * W.hlist[i]);
  const T kmarg = T(o.ksupport * (1.0 + 1e-6));
  // support term of the mixed test: kmarg2 max(h_i/2 + |h_j|/2, h_i)
  const float kmarg2 = (float)(o.ksupport * (1.0 + 4e-6));
  const float kA = kmarg2 * 0.5f * (float)hi, kB = kmarg2 * 0.5f, kC = kmarg2 * (float)hi;
  const double R = fmin(o.cutoff2 * hi_d, o.ksupport * fmax(0.5 * (hi_d + hmax[b]), hi_d)) * (1.0 + 1e-10);
  uint2* out = L.e + (size_t)i * LCAP;
  const T delT = T(g.del);
  const float xrf[3] = {W.xr[i], W.yr[i], W.zr[i]};
  int cnt = 0;
  for_segments_code<T>(g, cs, xrf, bi, R, [&](uint32_t j0, uint32_t j1, int code) {
    bool own;
    T ox, oy, oz;
    decode_offsets<T>(delT, code, own, ox, oy, oz);
    const T xsh[3] = {xs[0] + ox, xs[1] + oy, xs[2] + oz};
    // mixed: one threshold per candidate, min(list and CUTOFF2 boxes,
    // support box) -- the first exactly as the sweeps assume, the support
    // term (which the sweeps test again) with a wider margin
    const float Ti = own ? (float)supp : fminf((float)Lb, (float)supp);
    for (uint32_t wb = j0; wb < j1; wb += 32) {
      const int nb = (int)min(32u, j1 - wb);
      uint32_t mask = 0;
      if constexpr (sizeof(T) == 4) {
        mask = window_mask(K, wb, nb, xsh, Ti, kA, kB, kC);
      } else {
        for (int q = 0; q < nb; q++) {
          T xj[3], hj;
          JPos<T>::get(A, K, wb + q, xj, hj);
          const T dx[3] = {xsh[0] - xj[0], xsh[1] - xj[1], xsh[2] - xj[2]};
          if (!own && !in_box<3, T>(dx, Lb)) continue;
          if (!in_box<3, T>(dx, supp)) continue;
          const T hs = fmax(T(0.5) * (hi + fabs(hj)), hi);
          if (in_box<3, T>(dx, kmarg * hs)) mask |= 1u << q;
        }
      }
      if (mask) {
        if (cnt < LCAP) list_store(out + cnt, make_uint2(wb | ((uint32_t)code << 26), mask));
        cnt++;
      }
    }
  });
  L.cnt[i] = (cnt > LCAP) ? NL_OVERFLOW : (uint16_t)cnt;
}

// the fused listed pair of each sweep (mixed Gaussian path)
__device__ __forceinline__ void listed_pair(WMom<float>& s, uint32_t j, float ox, float oy, float oz) {
  s.listed(j, ox, oy, oz);
}
__device__ __forceinline__ void listed_pair(WDens<float>& s, uint32_t j, float ox, float oy, float oz) {
  dens_listed(s, j, ox, oy, oz);
}
__device__ __forceinline__ void listed_pair(WVel<float>& s, uint32_t j, float ox, float oy, float oz) {
  s.listed(j, ox, oy, oz);
}

// The stored windows of particle i (c of them), their set bits in order:
// pair(j, own, ox, oy, oz) per candidate, o = i's position shifted into the
// window's bucket.  The bit loop is flattened: every iteration hands each
// thread one pair, so the threads of a warp stay converged while they have
// pairs left.
template <typename T, class S, class F>
__device__ __forceinline__ void walk_windows(S& s, int i, const Geo& g, int c, const NList& L, F&& pair) {
  const uint2* ent = L.e + (size_t)i * LCAP;
  const T delT = T(g.del);
  int q = 0;
  // the next window's entry is loaded one window ahead, so that its load
  // (mostly an L2 or DRAM access: the lists are read once per sweep) is
  // in flight while the current window's pairs are summed
  constexpr bool ahead = PLUME_LIST_AHEAD && S::kListAhead;
  uint2 en = list_load(ent);
  uint2 nx = ahead ? list_load(ent + (c > 1 ? 1 : 0)) : en;
  uint32_t mask = en.y;
  bool own;
  T ox, oy, oz;
  auto shift = [&](int code) {
    decode_offsets<T>(delT, code, own, ox, oy, oz);
    ox += s.xpos()[0]; oy += s.xpos()[1]; oz += s.xpos()[2];
  };
  int pcode = (int)(en.x >> 26);
  shift(pcode);
  while (true) {
    if (mask == 0) {  // stored windows are never empty: one step suffices
      if constexpr (sizeof(T) == 4) s.flush();  // one partial per window
      if (++q >= c) break;
      if (ahead) {
        en = nx;
        nx = list_load(ent + min(q + 1, c - 1));  // the last one again at the end
      } else {
        en = list_load(ent + q);
      }
      mask = en.y;
      const int code = (int)(en.x >> 26);
      if (!S::kSkipDecode || code != pcode) {  // windows of one bucket share their offsets
        shift(code);
        pcode = code;
      }
    }
    const uint32_t j = (en.x & NL_JMASK) + (uint32_t)(__ffs(mask) - 1);
    mask &= mask - 1;
    pair(j, own, ox, oy, oz);
  }
}

// Visits the candidates of particle i in the walk's order: the particle's
// stored windows (set bits, in order), or the cell rows when its windows
// overflowed.  The mixed Gaussian path takes each listed candidate in one
// branch-free piece (its records loaded together, zero outside the
// support), with the momentum sweep's LANS terms chosen once per particle,
// outside the loop; otherwise s.math(j, dx, hj) for every candidate
// s.filter passes.
template <typename T, class S>
__device__ __forceinline__ void list_walk(S& s, int i, const Geo& g, const uint32_t* __restrict__ cs,
                                          const double* xi, const int* bi, double R, const NList& L) {
  const uint16_t c = L.cnt[i];
  if (c == NL_OVERFLOW) {
    // (the FP32 momentum sweep walks with carried bucket indices: measured
    // 12.03 vs 12.41 ms per step on the 134^3 plume through the code of the
    // list loop; the other sweeps and the adaptive pass divide)
    constexpr bool carry = sizeof(T) == 4 && std::is_same<S, WMom<T>>::value;
    for_segments<3, T, carry>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
      for (uint32_t j = j0; j < j1; j++) {
        T dx[3], hj;
        if (s.filter(j, own, ox, oy, oz, dx, hj)) s.math(j, dx, hj);
      }
      if constexpr (sizeof(T) == 4) s.flush();  // one partial per row segment
    });
    return;
  }
  if (c == 0) return;
  if constexpr (sizeof(T) == 4) {
    if (s.o.kernel != 1) {
      if constexpr (std::is_same<S, WMom<float>>::value) {
        if (s.lans)
          walk_windows<T>(s, i, g, c, L, [&](uint32_t j, bool, float ox, float oy, float oz) {
            s.template listed_l<true>(j, ox, oy, oz);
          });
        else
          walk_windows<T>(s, i, g, c, L, [&](uint32_t j, bool, float ox, float oy, float oz) {
            s.template listed_l<false>(j, ox, oy, oz);
          });
      } else {
        walk_windows<T>(s, i, g, c, L,
                        [&](uint32_t j, bool, float ox, float oy, float oz) { listed_pair(s, j, ox, oy, oz); });
      }
      return;
    }
  }
  walk_windows<T>(s, i, g, c, L, [&](uint32_t j, bool own, T ox, T oy, T oz) {
    T dx[3], hj;
    if (s.template filter<true>(j, own, ox, oy, oz, dx, hj)) s.math(j, dx, hj);
  });
}

// minimum resident blocks per SM of each list sweep (caps its registers),
// measured on the 134^3 plume at h ~ 1.5 dx (default window, 4^3 cells, ms
// per step): momentum 7 blocks = 72 registers 9.64 (6 = 80 registers 10.07);
// density 12 blocks = 40 registers 6.04 (8 = 64: 6.83, 10 = 48: 6.15);
// LANS filter 10 blocks = 48 registers 6.02 (8 = 64: 6.46, 11 = 40: 6.36).
// The spills the lower caps bring cost less than the latency the extra
// warps hide.
#ifndef PLUME_MINB_MOM
#define PLUME_MINB_MOM 7
#endif
#ifndef PLUME_MINB_DENS
#define PLUME_MINB_DENS 12
#endif
#ifndef PLUME_MINB_VEL
#define PLUME_MINB_VEL 10
#endif
// (the FP64 sweeps keep 6, 8 and 8 blocks: 80 and 64 registers)
template <typename T, template <typename> class SW>
struct SweepMinBlocks { static constexpr int v = 1; };
template <typename T>
struct SweepMinBlocks<T, WMom> { static constexpr int v = sizeof(T) == 4 ? PLUME_MINB_MOM : 6; };
template <typename T>
struct SweepMinBlocks<T, WDens> { static constexpr int v = sizeof(T) == 4 ? PLUME_MINB_DENS : 8; };
template <typename T>
struct SweepMinBlocks<T, WVel> { static constexpr int v = sizeof(T) == 4 ? PLUME_MINB_VEL : 8; };

template <typename T, template <typename> class SW, bool MULTI>
__global__ void __launch_bounds__(128, SweepMinBlocks<T, SW>::v) k_sweep3_list(Opt o, Geos<MULTI> geo, Dev A, Work W, Packed K,
                                                     const uint32_t* __restrict__ cs_all,
                                                     const double* __restrict__ hmax_all,
                                                     const int* __restrict__ d_real,
                                                     const uint32_t* __restrict__ real_idx, TimeState* ts_all,
                                                     NList L) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *d_real) return;
  const int i = (int)real_idx[r];
  const int m = geo.member(A, i);  // real_idx holds particles of active members only
  TimeState* ts = ts_all + m;
  const Geo& g = geo.of(m);
  const uint32_t* cs = MULTI ? cs_all + g.cell_base : cs_all;
  const double* hmax = MULTI ? hmax_all + g.bucket_base : hmax_all;
  SW<T> s(A, K, o);
  double xi[3], R;
  int bi[3];
  if (!s.setup(i, g, W, hmax, ts, xi, bi, R)) return;
  list_walk<T>(s, i, g, cs, xi, bi, R, L);
  s.template finish<false>(i, W, ts);
}

// ------------------------------------------------------------ warp list sweeps
// Mixed-path list sweeps with one warp per particle.  The particle's
// windows are taken 32 at a time, one per lane; an inclusive warp scan of
// the windows' set-bit counts places every listed candidate in a per-warp
// shared-memory queue (j | bucket-offset code << 26), in the walk's order,
// and the lanes then take the queue 32 pairs at a time.  Every pair of a
// batch is a listed candidate (no idle lanes but in a particle's last
// batch), consecutive lanes hold consecutive candidates of the same rows,
// so a batch's record loads fall on a few cache lines, and the particle's
// own fields are loaded once per warp (broadcast).  Each lane keeps its own
// compensated sums; finish<true> adds the lanes' sums in FP64.  The 27
// positions of i shifted into the neighbouring buckets are formed once per
// particle in shared memory; a particle whose windows overflowed walks its
// rows with ballot compaction (wp_walk).
constexpr int WL_QUEUE = 32 * 32 + 32;  // one chunk of 32 windows + a batch's remainder

template <typename T>
struct WLShared {
  uint32_t q[WP_WARPS][WL_QUEUE];
  float4 sh[WP_WARPS][27];
  WBuf<T> wb[WP_WARPS];
};

template <template <typename> class SW>
struct SweepMinBlocksW { static constexpr int v = 1; };
#ifndef PLUME_MINB_WMOM
#define PLUME_MINB_WMOM 5
#endif
#ifndef PLUME_MINB_WDENS
#define PLUME_MINB_WDENS 7
#endif
#ifndef PLUME_MINB_WVEL
#define PLUME_MINB_WVEL 7
#endif
template <>
struct SweepMinBlocksW<WMom> { static constexpr int v = PLUME_MINB_WMOM; };
template <>
struct SweepMinBlocksW<WDens> { static constexpr int v = PLUME_MINB_WDENS; };
template <>
struct SweepMinBlocksW<WVel> { static constexpr int v = PLUME_MINB_WVEL; };

template <template <typename> class SW, bool MULTI>
__global__ void __launch_bounds__(128, SweepMinBlocksW<SW>::v)
    k_sweep3_wl(Opt o, Geos<MULTI> geo, Dev A, Work W, Packed K, const uint32_t* __restrict__ cs_all,
                const double* __restrict__ hmax_all, const int* __restrict__ d_real,
                const uint32_t* __restrict__ real_idx, TimeState* ts_all, NList L) {
  using T = float;
  __shared__ WLShared<T> S;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * WP_WARPS + wid;
  if (r >= *d_real) return;  // whole warps leave together
  const int i = (int)real_idx[r];
  const int m = geo.member(A, i);  // real_idx holds particles of active members only
  TimeState* ts = ts_all + m;
  const Geo& g = geo.of(m);
  const uint32_t* cs = MULTI ? cs_all + g.cell_base : cs_all;
  const double* hmax = MULTI ? hmax_all + g.bucket_base : hmax_all;
  SW<T> s(A, K, o);
  double xi[3], R;
  int bi[3];
  if (!s.setup(i, g, W, hmax, ts, xi, bi, R)) return;  // the same for every lane
  const uint16_t c = L.cnt[i];
  if (c == NL_OVERFLOW) {
    wp_walk<T>(g, cs, xi, bi, R, S.wb[wid], s);
  } else if (c > 0) {
    uint32_t* q = S.q[wid];
    float4* sh = S.sh[wid];
    if (lane < 27) {  // lane = 9 kz + 3 ky + kx, code kx | ky << 2 | kz << 4
      bool own;
      T ox, oy, oz;
      decode_offsets<T>(T(g.del), lane % 3 | (lane / 3 % 3) << 2 | (lane / 9) << 4, own, ox, oy, oz);
      sh[lane] = make_float4(s.xpos()[0] + ox, s.xpos()[1] + oy, s.xpos()[2] + oz, 0.f);
    }
    __syncwarp();
    auto pair = [&](uint32_t e) {
      const uint32_t j = e & NL_JMASK;
      const int code = (int)(e >> 26);
      const float4 p = sh[(code & 3) + 3 * ((code >> 2) & 3) + 9 * (code >> 4)];
      T dx[3], hj;
      if (s.template filter<true>(j, code == OWN_CODE, p.x, p.y, p.z, dx, hj)) s.math(j, dx, hj);
    };
    const uint2* ent = L.e + (size_t)i * LCAP;
    int cnt = 0;  // queued candidates (the same in every lane)
    for (int w0 = 0; w0 < (int)c; w0 += 32) {
      const uint2 en = (w0 + lane < (int)c) ? ent[w0 + lane] : make_uint2(0u, 0u);
      uint32_t mask = en.y;
      const int pc = __popc(mask);
      int off = pc;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(WFULL, off, d);
        if (lane >= d) off += v;
      }
      const int tot = __shfl_sync(WFULL, off, 31);
      int pos = cnt + off - pc;
      const uint32_t base = en.x & NL_JMASK, codeb = en.x & ~NL_JMASK;
      while (mask) {
        q[pos++] = (base + (uint32_t)(__ffs(mask) - 1)) | codeb;
        mask &= mask - 1;
      }
      cnt += tot;
      __syncwarp();
      int b = 0;
      for (; b + 32 <= cnt; b += 32) {
        pair(q[b + lane]);
        s.flush();
      }
      const int rest = cnt - b;  // < 32: moved to the queue's front
      const uint32_t keep = (lane < rest) ? q[b + lane] : 0u;
      __syncwarp();
      if (lane < rest) q[lane] = keep;
      cnt = rest;
      __syncwarp();
    }
    if (lane < cnt) pair(q[lane]);
  }
  s.template finish<true>(i, W, ts);
}

// compacted indices of the need_neigh particles of the stepping members
// (sorted order kept)
__global__ void k_real_flags(Dev A, const int* __restrict__ d_count, int n, const TimeState* __restrict__ ts_all,
                             unsigned int* __restrict__ flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag[i] = (i < *d_count && need_neigh(A.bc[i]) && ts_all[A.mem[i]].active) ? 1u : 0u;
}
__global__ void k_real_scatter(const unsigned int* __restrict__ flag, const unsigned long long* __restrict__ offs,
                               int n, uint32_t* __restrict__ real_idx, int* __restrict__ d_real,
                               const unsigned long long* __restrict__ total) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *d_real = (int)*total;
  if (i >= n) return;
  if (flag[i]) real_idx[offs[i]] = (uint32_t)i;
}

// Processing order of the list build and the list sweeps for single runs:
// tiles of TILE_X x TILE_Y x TILE_Z fine cells (x fastest), the
// need_neigh particles of a tile consecutive.  The per-particle work does
// not depend on the order; a block of threads then draws its particles
// from a compact 3D region instead of a line of cells, so the candidate
// records the block's warps load overlap more in L1.
constexpr int TILE_X = 4, TILE_Y = 4, TILE_Z = 2;
__device__ __forceinline__ void tile_rows(const Geo& g, int t, int ntx, int nty, int& cx0, int& cx1, int& cy0,
                                          int& cy1, int& cz0, int& cz1) {
  const int tx = t % ntx, ty = (t / ntx) % nty, tz = t / (ntx * nty);
  cx0 = tx * TILE_X; cx1 = min(cx0 + TILE_X, g.G[0]);
  cy0 = ty * TILE_Y; cy1 = min(cy0 + TILE_Y, g.G[1]);
  cz0 = tz * TILE_Z; cz1 = min(cz0 + TILE_Z, g.G[2]);
}
__global__ void k_tile_count(Geo g, Dev A, const uint32_t* __restrict__ cs, const int* __restrict__ d_count,
                             const TimeState* __restrict__ ts, int ntx, int nty, int ntiles,
                             unsigned int* __restrict__ tcount) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  unsigned int c = 0;
  if (ts[0].active) {
    const uint32_t n = (uint32_t)*d_count;
    int cx0, cx1, cy0, cy1, cz0, cz1;
    tile_rows(g, t, ntx, nty, cx0, cx1, cy0, cy1, cz0, cz1);
    for (int cz = cz0; cz < cz1; cz++)
      for (int cy = cy0; cy < cy1; cy++) {
        const size_t row = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
        const uint32_t j1 = min(cs[row + cx1], n);
        for (uint32_t j = cs[row + cx0]; j < j1; j++) c += need_neigh(A.bc[j]) ? 1u : 0u;
      }
  }
  tcount[t] = c;
}
__global__ void k_tile_fill(Geo g, Dev A, const uint32_t* __restrict__ cs, const int* __restrict__ d_count,
                            const TimeState* __restrict__ ts, int ntx, int nty, int ntiles,
                            const unsigned long long* __restrict__ toffs, const unsigned long long* __restrict__ total,
                            uint32_t* __restrict__ real_idx, int* __restrict__ d_real) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) *d_real = (int)*total;
  if (t >= ntiles || !ts[0].active) return;
  const uint32_t n = (uint32_t)*d_count;
  unsigned long long o = toffs[t];
  int cx0, cx1, cy0, cy1, cz0, cz1;
  tile_rows(g, t, ntx, nty, cx0, cx1, cy0, cy1, cz0, cz1);
  for (int cz = cz0; cz < cz1; cz++)
    for (int cy = cy0; cy < cy1; cy++) {
      const size_t row = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      const uint32_t j1 = min(cs[row + cx1], n);
      for (uint32_t j = cs[row + cx0]; j < j1; j++)
        if (need_neigh(A.bc[j])) real_idx[o++] = j;
    }
}

// ------------------------------------------------------------ adaptive h, mixed
// adaptive_sml (neighs.cc:479-693) on the mixed path: one thread per
// need_neigh particle of the stepping members, over the compacted (and, for
// single runs, tile-ordered) index list, candidates from packed FP32 records
// P = (xr, yr, zr, m or -1 when the particle does not contribute to the
// density); the kernel support test and the weight on one reciprocal of
// H* = c_smooth h.  The fixed-point iteration, its stopping rule and the
// h update are those of k_adaptive (FP64 per particle).
__global__ void k_pack_adapt(Dev A, Packed K, Work W, int pgc, const int* __restrict__ d_count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *d_count) return;
  K.P[j] = make_float4(W.xr[j], W.yr[j], W.zr[j], contr_dens(A.bc[j], pgc) ? (float)A.mass[j] : -1.0f);
}

template <bool MULTI>
__global__ void __launch_bounds__(128) k_adaptive_mixed(Opt o, Geos<MULTI> geo, Dev A, Work W, Packed K,
                                                        const uint32_t* __restrict__ cs_all,
                                                        const int* __restrict__ d_real,
                                                        const uint32_t* __restrict__ real_idx, TimeState* ts_all,
                                                        const int* __restrict__ hstep, int force) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *d_real) return;
  if (!force && (*hstep % o.interval) != 0) return;
  const int i = (int)real_idx[r];
  const int m = geo.member(A, i);  // real_idx holds particles of active members only
  TimeState* ts = ts_all + m;
  const Geo& g = geo.of(m);
  const uint32_t* cs = MULTI ? cs_all + g.cell_base : cs_all;
  const double xi[3] = {A.x[i], A.y[i], A.z[i]};
  int bi[3];
  bucket_coords<3>(g, A.bkt[i], bi);
  float xs[3];
  Pos<3, float>::load(A, W, i, xs);
  const float Lb = float(o.list_factor * W.hlist[i]);
  const double mi = A.mass[i];
  double hcur = A.h[i];
  for (int loop = 0; loop < o.num_loop; loop++) {
    const double H_old = hcur;
    const double H_star_d = H_old * o.c_smooth;
    const float H_star = float(H_star_d);
    const float supp = float(o.cutoff2) * H_star;
    const float inv = 1.0f / H_star;
    const float rn = float(T1_INV_SQRT_PI) * inv;
    const float r3 = rn * rn * rn;
    Acc<float> rho_star;
    const double R = fmin(o.cutoff2, o.ksupport) * H_star_d * (1.0 + 1e-10);
    auto visit = [&](uint32_t j0, uint32_t j1, bool own, float ox, float oy, float oz) {
      const float xsh[3] = {xs[0] + ox, xs[1] + oy, xs[2] + oz};
      for (uint32_t j = j0; j < j1; j++) {
        const float4 p = K.P[j];
        if (p.w < 0.0f) continue;
        const float dx[3] = {xsh[0] - p.x, xsh[1] - p.y, xsh[2] - p.z};
        if (!own && !in_box<3, float>(dx, Lb)) continue;
        if (!in_box<3, float>(dx, supp)) continue;
        const float si[3] = {dx[0] * inv, dx[1] * inv, dx[2] * inv};
        float w;
        if (o.kernel != 1)
          w = (fabsf(si[0]) > 3.0f || fabsf(si[1]) > 3.0f || fabsf(si[2]) > 3.0f)
                  ? 0.0f
                  : r3 * __expf(-(si[0] * si[0] + si[1] * si[1] + si[2] * si[2]));
        else
          w = kw<3, float>(o.kernel, si, H_star);
        rho_star.add(w * p.w);
      }
    };
    walk_list_region<float>(g, cs, xi, bi, fmin(R, o.list_factor * W.hlist[i] * (1.0 + 1e-6)), visit);
    const double rs = (double)rho_star.get();
    const double H_new = o.eta * cbrt(mi / rs);
    hcur = 1.0 * H_new;
    if (!(H_new > 0) || !isfinite(H_new)) {
      set_status(ts, 4);
      break;
    }
    if (fabs((H_new - H_old) / H_old) < o.thresh) break;
  }
  A.h[i] = hcur;
}

// position records for the list build: P (xr, yr, zr, h)
__global__ void k_pack_pos(Dev A, Packed K, Work W, const int* __restrict__ d_count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *d_count) return;
  K.P[j] = make_float4(W.xr[j], W.yr[j], W.zr[j], f32_rz(A.h[j]));
}

}  // namespace plume
