// Godunov SPH (USE_GSPH 1) on the device: the per-particle gradients of
// calc_gradients and the momentum/energy step of mom_engr_update
// (mom_engr_update.cc:441-1146) with a Roe or HLLC Riemann problem per pair.
//
// Both are thread-per-particle walks over the fine cells of the candidate
// box, with the neighbour-list rule of search_neighs_consth (own bucket, or
// inside the list_factor h box of the 26 neighbours).  The gradients are
// FP64 on both paths; the momentum kernel is templated on the pair
// arithmetic like k_momentum (T = float: bucket-relative FP32 positions,
// FP32 Riemann problems, compensated FP32 sums, FP64 update).
#pragma once

#include "../../include/plume_gpu.h"
#include "sph_kernels.cuh"

namespace plume {

constexpr double C_SHOCK = 3.0;  // C_SHOCK, constant.h:103

// ---------------------------------------------------------------- gradients
// calc_gradients (calculate_gradient.cc:22-208): for every particle with a
// neighbour list (1D: the need_neigh particles, whose list is every
// particle, add_air.cc:470-479; 3D: every particle, neighs.cc:76, 136 under
// USE_GSPH) the sums
//   A_ab  = -sum_j dx_a dW_b(dx/h_i, h_i) m_j/rho_j
//   F_a,q = -sum_j (f_q,i - f_q,j) dW_a m_j/rho_j,   f = (rho, v, p),
// over j != i inside the CUTOFF2 h_i box; with more than 20 such j the
// gradient is inv(A) F (linsolve, sph_lib.cc:161-182: the cofactor matrix
// over the determinant in 3D, -1/A in 1D), else zero.  grad holds
// (D+2)*D doubles per row: q-major, x_k fastest.  T = double: the
// reference's arithmetic; T = float (mixed path): FP32 pair terms on
// bucket-relative positions with compensated sums, the solve in FP64.
template <int D, typename T>
__global__ void k_gsph_grad(Opt o, const Geo* __restrict__ geo, Dev A, Work W, const uint32_t* __restrict__ cs_all,
                            const int* __restrict__ d_count, const TimeState* __restrict__ ts_all,
                            double* __restrict__ grad) {
  constexpr int NQ = D + 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  const uint8_t bci = A.bc[i];
  if (bci == BC_DEAD) return;
  const int m = A.mem[i];
  if (!ts_all[m].active) return;
  double* gi = grad + (size_t)i * (NQ * D);
#pragma unroll
  for (int q = 0; q < NQ * D; q++) gi[q] = 0.0;
  if (D == 1 && !need_neigh(bci)) return;
  const Geo g = geo[m];
  const uint32_t* cs = cs_all + g.cell_base;
  const double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  bucket_coords<D>(g, A.bkt[i], bi);
  T xs[3];
  Pos<D, T>::load(A, W, i, xs);
  const double hi_d = A.h[i];
  const T hi = T(hi_d);
  const T supp = T(o.cutoff2) * hi;
  const T Lb = T(o.list_factor * W.hlist[i]);
  const T rhoi = T(A.rho[i]), pi = T(A.p[i]);
  const T vi[3] = {T(A.vx[i]), D == 3 ? T(A.vy[i]) : T(0), D == 3 ? T(A.vz[i]) : T(0)};
  Acc<T> AA[D * D], FF[D][NQ];
  // The sums only gain from j with a non-zero dW (inside the kernel support
  // of h_i), so the walk covers that reach; its in-list count is a lower
  // bound of the reference's count over the CUTOFF2 h_i box.  Only when it
  // is <= 20 does a second, count-only walk over the full box decide.
  int nreal = 0;
  const double Rk = fmin(o.cutoff2 * hi_d, o.ksupport * hi_d) * (1.0 + 1e-10);
  for_segments<D, T>(g, cs, xi, bi, Rk, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
    const T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
    for (uint32_t j = j0; j < j1; j++) {
      if (j == (uint32_t)i) continue;
      T dx[3];
      pair_dx<D, T>(xsh, xi, A, W, j, dx);
      if (!own && !in_box<D, T>(dx, Lb)) continue;
      if (!in_box<D, T>(dx, supp)) continue;
      nreal++;
      T sv[3], dw[3], dwm[3];
#pragma unroll
      for (int k = 0; k < D; k++) sv[k] = dx[k] / hi;
      kdw<D, T>(o.kernel, sv, hi, dw);
      const T mj = T(A.mass[j]), rhoj = T(A.rho[j]);
#pragma unroll
      for (int k = 0; k < D; k++) dwm[k] = dw[k] * mj / rhoj;
#pragma unroll
      for (int a = 0; a < D; a++)
#pragma unroll
        for (int b = 0; b < D; b++) AA[a * D + b].sub(dx[a] * dwm[b]);
      const T vj[3] = {T(A.vx[j]), D == 3 ? T(A.vy[j]) : T(0), D == 3 ? T(A.vz[j]) : T(0)};
      const T dr = rhoi - rhoj, dp = pi - T(A.p[j]);
#pragma unroll
      for (int a = 0; a < D; a++) {
        FF[a][0].sub(dr * dwm[a]);
#pragma unroll
        for (int b = 0; b < D; b++) FF[a][b + 1].sub((vi[b] - vj[b]) * dwm[a]);
        FF[a][NQ - 1].sub(dp * dwm[a]);
      }
    }
  });
  if (nreal <= 20) {
    nreal = 0;
    for_segments<D, T>(g, cs, xi, bi, o.cutoff2 * hi_d * (1.0 + 1e-10),
                       [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
      const T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
      for (uint32_t j = j0; j < j1; j++) {
        if (j == (uint32_t)i) continue;
        T dx[3];
        pair_dx<D, T>(xsh, xi, A, W, j, dx);
        if ((own || in_box<D, T>(dx, Lb)) && in_box<D, T>(dx, supp)) nreal++;
      }
    });
    if (nreal <= 20) return;
  }
  double Ad[D * D], Ai[D * D];
#pragma unroll
  for (int q = 0; q < D * D; q++) Ad[q] = (double)AA[q].get();
  if constexpr (D == 1) {
    Ai[0] = -1 / Ad[0];
  } else {
    // entry (a,b) = cofactor C_ab over the determinant, as inv3 returns it;
    // A is symmetric, so this is its inverse
    double C[9];
    C[0] = Ad[4] * Ad[8] - Ad[5] * Ad[7];
    C[1] = -(Ad[3] * Ad[8] - Ad[5] * Ad[6]);
    C[2] = Ad[3] * Ad[7] - Ad[4] * Ad[6];
    C[3] = -(Ad[1] * Ad[8] - Ad[2] * Ad[7]);
    C[4] = Ad[0] * Ad[8] - Ad[2] * Ad[6];
    C[5] = -(Ad[0] * Ad[7] - Ad[1] * Ad[6]);
    C[6] = Ad[1] * Ad[5] - Ad[2] * Ad[4];
    C[7] = -(Ad[0] * Ad[5] - Ad[2] * Ad[3]);
    C[8] = Ad[0] * Ad[4] - Ad[1] * Ad[3];
    const double id = 1.0 / (Ad[0] * C[0] + Ad[1] * C[1] + Ad[2] * C[2]);
#pragma unroll
    for (int q = 0; q < 9; q++) Ai[q] = C[q] * id;
  }
#pragma unroll
  for (int a = 0; a < D; a++)
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < D; b++) acc += Ai[a * D + b] * (double)FF[b][q].get();
      gi[q * D + a] = acc;
    }
}

// ---------------------------------------------------------------- Riemann
// One side of a pair's Riemann problem
template <typename T>
struct GSide {
  T rho, p, c, gam, h;
  T v[3];          // velocity of the step (smoothed under LANS)
  const double* g; // gradients (rho, v, p) x D, or null
};

// Roe_RP_Solver (sph_lib.cc:1694-1750): Roe averages with the Lagrangian
// sound speed rho_lr c_lr
template <typename T>
__device__ __forceinline__ void rp_roe(T dl, T dr, T pl, T pr, T ul, T ur, T gl, T gr, T& p_star, T& u_star) {
  const T rdl = sqrt(dl), rdr = sqrt(dr);
  const T den = T(1) / (rdl + rdr);
  const T plr = (pl * rdl + pr * rdr) * den;
  const T glr = (gl * rdl + gr * rdr) * den;
  const T dlr = (dl * rdl + dr * rdr) * den;
  T clr = sqrt(glr * plr / dlr);
  clr = dlr * clr;
  const T ulr = (ul * rdl + ur * rdr) * den;
  p_star = plr - T(0.5) * clr * (ur - ul);
  u_star = ulr - T(0.5) * (pr - pl) / clr;
}

// HLLC_RP_Solver (sph_lib.cc:1753-1908, HLL_WAVE_SPEED_EVA 0, USE_GSPH 1):
// wave speeds relative to the Roe velocity, the state of the region that
// holds the interface
template <typename T>
__device__ __forceinline__ void rp_hllc(T dl, T dr, T pl, T pr, T ul, T ur, T gl, T gr, T& p_star, T& u_star) {
  const T rdl = sqrt(dl), rdr = sqrt(dr);
  const T den = T(1) / (rdl + rdr);
  const T ulr = (ul * rdl + ur * rdr) * den;
  const T plr = (pl * rdl + pr * rdr) * den;
  const T glr = (gl * rdl + gr * rdr) * den;
  const T dlr = (dl * rdl + dr * rdr) * den;
  const T clr = sqrt(glr * plr / dlr);
  const T vl = ul - ulr, vr = ur - ulr;
  const T cl = sqrt(gl * pl / dl), cr = sqrt(gr * pr / dr);
  const T Sl = fmin(vl - cl, -clr);
  const T Sr = fmax(vr + cr, clr);
  const T Sm = (dr * vr * (Sr - vr) - dl * vl * (Sl - vl) + pl - pr) / (dr * (Sr - vr) - dl * (Sl - vl));
  const T ph = dl * (vl - Sl) * (vl - Sm) + pl;
  const T Ml = dl * ul, Mr = dr * ur;
  const T El = dl * (pl / (dl * (gl - T(1))) + T(0.5) * ul * ul);
  const T Er = dr * (pr / (dr * (gr - T(1))) + T(0.5) * ur * ur);
  if (Sl > T(0)) {
    p_star = pl;
    u_star = ul;
  } else if (Sl <= T(0) && Sm > T(0)) {
    p_star = Sm / (Sl - Sm) * ((Sl - vl) * Ml + (ph - pl)) + ph;
    u_star = (Sm / (Sl - Sm) * ((Sl - vl) * El + ph * Sm - pl * vl) + (Sm + ulr) * ph) / p_star;
  } else if (Sm <= T(0) && Sr > T(0)) {
    p_star = Sm / (Sr - Sm) * ((Sr - vr) * Mr + (ph - pr)) + ph;
    u_star = (Sm / (Sr - Sm) * ((Sr - vr) * Er + ph * Sm - pr * vr) + (Sm + ulr) * ph) / p_star;
  } else if (Sr <= T(0)) {
    p_star = pr;
    u_star = ur;
  } else {  // NaN wave speeds: the NaN reaches the state and its check
    p_star = T(NAN);
    u_star = T(NAN);
  }
}

// Generate_VanderCorput (sph_lib.cc:2214-2245): n brought below 65,537 by
// steps of 65,536, then its bits 0..15 mirrored about the binary point
// (bit k weighs 2^-(k+1)); the sample point of the random choice method
__host__ __device__ inline double vdc16(unsigned n) {
  while (n > 65536u) n -= 65536u;
  double v = 0.0, w = 0.5;
  for (int k = 0; k < 16; k++) {
    if (n & (1u << k)) v += w;
    w *= 0.5;
  }
  return v;
}

// HLLC_RP_Solver under USE_GSPH 2 (sph_lib.cc:1753-1885): the waves of
// rp_hllc, the solution sampled at x = 0.6 (sp - 1/2) |x_i - x_j| against
// the waves' positions S dt
template <typename T>
__device__ __forceinline__ void rp_hllc_rcm(T dl, T dr, T pl, T pr, T ul, T ur, T gl, T gr, T sp, T dt, T dist,
                                            T& p_star, T& u_star) {
  const T rdl = sqrt(dl), rdr = sqrt(dr);
  const T den = T(1) / (rdl + rdr);
  const T ulr = (ul * rdl + ur * rdr) * den;
  const T plr = (pl * rdl + pr * rdr) * den;
  const T glr = (gl * rdl + gr * rdr) * den;
  const T dlr = (dl * rdl + dr * rdr) * den;
  const T clr = sqrt(glr * plr / dlr);
  const T vl = ul - ulr, vr = ur - ulr;
  const T cl = sqrt(gl * pl / dl), cr = sqrt(gr * pr / dr);
  const T Sl = fmin(vl - cl, -clr);
  const T Sr = fmax(vr + cr, clr);
  const T Sm = (dr * vr * (Sr - vr) - dl * vl * (Sl - vl) + pl - pr) / (dr * (Sr - vr) - dl * (Sl - vl));
  const T ph = dl * (vl - Sl) * (vl - Sm) + pl;
  const T Ml = dl * ul, Mr = dr * ur;
  const T El = dl * (pl / (dl * (gl - T(1))) + T(0.5) * ul * ul);
  const T Er = dr * (pr / (dr * (gr - T(1))) + T(0.5) * ur * ur);
  const T xSl = Sl * dt, xSm = Sm * dt, xSr = Sr * dt;
  const T x = (sp - T(0.5)) * dist * T(0.6);
  if (xSl > x) {
    p_star = pl;
    u_star = ul;
  } else if (xSl <= x && xSm > x) {
    p_star = Sm / (Sl - Sm) * ((Sl - vl) * Ml + (ph - pl)) + ph;
    u_star = (Sm / (Sl - Sm) * ((Sl - vl) * El + ph * Sm - pl * vl) + (Sm + ulr) * ph) / p_star;
  } else if (xSm <= x && xSr > x) {
    p_star = Sm / (Sr - Sm) * ((Sr - vr) * Mr + (ph - pr)) + ph;
    u_star = (Sm / (Sr - Sm) * ((Sr - vr) * Er + ph * Sm - pr * vr) + (Sm + ulr) * ph) / p_star;
  } else if (xSr <= x) {
    p_star = pr;
    u_star = ur;
  } else {  // NaN wave speeds: the NaN reaches the state and its check
    p_star = T(NAN);
    u_star = T(NAN);
  }
}

// HLLC_RP_Solver_my (sph_lib.cc:1912-2088): HLLC for strong shocks on
// velocities relative to the Roe velocity, with the wave-speed estimate of
// HLL_WAVE_SPEED_EVA (wave: 2 Davis, 3 Toro, the two the reference runs
// with); p* = p_HLLC and u* = sqrt(2 (E*_l - e*_l)) in the star region, the
// side's own state outside it.
template <typename T>
__device__ __forceinline__ void rp_hllc_my(int wave, T dl, T dr, T pl, T pr, T ul, T ur, T gl, T gr, T& p_star,
                                           T& u_star) {
  const T rdl = sqrt(dl), rdr = sqrt(dr);
  const T den = T(1) / (rdl + rdr);
  const T cl = sqrt(gl * pl / dl), cr = sqrt(gr * pr / dr);
  const T ulr = (ul * rdl + ur * rdr) * den;
  ul = ul - ulr;
  ur = ur - ulr;
  T Sl, Sr;
  if (wave == 2) {
    Sl = fmin(ul - cl, ur - cr);
    Sr = fmax(ul + cl, ur + cr);
  } else {
    const T plr = (pl * rdl + pr * rdr) * den;
    const T glr = (gl * rdl + gr * rdr) * den;
    const T dlr = (dl * rdl + dr * rdr) * den;
    const T clr = sqrt(glr * plr / dlr);
    const T p_refs = fmax(T(0), T(0.5) * (pl + pr) + T(0.25) * (ul - ur) * (dr + dl) * clr);
    const T ql = p_refs < pl ? T(1) : sqrt(T(1) + T(0.5) * (gl + T(1)) / gl * (p_refs / pl - T(1)));
    const T qr = p_refs < pr ? T(1) : sqrt(T(1) + T(0.5) * (gr + T(1)) / gr * (p_refs / pr - T(1)));
    Sl = ul - cl * ql;
    Sr = ur + cr * qr;
  }
  const T alf_l = dl * (Sl - ul), alf_r = dr * (Sr - ur);
  const T Sm = (ur * alf_r - ul * alf_l + pl - pr) / (alf_r - alf_l);
  const T p_hllc = (pr * alf_r - pl * alf_l - alf_r * alf_l * (ul - ur)) / (alf_r - alf_l);
  const T dl_star = alf_l / (Sl - Sm);
  const T el_star = p_hllc / (dl_star * (gl - T(1)));
  const T el = pl / (dl * (gl - T(1)));
  const T El_star = el + (Sm - ul) * (Sm + pl / alf_l);
  const T u_hllc = sqrt(T(2) * (El_star - el_star));
  if (Sl > T(0)) {
    p_star = pl;
    u_star = ul;
  } else if (Sl <= T(0) && Sr > T(0)) {
    p_star = p_hllc;
    u_star = u_hllc;
  } else if (Sr <= T(0)) {
    p_star = pr;
    u_star = ur;
  } else {  // NaN wave speeds: the NaN reaches the state and its check
    p_star = T(NAN);
    u_star = T(NAN);
  }
}

// VanLeer_RP_Solver (sph_lib.cc:2094-2210): Van Leer's iterative solver on
// the Lagrangian sound speeds C = rho c (c the particles' own sound speeds):
// the acoustic estimate of p*, accepted when within 1 % of both pressures,
// else secant-like updates with the shock / rarefaction impedances W and
// slopes Z until p* moves by less than 1 %.  The reference iterates without
// a limit; here a problem that has not converged after
// PLUME_VANLEER_MAX_ITER iterations gives NaN, which the step reports.
template <typename T>
__device__ __forceinline__ void rp_vanleer(T dl, T dr, T pl, T pr, T ul, T ur, T gl, T gr, T csl, T csr,
                                           T& p_star, T& u_star) {
  const T Cl = csl * dl, Cr = csr * dr;
  T p = (Cl * pr + Cr * pl - Cr * Cl * (ul - ur)) / (Cl + Cr);
  T md = fabs(p - pl) / pl;
  const T md2 = fabs(p - pr) / pr;
  if (md2 > md) md = md2;
  if (md < T(0.01)) {
    u_star = T(0.5) * (ul + ur);
    p_star = p;
    return;
  }
  const T G1l = T(0.5) * (gl + T(1)) / gl, G2l = T(0.5) * (gl - T(1)) / gl, G3l = T(1) - G2l;
  const T G1r = T(0.5) * (gr + T(1)) / gr, G2r = T(0.5) * (gr - T(1)) / gr, G3r = T(1) - G2r;
  const T Cl2 = Cl * Cl, Cr2 = Cr * Cr;
  T Zl = 0, Zr = 0, vl = 0, vr = 0, err = T(1);
  int it = 0;
  while (err > T(0.01)) {
    if (++it > PLUME_VANLEER_MAX_ITER) {
      p_star = T(NAN);
      u_star = T(NAN);
      return;
    }
    const T Rl = p / pl, Rr = p / pr;
    const T Wl = (p >= pl) ? Cl * pow(T(1) + G1l * (p - pl) / pl, T(0.5))
                           : G2l * (T(1) - Rl) / (T(1) - pow(Rl, G2l)) * Cl;
    const T Wr = (p >= pr) ? Cr * pow(T(1) + G1r * (p - pr) / pr, T(0.5))
                           : G2r * (T(1) - Rr) / (T(1) - pow(Rr, G2r)) * Cr;
    const T Wl2 = Wl * Wl, Wr2 = Wr * Wr;
    Zl = (p >= pl) ? T(2) * Wl2 / (Wl2 + Cl2) * Wl : Cl * pow(Rl, G3l);
    Zr = (p >= pr) ? T(2) * Wr2 / (Wr2 + Cr2) * Wr : Cr * pow(Rr, G3r);
    vl = ul + (p - pl) / Wl;
    vr = ur - (p - pr) / Wr;
    const T pn = p - (Zl * Zr * (vl - vr)) / (Zl + Zr);
    err = fabs(pn - p) / p;
    p = pn;
  }
  u_star = (Zl * vl + Zr * vr) / (Zl + Zr);
  p_star = p;
}

// Riemann_Solver (sph_lib.cc:2247-2598, USE_GSPH 1, RP_MASS_WEIGHTED 0,
// SWITCH_OFF_AV_FOR_EXPAN 0, SHEAR_VEL_APP 2) for the pair (i = right side,
// j = left side) at distance vector dx = x_i - x_j: states projected on
// e = dx/|dx|; unless the states are zeroth order, the gradients projected
// on e and limited (opposite velocity slopes; C_SHOCK (u_j - u_i), or its
// absolute value, above the smaller sound speed), the interface put at s*
// (GSPH_SPECIFIC_VOL_APP 0 / 1 / 3, Compute_sij_star sph_lib.cc:1655-1692)
// and the states moved to it over c dt/2, with the MINI_DERIVATIVE_COND
// fallback; the solver's u* put back along e with the Roe-averaged
// transverse velocity.
template <int D, typename T>
__device__ __forceinline__ void gsph_riemann(const Opt& o, const T* dx, const GSide<T>& I, const GSide<T>& J,
                                             T dt_half, T& p_star, T* v_star, T sp = T(0.5)) {
  const bool rcm = o.method == 2;  // USE_GSPH 2: interface and sampling at sp
  constexpr int NQ = D + 2;
  T dist = 0;
#pragma unroll
  for (int k = 0; k < D; k++) dist += dx[k] * dx[k];
  dist = sqrt(dist);
  T e[3];
#pragma unroll
  for (int k = 0; k < D; k++) e[k] = dx[k] / dist;
  T ui = 0, uj = 0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    ui += I.v[k] * e[k];
    uj += J.v[k] * e[k];
  }
  T dr = I.rho, ur = ui, pr = I.p, dl = J.rho, ul = uj, pl = J.p;
  const int recon = o.gsph_recon;
  if (recon != 4) {
    T drhoi = 0, dpi = 0, drhoj = 0, dpj = 0, dvi[3] = {0, 0, 0}, dvj[3] = {0, 0, 0};
    if (I.g && J.g) {
#pragma unroll
      for (int k = 0; k < D; k++) {
        drhoi += T(I.g[k]) * e[k];
        drhoj += T(J.g[k]) * e[k];
        dpi += T(I.g[(NQ - 1) * D + k]) * e[k];
        dpj += T(J.g[(NQ - 1) * D + k]) * e[k];
#pragma unroll
        for (int c = 0; c < D; c++) {
          dvi[c] += T(I.g[(1 + c) * D + k]) * e[k];
          dvj[c] += T(J.g[(1 + c) * D + k]) * e[k];
        }
      }
    }
    T ddui = 0, dduj = 0;
#pragma unroll
    for (int c = 0; c < D; c++) {
      ddui += dvi[c] * e[c];
      dduj += dvj[c] * e[c];
    }
    if (ddui * dduj < T(0)) ddui = dduj = T(0);
    T du = uj - ui;
    if (o.gsph_mono) du = fabs(du);
    if (T(C_SHOCK) * du > fmin(I.c, J.c)) drhoi = dpi = ddui = drhoj = dpj = dduj = T(0);
    const T Si = T(0.5) * dist, Sj = -Si;
    T sij = 0;
    const T hij = T(0.5) * (I.h + J.h), Vi = T(1) / I.rho, Vj = T(1) / J.rho;
    if (o.gsph_vol == 1) {
      const T Cc = (Vi - Vj) / dist, Dd = (Vi + Vj) * T(0.5), hsq = hij * hij;
      const T Vsq = T(0.25) * hsq * Cc * Cc + Dd * Dd;
      sij = T(0.5) * (hsq * Cc * Dd) / Vsq;
    } else if (o.gsph_vol == 3) {
      const T DVi = -Vi * Vi * drhoi, DVj = -Vj * Vj * drhoj;
      const T d2 = dist * dist, d3 = d2 * dist;
      const T Aa = T(-2.0) * (Vi - Vj) / d3 + (DVi + DVj) / d2;
      const T Bb = T(0.5) * (DVi - DVj) / dist;
      const T Cc = T(1.5) * (Vi - Vj) / dist - T(0.25) * (DVi + DVj);
      const T Dd = T(0.5) * (Vi + Vj) - T(0.125) * (DVi - DVj) * dist;
      const T hsq = hij * hij, h4 = hsq * hsq, h6 = h4 * hsq;
      const T Vsq = T(0.234375) * h6 * Aa * Aa + T(0.1875) * h4 * (T(2.0) * Aa * Cc + Bb * Bb) +
                    T(0.25) * hsq * (T(2.0) * Bb * Dd + Cc * Cc) + Dd * Dd;
      sij = (T(0.46875) * h6 * Aa * Bb + T(0.375) * h4 * (Aa * Dd + Bb * Cc) + T(0.5) * hsq * Cc * Dd) / Vsq;
    }
    if (rcm) sij = (sp - T(0.5)) * dist;
    const T delta_i = sij + I.c * dt_half - Si;
    const T delta_j = sij - J.c * dt_half - Sj;
    dr = I.rho + drhoi * delta_i;
    ur = ui + ddui * delta_i;
    pr = I.p + dpi * delta_i;
    dl = J.rho + drhoj * delta_j;
    ul = uj + dduj * delta_j;
    pl = J.p + dpj * delta_j;
    if (recon == 3) {
      if (dr < T(0) || dl < T(0) || pr < T(0) || pl < T(0)) {
        dr = I.rho; ur = ui; pr = I.p; dl = J.rho; ul = uj; pl = J.p;
      }
    } else if (recon == 2) {
      if (dr < T(0) || dl < T(0)) { dr = I.rho; dl = J.rho; }
      if (pr < T(0) || pl < T(0)) { pr = I.p; pl = J.p; }
    } else if (recon == 1 || recon == 10) {
      if (dr < T(0)) dr = I.rho;
      if (dl < T(0)) dl = J.rho;
      if (pr < T(0)) pr = I.p;
      if (pl < T(0)) pl = J.p;
      if (recon == 10 && T(3.0) * fabs(ul - ur) > fmin(I.c, J.c)) {
        ul = uj;
        ur = ui;
      }
    }
  }
  T u_star;
  if (rcm)
    rp_hllc_rcm<T>(dl, dr, pl, pr, ul, ur, J.gam, I.gam, sp, T(2) * dt_half, dist, p_star, u_star);
  else if (o.gsph_solver == 1)
    rp_hllc<T>(dl, dr, pl, pr, ul, ur, J.gam, I.gam, p_star, u_star);
  else if (o.gsph_solver == 2)
    rp_hllc_my<T>(o.gsph_wave, dl, dr, pl, pr, ul, ur, J.gam, I.gam, p_star, u_star);
  else if (o.gsph_solver == 3)
    rp_vanleer<T>(dl, dr, pl, pr, ul, ur, J.gam, I.gam, J.c, I.c, p_star, u_star);
  else
    rp_roe<T>(dl, dr, pl, pr, ul, ur, J.gam, I.gam, p_star, u_star);
  const T rdl = sqrt(dl), rdr = sqrt(dr);
  const T den = T(1) / (rdl + rdr);
  const T ulr = (ul * rdl + ur * rdr) * den;
#pragma unroll
  for (int k = 0; k < D; k++) {
    const T vlr = (J.v[k] * rdl + I.v[k] * rdr) * den;
    v_star[k] = e[k] * u_star + vlr - ulr * e[k];
  }
}

// ---------------------------------------------------------------- momentum
// GSPH momentum and energy (mom_engr_update.cc:441-1146, ME_UPDATE_SML 2,
// ADAPTIVE_SML 1, HAVE_ENERGY_CUT 0).  Over particle i's list entries
// j != i inside the CUTOFF2 h_i box whose V_i^2 dW(dx/h_ij, h_ij) is
// non-zero (h_ij = (h_i + h_j)/2), with F_j = p* (V_i^2 + V_j^2) dW - tau dW
// (tau the LANS stress SPH_epsilon_mom(v_i - v_j, V_j), zero without LANS):
//   rhs_v = -sum_j m_j F_j
//   rhs_e = -sum_j m_j (v*_j - xdot*) . F_j + LANS heat flux,
//           xdot* = v_i + dt/2 (rhs_v + g).
// The reference walks the list twice, solving each Riemann problem again
// once rhs_v is known; here one walk accumulates sum m_j v*_j . F_j and
// rhs_v, and rhs_e = -sum m_j v*_j . F_j - xdot* . rhs_v + heat follows
// (the same sum, regrouped).  Then v_new = v + dt (rhs_v + g e_D),
// e_new = e + dt (rhs_e + v_i,D g) into W.nv*, W.ne for k_commit_mom.
// grad: the step's gradients, or null for zeroth-order states.
template <int D, typename T>
__global__ void k_gsph_mom(Opt o, const Geo* __restrict__ geo, Dev A, Work W, const uint32_t* __restrict__ cs_all,
                           const double* __restrict__ hmax_all, const int* __restrict__ d_count,
                           TimeState* ts_all, const double* __restrict__ grad) {
  constexpr int NQ = D + 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Geo g = geo[m];
  const uint32_t* cs = cs_all + g.cell_base;
  const double* hmax = hmax_all + g.bucket_base;
  const double dt = ts->dtime;
  const double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  const int b = A.bkt[i];
  bucket_coords<D>(g, b, bi);
  T xs[3];
  Pos<D, T>::load(A, W, i, xs);
  const double hi_d = A.h[i];
  const double rho_i_d = A.rho[i];
  if (!(rho_i_d > 0)) {
    set_status(ts, 4);
    return;
  }
  const T hi = T(hi_d);
  const T supp = T(o.cutoff2) * hi;
  const T Lb = T(o.list_factor * W.hlist[i]);
  const T Vi = T(1.0) / T(rho_i_d);
  const bool lans = o.lans != 0;
  GSide<T> I;
  I.rho = T(rho_i_d); I.p = T(A.p[i]); I.c = T(A.c[i]); I.gam = T(A.gam[i]); I.h = hi;
  I.v[0] = T(lans ? A.vsx[i] : A.vx[i]);
  if (D == 3) {
    I.v[1] = T(lans ? A.vsy[i] : A.vy[i]);
    I.v[2] = T(lans ? A.vsz[i] : A.vz[i]);
  }
  I.g = grad ? grad + (size_t)i * (NQ * D) : nullptr;
  const T tempi = T(A.T[i]), cpi = T(A.cp[i]);
  const T dt_half = T(0.5 * dt);
  // random choice method: the step's sample point (mom_engr_update.cc:513-516)
  const T sp = T(o.method == 2 ? vdc16((unsigned)ts->step) : 0.5);
  const double hm = hmax[D == 3 ? b : 0];
  const double R = fmin(o.cutoff2 * hi_d, o.ksupport * 0.5 * (hi_d + hm)) * (1.0 + 1e-10);
  const double grav = -o.g;
  Acc<T> rhs_v[3], vF, heat_sum;
  for_segments<D, T>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
    const T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
    for (uint32_t j = j0; j < j1; j++) {
      if (j == (uint32_t)i) continue;
      T dx[3];
      pair_dx<D, T>(xsh, xi, A, W, j, dx);
      if (!own && !in_box<D, T>(dx, Lb)) continue;
      if (!in_box<D, T>(dx, supp)) continue;
      const T hj = T(A.h[j]);
      const T hij = T(0.5) * (hi + hj);
      const T Vj = T(1.0) / T(A.rho[j]);
      T si[3], dw[3], vsqi[3], vsqj[3];
#pragma unroll
      for (int k = 0; k < D; k++) si[k] = dx[k] / hij;
      kdw<D, T>(o.kernel, si, hij, dw);
      T max_dw = 0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        vsqi[k] = Vi * Vi * dw[k];
        vsqj[k] = Vj * Vj * dw[k];
        max_dw = fmax(max_dw, fabs(vsqi[k]));
      }
      if (!(max_dw > T(0))) continue;
      GSide<T> J;
      J.rho = T(A.rho[j]); J.p = T(A.p[j]); J.c = T(A.c[j]); J.gam = T(A.gam[j]); J.h = hj;
      J.v[0] = T(lans ? A.vsx[j] : A.vx[j]);
      if (D == 3) {
        J.v[1] = T(lans ? A.vsy[j] : A.vy[j]);
        J.v[2] = T(lans ? A.vsz[j] : A.vz[j]);
      }
      J.g = grad ? grad + (size_t)j * (NQ * D) : nullptr;
      T p_star, v_star[3];
      gsph_riemann<D, T>(o, dx, I, J, dt_half, p_star, v_star, sp);
      T velij[3], tau = 0;
#pragma unroll
      for (int k = 0; k < D; k++) velij[k] = I.v[k] - J.v[k];
      if (lans) {
        T dotv = 0;
#pragma unroll
        for (int k = 0; k < D; k++) dotv += velij[k] * velij[k];
        tau = T(EPS_HALF) * dotv * Vj;
      }
      const T mj = T(A.mass[j]);
      T vf = 0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        const T F = mj * (p_star * (vsqi[k] + vsqj[k]) - tau * dw[k]);
        rhs_v[k].sub(F);
        vf += v_star[k] * F;
      }
      vF.add(vf);
      if (lans) {
        // SPH_epsilon_heat_conductivity (sph_lib.cc:1399-1440) with h_ab,
        // c_ab; compute_F (sph_lib.cc:257-281) of the same dW
        const T cab = T(0.5) * (I.c + J.c);
        const T Cp_ij = T(0.5) * (T(A.cp[j]) + cpi);
        T dotvr = 0, dotrr = 0, dotvv = 0, kij = 0;
#pragma unroll
        for (int k = 0; k < D; k++) dotvr += fabs(velij[k] * dx[k]);
        if (dotvr != T(0)) {
#pragma unroll
          for (int k = 0; k < D; k++) dotrr += dx[k] * dx[k];
#pragma unroll
          for (int k = 0; k < D; k++) dotvv += velij[k] * velij[k];
          const T kab = (D == 3) ? T(10.0) * T(EPS_HALF) * Cp_ij * dotrr * dotvv / (T(PRANDTL) * dotvr) : T(0);
          kij = kab / (hij * cab);
        }
        T W_r = 0, r_sq = 0, Fij = 0;
#pragma unroll
        for (int k = 0; k < D; k++) W_r += dw[k] * dx[k];
        if (W_r != T(0)) {
#pragma unroll
          for (int k = 0; k < D; k++) r_sq += dx[k] * dx[k];
          Fij = W_r / r_sq;
        }
        heat_sum.add(mj * Vj * Vi * kij * (tempi - T(A.T[j])) * Fij);
      }
    }
  });
  double rv[3], xdot_rv = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    rv[k] = (double)rhs_v[k].get();
    const double xdot = (double)I.v[k] + 0.5 * dt * (rv[k] + (k == D - 1 ? grav : 0.0));
    xdot_rv += xdot * rv[k];
  }
  const double rhs_e = -(double)vF.get() - xdot_rv + (double)heat_sum.get();
  const double vi[3] = {A.vx[i], D == 3 ? A.vy[i] : 0.0, D == 3 ? A.vz[i] : 0.0};
  double unew[3];
#pragma unroll
  for (int k = 0; k < D; k++) unew[k] = vi[k] + dt * rv[k];
  unew[D - 1] += dt * grav;
  W.nv0[i] = unew[0];
  if (D == 3) { W.nv1[i] = unew[1]; W.nv2[i] = unew[2]; }
  W.ne[i] = A.e[i] + dt * (rhs_e + (double)I.v[D - 1] * grav);
}

}  // namespace plume
