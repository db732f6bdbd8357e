// sph_adjoint.cuh -- hand-written reverse-mode (adjoint) kernels of the 3D
// FP64 particle step.
//
// The differentiated map is one step with its discrete decisions frozen: the
// neighbour lists, the particle that sets dt, the erupt-to-real conversions
// (h <- sml2) and the deletions of the recorded forward run.  Inside that
// map every formula of the forward kernels is differentiated exactly (the
// Gaussian's box cut-off and the branch tests are constant almost
// everywhere).  Stages of a step and what they overwrite (need_neigh
// particles only):
//   A adaptive h           h                       (every sml_interval steps)
//   M momentum/energy      v, e (+ EOS outputs, which D overwrites unused)
//   D density / Y / e      rho, Y, e, p, c, T, cp
//   V LANS filter          vs
//   P position             x (+ h of converted erupt particles)
// The backward of a stage reads the adjoint of its outputs, zeroes the
// adjoint of what it overwrote (a pointwise kernel), then adds the adjoint
// of every input (a pair kernel over the same neighbour windows as the
// forward, j-side terms scattered with FP64 atomics).  Formulas follow the
// forward kernels (sph_warp.cuh), which restate the reference:
// mom_engr_update.cc:96-354, density_massfrac.cc:64-352,
// smooth_velocity.cc:25-165, update_pos.cc:34-168, neighs.cc:479-693,
// particle.cc:528-604, timestep.cc:94-183.
#pragma once
#include "sph_warp.cuh"

namespace plume {

// adjoint of the per-particle fields (sorted order of a step)
struct Adj {
  double *x, *y, *z, *vx, *vy, *vz, *vsx, *vsy, *vsz, *m, *h, *rho, *e, *p, *Y, *c, *T, *cp;
};

// Gaussian W(dx, h) = (T1 / h)^3 exp(-|dx|^2 / h^2), zero when any
// |dx_k| / h > 3 (sph_lib.cc:210-230); returns W, its gradient in dx and
// its derivative in h at fixed dx
__device__ __forceinline__ double gw3(const double* dx, double h, double* dW, double& dWdh) {
  double s[3], q = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s[k] = dx[k] / h;
    q += s[k] * s[k];
  }
  if (fabs(s[0]) > KCUTOFF || fabs(s[1]) > KCUTOFF || fabs(s[2]) > KCUTOFF) {
    dW[0] = dW[1] = dW[2] = 0;
    dWdh = 0;
    return 0;
  }
  const double r = T1_INV_SQRT_PI / h;
  const double W = r * r * r * exp(-q);
#pragma unroll
  for (int k = 0; k < 3; k++) dW[k] = -2.0 * s[k] / h * W;
  dWdh = W * (-3.0 + 2.0 * q) / h;
  return W;
}

// Adjoint of the EOS (particle.cc:528-604 as eos() in sph_device.cuh) at
// (rho, Y, e): adds to rhob, Yb, eb and ng0b the pull-back of the adjoints
// of p, c, T and (LANS) cp.
__device__ __forceinline__ void eos_vjp(const Opt& o, double rho, double Y, double e, double pb, double cb,
                                        double Tb, double cpb, bool lans, double& rhob, double& Yb,
                                        double& eb, double& ng0b) {
  const double ng0 = o.ng0;
  const double na = 1 - Y;
  const double ng = ng0 * Y;
  const double ns = Y - ng;
  const double Cvm = ns * o.cvs + ng * o.cvg + na * o.cva;
  const double Rm = ng * o.rg + na * o.ra;
  const double den = ng + na;
  const double gam = 1 + Rm / Cvm;
  const double desmg = rho * den;
  const double p = Rm / den * desmg * e / Cvm;
  const double c = sqrt(gam * p / desmg);
  const double T = e / Cvm;
  double gamb = 0, desmgb = 0, Rmb = 0, Cvmb = lans ? cpb : 0.0, denb = 0;
  if (cb != 0 && c > 0) {
    const double k = cb / (2.0 * c * desmg);
    gamb += k * p;
    pb += k * gam;
    desmgb -= k * gam * p / desmg;
  }
  Rmb += pb * rho * e / Cvm;
  rhob += pb * Rm * e / Cvm;
  eb += pb * Rm * rho / Cvm;
  Cvmb -= pb * p / Cvm;
  rhob += desmgb * den;
  denb += desmgb * rho;
  Rmb += gamb / Cvm;
  Cvmb -= gamb * Rm / (Cvm * Cvm);
  eb += Tb / Cvm;
  Cvmb -= Tb * T / Cvm;
  Yb += Cvmb * ((1 - ng0) * o.cvs + ng0 * o.cvg - o.cva) + Rmb * (ng0 * o.rg - o.ra) + denb * (ng0 - 1);
  ng0b += Cvmb * Y * (o.cvg - o.cvs) + Rmb * Y * o.rg + denb * Y;
}

// block-wide sum into one FP64 atomic (blockDim.x == 128)
__device__ __forceinline__ void block_add(double v, double* out) {
  __shared__ double red[4];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    const double s = red[0] + red[1] + red[2] + red[3];
    if (s != 0) atomicAdd(out, s);
  }
}

// adjoint inputs shared by the pair kernels of one stage
struct AdjIn {
  const double *vx, *vy, *vz, *e;   // momentum: adjoints of the new v and e
  const double *rho, *Y, *ee;       // density: adjoints of the new rho, Y, e
  const double *vsx, *vsy, *vsz;    // LANS filter: adjoints of the new vs
  const double *rho_new, *Y_new, *e_new;     // density outputs (recorded)
  const double *vsx_new, *vsy_new, *vsz_new; // LANS filter outputs (recorded)
  const double *wnd, *wnv;          // recorded normalisations
  double* dtbar;                    // adjoint of the step's dt
  double* ng0bar;
};

// ---------------------------------------------------------------- momentum
// Adjoint of WMom (mom_engr_update.cc:96-354 with LANS terms): i-side terms
// accumulated in registers, j-side terms scattered; the forward sums are
// formed again for the adjoint of dt.
struct VMom {
  WMom<double> f;
  static constexpr bool kListAhead = false;  // the list walk's plain entry loads
  static constexpr bool kSkipDecode = false;
  __device__ __forceinline__ const double* xpos() const { return f.xs; }
  const Adj& B;
  const AdjIn& in;
  double dt;
  double obv[3], obe;                        // adjoints of v_new, e_new
  double xb[3], hb, rhob, Vib, pvb, cb, Tb, cpb, velb[3];
  double rv[3], re;
  __device__ VMom(const Dev& A, const Packed& K, const Opt& o, const Adj& B_, const AdjIn& in_, double dt_)
      : f(A, K, o), B(B_), in(in_), dt(dt_) {}
  __device__ __forceinline__ bool setup(int ii, const Geo& g, const Work& W, const double* hmax, TimeState* ts,
                                        double* xi, int* bi, double& R) {
    if (!f.setup(ii, g, W, hmax, ts, xi, bi, R)) return false;
    obv[0] = in.vx[ii]; obv[1] = in.vy[ii]; obv[2] = in.vz[ii];
    obe = in.e[ii];
    xb[0] = xb[1] = xb[2] = 0;
    hb = rhob = Vib = pvb = cb = Tb = cpb = 0;
    velb[0] = velb[1] = velb[2] = 0;
    rv[0] = rv[1] = rv[2] = 0;
    re = 0;
    return true;
  }
  template <bool LISTED = false>
  __device__ __forceinline__ bool filter(uint32_t j, bool own, double ox, double oy, double oz, double* dx,
                                         double& hj) const {
    return f.template filter<LISTED>(j, own, ox, oy, oz, dx, hj);
  }
  __device__ __forceinline__ void math(uint32_t j, const double* dx, double hj) {
    const Dev& A = f.A;
    const double alpha = f.alpha, beta = f.beta, ata = f.ata;
    const bool lans = f.lans;
    double mj, rhoj, Vj, pVVj, cj, Tj, cpj, vj[3];
    f.load_j(j, mj, rhoj, Vj, pVVj, cj, Tj, cpj, vj);
    const double hi = f.hi, Vi = f.Vi;
    const double h = 0.5 * (hi + hj);
    double dist_sq = 0, velij[3], vrab = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      dist_sq += dx[k] * dx[k];
      velij[k] = f.veli[k] - vj[k];
      vrab += dx[k] * velij[k];
    }
    const double rhoab = 0.5 * (f.rhoi + rhoj);
    const double cab = 0.5 * (f.ci + cj);
    const double Dn = dist_sq + ata * h * h;
    const double miu = h * vrab / Dn;
    const bool av = vrab < 0;
    const double vis_av = av ? (beta * miu - alpha * cab) * miu / rhoab : 0.0;
    const double dotv = lans ? velij[0] * velij[0] + velij[1] * velij[1] + velij[2] * velij[2] : 0.0;
    const double vis = vis_av - (lans ? EPS_HALF * dotv * Vj : 0.0);
    const double P = mj * (pVVj + f.pvsqi + vis);
    double dW[3], dWdh;
    const double W = gw3(dx, h, dW, dWdh);
    const double* dwdx = dW;  // d_weight = dW/dx
    // LANS heat term
    double Cp_ij = 0, dotvr = 0, kab = 0, kij = 0, W_r = 0, F = 0, heat = 0;
    if (lans) {
      Cp_ij = 0.5 * (cpj + f.Cp_i);
#pragma unroll
      for (int k = 0; k < 3; k++) dotvr += fabs(velij[k] * dx[k]);
      if (dotvr != 0) {
        kab = 10.0 * EPS_HALF * Cp_ij * dist_sq * dotv / (PRANDTL * dotvr);
        kij = kab / (h * cab);
      }
#pragma unroll
      for (int k = 0; k < 3; k++) W_r += dwdx[k] * dx[k];
      if (W_r != 0) F = W_r / dist_sq;
      heat = mj * Vj * Vi * kij * (f.tempi - Tj) * F;
    }
    double sdv = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      rv[k] -= P * dwdx[k];
      sdv += dwdx[k] * velij[k];
    }
    re += 0.5 * P * sdv + heat;
    // ---- backward of the pair
    const double rvb[3] = {dt * obv[0], dt * obv[1], dt * obv[2]};
    const double reb = dt * obe;
    double Pb = 0.5 * reb * sdv, dwdxb[3], velijb[3], dxb[3] = {0, 0, 0};
    double hpb = 0, dist_sqb = 0, mjb = 0, Vjb = 0, rhojb = 0, cjb = 0, Tjb = 0, cpjb = 0, pjb = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      Pb -= rvb[k] * dwdx[k];
      dwdxb[k] = -rvb[k] * P + 0.5 * reb * P * velij[k];
      velijb[k] = 0.5 * reb * P * dwdx[k];
    }
    if (lans) {
      const double hb_ = reb;  // adjoint of heat
      const double tdiff = f.tempi - Tj;
      const double A0 = mj * Vj * Vi;
      mjb += hb_ * Vj * Vi * kij * tdiff * F;
      Vjb += hb_ * mj * Vi * kij * tdiff * F;
      Vib += hb_ * mj * Vj * kij * tdiff * F;
      const double kijb = hb_ * A0 * tdiff * F;
      Tb += hb_ * A0 * kij * F;
      Tjb -= hb_ * A0 * kij * F;
      const double Fb = hb_ * A0 * kij * tdiff;
      if (W_r != 0) {
        const double W_rb = Fb / dist_sq;
        dist_sqb -= Fb * W_r / (dist_sq * dist_sq);
#pragma unroll
        for (int k = 0; k < 3; k++) {
          dwdxb[k] += W_rb * dx[k];
          dxb[k] += W_rb * dwdx[k];
        }
      }
      if (dotvr != 0) {
        const double kabb = kijb / (h * cab);
        hpb -= kijb * kij / h;
        const double cabb_h = -kijb * kij / cab;
        cb += 0.5 * cabb_h;
        cjb += 0.5 * cabb_h;
        const double Kc = 10.0 * EPS_HALF / PRANDTL;
        const double Cp_ijb = kabb * Kc * dist_sq * dotv / dotvr;
        dist_sqb += kabb * Kc * Cp_ij * dotv / dotvr;
        const double dotvb_h = kabb * Kc * Cp_ij * dist_sq / dotvr;
        const double dotvrb = -kabb * kab / dotvr;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const double t = velij[k] * dx[k];
          const double sg = (t > 0) ? 1.0 : ((t < 0) ? -1.0 : 0.0);
          velijb[k] += dotvrb * sg * dx[k] + 2.0 * dotvb_h * velij[k];
          dxb[k] += dotvrb * sg * velij[k];
        }
        cpb += 0.5 * Cp_ijb;
        cpjb += 0.5 * Cp_ijb;
      }
    }
    // P = mj (pVVj + pvsqi + vis)
    mjb += Pb * (pVVj + f.pvsqi + vis);
    const double pVVjb = Pb * mj;
    pvb += Pb * mj;
    const double visb = Pb * mj;
    if (lans) {
      const double dotvb = -EPS_HALF * visb * Vj;
      Vjb -= EPS_HALF * visb * dotv;
#pragma unroll
      for (int k = 0; k < 3; k++) velijb[k] += 2.0 * dotvb * velij[k];
    }
    if (av) {
      const double miub = visb * (2.0 * beta * miu - alpha * cab) / rhoab;
      const double cabb = -visb * alpha * miu / rhoab;
      const double rhoabb = -visb * vis_av / rhoab;
      cb += 0.5 * cabb;
      cjb += 0.5 * cabb;
      rhob += 0.5 * rhoabb;
      rhojb += 0.5 * rhoabb;
      hpb += miub * (vrab / Dn - 2.0 * ata * h * h * vrab / (Dn * Dn));
      const double vrabb = miub * h / Dn;
      dist_sqb -= miub * h * vrab / (Dn * Dn);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        dxb[k] += vrabb * velij[k];
        velijb[k] += vrabb * dx[k];
      }
    }
    // dwdx_k = -2 dx_k W / h^2
    if (W != 0) {
      double sdw = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) sdw += dwdxb[k] * dx[k];
      const double ih2 = 1.0 / (h * h);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        dxb[k] += -2.0 * ih2 * (dwdxb[k] * W + sdw * dW[k]);
        hpb += dwdxb[k] * (4.0 * dx[k] * ih2 / h * W - 2.0 * dx[k] * ih2 * dWdh);
      }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) dxb[k] += 2.0 * dist_sqb * dx[k];
    // pVVj = p_j Vj^2, Vj = 1/rho_j
    const double pj = pVVj / (Vj * Vj);
    pjb += pVVjb * Vj * Vj;
    Vjb += 2.0 * pVVjb * pj * Vj;
    rhojb -= Vjb * Vj * Vj;
    // scatter j, keep i
#pragma unroll
    for (int k = 0; k < 3; k++) {
      xb[k] += dxb[k];
      velb[k] += velijb[k];
    }
    hb += 0.5 * hpb;
    atomicAdd(&B.x[j], -dxb[0]);
    atomicAdd(&B.y[j], -dxb[1]);
    atomicAdd(&B.z[j], -dxb[2]);
    atomicAdd(&B.h[j], 0.5 * hpb);
    atomicAdd(&B.m[j], mjb);
    atomicAdd(&B.rho[j], rhojb);
    atomicAdd(&B.p[j], pjb);
    atomicAdd(&B.c[j], cjb);
    if (lans) {
      atomicAdd(&B.T[j], Tjb);
      atomicAdd(&B.cp[j], cpjb);
      atomicAdd(&B.vsx[j], -velijb[0]);
      atomicAdd(&B.vsy[j], -velijb[1]);
      atomicAdd(&B.vsz[j], -velijb[2]);
    } else {
      atomicAdd(&B.vx[j], -velijb[0]);
      atomicAdd(&B.vy[j], -velijb[1]);
      atomicAdd(&B.vz[j], -velijb[2]);
    }
    (void)A;
  }
  // i-side: everything accumulated, plus the finish (v_new = v + dt rv +
  // dt g e_z, e_new = e + dt (re + veli_z g)); returns this particle's
  // share of the adjoint of dt
  __device__ __forceinline__ double finish(int ii) {
    const double grav = -f.o.g;
    const bool lans = f.lans;
    const double Vi = f.Vi, pi = f.pvsqi / (Vi * Vi);
    // pvsqi = p_i Vi^2
    double pib = pvb * Vi * Vi;
    double Vib_t = Vib + 2.0 * pvb * pi * Vi;
    double rhoib = rhob - Vib_t * Vi * Vi;
    velb[2] += dt * grav * obe;  // veli_z in the energy update
    atomicAdd(&B.x[ii], xb[0]);
    atomicAdd(&B.y[ii], xb[1]);
    atomicAdd(&B.z[ii], xb[2]);
    atomicAdd(&B.h[ii], hb);
    atomicAdd(&B.rho[ii], rhoib);
    atomicAdd(&B.p[ii], pib);
    atomicAdd(&B.c[ii], cb);
    if (lans) {
      atomicAdd(&B.T[ii], Tb);
      atomicAdd(&B.cp[ii], cpb);
      atomicAdd(&B.vsx[ii], velb[0]);
      atomicAdd(&B.vsy[ii], velb[1]);
      atomicAdd(&B.vsz[ii], velb[2]);
    } else {
      atomicAdd(&B.vx[ii], velb[0]);
      atomicAdd(&B.vy[ii], velb[1]);
      atomicAdd(&B.vz[ii], velb[2]);
    }
    return rv[0] * obv[0] + rv[1] * obv[1] + (rv[2] + grav) * obv[2] + (re + f.veli[2] * grav) * obe;
  }
};

// ---------------------------------------------------------------- density
// Adjoint of WDens (density_massfrac.cc:64-333): rho = r1 + r2 (phase 1 /
// phase 2 sums of m_j W(dx, h_ij)), Y = r2 / rho, e = sum (m_j/rho_j) e_j
// W(dx, h_ij/4) / sum (m_j/rho_j) W(dx, h_ij/4).
struct VDens {
  WDens<double> f;
  static constexpr bool kListAhead = false;  // the list walk's plain entry loads
  static constexpr bool kSkipDecode = false;
  __device__ __forceinline__ const double* xpos() const { return f.xs; }
  const Adj& B;
  const AdjIn& in;
  double r1b, r2b, wnb, enb;
  double xb[3], hb;
  __device__ VDens(const Dev& A, const Packed& K, const Opt& o, const Adj& B_, const AdjIn& in_, double)
      : f(A, K, o), B(B_), in(in_) {}
  __device__ __forceinline__ bool setup(int ii, const Geo& g, const Work& W, const double* hmax, TimeState* ts,
                                        double* xi, int* bi, double& R) {
    if (!f.setup(ii, g, W, hmax, ts, xi, bi, R)) return false;
    const double rb = in.rho[ii], Yb = in.Y[ii];
    const double rho2 = in.rho_new[ii], Y2 = in.Y_new[ii];
    r1b = rb - Yb * Y2 / rho2;
    r2b = rb + Yb * (1.0 - Y2) / rho2;
    wnb = enb = 0;
    if (f.esm) {
      const double eb = in.ee[ii], wn = in.wnd[ii], nE = in.e_new[ii];
      enb = eb / wn;
      wnb = -eb * nE / wn;
    }
    xb[0] = xb[1] = xb[2] = 0;
    hb = 0;
    return true;
  }
  template <bool LISTED = false>
  __device__ __forceinline__ bool filter(uint32_t j, bool own, double ox, double oy, double oz, double* dx,
                                         double& hj) const {
    return f.template filter<LISTED>(j, own, ox, oy, oz, dx, hj);
  }
  __device__ __forceinline__ void math(uint32_t j, const double* dx, double hj) {
    const Dev& A = f.A;
    const double mj = A.mass[j], rhoj = A.rho[j], ej = A.e[j];
    const double hh = 0.5 * (f.hi + hj);
    double dW[3], dWdh;
    const double W = gw3(dx, hh, dW, dWdh);
    const double rphb = (A.phase[j] == 1) ? r1b : r2b;
    const double Wb = rphb * mj;
    double mjb = rphb * W, rhojb = 0, ejb = 0, hhb = Wb * dWdh;
    double dxb[3] = {Wb * dW[0], Wb * dW[1], Wb * dW[2]};
    if (f.esm) {
      double dWe[3], dWedh;
      const double We = gw3(dx, 0.25 * hh, dWe, dWedh);
      const double a = We * mj / rhoj;
      const double ab = wnb + enb * ej;
      ejb = enb * a;
      const double Web = ab * mj / rhoj;
      mjb += ab * We / rhoj;
      rhojb = -ab * We * mj / (rhoj * rhoj);
#pragma unroll
      for (int k = 0; k < 3; k++) dxb[k] += Web * dWe[k];
      hhb += Web * dWedh * 0.25;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) xb[k] += dxb[k];
    hb += 0.5 * hhb;
    atomicAdd(&B.x[j], -dxb[0]);
    atomicAdd(&B.y[j], -dxb[1]);
    atomicAdd(&B.z[j], -dxb[2]);
    atomicAdd(&B.h[j], 0.5 * hhb);
    atomicAdd(&B.m[j], mjb);
    if (rhojb != 0) atomicAdd(&B.rho[j], rhojb);
    if (ejb != 0) atomicAdd(&B.e[j], ejb);
  }
  __device__ __forceinline__ double finish(int ii) {
    atomicAdd(&B.x[ii], xb[0]);
    atomicAdd(&B.y[ii], xb[1]);
    atomicAdd(&B.z[ii], xb[2]);
    atomicAdd(&B.h[ii], hb);
    return 0;
  }
};

// ---------------------------------------------------------------- LANS filter
// Adjoint of WVel (smooth_velocity.cc:25-165): vs_i = v_i + sum w_j (v_j -
// v_i) / sum w_j, w_j = (m_j / rho_j) W(dx, h_i).
struct VVel {
  WVel<double> f;
  static constexpr bool kListAhead = false;  // the list walk's plain entry loads
  static constexpr bool kSkipDecode = false;
  __device__ __forceinline__ const double* xpos() const { return f.xs; }
  const Adj& B;
  const AdjIn& in;
  double ob[3], dvb[3], wnb, vib[3];
  double xb[3], hb;
  __device__ VVel(const Dev& A, const Packed& K, const Opt& o, const Adj& B_, const AdjIn& in_, double)
      : f(A, K, o), B(B_), in(in_) {}
  __device__ __forceinline__ bool setup(int ii, const Geo& g, const Work& W, const double* hmax, TimeState* ts,
                                        double* xi, int* bi, double& R) {
    if (!f.setup(ii, g, W, hmax, ts, xi, bi, R)) return false;
    ob[0] = in.vsx[ii]; ob[1] = in.vsy[ii]; ob[2] = in.vsz[ii];
    const double wn = in.wnv[ii];
    const double avg[3] = {in.vsx_new[ii] - f.vi_d[0], in.vsy_new[ii] - f.vi_d[1], in.vsz_new[ii] - f.vi_d[2]};
    wnb = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      dvb[k] = ob[k] / wn;
      wnb -= ob[k] * avg[k] / wn;
      vib[k] = ob[k];  // vs = v_i + ...
    }
    xb[0] = xb[1] = xb[2] = 0;
    hb = 0;
    return true;
  }
  template <bool LISTED = false>
  __device__ __forceinline__ bool filter(uint32_t j, bool own, double ox, double oy, double oz, double* dx,
                                         double& flag) const {
    return f.template filter<LISTED>(j, own, ox, oy, oz, dx, flag);
  }
  __device__ __forceinline__ void math(uint32_t j, const double* dx, double) {
    const Dev& A = f.A;
    const double mj = A.mass[j], rhoj = A.rho[j];
    const double vj[3] = {A.vx[j], A.vy[j], A.vz[j]};
    double dW[3], dWdh;
    const double W = gw3(dx, f.hi, dW, dWdh);
    const double mvw = W * mj / rhoj;
    double mvwb = wnb;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      mvwb += dvb[k] * (vj[k] - f.vi_d[k]);
      vib[k] -= mvw * dvb[k];
    }
    const double Wb = mvwb * mj / rhoj;
    const double dxb[3] = {Wb * dW[0], Wb * dW[1], Wb * dW[2]};
#pragma unroll
    for (int k = 0; k < 3; k++) xb[k] += dxb[k];
    hb += Wb * dWdh;
    atomicAdd(&B.x[j], -dxb[0]);
    atomicAdd(&B.y[j], -dxb[1]);
    atomicAdd(&B.z[j], -dxb[2]);
    atomicAdd(&B.m[j], mvwb * W / rhoj);
    atomicAdd(&B.rho[j], -mvwb * W * mj / (rhoj * rhoj));
    atomicAdd(&B.vx[j], mvw * dvb[0]);
    atomicAdd(&B.vy[j], mvw * dvb[1]);
    atomicAdd(&B.vz[j], mvw * dvb[2]);
  }
  __device__ __forceinline__ double finish(int ii) {
    atomicAdd(&B.x[ii], xb[0]);
    atomicAdd(&B.y[ii], xb[1]);
    atomicAdd(&B.z[ii], xb[2]);
    atomicAdd(&B.h[ii], hb);
    atomicAdd(&B.vx[ii], vib[0]);
    atomicAdd(&B.vy[ii], vib[1]);
    atomicAdd(&B.vz[ii], vib[2]);
    return 0;
  }
};

// driver: one thread per need_neigh particle over the step's windows; the
// functor's finish returns the particle's share of the adjoint of dt
template <class SV>
__global__ void __launch_bounds__(128) k_adj_sweep(Opt o, Geo g, Dev A, Work W, Packed K,
                                                   const uint32_t* __restrict__ cs, const double* __restrict__ hmax,
                                                   const int* __restrict__ d_real,
                                                   const uint32_t* __restrict__ real_idx, TimeState* ts, NList L,
                                                   Adj B, AdjIn in, double dt) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double dtb = 0;
  if (r < *d_real) {
    const int i = (int)real_idx[r];
    SV s(A, K, o, B, in, dt);
    double xi[3], R;
    int bi[3];
    if (s.setup(i, g, W, hmax, ts, xi, bi, R)) {
      list_walk<double>(s, i, g, cs, xi, bi, R, L);
      dtb = s.finish(i);
    }
  }
  block_add(dtb, in.dtbar);
}

// ---------------------------------------------------------------- pointwise
// P: x_new = x + dt u (u = vs for real particles under LANS, v for erupt
// particles while erupting); converted erupt particles get h = sml2.
// bc0 = bc before the update, bc1 = after.
__global__ void k_adj_pos(Dev S, const uint8_t* __restrict__ bc1, const double* __restrict__ vsx,
                          const double* __restrict__ vsy, const double* __restrict__ vsz, const double* __restrict__ vx,
                          const double* __restrict__ vy, const double* __restrict__ vz, int n, double dt, int erupt,
                          int lans, Adj B, double* dtbar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double dtb = 0;
  if (i < n && bc1[i] != BC_DEAD) {
    const uint8_t b0 = S.bc[i];
    const double xb[3] = {B.x[i], B.y[i], B.z[i]};
    if (is_real(b0)) {
      if (lans) {
        dtb = xb[0] * vsx[i] + xb[1] * vsy[i] + xb[2] * vsz[i];
        B.vsx[i] += dt * xb[0]; B.vsy[i] += dt * xb[1]; B.vsz[i] += dt * xb[2];
      } else {
        dtb = xb[0] * vx[i] + xb[1] * vy[i] + xb[2] * vz[i];
        B.vx[i] += dt * xb[0]; B.vy[i] += dt * xb[1]; B.vz[i] += dt * xb[2];
      }
    } else if (b0 == 0 && erupt) {
      dtb = xb[0] * vx[i] + xb[1] * vy[i] + xb[2] * vz[i];
      B.vx[i] += dt * xb[0]; B.vy[i] += dt * xb[1]; B.vz[i] += dt * xb[2];
      if (bc1[i] == 100) B.h[i] = 0;  // h <- sml2
    }
  }
  block_add(dtb, dtbar);
}

// V: take the adjoint of the new vs out (need_neigh particles)
__global__ void k_adj_vel_pre(Dev S, int n, Adj B, double* ox, double* oy, double* oz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !need_neigh(S.bc[i])) return;
  ox[i] = B.vsx[i]; oy[i] = B.vsy[i]; oz[i] = B.vsz[i];
  B.vsx[i] = 0; B.vsy[i] = 0; B.vsz[i] = 0;
}

// D: EOS of the density commit, then take the adjoint of the new rho, Y, e
// out (need_neigh particles); p, c, T, cp written before D are dead
__global__ void k_adj_dens_pre(Opt o, Dev S, const double* __restrict__ rho2, const double* __restrict__ Y2,
                               const double* __restrict__ e2, int n, Adj B, double* orho, double* oY, double* oe,
                               double* ng0bar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ngb = 0;
  if (i < n && need_neigh(S.bc[i])) {
    double rb = B.rho[i], Yb = B.Y[i], eb = B.e[i];
    eos_vjp(o, rho2[i], Y2[i], e2[i], B.p[i], B.c[i], B.T[i], B.cp[i], o.lans != 0, rb, Yb, eb, ngb);
    orho[i] = rb;
    oY[i] = Yb;
    if (o.esmooth) {
      oe[i] = eb;
      B.e[i] = 0;
    } else {
      oe[i] = 0;
      B.e[i] = eb;
    }
    B.rho[i] = 0;
    B.Y[i] = 0;
    B.p[i] = 0; B.c[i] = 0; B.T[i] = 0; B.cp[i] = 0;
  }
  block_add(ngb, ng0bar);
}

// M: copy the adjoint of the new v, e (they also pass to the old v, e)
__global__ void k_adj_mom_pre(Dev S, int n, Adj B, double* ox, double* oy, double* oz, double* oe) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool nn = need_neigh(S.bc[i]);
  ox[i] = nn ? B.vx[i] : 0.0;
  oy[i] = nn ? B.vy[i] : 0.0;
  oz[i] = nn ? B.vz[i] : 0.0;
  oe[i] = nn ? B.e[i] : 0.0;
}

// A: take the adjoint of the new h out (particles that iterated)
__global__ void k_adj_adapt_pre(Dev S, const uint8_t* __restrict__ nit, int n, Adj B, double* oh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool it = need_neigh(S.bc[i]) && nit[i] > 0;
  oh[i] = it ? B.h[i] : 0.0;
  if (it) B.h[i] = 0;
}

// A: adjoint of adaptive_sml's iterations h_{k+1} = eta (m_i / rho*_k)^(1/3),
// rho*_k = sum_j m_j W(dx, c_smooth h_k), from the recorded iterates; the
// iteration count and the list rule are those of the forward run
__global__ void k_adj_adaptive(Opt o, Geo g, Dev S, Work W, const uint32_t* __restrict__ cs, int n,
                               const double* __restrict__ hit, const uint8_t* __restrict__ nit, int nrow,
                               const double* __restrict__ ohb, Adj B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !need_neigh(S.bc[i])) return;
  const int K = nit[i];
  if (K == 0) return;
  double hb = ohb[i];
  const double xi[3] = {S.x[i], S.y[i], S.z[i]};
  int bi[3];
  bucket_coords<3>(g, S.bkt[i], bi);
  const double Lb = o.list_factor * W.hlist[i];
  const double mi = S.mass[i];
  double xb[3] = {0, 0, 0}, mib = 0;
  for (int k = K - 1; k >= 0; k--) {
    const double hk = hit[(size_t)k * nrow + i];
    const double hn = hit[(size_t)(k + 1) * nrow + i];
    if (hb == 0) continue;  // nothing flows back (h_k only enters iteration k)
    const double H = hk * o.c_smooth;
    const double rs = mi * (o.eta / hn) * (o.eta / hn) * (o.eta / hn);
    const double rsb = -hb * hn / (3.0 * rs);
    mib += hb * hn / (3.0 * mi);
    const double supp = o.cutoff2 * H;
    const double R = fmin(o.cutoff2, o.ksupport) * H * (1.0 + 1e-10);
    double Hb = 0;
    for_segments<3, double>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, double, double, double) {
      for (uint32_t j = j0; j < j1; j++) {
        if (!contr_dens(S.bc[j], o.pgc)) continue;
        const double dx[3] = {xi[0] - S.x[j], xi[1] - S.y[j], xi[2] - S.z[j]};
        if (!own && !in_box<3, double>(dx, Lb)) continue;
        if (!in_box<3, double>(dx, supp)) continue;
        double dW[3], dWdh;
        const double Wv = gw3(dx, H, dW, dWdh);
        if (Wv == 0) continue;
        const double mj = S.mass[j];
        const double dxb[3] = {rsb * mj * dW[0], rsb * mj * dW[1], rsb * mj * dW[2]};
        xb[0] += dxb[0]; xb[1] += dxb[1]; xb[2] += dxb[2];
        Hb += rsb * mj * dWdh;
        atomicAdd(&B.m[j], rsb * Wv);
        atomicAdd(&B.x[j], -dxb[0]);
        atomicAdd(&B.y[j], -dxb[1]);
        atomicAdd(&B.z[j], -dxb[2]);
      }
    });
    hb = o.c_smooth * Hb;
  }
  atomicAdd(&B.h[i], hb);
  atomicAdd(&B.m[i], mib);
  atomicAdd(&B.x[i], xb[0]);
  atomicAdd(&B.y[i], xb[1]);
  atomicAdd(&B.z[i], xb[2]);
}

// dt = cfl h_k / c_k of the particle k that set it (timestep.cc:94-135)
__global__ void k_adj_dt(Dev S, const int* __restrict__ argmin, double cfl, const double* __restrict__ dtbar,
                         Adj B) {
  const int k = *argmin;
  if (k == 0x7fffffff) return;  // no particle updates its state
  const double hk = S.h[k], ck = S.c[k], db = *dtbar;
  B.h[k] += cfl * db / ck;
  B.c[k] -= cfl * hk * db / (ck * ck);
}

// the particle k with h_k / c_k == the step's minimum (smallest index on ties)
__global__ void k_dt_argmin(Dev A, const int* __restrict__ d_count, const TimeState* ts, int* argmin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count || !need_neigh(A.bc[i])) return;
  const double m = __longlong_as_double((long long)ts->dtmin_bits);
  if (A.h[i] / A.c[i] == m) atomicMin(argmin, i);
}

// adjoint rows back to the order before the step's sort (rows that were not
// alive at the sort stay zero)
__global__ void k_adj_unperm(Adj cur, Adj prev, const uint32_t* __restrict__ perm, int nlive) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nlive) return;
  const uint32_t q = perm[p];
  double* const c[18] = {cur.x, cur.y, cur.z, cur.vx, cur.vy, cur.vz, cur.vsx, cur.vsy, cur.vsz,
                         cur.m, cur.h, cur.rho, cur.e, cur.p, cur.Y, cur.c, cur.T, cur.cp};
  double* const d[18] = {prev.x, prev.y, prev.z, prev.vx, prev.vy, prev.vz, prev.vsx, prev.vsy, prev.vsz,
                         prev.m, prev.h, prev.rho, prev.e, prev.p, prev.Y, prev.c, prev.T, prev.cp};
#pragma unroll
  for (int f = 0; f < 18; f++) d[f][q] = c[f][p];
}

}  // namespace plume
