// physics.cuh -- per-ion device physics shared by the FP64 and mixed forms:
// Boris rotation, mean relative speed, Philox ion-neutral collision.
#pragma once

#include "common.cuh"

template <typename R> __device__ __forceinline__ R unitR(uint32_t r);
template <> __device__ __forceinline__ double unitR<double>(uint32_t r) { return ch_unit(r); }
template <> __device__ __forceinline__ float unitR<float>(uint32_t r) { return ch_unitf(r); }

__device__ __forceinline__ double ch_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float ch_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double ch_log(double x) { return log(x); }
// FP32 form: the hardware log2 (absolute error near 1e-7 on the unit
// interval, ample for waiting times and Box-Muller radii of the FP32 form)
__device__ __forceinline__ float ch_log(float x) { return __logf(x); }
__device__ __forceinline__ double ch_exp(double x) { return exp(x); }
__device__ __forceinline__ float ch_exp(float x) { return expf(x); }
__device__ __forceinline__ double ch_erf(double x) { return erf(x); }
// Quick forms for the collision draws of the FP32 form: the hardware
// approximate square root (PTX sqrt.approx.f32) and the full-range
// approximate division (__fdividef, 2 ulp).  The draws are statistical and
// their FP32 form is already rounded at 2^-24; the FP64 form stays exact.
__device__ __forceinline__ double ch_qsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float ch_qsqrt(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double ch_qdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float ch_qdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float ch_erf(float x) { return erff(x); }
__device__ __forceinline__ void ch_sincos2pi(double u, double* s, double* c) { sincos(2.0 * CH_PI * u, s, c); }
// FP32 form, u in [0, 1): the hardware sine/cosine on the angle 2 pi (u -
// 1/2) in [-pi, pi), where its absolute error stays near 2^-21, and the half
// turn restored by the signs.
__device__ __forceinline__ void ch_sincos2pi(float u, float* s, float* c) {
  float sh, ch;
  __sincosf(6.2831853071795865f * (u - 0.5f), &sh, &ch);
  *s = -sh;
  *c = -ch;
}

// E|w - V| for |w - vn0| = w and V Maxwellian with per-component std sigma:
// sigma sqrt(2/pi) exp(-a^2) + (w + sigma^2/w) erf(a), a = w/(sigma sqrt 2);
// series 2 sigma sqrt(2/pi)(1 + a^2/3) for small a.
template <typename R>
__device__ __forceinline__ R ch_gmean(R w, R sigma) {
  if (!(sigma > R(0))) return w;
  const R a = w / (sigma * R(1.4142135623730951));
  const R c = sigma * R(0.7978845608028654);
  if (a < R(1e-4)) return R(2) * c * (R(1) + a * a / R(3));
  return c * ch_exp(-a * a) + (w + sigma * sigma / w) * ch_erf(a);
}

// FP32 form of the same mean: erf(a) = 1 - P(t) e^{-a^2} with t = 1/(1 + p a)
// (Abramowitz & Stegun 7.1.26, |error| <= 1.5e-7) shares the exponential of
// the first term; below a = 0.3 the series 2 sigma sqrt(2/pi)(1 + a^2/3 -
// a^4/30 + a^6/210) avoids the cancellation in 1 - P e^{-a^2}.  Relative
// error below 1e-6 against the FP64 form.
// Every operation is rounded as written (the _rn intrinsics are neither
// contracted nor reordered by the compiler), so each kernel that evaluates
// g of the same velocity gets the same bits: the collision-rate sum S formed
// by one step and the S formed from the ions it wrote agree exactly.
template <>
__device__ __forceinline__ float ch_gmean<float>(float w, float sigma) {
  if (!(sigma > 0.0f)) return w;
  const float a = __fdividef(w, __fmul_rn(sigma, 1.41421356f));
  const float c = __fmul_rn(sigma, 0.797884561f);
  const float a2 = __fmul_rn(a, a);
  if (a < 0.3f)
    return __fmul_rn(__fmul_rn(2.0f, c),
                     __fmaf_rn(a2, __fmaf_rn(a2, __fmaf_rn(a2, 0.00476190476f, -0.0333333333f), 0.333333333f), 1.0f));
  const float e = __expf(-a2);
  const float t = __fdividef(1.0f, __fmaf_rn(0.3275911f, a, 1.0f));
  float h = __fmaf_rn(t, 1.061405429f, -1.453152027f);
  h = __fmaf_rn(t, h, 1.421413741f);
  h = __fmaf_rn(t, h, -0.284496736f);
  h = __fmaf_rn(t, h, 0.254829592f);
  const float P = __fmul_rn(t, h);
  return __fmaf_rn(c, e, __fmul_rn(__fadd_rn(w, __fdividef(__fmul_rn(sigma, sigma), w)), __fmaf_rn(-P, e, 1.0f)));
}

// |v - vn0| of the FP32 form, rounded as written (see ch_gmean<float>).
__device__ __forceinline__ float ch_relspeed_rn(float vx, float vy, float vz, float ux, float uy, float uz) {
  const float qx = __fsub_rn(vx, ux), qy = __fsub_rn(vy, uy), qz = __fsub_rn(vz, uz);
  return ch_qsqrt(__fmaf_rn(qz, qz, __fmaf_rn(qy, qy, __fmul_rn(qx, qx))));
}
template <typename R>
__device__ __forceinline__ R ch_relspeed(R vx, R vy, R vz, R ux, R uy, R uz) {
  const R qx = vx - ux, qy = vy - uy, qz = vz - uz;
  return ch_qsqrt(qx * qx + qy * qy + qz * qz);
}
template <>
__device__ __forceinline__ float ch_relspeed<float>(float vx, float vy, float vz, float ux, float uy, float uz) {
  return ch_relspeed_rn(vx, vy, vz, ux, uy, uz);
}

template <typename R>
__device__ __forceinline__ R ch_neutral_density(const StepConsts& c, R x_abs) {
  if (c.nn_profile != CH_NN_GAUSSIAN_X) return R(1);
  const R u = (x_abs - ch_pick<R>(c.nn_center, c.f.nn_center)) / ch_pick<R>(c.nn_sigma, c.f.nn_sigma);
  const R v = ch_exp(R(-0.5) * u * u);
  const R fl = ch_pick<R>(c.nn_floor, c.f.nn_floor);
  return v > fl ? v : fl;
}

// Boris push (src/particles.c:374-447), E already includes the push scale.
template <typename R>
__device__ __forceinline__ void ch_boris(const StepConsts& c, const R E[3], R v[3]) {
  const R ts = R(c.tscale);
  R vm0 = v[0] + ts * E[0], vm1 = v[1] + ts * E[1], vm2 = v[2] + ts * E[2];
  R vp0, vp1, vp2;
  if (c.faithful & CH_FAITHFUL_D2) {
    vp0 = vm0; vp1 = vm1; vp2 = vm2;
  } else {
    const R t0 = R(c.t[0]), t1 = R(c.t[1]), t2 = R(c.t[2]);
    const R s0 = R(c.s[0]), s1 = R(c.s[1]), s2 = R(c.s[2]);
    const R q0 = vm0 + (vm1 * t2 - vm2 * t1);
    const R q1 = vm1 + (vm2 * t0 - vm0 * t2);
    const R q2 = vm2 + (vm0 * t1 - vm1 * t0);
    vp0 = vm0 + (q1 * s2 - q2 * s1);
    vp1 = vm1 + (q2 * s0 - q0 * s2);
    vp2 = vm2 + (q0 * s1 - q1 * s0);
  }
  v[0] = vp0 + ts * E[0];
  v[1] = vp1 + ts * E[1];
  v[2] = vp2 + ts * E[2];
}

// Collisions of one ion over one step (src/particles.c:471-624 in its
// many-ion limit): the ion's events form a Poisson process in the step's unit
// time with rate lambda(v) = lscale g(|v - vn0|), lscale = Nc rho_n(x) / S.
// Event e draws its exponential waiting time from Philox block e << 8 and
// its neutral V ~ |v - V| N(V) from blocks (e << 8) | (1 + 2 it), (2 + 2 it);
// the centre-of-mass scatter and the 10 vT refusal follow the reference.
// Returns the accepted collisions; *refused counts refused events.
#define CH_MAX_EVENTS 32
template <typename R>
__device__ __noinline__ int ch_collide(const StepConsts& c, uint32_t id, R lscale, R v[3], unsigned* refused) {
  const R sig = ch_pick<R>(c.vnT, c.f.vnT);
  const R vn0x = ch_pick<R>(c.vn0[0], c.f.vn0[0]), vn0y = ch_pick<R>(c.vn0[1], c.f.vn0[1]),
          vn0z = ch_pick<R>(c.vn0[2], c.f.vn0[2]);
  const R m1 = ch_pick<R>(c.m1, c.f.m1);
  const R mi = ch_pick<R>(c.mi, c.f.mi), mn = ch_pick<R>(c.mn, c.f.mn), M = mn + mi;
  R t = R(0);
  int ncol = 0;
  for (uint32_t e = 0; e < CH_MAX_EVENTS; ++e) {
    const R vix = v[0], viy = v[1], viz = v[2];
    const R wx = vix - vn0x, wy = viy - vn0y, wz = viz - vn0z;
    const R w = ch_sqrt(wx * wx + wy * wy + wz * wz);
    const R lam = lscale * ch_gmean<R>(w, sig);
    if (!(lam > R(0))) break;
    const U4 r0 = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8), c.run, c.seed_lo, c.seed_hi);
    t += -ch_log(unitR<R>(r0.x)) / lam;
    if (!(t < R(1))) break;
    R Vx = 0, Vy = 0, Vz = 0, uz = 0, uphi = 0;
    bool ok = false;
    for (uint32_t it = 0; it < 64 && !ok; ++it) {
      const U4 a = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8) | (1 + 2 * it), c.run, c.seed_lo,
                             c.seed_hi);
      const U4 b = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8) | (2 + 2 * it), c.run, c.seed_lo,
                             c.seed_hi);
      R nx, ny, nz;
      if (unitR<R>(a.x) * (w + m1) < w) {
        // plain Maxwellian proposal, Box-Muller
        R s1, c1, s2, c2;
        const R r1 = ch_sqrt(R(-2) * ch_log(unitR<R>(a.y)));
        ch_sincos2pi(unitR<R>(a.z), &s1, &c1);
        const R r2 = ch_sqrt(R(-2) * ch_log(unitR<R>(a.w)));
        ch_sincos2pi(unitR<R>(b.x), &s2, &c2);
        nx = sig * (r1 * c1); ny = sig * (r1 * s1); nz = sig * (r2 * c2);
      } else {
        // speed-weighted proposal: |V - vn0|^2 / (2 sigma^2) ~ Gamma(2, 1)
        const R sp = sig * ch_sqrt(R(-2) * ch_log(unitR<R>(a.y) * unitR<R>(a.z)));
        const R ct = R(2) * unitR<R>(a.w) - R(1);
        R st = R(1) - ct * ct;
        st = ch_sqrt(st > R(0) ? st : R(0));
        R sph, cph;
        ch_sincos2pi(unitR<R>(b.x), &sph, &cph);
        nx = sp * st * cph; ny = sp * st * sph; nz = sp * ct;
      }
      Vx = vn0x + nx; Vy = vn0y + ny; Vz = vn0z + nz;
      const R dV = ch_sqrt(nx * nx + ny * ny + nz * nz);
      const R rx = vix - Vx, ry = viy - Vy, rz = viz - Vz;
      const R D = ch_sqrt(rx * rx + ry * ry + rz * rz);
      if (unitR<R>(b.y) * (w + dV) < D) {
        ok = true;
        uz = R(2) * unitR<R>(b.z) - R(1);
        uphi = unitR<R>(b.w);
      }
    }
    if (!ok) { ++*refused; continue; }
    // centre-of-mass scatter (src/particles.c:552-591)
    const R vrx = vix - Vx, vry = viy - Vy, vrz = viz - Vz;
    const R vrr = ch_sqrt(vrx * vrx + vry * vry + vrz * vrz);
    const R vcx = (vix * mi + Vx * mn) / M, vcy = (viy * mi + Vy * mn) / M, vcz = (viz * mi + Vz * mn) / M;
    const R ax = vix - vcx, ay = viy - vcy, az = viz - vcz;
    const R vcr = ch_sqrt(ax * ax + ay * ay + az * az);
    R up = R(1) - uz * uz;
    const R uperp = ch_sqrt(up > R(0) ? up : R(0));
    R sph, cph;
    ch_sincos2pi(uphi, &sph, &cph);
    const R ux = uperp * cph, uy = uperp * sph;
    const R costht = vrr > R(0) ? vrz / vrr : R(1);
    R st2 = R(1) - costht * costht;
    const R sintht = ch_sqrt(st2 > R(0) ? st2 : R(0));
    R cosphi = R(1), sinphi = R(0);
    if (vrr * sintht > R(0)) {
      cosphi = vrx / (vrr * sintht);
      sinphi = vry / (vrr * sintht);
    }
    const R ux1 = uz * sintht + ux * costht, uy1 = uy, uz1 = uz * costht - ux * sintht;
    const R ux2 = ux1 * cosphi - uy1 * sinphi, uy2 = ux1 * sinphi + uy1 * cosphi, uz2 = uz1;
    const R vfx = vcx + vcr * ux2, vfy = vcy + vcr * uy2, vfz = vcz + vcr * uz2;
    const R vfr = ch_sqrt(vfx * vfx + vfy * vfy + vfz * vfz);
    if (vfr / ch_pick<R>(c.viTr, c.f.viTr) > R(10)) { ++*refused; continue; }
    v[0] = vfx; v[1] = vfy; v[2] = vfz;
    ++ncol;
  }
  return ncol;
}

// One round of the collision event process of one ion, for queues that
// advance every queued ion by one proposal per round (so that a warp does
// not wait on the unluckiest lane's rejection loop).  State: event e,
// proposal it of that event, elapsed time t (the waiting time of event e is
// already in t).  The round draws proposal it of event e from the same
// Philox blocks as ch_collide; if it is accepted the scatter (or refusal) is
// applied and the waiting time of event e + 1 is added.  Returns true when
// the ion has no further event in this step; gfin is then the mean relative
// speed g of its final velocity.  Quick square roots and divisions
// (ch_qsqrt, ch_qdiv) and two identities of the scatter, |v - v_cm| =
// mn / M |v - V| and the refusal |v'| > 10 viT compared in squares, keep
// the FP32 rounds short.
template <typename R>
__device__ __forceinline__ bool ch_collide_round(const StepConsts& c, uint32_t id, R lscale, R v[3], R& t,
                                                 uint32_t& e, uint32_t& it, unsigned* ncol, unsigned* refused,
                                                 R& gfin) {
  const R sig = ch_pick<R>(c.vnT, c.f.vnT);
  const R vn0x = ch_pick<R>(c.vn0[0], c.f.vn0[0]), vn0y = ch_pick<R>(c.vn0[1], c.f.vn0[1]),
          vn0z = ch_pick<R>(c.vn0[2], c.f.vn0[2]);
  const R m1 = ch_pick<R>(c.m1, c.f.m1);
  const R vix = v[0], viy = v[1], viz = v[2];
  const R wx = vix - vn0x, wy = viy - vn0y, wz = viz - vn0z;
  const R w = ch_qsqrt(wx * wx + wy * wy + wz * wz);
  const U4 a = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8) | (1 + 2 * it), c.run, c.seed_lo, c.seed_hi);
  const U4 b = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8) | (2 + 2 * it), c.run, c.seed_lo, c.seed_hi);
  // The two proposals of ch_collide, written so that the lanes of a warp
  // that take different ones share a radius, one logarithm and the sine /
  // cosine of b.x (the same draws, the same formulas):
  //   Maxwellian: r = sig sqrt(-2 ln a.y), (cos, sin)(2 pi a.z) in x, y;
  //               z = sig sqrt(-2 ln a.w) cos(2 pi b.x);
  //   speed-weighted: r = sig sqrt(-2 ln(a.y a.z)), polar cosine 2 a.w - 1,
  //               azimuth 2 pi b.x.
  const bool maxw = unitR<R>(a.x) * (w + m1) < w;
  const R ua = unitR<R>(a.y), ub = unitR<R>(a.z);
  const R r = sig * ch_qsqrt(R(-2) * ch_log(maxw ? ua : ua * ub));
  R sb, cb;
  ch_sincos2pi(unitR<R>(b.x), &sb, &cb);
  R nx, ny, nz;
  if (maxw) {
    R s1, c1;
    ch_sincos2pi(ub, &s1, &c1);
    nx = r * c1; ny = r * s1;
    nz = sig * ch_qsqrt(R(-2) * ch_log(unitR<R>(a.w))) * cb;
  } else {
    const R ct = R(2) * unitR<R>(a.w) - R(1);
    R st = R(1) - ct * ct;
    st = ch_qsqrt(st > R(0) ? st : R(0));
    nx = r * st * cb; ny = r * st * sb; nz = r * ct;
  }
  const R Vx = vn0x + nx, Vy = vn0y + ny, Vz = vn0z + nz;
  const R dV = ch_qsqrt(nx * nx + ny * ny + nz * nz);
  const R rx = vix - Vx, ry = viy - Vy, rz = viz - Vz;
  const R D = ch_qsqrt(rx * rx + ry * ry + rz * rz);
  const bool accept = unitR<R>(b.y) * (w + dV) < D;
  if (!accept && it + 1 < 64) {
    ++it;
    return false;
  }
  if (accept) {
    // centre-of-mass scatter (src/particles.c:552-591)
    const R uz = R(2) * unitR<R>(b.z) - R(1);
    const R vrr = D;
    const R wi = ch_pick<R>(c.mi / (c.mi + c.mn), c.f.wi), wn = ch_pick<R>(c.mn / (c.mi + c.mn), c.f.wn);
    const R vcx = vix * wi + Vx * wn, vcy = viy * wi + Vy * wn, vcz = viz * wi + Vz * wn;
    const R vcr = wn * vrr;  // v - v_cm = wn (v - V)
    R up = R(1) - uz * uz;
    const R uperp = ch_qsqrt(up > R(0) ? up : R(0));
    R sph, cph;
    ch_sincos2pi(unitR<R>(b.w), &sph, &cph);
    const R ux = uperp * cph, uy = uperp * sph;
    const R costht = vrr > R(0) ? ch_qdiv(rz, vrr) : R(1);
    R st2 = R(1) - costht * costht;
    const R sintht = ch_qsqrt(st2 > R(0) ? st2 : R(0));
    R cosphi = R(1), sinphi = R(0);
    if (vrr * sintht > R(0)) {
      const R inv = ch_qdiv(R(1), vrr * sintht);
      cosphi = rx * inv;
      sinphi = ry * inv;
    }
    const R ux1 = uz * sintht + ux * costht, uy1 = uy, uz1 = uz * costht - ux * sintht;
    const R ux2 = ux1 * cosphi - uy1 * sinphi, uy2 = ux1 * sinphi + uy1 * cosphi, uz2 = uz1;
    const R vfx = vcx + vcr * ux2, vfy = vcy + vcr * uy2, vfz = vcz + vcr * uz2;
    if (vfx * vfx + vfy * vfy + vfz * vfz > ch_pick<R>(R(100) * c.viTr * c.viTr, c.f.vlim2)) {
      ++*refused;  // src/particles.c:597-606
    } else {
      v[0] = vfx; v[1] = vfy; v[2] = vfz;
      ++*ncol;
    }
  } else {
    ++*refused;  // 64 proposals without acceptance
  }
  // the next event's waiting time
  ++e;
  it = 0;
  gfin = ch_gmean<R>(ch_relspeed<R>(v[0], v[1], v[2], vn0x, vn0y, vn0z), sig);
  if (e >= CH_MAX_EVENTS) return true;
  const R lam = lscale * gfin;
  if (!(lam > R(0))) return true;
  const U4 r0 = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8), c.run, c.seed_lo, c.seed_hi);
  t += ch_qdiv(-ch_log(unitR<R>(r0.x)), lam);
  return !(t < R(1));
}

