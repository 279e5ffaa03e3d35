// su2_kernels.cuh -- device kernels of the checkerboard update sweep, the
// measurement reductions and the gradient flow, templated on the field
// precision R (double: plain FP64 path, float: precision form with FP64
// reductions) and on the field content CC (a compile-time content mask, or
// C_GENERIC to read it at run time).
//
// One thread owns one site of the parity being updated.  Sites of one parity
// never read each other's updated field (checkerboard), so a half-sweep is
// one launch, exactly as the reference's sequential site loop over that
// parity (update.c:35-259).
#pragma once

#include "su2_common.cuh"

namespace su2 {

#define HAS(bit) SU2_HAS(CC, cp.content, bit)
#define NHIGGS (HAS(C_H2) ? 2 : (HAS(C_H1) ? 1 : 0))

constexpr int BLOCK = 128;
// resident blocks per SM asked of the compiler: 8 x 128 threads caps FP32
// kernels at 64 registers (half occupancy); FP64 ones at 128
template <typename R>
struct MinBlocks {
  static constexpr int value = sizeof(R) == 4 ? 8 : 4;
};

// launch shapes of the update kernels the autotuner chooses from:
// (threads per block, resident blocks per SM asked of the compiler, which
// sets the register budget: 65536 / (threads * blocks))
constexpr int NVARIANTS = 4;
template <typename R, int V>
struct Variant;
template <typename R> struct Variant<R, 0> { static constexpr int BS = 128, MINB = sizeof(R) == 4 ? 8 : 4; };
template <typename R> struct Variant<R, 1> { static constexpr int BS = 128, MINB = sizeof(R) == 4 ? 5 : 3; };
template <typename R> struct Variant<R, 2> { static constexpr int BS = 256, MINB = sizeof(R) == 4 ? 4 : 2; };
template <typename R> struct Variant<R, 3> { static constexpr int BS = 64, MINB = sizeof(R) == 4 ? 12 : 6; };
// threads per block of each variant, for host code that builds tile tables
constexpr int kVariantBS[NVARIANTS] = {128, 128, 256, 64};
constexpr int NSUMS = 24;

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ inline void warp_count(unsigned long long* ctr, int v) {
  // every lane of the warp reaches this call (no early returns in kernels)
  int s = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(ctr, (unsigned long long)s);
}

// sum of v over the block, result valid in thread 0; blockDim.x <= 1024
__device__ inline double block_sum(double v) {
  __shared__ double sm[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sm[w] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  if (w == 0) {
    v = lane < nw ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// ---------------------------------------------------------------------------
// SU(2) gauge part
// ---------------------------------------------------------------------------
// su2staple_wilson (staples.c:84-115)
template <typename R>
__device__ inline Q<R> wilson_staple(const Fields<R>& f, const Geom& g, const int* c, int i, int mu) {
  Q<R> tot{(R)0, (R)0, (R)0, (R)0};
  int xp = shifted(g, c, mu, 1);
#pragma unroll
  for (int nu = 0; nu < 3; nu++) {
    if (nu == mu) continue;
    int xn = shifted(g, c, nu, 1);
    int xpm = shifted(g, c, mu, 1, nu, -1);
    int xm = shifted(g, c, nu, -1);
    Q<R> up = qmul(qmul(ldro4<R>(lk(f, nu), xp), qdag(ldro4<R>(lk(f, mu), xn))), qdag(ldro4<R>(lk(f, nu), i)));
    tot = qadd(tot, up);
    Q<R> lo = qmul(qmul(qdag(ldro4<R>(lk(f, nu), xpm)), qdag(ldro4<R>(lk(f, mu), xm))), ldro4<R>(lk(f, nu), xm));
    tot = qadd(tot, lo);
  }
  return tot;
}

// hopping_triplet_forward (su2u1.c:605-617): -Sigma(x) . R(U_mu(x)) Sigma(x+mu)
template <typename R>
__device__ inline R hop_triplet_fwd_u(const Fields<R>& f, const Geom& g, const int* c, int i, int mu,
                                      const Q<R>& U) {
  V3<R> r = qrot(U, ldro3(f, shifted(g, c, mu, 1)));
  return -dot3(ld3(f, i), r);
}

// su2link_staple (staples.c:134-193)
template <typename R, int CC>
__device__ inline Q<R> link_staple(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                   int mu) {
  Q<R> V = qscale(wilson_staple(f, g, c, i, mu), (R)-0.5 * cp.beta);
  const int nh = NHIGGS;
  if (nh > 0) {
    int xp = shifted(g, c, mu, 1);
    for (int h = 0; h < nh; h++) {
      Q<R> nphi = ldro4<R>(php(f, h), xp);
      if (HAS(C_U1)) nphi = qmul(nphi, u1phase(a1p(f, mu)[i]));
      Q<R> t = qmul(nphi, qdag(ldro4<R>(php(f, h), i)));
      V.a -= (R)0.5 * t.a;
      V.b -= (R)0.5 * t.b;
      V.c -= (R)0.5 * t.c;
      V.d -= (R)0.5 * t.d;
    }
  }
  return V;
}

// su2ptrace (su2u1.c:108-116) at site x (index i, coords c)
template <typename R>
__device__ inline R ptrace(const Fields<R>& f, const Geom& g, const int* c, int i, int mu, int nu) {
  Q<R> s = qmul(qmul(ld4<R>(lk(f, mu), i), ld4<R>(lk(f, nu), shifted(g, c, mu, 1))),
                qdag(ld4<R>(lk(f, mu), shifted(g, c, nu, 1))));
  return (R)2 * qdot0(s, qdag(ld4<R>(lk(f, nu), i)));
}

// ---------------------------------------------------------------------------
// doublet
// ---------------------------------------------------------------------------
template <typename R>
__device__ inline R doubletsq(const Q<R>& a) {
  return (R)0.5 * (a.a * a.a + a.b * a.b + a.c * a.c + a.d * a.d);
}
template <typename R>
__device__ inline R tripletsq(const V3<R>& a) {
  return (R)0.5 * (a.x * a.x + a.y * a.y + a.z * a.z);
}

// hopping_trace(_su2u1) (su2u1.c:388-418): Re Tr Phi1^+ U Phi2 e^{-i a s3}
template <typename R, int CC>
__device__ inline R hop_trace(const CoupT<R>& cp, const Q<R>& p1, const Q<R>& u, const Q<R>& p2, R alpha) {
  Q<R> t = qmul(u, p2);
  if (HAS(C_U1)) t = qmul(t, u1phase(alpha));
  return qdot0(qdag(p1), t);
}
template <typename R, int CC>
__device__ inline R hop_doublet_fwd(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                    int mu, int h) {
  R al = HAS(C_U1) ? a1p(f, mu)[i] : (R)0;
  return -hop_trace<R, CC>(cp, ld4<R>(php(f, h), i), ld4<R>(lk(f, mu), i), ld4<R>(php(f, h), shifted(g, c, mu, 1)), al);
}
template <typename R, int CC>
__device__ inline R hop_doublet_bwd(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                    int mu, int h) {
  int pm = shifted(g, c, mu, -1);
  R al = HAS(C_U1) ? a1p(f, mu)[pm] : (R)0;
  return -hop_trace<R, CC>(cp, ld4<R>(php(f, h), pm), ld4<R>(lk(f, mu), pm), ld4<R>(php(f, h), i), al);
}
template <typename R, int CC>
__device__ inline R covariant_doublet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                      int h) {
  R tot = 0, mod = doubletsq(ld4<R>(php(f, h), i));
#pragma unroll
  for (int d = 0; d < 3; d++) tot += (R)2 * mod + hop_doublet_fwd<R, CC>(f, g, cp, c, i, d, h);
  return tot;
}

// potential_singlet (su2u1.c:708-723)
template <typename R, int CC>
__device__ inline R potential_singlet(const Fields<R>& f, const CoupT<R>& cp, int i) {
  R S = f.sing[i];
  R pot = (R)cp.b1s * S + (R)0.5 * (R)cp.msqs * S * S + (R)(1.0 / 3.0) * (R)cp.b3s * S * S * S +
          (R)0.25 * (R)cp.b4s * S * S * S * S;
  if (NHIGGS == 1) {
    R mod = doubletsq(ld4<R>(php(f, 0), i));
    pot += (R)0.5 * (R)cp.a1s * S * mod + (R)0.5 * (R)cp.a2s * S * S * mod;
  }
  return pot;
}

// higgspotential (su2u1.c:528-572)
template <typename R, int CC>
__device__ inline R higgspotential(const Fields<R>& f, const CoupT<R>& cp, int i) {
  R pot = 0, mod = 0;
  const int nh = NHIGGS;
  if (nh > 0) {
    Q<R> h1 = ld4<R>(php(f, 0), i);
    mod = doubletsq(h1);
    pot += (R)cp.msq * mod + (R)cp.lam * mod * mod;
    if (nh == 2) {
      Q<R> h2 = ld4<R>(php(f, 1), i);
      R f11 = mod, f22 = doubletsq(h2);
      R Re = (R)0.5 * (h1.a * h2.a + h1.b * h2.b + h1.c * h2.c + h1.d * h2.d);
      R Im = (R)0.5 * (h1.d * h2.a + h1.c * h2.b - h1.b * h2.c - h1.a * h2.d);
      pot += (R)cp.msq2 * f22 + (R)cp.m12re * Re - (R)cp.m12im * Im + (R)cp.lam2 * f22 * f22 +
             (R)cp.lam3 * f11 * f22 + (R)cp.lam4 * (Re * Re + Im * Im) + (R)cp.lam5re * (Re * Re - Im * Im) -
             (R)2 * (R)cp.lam5im * Re * Im + f11 * ((R)cp.lam6re * Re - (R)cp.lam6im * Im) +
             f22 * ((R)cp.lam7re * Re + (R)cp.lam7im * Im);
    }
  }
  if (HAS(C_T)) {
    R mt = tripletsq(ld3(f, i));
    pot += (R)cp.msqT * mt + (R)cp.b4 * mt * mt;
    if (nh > 0) pot += (R)cp.a2 * mod * mt;
  }
  if (HAS(C_S)) pot += potential_singlet<R, CC>(f, cp, i);
  return pot;
}

// localact_doublet (su2u1.c:495-510)
template <typename R, int CC>
__device__ inline R localact_doublet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                     int h) {
  R tot = covariant_doublet<R, CC>(f, g, cp, c, i, h);
#pragma unroll
  for (int d = 0; d < 3; d++) tot += hop_doublet_bwd<R, CC>(f, g, cp, c, i, d, h);
  tot += higgspotential<R, CC>(f, cp, i);
  return tot;
}

// staple_doublet (staples.c:243-302)
template <typename R, int CC>
__device__ inline Q<R> staple_doublet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                      int h) {
  Q<R> res{(R)0, (R)0, (R)0, (R)0};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    int xp = shifted(g, c, d, 1), xm = shifted(g, c, d, -1);
    Q<R> w = qmul(ldro4<R>(lk(f, d), i), ldro4<R>(php(f, h), xp));
    if (HAS(C_U1)) w = qmul(w, u1phase(a1p(f, d)[i]));
    res.a -= w.a; res.b -= w.b; res.c -= w.c; res.d -= w.d;
    w = qmul(qdag(ldro4<R>(lk(f, d), xm)), ldro4<R>(php(f, h), xm));
    if (HAS(C_U1)) w = qmul(w, qdag(u1phase(a1p(f, d)[xm])));
    res.a -= w.a; res.b -= w.b; res.c -= w.c; res.d -= w.d;
  }
  return res;
}

// ---------------------------------------------------------------------------
// triplet
// ---------------------------------------------------------------------------
template <typename R>
__device__ inline R hop_triplet_fwd(const Fields<R>& f, const Geom& g, const int* c, int i, int mu) {
  return hop_triplet_fwd_u(f, g, c, i, mu, ld4<R>(lk(f, mu), i));
}
template <typename R>
__device__ inline R covariant_triplet(const Fields<R>& f, const Geom& g, const int* c, int i) {
  R tot = 0, mod = tripletsq(ld3(f, i));
#pragma unroll
  for (int d = 0; d < 3; d++) tot += (R)2 * mod + hop_triplet_fwd(f, g, c, i, d);
  return tot;
}

// localact_su2link (su2u1.c:166-198)
template <typename R, int CC>
__device__ inline R localact_su2link(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                     int mu) {
  R tot = 0;
#pragma unroll
  for (int nu = 0; nu < 3; nu++) {
    if (nu == mu) continue;
    tot += ((R)1 - (R)0.5 * ptrace(f, g, c, i, mu, nu));
    int cm[3];
    shift_coords(g, c, nu, -1, cm);
    tot += ((R)1 - (R)0.5 * ptrace(f, g, cm, shifted(g, c, nu, -1), mu, nu));
  }
  tot *= (R)cp.beta;
  for (int h = 0; h < NHIGGS; h++) tot += hop_doublet_fwd<R, CC>(f, g, cp, c, i, mu, h);
  if (HAS(C_T)) tot += hop_triplet_fwd(f, g, c, i, mu);
  return tot;
}

// ---------------------------------------------------------------------------
// U(1)
// ---------------------------------------------------------------------------
template <typename R>
__device__ inline R u1ptrace(const Fields<R>& f, const Geom& g, const int* c, int i, int d1, int d2) {
  return a1p(f, d1)[i] + a1p(f, d2)[shifted(g, c, d1, 1)] - a1p(f, d1)[shifted(g, c, d2, 1)] - a1p(f, d2)[i];
}
// local_u1wilson (su2u1.c:316-328)
template <typename R>
__device__ inline R local_u1wilson(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i) {
  R res = 0;
#pragma unroll
  for (int d1 = 0; d1 < 3; d1++)
#pragma unroll
    for (int d2 = 0; d2 < d1; d2++) res += ((R)1 - mcos((R)cp.r_u1 * u1ptrace(f, g, c, i, d2, d1)));
  return (R)cp.betau1 * res;
}
// localact_u1link (su2u1.c:336-354)
template <typename R, int CC>
__device__ inline R localact_u1link(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                    int mu) {
  R tot = 0;
#pragma unroll
  for (int nu = 0; nu < 3; nu++) {
    if (nu == mu) continue;
    tot += ((R)1 - mcos((R)cp.r_u1 * u1ptrace(f, g, c, i, mu, nu)));
    int cm[3];
    shift_coords(g, c, nu, -1, cm);
    tot += ((R)1 - mcos((R)cp.r_u1 * u1ptrace(f, g, cm, shifted(g, c, nu, -1), mu, nu)));
  }
  tot *= (R)cp.betau1;
  for (int h = 0; h < NHIGGS; h++) tot += hop_doublet_fwd<R, CC>(f, g, cp, c, i, mu, h);
  return tot;
}

// ---------------------------------------------------------------------------
// real root of a x^3 + b x^2 + c x + d (polysolve3, overrelax.c:14-34):
// Cardano's formula followed by Newton steps on the cubic (one in FP64, two
// in FP32).  The reference evaluates Cardano's formula in long double: the
// leading coefficient of these cubics is lambda/4 (~5e-4), so the formula
// cancels, and in double it lands up to ~1e-11 away (relative) from the
// long-double root.  The cubic itself is well conditioned near its root
// (the linear coefficient dominates), so a Newton step brings the double
// result to the root within rounding, matching the reference's long-double
// value to ~1e-15.
// ---------------------------------------------------------------------------
template <typename R>
__device__ inline R polysolve3(R a, R b, R c, R d, int* fallback) {
  R discr = (R)18 * a * b * c * d - (R)4 * b * b * b * d + b * b * c * c - (R)4 * a * c * c * c - (R)27 * a * a * d * d;
  R del1 = (R)2 * b * b * b - (R)9 * a * b * c + (R)27 * a * a * d;
  R x;
  if (discr < (R)0) {
    R A = (R)0.5 * (del1 + a * msqrt((R)(-27) * discr));
    A = mcbrt(A);
    x = -(b + A + (b * b - (R)3 * a * c) / A) / ((R)3 * a);
#pragma unroll
    for (int it = 0; it < (sizeof(R) == 4 ? 2 : 1); it++) {
      R fx = ((a * x + b) * x + c) * x + d;
      R dfx = ((R)3 * a * x + (R)2 * b) * x + c;
      x -= fx / dfx;
    }
  } else {
    x = b / a;
    *fallback = 1;
  }
  return x;
}

// ---------------------------------------------------------------------------
// local updates.  The overrelaxation updates take their random-number source
// as a template parameter: the sweep kernels pass the site's stream
// (SiteRng), the per-site verification kernel ZeroRng, whose uniforms are
// all 0, so that every proposal is accepted and can be read back.
// ---------------------------------------------------------------------------
template <typename R>
struct ZeroRng {
  __device__ R uni() { return (R)0; }
};
// heatbath_su2link (heatbath.c:15-124): Kennedy-Pendleton; the uniforms are
// drawn in the reference's order (4 per trial, 3 per sphere trial, 1 for the
// triplet accept/reject).  The first trial's four are drawn before the staple
// is gathered: the same values in the same order (each site's stream is
// positional), with the generator's arithmetic free to run while the loads
// are in flight.  The other local updates draw early in the same way.
template <typename R, int CC>
__device__ inline int heatbath(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i, int mu,
                               SiteRng<R>& rng, int* kpcap, int* err) {
  R u0 = rng.uni(), u1 = rng.uni(), u2 = rng.uni(), u3 = rng.uni();  // the first trial's
  Q<R> old{};
  R oldact = 0;
  if (HAS(C_T)) {
    old = ld4<R>(lk(f, mu), i);
    oldact = hop_triplet_fwd_u(f, g, c, i, mu, old);
  }
  Q<R> V = link_staple<R, CC>(f, g, cp, c, i, mu);
  R a = msqrt(qsq(V));
  V = qscale(V, (R)-1 / a);
  a *= (R)2;
  R a0, r1, r2, r3, d;
  int loop = 1;
  do {
    if (loop > 1) {
      u0 = rng.uni();
      u1 = rng.uni();
      u2 = rng.uni();
      u3 = rng.uni();
    }
    r1 = -mlog((R)1 - u0) / a;
    r2 = -mlog((R)1 - u1) / a;
    r3 = mcos2pi(u2);
    r3 *= r3;
    d = r1 * r3 + r2;
    r3 = (R)1 - u3;
    loop++;
  } while (r3 * r3 > (R)1 - (R)0.5 * d && loop <= 200);
  R rad;
  if (loop > 200) {
    a0 = (R)1e-9;
    *kpcap = 1;
    rad = (R)1 - a0 * a0;
  } else {
    a0 = (R)1 - d;
    // FP32: 1 - a0^2 = d (2 - d) without the cancellation near a0 = 1
    rad = sizeof(R) == 8 ? (R)1 - a0 * a0 : d * ((R)2 - d);
  }
  if (rad < (R)0) return 0;
  rad = msqrt(rad);
  Q<R> nl;
  if constexpr (sizeof(R) == 8) {
    // uniform direction on S^2 by rejection from the cube (heatbath.c:82-93)
    d = 2;
    int it = 0;
    while (d > (R)1 || d == (R)0) {
      r1 = (R)2 * rng.uni() - (R)1;
      r2 = (R)2 * rng.uni() - (R)1;
      r3 = (R)2 * rng.uni() - (R)1;
      d = r1 * r1 + r2 * r2 + r3 * r3;
      if (++it > 4096) {  // probability (1 - pi/6)^4096: never; guards a NaN state
        *err = 1;
        return 0;
      }
    }
    d = msqrt(d);
    nl = Q<R>{a0, r1 * (rad / d), r2 * (rad / d), r3 * (rad / d)};
  } else {
    // FP32 form: the same uniform direction drawn directly (Archimedes:
    // cos(theta) uniform on [-1,1], azimuth uniform), no rejection loop to
    // diverge a warp
    float z = 2.0f * rng.uni() - 1.0f;
    float ph = rng.uni();
    float sn, cs;
    sincospif(2.0f * ph, &sn, &cs);
    float s = sqrtf(fmaxf(0.0f, 1.0f - z * z)) * rad;
    nl = Q<R>{a0, s * cs, s * sn, z * rad};
  }
  Q<R> U = unitize(qmul(nl, qdag(V)));
  st4<R>(lk(f, mu), i, U);
  if (HAS(C_T)) {
    R diff = oldact - hop_triplet_fwd_u(f, g, c, i, mu, U);
    if (rng.uni() < mexp(diff)) return 1;
    st4<R>(lk(f, mu), i, old);
    return 0;
  }
  return 1;
}

// FP32 form: every link written is re-normalised to unit length, so rounding
// never accumulates in the SU(2) constraint (the FP64 path writes the
// reference's arithmetic unchanged)
template <typename R>
__device__ inline Q<R> unitize(const Q<R>& q) {
  if (sizeof(R) == 8) return q;
  return qscale(q, (R)rsqrtf((float)qsq(q)));
}

// Metropolis decision (metropolis.c:15-167)
template <typename R>
__device__ inline int metro_accept(R diff, SiteRng<R>& rng) {
  if (diff < (R)0) return 1;
  if (diff > (R)0 && mexp(-diff) > rng.uni()) return 1;
  return 0;
}
// the same with the decision's uniform u drawn beforehand (it is the site's
// last draw of the pass, so drawing it whatever diff turns out to be changes
// no other draw)
template <typename R>
__device__ inline int metro_accept_u(R diff, R u) {
  if (diff < (R)0) return 1;
  if (diff > (R)0 && mexp(-diff) > u) return 1;
  return 0;
}

// metro_su2link (metropolis.c:15-41) with random_su2link (init.c:43-58)
template <typename R, int CC>
__device__ inline int metro_link(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i, int mu,
                                 SiteRng<R>& rng) {
  Q<R> old = ld4<R>(lk(f, mu), i);
  R a0 = localact_su2link<R, CC>(f, g, cp, c, i, mu);
  Q<R> u;
  u.a = (R)10 * (rng.uni() - (R)0.5);
  u.b = (R)1 * (rng.uni() - (R)0.5);
  u.c = (R)1 * (rng.uni() - (R)0.5);
  u.d = (R)1 * (rng.uni() - (R)0.5);
  R n = msqrt(u.a * u.a + u.b * u.b + u.c * u.c + u.d * u.d);
  u = Q<R>{u.a / n, u.b / n, u.c / n, u.d / n};
  st4<R>(lk(f, mu), i, unitize(qmul(old, u)));
  R a1 = localact_su2link<R, CC>(f, g, cp, c, i, mu);
  if (metro_accept(a1 - a0, rng)) return 1;
  st4<R>(lk(f, mu), i, old);
  return 0;
}

// metro_u1link (metropolis.c:48-70)
template <typename R, int CC>
__device__ inline int metro_u1(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i, int mu,
                               SiteRng<R>& rng) {
  R old = a1p(f, mu)[i];
  R a0 = localact_u1link<R, CC>(f, g, cp, c, i, mu);
  a1p(f, mu)[i] = old + (R)0.95 * (rng.uni() - (R)0.5);
  R a1 = localact_u1link<R, CC>(f, g, cp, c, i, mu);
  if (metro_accept(a1 - a0, rng)) return 1;
  a1p(f, mu)[i] = old;
  return 0;
}

// metro_doublet (metropolis.c:77-106)
template <typename R, int CC>
__device__ inline int metro_doublet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                    int h, SiteRng<R>& rng) {
  const R d0 = rng.uni() - (R)0.5, d1 = rng.uni() - (R)0.5, d2 = rng.uni() - (R)0.5, d3 = rng.uni() - (R)0.5;
  Q<R> old = ld4<R>(php(f, h), i);
  R a0 = localact_doublet<R, CC>(f, g, cp, c, i, h);
  Q<R> nw = old;
  nw.a += (R)1 * d0;
  nw.b += (R)1 * d1;
  nw.c += (R)1 * d2;
  nw.d += (R)1 * d3;
  st4<R>(php(f, h), i, nw);
  R a1 = localact_doublet<R, CC>(f, g, cp, c, i, h);
  if (metro_accept(a1 - a0, rng)) return 1;
  st4<R>(php(f, h), i, old);
  return 0;
}

// overrelax_doublet (overrelax.c:54-128)
template <typename R, int CC, typename RNG>
__device__ inline int overrelax_doublet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                        RNG& rng, int* fallback) {
  const R u = rng.uni();
  Q<R> s = staple_doublet<R, CC>(f, g, cp, c, i, 0);
  Q<R> p = ld4<R>(php(f, 0), i);
  R F = msqrt(s.a * s.a + s.b * s.b + s.c * s.c + s.d * s.d);
  // FP32: one reciprocal instead of nine divisions (the FP64 path divides as
  // the reference does)
  const bool f32 = sizeof(R) == 4;
  const R iF = f32 ? (R)1 / F : (R)0;
  R X = f32 ? (p.a * s.a + p.b * s.b + p.c * s.c + p.d * s.d) * iF : (p.a * s.a + p.b * s.b + p.c * s.c + p.d * s.d) / F;
  R y0 = f32 ? p.a - X * s.a * iF : p.a - X * s.a / F;
  R y1 = f32 ? p.b - X * s.b * iF : p.b - X * s.b / F;
  R y2 = f32 ? p.c - X * s.c * iF : p.c - X * s.c / F;
  R y3 = f32 ? p.d - X * s.d * iF : p.d - X * s.d / F;
  R Ysq = y0 * y0 + y1 * y1 + y2 * y2 + y3 * y3;
  R B = (R)0.5 * (R)cp.msq + (R)3;
  if (HAS(C_T)) B += (R)0.5 * (R)cp.a2 * tripletsq(ld3(f, i));
  if (HAS(C_S)) {
    R S = f.sing[i];
    B += (R)0.25 * (R)cp.a1s * S + (R)0.25 * (R)cp.a2s * S * S;
  }
  R C = (R)0.25 * (R)cp.lam;
  R cc = B + (R)2 * Ysq * C;
  R newX = polysolve3<R>(C, C * X, cc + C * X * X, F + cc * X + C * X * X * X, fallback);
  R dV = F + (R)2 * B * X + (R)4 * C * (X * X * X + Ysq * X);
  R dVn = F + (R)2 * B * newX + (R)4 * C * (newX * newX * newX + Ysq * newX);
  if (mabs(dV / dVn) >= u) {
    R k = (newX + X);
    st4<R>(php(f, 0), i, f32 ? Q<R>{-p.a + k * s.a * iF, -p.b + k * s.b * iF, -p.c + k * s.c * iF, -p.d + k * s.d * iF}
                             : Q<R>{-p.a + k * s.a / F, -p.b + k * s.b / F, -p.c + k * s.c / F, -p.d + k * s.d / F});
    return 1;
  }
  return 0;
}

// overrelax_higgs2 (overrelax.c:295-417)
template <typename R, int CC, typename RNG>
__device__ inline int overrelax_higgs2(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                       int h, RNG& rng, int* fallback) {
  const R u = rng.uni();
  Q<R> s = staple_doublet<R, CC>(f, g, cp, c, i, h);
  Q<R> fv = ld4<R>(php(f, h), i);
  Q<R> H;
  R l67re, l67im, lore, loim, lam12, msq;
  int sign;
  if (h == 0) {
    H = ld4<R>(php(f, 1), i);
    sign = -1;
    lam12 = cp.lam; msq = cp.msq;
    l67re = cp.lam7re; l67im = cp.lam7im; lore = cp.lam6re; loim = -cp.lam6im;
  } else {
    H = ld4<R>(php(f, 0), i);
    sign = 1;
    lam12 = cp.lam2; msq = cp.msq2;
    l67re = cp.lam6re; l67im = -cp.lam6im; lore = cp.lam7re; loim = cp.lam7im;
  }
  R Hv[4] = {H.a, H.b, H.c, H.d};
  R G[4] = {sign * Hv[3], sign * Hv[2], -(R)sign * Hv[1], -(R)sign * Hv[0]};
  R Hsq = doubletsq(H);
  R sv[4] = {s.a, s.b, s.c, s.d}, fr[4] = {fv.a, fv.b, fv.c, fv.d};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    sv[k] += (R)0.5 * ((R)cp.m12re + Hsq * l67re) * Hv[k];
    sv[k] += (R)0.5 * (-(R)cp.m12im + Hsq * l67im) * G[k];
    sv[k] = -sv[k];
  }
  R F = msqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2] + sv[3] * sv[3]);
  R X = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) { sv[k] /= F; X += fr[k] * sv[k]; }
  R Y[4], Ysq = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) { Y[k] = fr[k] - X * sv[k]; Ysq += Y[k] * Y[k]; }
  R Hf = 0, Gf = 0, HY = 0, GY = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) { Hf += Hv[k] * sv[k]; Gf += G[k] * sv[k]; HY += Hv[k] * Y[k]; GY += G[k] * Y[k]; }
  R b4 = (R)0.25 * lam12;
  R b3 = (R)0.25 * (Hf * lore + Gf * loim);
  R b2 = (R)0.5 * msq + (R)3 + (R)0.5 * Ysq * lam12 + (R)0.25 * (HY * lore + GY * loim);
  R b1 = -F + (R)0.25 * Ysq * (Hf * lore + Gf * loim);
  b2 += (R)0.5 * Hsq * (R)cp.lam3 + (R)0.25 * (R)cp.lam4 * (Hf * Hf + Gf * Gf) +
        (R)0.25 * (R)cp.lam5re * (Hf * Hf - Gf * Gf) - (R)0.5 * (R)cp.lam5im * Gf * Hf;
  b1 += (R)0.5 * Hf * (HY * (R)cp.lam4 + HY * (R)cp.lam5re - GY * (R)cp.lam5im) +
        (R)0.5 * Gf * (GY * (R)cp.lam4 - GY * (R)cp.lam5re - HY * (R)cp.lam5im);
  R Xn = polysolve3<R>(b4, b3 + b4 * X, b2 + b3 * X + b4 * X * X, b1 + b2 * X + b3 * X * X + b4 * X * X * X, fallback);
  R dV = (R)4 * b4 * X * X * X + (R)3 * b3 * X * X + (R)2 * b2 * X + b1;
  R dVn = (R)4 * b4 * Xn * Xn * Xn + (R)3 * b3 * Xn * Xn + (R)2 * b2 * Xn + b1;
  if (mabs(dV / dVn) >= u) {
    st4<R>(php(f, h), i, Q<R>{fr[0] + sv[0] * (Xn - X), fr[1] + sv[1] * (Xn - X), fr[2] + sv[2] * (Xn - X),
                             fr[3] + sv[3] * (Xn - X)});
    return 1;
  }
  return 0;
}

// overrelax_triplet (overrelax.c:137-236); no portal term in B (the
// reference's "#ifdef HIGGS" there is never defined)
// The triplet's staple s = -sum_d [R(U_d(x)) t(x+d) + R(U_d(x-d))^T t(x-d)]:
// with it the local action (localact_triplet, su2u1.c:657-679) is
// t.s + B t^2 + C t^4 (+ the portal a2 phi^2 t^2 / 2), B = 3 + msqT / 2,
// C = b4 / 4, the form overrelax.c:137-236 works with.
template <typename R>
__device__ inline V3<R> staple_triplet(const Fields<R>& f, const Geom& g, const int* c, int i) {
  V3<R> s{(R)0, (R)0, (R)0};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    int xp = shifted(g, c, d, 1), xm = shifted(g, c, d, -1);
    V3<R> r = qrot(ldro4<R>(lk(f, d), i), ldro3(f, xp));
    s.x -= r.x; s.y -= r.y; s.z -= r.z;
    r = qrot(qdag(ldro4<R>(lk(f, d), xm)), ldro3(f, xm));
    s.x -= r.x; s.y -= r.y; s.z -= r.z;
  }
  return s;
}

template <typename R, int CC, typename RNG>
__device__ inline int overrelax_triplet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                        RNG& rng, int* fallback) {
  const R u = rng.uni();
  V3<R> s = staple_triplet(f, g, c, i);
  V3<R> t = ld3(f, i);
  R F = msqrt(s.x * s.x + s.y * s.y + s.z * s.z);
  // FP32: one reciprocal instead of seven divisions (the FP64 path divides as
  // the reference does)
  const bool f32 = sizeof(R) == 4;
  const R iF = f32 ? (R)1 / F : (R)0;
  R X = f32 ? (t.x * s.x + t.y * s.y + t.z * s.z) * iF : (t.x * s.x + t.y * s.y + t.z * s.z) / F;
  R y0 = f32 ? t.x - X * s.x * iF : t.x - X * s.x / F;
  R y1 = f32 ? t.y - X * s.y * iF : t.y - X * s.y / F;
  R y2 = f32 ? t.z - X * s.z * iF : t.z - X * s.z / F;
  R Ysq = y0 * y0 + y1 * y1 + y2 * y2;
  R B = (R)0.5 * (R)cp.msqT + (R)3;
  R C = (R)0.25 * (R)cp.b4;
  R cc = B + (R)2 * Ysq * C;
  R newX = polysolve3<R>(C, C * X, cc + C * X * X, F + cc * X + C * X * X * X, fallback);
  R dV = F + (R)2 * B * X + (R)4 * C * (X * X * X + Ysq * X);
  R dVn = F + (R)2 * B * newX + (R)4 * C * (newX * newX * newX + Ysq * newX);
  if (mabs(dV / dVn) >= u) {
    R k = newX + X;
    st3(f, i, f32 ? V3<R>{-t.x + k * s.x * iF, -t.y + k * s.y * iF, -t.z + k * s.z * iF}
                  : V3<R>{-t.x + k * s.x / F, -t.y + k * s.y / F, -t.z + k * s.z / F});
    return 1;
  }
  return 0;
}

// metro_triplet (metropolis.c:113-143).  The reference evaluates
// localact_triplet before and after the change; in their difference every
// term but t.s and the powers of t^2 cancels, so it is formed directly from
// the staple: dS = (t'-t).s + (t'^2-t^2) (B + C (t'^2+t^2)) (+ portal).  One
// gather of the neighbours instead of two, the field written only on accept.
template <typename R, int CC>
__device__ inline int metro_triplet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                    SiteRng<R>& rng) {
  const R e0 = rng.uni() - (R)0.5, e1 = rng.uni() - (R)0.5, e2 = rng.uni() - (R)0.5;
  // FP32: the decision's uniform is the fourth word of the same generator
  // block, drawn with the proposal; FP64 draws it only when it is needed
  const R ua = sizeof(R) == 4 ? rng.uni() : (R)0;
  V3<R> s = staple_triplet(f, g, c, i);
  V3<R> old = ld3(f, i);
  V3<R> nw = old;
  nw.x += (R)1 * e0;
  nw.y += (R)1 * e1;
  nw.z += (R)1 * e2;
  const R dx = nw.x - old.x, dy = nw.y - old.y, dz = nw.z - old.z;
  const R dsq = dx * (nw.x + old.x) + dy * (nw.y + old.y) + dz * (nw.z + old.z);
  const R ssq = (nw.x * nw.x + nw.y * nw.y + nw.z * nw.z) + (old.x * old.x + old.y * old.y + old.z * old.z);
  R B = (R)0.5 * (R)cp.msqT + (R)3;
  if (NHIGGS > 0) B += (R)0.5 * (R)cp.a2 * doubletsq(ld4<R>(php(f, 0), i));
  const R dS = dx * s.x + dy * s.y + dz * s.z + dsq * (B + (R)0.25 * (R)cp.b4 * ssq);
  if (sizeof(R) == 4 ? metro_accept_u(dS, ua) : metro_accept(dS, rng)) {
    st3(f, i, nw);
    return 1;
  }
  return 0;
}

// localact_singlet (su2u1.c:688-705)
template <typename R, int CC>
__device__ inline R localact_singlet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i) {
  R S = f.sing[i], res = (R)3 * S * S;
#pragma unroll
  for (int d = 0; d < 3; d++) res -= S * (f.sing[shifted(g, c, d, 1)] + f.sing[shifted(g, c, d, -1)]);
  res += potential_singlet<R, CC>(f, cp, i);
  return res;
}

// overrelax_singlet (overrelax.c:243-285)
template <typename R, int CC, typename RNG>
__device__ inline int overrelax_singlet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                        RNG& rng, int* fallback) {
  const R u = rng.uni();
  R S = f.sing[i];
  R c1 = (R)cp.b1s;
#pragma unroll
  for (int d = 0; d < 3; d++) c1 -= (f.sing[shifted(g, c, d, 1)] + f.sing[shifted(g, c, d, -1)]);
  R c2 = (R)3 + (R)0.5 * (R)cp.msqs;
  R c3 = (R)(1.0 / 3.0) * (R)cp.b3s;
  R c4 = (R)0.25 * (R)cp.b4s;
  if (NHIGGS == 1) {
    R phisq = doubletsq(ld4<R>(php(f, 0), i));
    c1 += (R)0.5 * (R)cp.a1s * phisq;
    c2 += (R)0.5 * (R)cp.a2s * phisq;
  }
  R d0 = c1 + c2 * S + c3 * S * S + c4 * S * S * S;
  R d1 = c2 + c3 * S + c4 * S * S;
  R d2 = c3 + c4 * S;
  R Y = polysolve3<R>(c4, d2, d1, d0, fallback);
  R dV = c1 + (R)2 * c2 * S + (R)3 * c3 * S * S + (R)4 * c4 * S * S * S;
  R dVn = c1 + (R)2 * c2 * Y + (R)3 * c3 * Y * Y + (R)4 * c4 * Y * Y * Y;
  if (mabs(dV / dVn) >= u) {
    f.sing[i] = Y;
    return 1;
  }
  return 0;
}

// metro_singlet (metropolis.c:148-167)
template <typename R, int CC>
__device__ inline int metro_singlet(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                    SiteRng<R>& rng) {
  R old = f.sing[i];
  R a0 = localact_singlet<R, CC>(f, g, cp, c, i);
  f.sing[i] = old + (R)1 * (rng.uni() - (R)0.5);
  R a1 = localact_singlet<R, CC>(f, g, cp, c, i);
  if (metro_accept(a1 - a0, rng)) return 1;
  f.sing[i] = old;
  return 0;
}

// order-parameter contribution of one site (calc_orderparam, multicanonical.c:709-751)
template <typename R>
__device__ inline double orderparam_site(const Fields<R>& f, int op, int i) {
  switch (op) {
    case 2: return (double)tripletsq(ld3(f, i));
    case 3: return (double)doubletsq(ld4<R>(php(f, 0), i)) - (double)tripletsq(ld3(f, i));
    case 1: return (double)doubletsq(ld4<R>(php(f, 0), i));
    case 4: return (double)doubletsq(ld4<R>(php(f, 1), i));
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// half-sweep kernels
// ---------------------------------------------------------------------------
struct PassArgs;
__device__ inline void muca_fused_finish(const PassArgs& a, double s);

struct PassArgs {
  Geom g;
  CoupT<double> cpd;  // couplings for FP64 kernels
  CoupT<float> cpf;   // the same for FP32 kernels
  RngKey rk;
  int parity;
  int sub;      // direction for links, doublet index for doublets
  int alg;      // algorithm (links) or forced Metropolis flag (scalars)
  uint32_t pass;
  int t_lo, t_hi;       // site range inside the parity
  void* backup;             // multicanonical backup of the updated field (or null)
  int op;                   // order parameter to reduce (0: none)
  double* partials;         // per-block order-parameter sums (or null)
  unsigned long long* ctr;  // device counters
  int* err;                 // device error flag
  // the multicanonical check decided inside the pass (muca_fused_finish):
  // the weight (null: no decision in this launch), arrival counters, the
  // check's number and the volume the order parameter is divided by
  MucaDev* muca;
  unsigned* arrive;
  uint32_t check;
  double vol;
};

template <typename R>
__device__ inline const CoupT<R>& coup(const PassArgs& a);
template <>
__device__ inline const CoupT<double>& coup<double>(const PassArgs& a) { return a.cpd; }
template <>
__device__ inline const CoupT<float>& coup<float>(const PassArgs& a) { return a.cpf; }

// MU: the link direction of the pass, a template parameter so that every
// neighbour offset and field pointer of the staple is fixed at compile time
template <typename R, int CC, int MU, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_link(Fields<R> f, PassArgs a) {
  const CoupT<R>& cp = coup<R>(a);
  int t = a.t_lo + (int)blockIdx.x * blockDim.x + threadIdx.x;
  int acc = 0, cap = 0, err = 0;
  if (t < a.t_hi) {
    int c[3];
    site_coords(a.g, a.parity, t, c);
    int i = a.parity * a.g.half + t;
    SiteRng<R> rng(a.rk, *a.rk.sweep, (uint32_t)i, a.pass);
    if (a.alg == ALG_HEATBATH) acc = heatbath<R, CC>(f, a.g, cp, c, i, MU, rng, &cap, &err);
    else acc = metro_link<R, CC>(f, a.g, cp, c, i, MU, rng);
  }
  warp_count(a.ctr + 1, acc);
  warp_count(a.ctr + 22, cap);
  if (err) atomicOr(a.err, 1);
}

template <typename R, int CC, int MU, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_u1(Fields<R> f, PassArgs a) {
  const CoupT<R>& cp = coup<R>(a);
  int t = a.t_lo + (int)blockIdx.x * blockDim.x + threadIdx.x;
  int acc = 0;
  if (t < a.t_hi) {
    int c[3];
    site_coords(a.g, a.parity, t, c);
    int i = a.parity * a.g.half + t;
    SiteRng<R> rng(a.rk, *a.rk.sweep, (uint32_t)i, a.pass);
    acc = metro_u1<R, CC>(f, a.g, cp, c, i, MU, rng);
  }
  warp_count(a.ctr + 3, acc);
}

// one parity (or a contiguous block of it) of one doublet / the triplet /
// the singlet; optional multicanonical backup of the old values and block
// sums of the order parameter over the new ones
template <typename R, int CC, int FIELD, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_scalar(Fields<R> f, PassArgs a) {
  const CoupT<R>& cp = coup<R>(a);
  int t = a.t_lo + (int)blockIdx.x * blockDim.x + threadIdx.x;
  int acc = 0, fb = 0;
  double opv = 0.0;
  bool orr = false;
  if (t < a.t_hi) {
    int c[3];
    site_coords(a.g, a.parity, t, c);
    int i = a.parity * a.g.half + t;
    SiteRng<R> rng(a.rk, *a.rk.sweep, (uint32_t)i, a.pass);
    if (FIELD == 0) {
      const int h = a.sub;
      if (a.backup) ((V4<R>*)a.backup)[i] = php(f, h)[i];
      orr = cp.alg_d == ALG_OR && !a.alg;
      if (orr) acc = NHIGGS == 2 ? overrelax_higgs2<R, CC>(f, a.g, cp, c, i, h, rng, &fb)
                                 : overrelax_doublet<R, CC>(f, a.g, cp, c, i, rng, &fb);
      else acc = metro_doublet<R, CC>(f, a.g, cp, c, i, h, rng);
    } else if (FIELD == 1) {
      if (a.backup) {
        R* b = (R*)a.backup;
        b[3 * i] = f.trip[0][i]; b[3 * i + 1] = f.trip[1][i]; b[3 * i + 2] = f.trip[2][i];
      }
      orr = cp.alg_t == ALG_OR && !a.alg;
      if (orr) acc = overrelax_triplet<R, CC>(f, a.g, cp, c, i, rng, &fb);
      else acc = metro_triplet<R, CC>(f, a.g, cp, c, i, rng);
    } else {
      orr = cp.alg_s == ALG_OR && !a.alg;
      if (orr) acc = overrelax_singlet<R, CC>(f, a.g, cp, c, i, rng, &fb);
      else acc = metro_singlet<R, CC>(f, a.g, cp, c, i, rng);
    }
    if (a.partials) opv = orderparam_site<R>(f, a.op, i);
  }
  // counters: doublet OR/Metropolis (+h), triplet, singlet
  int base_or = FIELD == 0 ? 10 + a.sub : (FIELD == 1 ? 15 : 19);
  int base_mt = FIELD == 0 ? 6 + a.sub : (FIELD == 1 ? 13 : 17);
  bool any_or = (FIELD == 0 ? cp.alg_d : (FIELD == 1 ? cp.alg_t : cp.alg_s)) == ALG_OR && !a.alg;
  warp_count(a.ctr + (any_or ? base_or : base_mt), acc);
  warp_count(a.ctr + 23, fb);
  if (a.partials) {
    double s = block_sum(opv);
    if (a.muca) muca_fused_finish(a, s);
    else if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  }
}

// order parameter of a whole parity (calc_orderparam)
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_orderparam(Fields<R> f, Geom g, int parity, int op, double* partials) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < g.half) v = orderparam_site<R>(f, op, parity * g.half + t);
  double s = block_sum(v);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// restore a block of the parity from the backup if the last check rejected
// (a small grid striding over the block: when the check accepted, which is
// the common case, the launch is over as soon as its few blocks have read
// the flag)
template <typename R, int FIELD>
__global__ void k_muca_restore(Fields<R> f, const MucaDev* m, const void* backup, int h, int lo, int hi) {
  if (m->last_accept) return;
  for (int i = lo + (int)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (int)(gridDim.x * blockDim.x)) {
    if (FIELD == 0) {
      php(f, h)[i] = ((const V4<R>*)backup)[i];
    } else {
      const R* b = (const R*)backup;
      f.trip[0][i] = b[3 * i]; f.trip[1][i] = b[3 * i + 1]; f.trip[2][i] = b[3 * i + 2];
    }
  }
}

// ---------------------------------------------------------------------------
// multicanonical decision (multicanonical.c:337-704, update.c:13-30), one block
// ---------------------------------------------------------------------------
__device__ inline void muca_linearize(MucaDev* w) {
  w->slope[0] = 0;
  w->slope[w->bins + 1] = 0;
  w->b[0] = w->W[0];
  w->b[w->bins + 1] = w->W[w->bins + 1];
  for (int i = 1; i < w->bins + 1; i++) {
    w->slope[i] = (w->W[i + 1] - w->W[i]) / (w->pos[i + 1] - w->pos[i]);
    w->b[i] = w->W[i] - w->slope[i] * w->pos[i];
  }
}
__device__ inline int muca_whichbin(const MucaDev* w, double val) {
  if (val < w->min) return 0;
  if (val >= w->max) return w->bins + 1;
  int bmin = 1, bmax = w->bins;
  while (bmin <= bmax) {
    int bin = bmin + (bmax - bmin) / 2;
    double cur = w->pos[bin], nxt = w->pos[bin + 1];
    if ((val < nxt && val > cur) || (fabs(val - cur) < 1e-12)) return bin;
    if (val > cur) bmin = bin + 1;
    else bmax = bin - 1;
  }
  return w->bins;
}
__device__ inline double muca_get_weight(const MucaDev* w, double val) {
  if (val >= w->max) return w->b[w->bins + 1];
  if (val < w->min) return w->b[0];
  int bin = muca_whichbin(w, val);
  if (bin >= w->bins + 1) return w->b[w->bins + 1];
  return w->b[bin] + w->slope[bin] * val;
}
__device__ inline void muca_accumulate(MucaDev* w, double val) {
  int bin = muca_whichbin(w, val);
  if (bin == 0) {
    double dmin = w->pos[2] - w->pos[1];
    if (val < w->pos[1] - 0.5 * dmin) return;
    bin += 1;
  } else if (bin < w->bins + 1) {
    if (val - w->pos[bin] > w->pos[bin + 1] - val) bin = bin + 1;
  } else {
    double dmax = w->pos[w->bins + 1] - w->pos[w->bins];
    if (val > w->pos[w->bins + 1] + 0.5 * dmax) return;
  }
  if (w->mode == 1) {
    w->hits[bin] += 5;
    if (bin > 1) w->hits[bin - 1] += 3;
    if (bin > 2) w->hits[bin - 2] += 1;
    if (bin < w->bins) w->hits[bin + 1] += 3;
    if (bin < w->bins - 1) w->hits[bin + 2] += 1;
  } else if (w->mode == 2) {
    w->hits[bin]++;
    w->hgram[bin] += exp(muca_get_weight(w, val));
  }
}
__device__ inline void muca_update_fast(MucaDev* w) {
  int first = -1;
  double delta = 0.0;
  for (int i = 0; i < w->bins + 2; i++) {
    if (w->pos[i] >= w->wrk_min && w->wrk_max >= w->pos[i]) {
      if (first < 0) first = i;
      delta = (w->hits[i] - w->hits[first]) * w->delta / ((double)w->bins);
      w->W[i] += delta;
    } else if (w->wrk_max < w->pos[i]) {
      w->W[i] += delta;
    }
  }
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  muca_linearize(w);
  int tunnel = 0;
  if (w->last_max && w->hits[1] > 0) { w->last_max = 0; tunnel = 1; }
  else if (!w->last_max && w->hits[w->bins] > 0) { w->last_max = 1; tunnel = 1; }
  if (tunnel) w->delta /= 1.5;
  for (int i = 0; i < w->bins + 2; i++) w->hits[i] = 0;
}
__device__ inline void muca_update_slow(MucaDev* w) {
  int n = w->bins + 2;
  double* wold = w->wold;
  for (int i = 0; i < n; i++) wold[i] = w->W[i];
  double dmin = w->pos[2] - w->pos[1];
  w->hgram[1] /= dmin;
  for (int i = 2; i < w->bins + 1; i++) w->hgram[i] /= (w->pos[i + 1] - w->pos[i - 1]);
  int first = -1, last = -1, hits_min = 8;
  for (int i = 1; i < w->bins + 1; i++) {
    if (w->pos[i] >= w->wrk_min && w->wrk_max >= w->pos[i]) {
      if (first < 0) { first = i; continue; }
      w->nsum[i] += w->hits[i];
      int gg = 0;
      if (w->hits[i] >= hits_min && w->hits[i - 1] >= hits_min) {
        gg = w->hits[i] + w->hits[i - 1];
      } else {
        w->W[i] = wold[i] - wold[i - 1] + w->W[i - 1];
        continue;
      }
      long long gsum_new = w->gsum[i] + gg;
      double ln = w->hgram[i - 1] / w->hgram[i];
      ln = -1.0 * gg * log(ln);
      w->W[i] = w->W[i - 1] + ((wold[i] - wold[i - 1]) * w->gsum[i] + ln) / ((double)gsum_new);
      w->gsum[i] = gsum_new;
    } else if (w->wrk_max < w->pos[i]) {
      if (last < 0) last = i - 1;
      w->W[i] += w->W[last] - wold[last];
    }
  }
  for (int i = 0; i < n; i++) { w->hits[i] = 0; w->hgram[i] = 0.0; }
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  for (int i = 0; i < n; i++) wold[i] = w->W[i];
  double corr = 0.0;
  if (first < 1) {  // no bin inside the work range: nothing to overcorrect
    muca_linearize(w);
    return;
  }
  if (first == 1) dmin = w->pos[first + 1] - w->pos[first];
  else dmin = w->pos[first + 1] - w->pos[first - 1];
  for (int i = first + 1; i < w->bins + 1; i++) {
    if (i <= last) {
      double diff1 = w->pos[i + 1] - w->pos[i - 1];
      corr = 2.0 * log((dmin / diff1) * w->nsum[i] / w->nsum[first]);
    }
    w->W[i] += corr;
  }
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  muca_linearize(w);
  for (int i = 0; i < n; i++) w->W[i] = wold[i];
}

// muca_check (update.c:13-30) once the parity's order parameter `tot` is
// known, by a whole block (every thread calls it; blockDim.x >= 2): weight
// difference, global draw (site 0xffffffff, block = check), accept/reject,
// hits and weight recursion.  The weights of the new and the old value
// (get_weight, multicanonical.c:350-379) are looked up with the bins tested
// by all threads at once -- one pass of independent loads instead of a
// binary search of dependent ones, which on the critical path of every
// check cost more than the update itself.  The bin found is the one the
// reference's binary search (whichbin, multicanonical.c:671-704) returns:
// the unique bin with pos[b] < val < pos[b+1]; a value within 1e-12 of a bin
// edge (where the search may stop at either neighbour) or in no bin takes
// the sequential search.  `sweep` is the chain's sweep number (the global
// draw's counter); the decision (1 accept) is returned to every thread.
// What the decision reads of the weight besides the bins it searches, and
// this thread's first bin k = 1 + threadIdx.x (pos[k], pos[k + 1], b[k],
// slope[k]) -- loaded by the deciding block while it still sums the order
// parameter, so that the decision itself waits on no global load in the
// common case (a value strictly inside a bin of the first blockDim.x)
struct MucaPre {
  double pv0, pv1, mn, mx;
  int bins, mode;
  double cur, nxt, bk, sk;
};
__device__ inline MucaPre muca_preload(const MucaDev* w) {
  MucaPre p;
  p.pv0 = w->param_value[0];
  p.pv1 = w->param_value[1];
  p.mn = w->min;
  p.mx = w->max;
  p.bins = w->bins;
  p.mode = w->mode;
  p.cur = p.nxt = p.bk = p.sk = 0.0;
  const int k = 1 + (int)threadIdx.x;
  if (k <= p.bins) {
    p.cur = w->pos[k];
    p.nxt = w->pos[k + 1];
    p.bk = w->b[k];
    p.sk = w->slope[k];
  }
  return p;
}
__device__ inline int muca_decide_block(MucaDev* w, const MucaPre& pre, double tot, int parity, const RngKey& rk,
                                        uint32_t pass, uint32_t check, uint32_t sweep, unsigned long long* ctr) {
  __shared__ int s_bin[2], s_fuzzy[2], s_accept;
  __shared__ double s_W[2];
  const int bins = pre.bins;
  const double old = pre.pv0 + pre.pv1;
  const double nw = tot + (parity ? pre.pv0 : pre.pv1);
  if (threadIdx.x < 2) {
    s_bin[threadIdx.x] = -1;
    s_fuzzy[threadIdx.x] = 0;
  }
  __syncthreads();
  for (int k = 1 + (int)threadIdx.x; k <= bins; k += (int)blockDim.x) {
    const bool first = k == 1 + (int)threadIdx.x;
    const double cur = first ? pre.cur : w->pos[k], nxt = first ? pre.nxt : w->pos[k + 1];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const double v = j ? old : nw;
      if (v < nxt && v > cur) s_bin[j] = k;
      if (fabs(v - cur) < 1e-12 || fabs(v - nxt) < 1e-12) s_fuzzy[j] = 1;
    }
  }
  __syncthreads();
  // W = b[bin] + slope[bin] v (get_weight): by the thread that holds the bin,
  // or with loads by thread j for the other cases
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const double v = j ? old : nw;
    const bool inside = !(v >= pre.mx) && !(v < pre.mn);
    const bool direct = inside && s_bin[j] >= 1 && !s_fuzzy[j] && s_bin[j] <= (int)blockDim.x;
    if (direct && s_bin[j] == 1 + (int)threadIdx.x) s_W[j] = pre.bk + pre.sk * v;
    if (!direct && (int)threadIdx.x == j) {
      double W;
      if (v >= pre.mx) W = w->b[bins + 1];
      else if (v < pre.mn) W = w->b[0];
      else {
        const int bin = (s_bin[j] < 0 || s_fuzzy[j]) ? muca_whichbin(w, v) : s_bin[j];
        W = bin >= bins + 1 ? w->b[bins + 1] : w->b[bin] + w->slope[bin] * v;
      }
      s_W[j] = W;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    w->param_value[parity] = tot;
    const double Wn = s_W[0], Wo = s_W[1];
    double u = philox_uniform53(rk.k0, rk.k1, GLOBAL_SITE, pass, check, sweep, rk.chain, 0);
    int accept = exp(-(Wn - Wo)) > u ? 1 : 0;
    if (pre.mode != 0) {
      double val = accept ? nw : old;
      muca_accumulate(w, val);
      w->muca_count++;
      if (w->muca_count % w->update_interval == 0) {
        if (pre.mode == 1) muca_update_fast(w);
        else if (pre.mode == 2) muca_update_slow(w);
        w->muca_count = 0;
        w->weight_updates++;
      }
      // the recursion may have changed the other parity's value: read it back
      if (!accept) w->param_value[parity] = old - w->param_value[1 - parity];
    } else if (!accept) {
      w->param_value[parity] = old - (parity ? pre.pv0 : pre.pv1);
    }
    w->last_accept = accept;
    // fire-and-forget adds: this thread alone writes the chain's counters here
    atomicAdd(ctr + 20, 1ull);
    atomicAdd(ctr + 21, (unsigned long long)accept);
    s_accept = accept;
  }
  __syncthreads();
  return s_accept;
}

// sum of x[0..n) by the block's first 64 threads (blockDim.x >= 64) in a
// fixed order -- lane l adds x[l], x[l + 64], ..., then a tree over the 64
// lane sums -- valid in thread 0.  The loads bypass L1: the values were
// written by other blocks of the same launch.
__device__ inline double fixed_sum64(const double* x, int n) {
  __shared__ double red[64];
  if (threadIdx.x < 64) {
    // lane k adds x[k], x[k + 64], ... in that order; the loads are issued
    // sixteen at a time
    double v = 0.0;
    for (int k = threadIdx.x; k < n; k += 64 * 16) {
      double t[16];
#pragma unroll
      for (int j = 0; j < 16; j++) t[j] = k + 64 * j < n ? __ldcg(x + k + 64 * j) : 0.0;
#pragma unroll
      for (int j = 0; j < 16; j++)
        if (k + 64 * j < n) v += t[j];
    }
    red[threadIdx.x] = v;
  }
  __syncthreads();
#pragma unroll
  for (int h = 32; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  return red[0];
}

// The multicanonical check of a whole parity decided by the update launch
// itself, without a kernel of its own: every block leaves its order-parameter
// sum in partials[block]; the last block to finish in each chunk of
// MUCA_CHUNK blocks adds the chunk's sums (fixed order) into
// partials[blocks + chunk]; the last chunk to finish adds the chunk sums
// (fixed order) and decides.  Arrival counts are atomic adds after a fence,
// and each count is put back to 0 by the block that completes it, ready for
// the next launch (and for graph replays).
constexpr int MUCA_CHUNK = 64;
constexpr int MUCA_MAX_CHUNKS = 3071;  // arrival counters after the chunk count (host buffer size)
__device__ inline void muca_fused_finish(const PassArgs& a, double s) {
  __shared__ int s_last;
  const unsigned nb = gridDim.x, b = blockIdx.x;
  const unsigned chunk = b / MUCA_CHUNK, c0 = chunk * MUCA_CHUNK;
  const unsigned csize = min(nb - c0, (unsigned)MUCA_CHUNK);
  const unsigned nchunks = (nb + MUCA_CHUNK - 1) / MUCA_CHUNK;
  if (threadIdx.x == 0) {
    a.partials[b] = s;
    __threadfence();
    s_last = atomicAdd(a.arrive + 1 + chunk, 1u) == csize - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // the weight, loaded while the sums are formed (only the final block uses it)
  const MucaPre pre = muca_preload(a.muca);
  const double cs = fixed_sum64(a.partials + c0, (int)csize);
  if (threadIdx.x == 0) {
    a.arrive[1 + chunk] = 0;
    a.partials[nb + chunk] = cs;
    __threadfence();
    s_last = atomicAdd(a.arrive, 1u) == nchunks - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const double tot = fixed_sum64(a.partials + nb, (int)nchunks);  // the same value in every thread
  if (threadIdx.x == 0) a.arrive[0] = 0;
  muca_decide_block(a.muca, pre, tot / a.vol, a.parity, a.rk, a.pass, a.check, *a.rk.sweep, a.ctr);
}

#ifdef SU2_WITH_GLOBAL
// muca_check (update.c:13-30) as a kernel of its own, for checks that cover
// part of a parity: the partial sums added in a fixed order, then the
// decision.  One block.
__global__ void k_muca_decide(MucaDev* w, const double* partials, int np, double vol, int parity, RngKey rk,
                              uint32_t pass, uint32_t check, unsigned long long* ctr) {
  __shared__ double red[256];
  const MucaPre pre = muca_preload(w);
  double v = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) v += partials[k];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  muca_decide_block(w, pre, red[0] / vol, parity, rk, pass, check, *rk.sweep, ctr);
}

// calc_orderparam for the host API: store the parity sum
__global__ void k_muca_set_param(MucaDev* w, const double* partials, int np, double vol, int parity) {
  __shared__ double red[256];
  double v = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) v += partials[k];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) w->param_value[parity] = red[0] / vol;
}

#endif  // SU2_WITH_GLOBAL

// ---------------------------------------------------------------------------
// measurements (measure.c:71-243)
// ---------------------------------------------------------------------------
// The projected U(1) links (magfield.c:32-184) and the plaquette angle
// alpha_proj (magfield.c:189-216).  The reference forms each projected link
// Pi(x) U_mu(x) Pi(x+mu), Pi = (1 + n.sigma)/2, n = Sigma/|Sigma| (projector(),
// project_u1()), as a complex 2x2 matrix, multiplies the four of a plaquette
// and takes the argument of the trace.  Pi is the rank-one projector |n><n|
// onto the +1 eigenvector of n.sigma, so the product collapses to
//   tr = z(x,d1) z(x+d1,d2) conj(z(x+d2,d1)) conj(z(x,d2)),
//   z(a,mu) = <n_a| U_mu(a) |n_{a+mu}>,
// the same number (the phase of each |n> cancels around the closed loop),
// from 4 spinors and 4 overlaps instead of 8 projectors and 11 matrix
// products.  Each site's spinor takes the chart that avoids the pole opposite
// to Sigma: (|S| + S3, S1 + i S2) or (S1 - i S2, |S| - S3), normalised.
template <typename R>
struct Spinor {
  R r0, i0, r1, i1;
};
template <typename R>
__device__ inline Spinor<R> proj_spinor(const V3<R>& a) {
  const R m = msqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  Spinor<R> s;
  if (a.z >= 0) {
    const R k = (R)1 / msqrt((R)2 * m * (m + a.z));
    s.r0 = (m + a.z) * k; s.i0 = 0; s.r1 = a.x * k; s.i1 = a.y * k;
  } else {
    const R k = (R)1 / msqrt((R)2 * m * (m - a.z));
    s.r0 = a.x * k; s.i0 = -a.y * k; s.r1 = (m - a.z) * k; s.i1 = 0;
  }
  return s;
}
// z = <va| U |vb>, U = [[a + i d, c + i b], [-c + i b, a - i d]] (the SU(2)
// matrix of the link quaternion, as project_u1 builds it)
template <typename R>
__device__ inline void link_overlap(const Spinor<R>& va, const Q<R>& u, const Spinor<R>& vb, R& zr, R& zi) {
  const R w0r = u.a * vb.r0 - u.d * vb.i0 + u.c * vb.r1 - u.b * vb.i1;
  const R w0i = u.a * vb.i0 + u.d * vb.r0 + u.c * vb.i1 + u.b * vb.r1;
  const R w1r = -u.c * vb.r0 - u.b * vb.i0 + u.a * vb.r1 + u.d * vb.i1;
  const R w1i = -u.c * vb.i0 + u.b * vb.r0 + u.a * vb.i1 - u.d * vb.r1;
  zr = va.r0 * w0r + va.i0 * w0i + va.r1 * w1r + va.i1 * w1i;
  zi = va.r0 * w0i - va.i0 * w0r + va.r1 * w1i - va.i1 * w1r;
}
template <typename R>
__device__ inline R alpha_proj(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i, int d1,
                               int d2) {
  int c1[3];
  shift_coords(g, c, d1, 1, c1);
  const int i1 = shifted(g, c, d1, 1), i2 = shifted(g, c, d2, 1), i12 = shifted(g, c1, d2, 1);
  const Spinor<R> sx = proj_spinor(ld3(f, i)), s1 = proj_spinor(ld3(f, i1)), s2 = proj_spinor(ld3(f, i2)),
                  s12 = proj_spinor(ld3(f, i12));
  R z1r, z1i, z2r, z2i, z3r, z3i, z4r, z4i;
  link_overlap(sx, ld4<R>(lk(f, d1), i), s1, z1r, z1i);
  link_overlap(s1, ld4<R>(lk(f, d2), i1), s12, z2r, z2i);
  link_overlap(s2, ld4<R>(lk(f, d1), i2), s12, z3r, z3i);
  link_overlap(sx, ld4<R>(lk(f, d2), i), s2, z4r, z4i);
  // (z1 z2) conj(z3 z4)
  const R pr = z1r * z2r - z1i * z2i, pi = z1r * z2i + z1i * z2r;
  const R qr = z3r * z4r - z3i * z4i, qi = z3r * z4i + z3i * z4r;
  const R tr = pr * qr + pi * qi, ti = pi * qr - pr * qi;
  return matan2(ti, tr) * msqrt((R)cp.beta);
}

// alpha(x; 0,1), alpha(x; 0,2), alpha(x; 1,2) for every site
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_alpha(Fields<R> f, Geom g, CoupT<R> cp, double* alpha) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.V) return;
  int parity = t >= g.half;
  int tp = t - parity * g.half;
  int c[3];
  site_coords(g, parity, tp, c);
  alpha[t] = (double)alpha_proj(f, g, cp, c, t, 0, 1);
  alpha[g.V + t] = (double)alpha_proj(f, g, cp, c, t, 0, 2);
  alpha[2 * g.V + t] = (double)alpha_proj(f, g, cp, c, t, 1, 2);
}

// which of the NSUMS volume sums a content produces
template <int CC>
__device__ inline bool sum_active(int k, int rt) {
  const bool h1 = SU2_HAS(CC, rt, C_H1), h2 = SU2_HAS(CC, rt, C_H2), t = SU2_HAS(CC, rt, C_T),
             s = SU2_HAS(CC, rt, C_S), u = SU2_HAS(CC, rt, C_U1);
  const int nh = h2 ? 2 : (h1 ? 1 : 0);
  switch (k) {
    case 0: case 1: return true;
    case 2: return u;
    case 3: case 4: case 5: return nh > 0;
    case 6: case 7: case 8: case 9: case 10: return nh > 1;
    case 11: case 12: case 13: case 15: case 16: return t;
    case 14: return t && nh > 0;
    case 17: case 18: case 19: case 20: case 21: return s;
    case 22: case 23: return s && nh == 1;
  }
  return false;
}

// per-site terms of measure() summed over the block into partials[k][block]
// Sources of the projected U(1) field strengths alpha_proj (magfield.c:189-216)
// of the magnetic charge: planes filled by k_alpha (plane 0 = (0,1), 1 = (0,2),
// 2 = (1,2)), or the projections computed where they are needed.
struct AlphaPlanes {
  const double* a;
  int V;
  template <typename R>
  __device__ double operator()(const Fields<R>&, const Geom&, const CoupT<R>&, const int*, int n, int plane) const {
    return a[plane * V + n];
  }
};
struct AlphaOnTheFly {
  template <typename R>
  __device__ double operator()(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* cn, int n,
                               int plane) const {
    const int d1 = plane == 2 ? 1 : 0, d2 = plane == 0 ? 1 : 2;
    return (double)alpha_proj(f, g, cp, cn, n, d1, d2);
  }
};

// magcharge_cube (magfield.c:262-280): the divergence of the magnetic field
// of the projected U(1) over the cube at site i (coordinates c)
template <typename R, typename AF>
__device__ inline double magcharge_site(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                        const AF& alpha) {
  int c0[3], c1[3], c2[3];
  shift_coords(g, c, 0, 1, c0);
  shift_coords(g, c, 1, 1, c1);
  shift_coords(g, c, 2, 1, c2);
  int n0 = shifted(g, c, 0, 1), n1 = shifted(g, c, 1, 1), n2 = shifted(g, c, 2, 1);
  double q = 0.0;
  double B1 = alpha(f, g, cp, c, i, 2), B2 = alpha(f, g, cp, c0, n0, 2);
  q += B2 - B1;
  B1 = -alpha(f, g, cp, c, i, 1);
  B2 = -alpha(f, g, cp, c1, n1, 1);
  q += B2 - B1;
  B1 = alpha(f, g, cp, c, i, 0);
  B2 = alpha(f, g, cp, c2, n2, 0);
  q += B2 - B1;
  return q;
}

// magcharge_cube with the projections computed here: the cube's 8 corner
// spinors and 12 edge overlaps once each (each edge borders two of the six
// faces), then the six face angles as alpha_proj forms them
template <typename R>
__device__ inline R face_angle(R ar, R ai, R br, R bi, R cr, R ci, R dr, R di, R sqrt_beta) {
  const R pr = ar * br - ai * bi, pi = ar * bi + ai * br;
  const R qr = cr * dr - ci * di, qi = cr * di + ci * dr;
  return matan2(pi * qr - pr * qi, pr * qr + pi * qi) * sqrt_beta;
}
template <typename R>
__device__ inline double magcharge_site(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, const int* c, int i,
                                        const AlphaOnTheFly&) {
  int c0[3], c1[3], c01[3];
  shift_coords(g, c, 0, 1, c0);
  shift_coords(g, c, 1, 1, c1);
  shift_coords(g, c0, 1, 1, c01);
  const int i0 = shifted(g, c, 0, 1), i1 = shifted(g, c, 1, 1), i2 = shifted(g, c, 2, 1);
  const int i01 = shifted(g, c0, 1, 1), i02 = shifted(g, c0, 2, 1), i12 = shifted(g, c1, 2, 1);
  const int i012 = shifted(g, c01, 2, 1);
  const Spinor<R> sx = proj_spinor(ld3(f, i)), s0 = proj_spinor(ld3(f, i0)), s1 = proj_spinor(ld3(f, i1)),
                  s2 = proj_spinor(ld3(f, i2)), s01 = proj_spinor(ld3(f, i01)), s02 = proj_spinor(ld3(f, i02)),
                  s12 = proj_spinor(ld3(f, i12)), s012 = proj_spinor(ld3(f, i012));
  // z(y, mu) = <n_y| U_mu(y) |n_{y+mu}> on the cube's edges
  R x0r, x0i, x1r, x1i, x2r, x2i, a1r, a1i, a2r, a2i, b0r, b0i, b2r, b2i, e0r, e0i, e1r, e1i, f2r, f2i, g1r, g1i,
      h0r, h0i;
  link_overlap(sx, ld4<R>(lk(f, 0), i), s0, x0r, x0i);       // (x, 0)
  link_overlap(sx, ld4<R>(lk(f, 1), i), s1, x1r, x1i);       // (x, 1)
  link_overlap(sx, ld4<R>(lk(f, 2), i), s2, x2r, x2i);       // (x, 2)
  link_overlap(s0, ld4<R>(lk(f, 1), i0), s01, a1r, a1i);     // (x+0, 1)
  link_overlap(s0, ld4<R>(lk(f, 2), i0), s02, a2r, a2i);     // (x+0, 2)
  link_overlap(s1, ld4<R>(lk(f, 0), i1), s01, b0r, b0i);     // (x+1, 0)
  link_overlap(s1, ld4<R>(lk(f, 2), i1), s12, b2r, b2i);     // (x+1, 2)
  link_overlap(s2, ld4<R>(lk(f, 0), i2), s02, e0r, e0i);     // (x+2, 0)
  link_overlap(s2, ld4<R>(lk(f, 1), i2), s12, e1r, e1i);     // (x+2, 1)
  link_overlap(s01, ld4<R>(lk(f, 2), i01), s012, f2r, f2i);  // (x+0+1, 2)
  link_overlap(s02, ld4<R>(lk(f, 1), i02), s012, g1r, g1i);  // (x+0+2, 1)
  link_overlap(s12, ld4<R>(lk(f, 0), i12), s012, h0r, h0i);  // (x+1+2, 0)
  const R sb = msqrt((R)cp.beta);
  // the charge in the field precision (the angles are): a site's terms are
  // combined in R, the volume sums are FP64
  R q = 0;
  // plane (1,2) at x + 0 minus at x
  R B1 = face_angle(x1r, x1i, b2r, b2i, e1r, e1i, x2r, x2i, sb);
  R B2 = face_angle(a1r, a1i, f2r, f2i, g1r, g1i, a2r, a2i, sb);
  q += B2 - B1;
  // plane (0,2): at x minus at x + 1
  B1 = -face_angle(x0r, x0i, a2r, a2i, e0r, e0i, x2r, x2i, sb);
  B2 = -face_angle(b0r, b0i, f2r, f2i, h0r, h0i, b2r, b2i, sb);
  q += B2 - B1;
  // plane (0,1) at x + 2 minus at x
  B1 = face_angle(x0r, x0i, a1r, a1i, b0r, b0i, x1r, x1i, sb);
  B2 = face_angle(e0r, e0i, g1r, g1i, h0r, h0i, e1r, e1i, sb);
  q += B2 - B1;
  return (double)q;
}

// measure_local (measure.c:368-487): per site (storage order) Tr Sigma^2 and
// the magnetic charge in units of 2 pi sqrt(beta) -- an integer up to rounding
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_measure_local(Fields<R> f, Geom g, CoupT<R> cp, double denom,
                                                         double* out) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.V) return;
  int parity = t >= g.half;
  int c[3];
  site_coords(g, parity, t - parity * g.half, c);
  out[2 * (size_t)t] = (double)tripletsq(ld3(f, t));
  out[2 * (size_t)t + 1] = magcharge_site(f, g, cp, c, t, AlphaOnTheFly{}) / denom;
}

// measure_along_z (z_coord.c:206-300): sums over the plane z of phi^2 (first
// doublet), Tr Sigma^2, S and S^2; one block per plane, the plane's sites
// enumerated by the two other coordinates (lower direction fastest) and summed
// in a fixed order.  out[z][4], columns of absent fields zero.
constexpr int ZBLOCK = 256;
template <typename R>
__global__ void __launch_bounds__(ZBLOCK) k_measure_z(Fields<R> f, Geom g, int content, int zdir, double* out) {
  const int z = blockIdx.x;
  const int dlo = zdir == 0 ? 1 : 0, dhi = zdir == 2 ? 1 : 2;
  const int La = g.L[dlo], area = g.V / g.L[zdir];
  const bool h = content & (C_H1 | C_H2), tr = content & C_T, sg = content & C_S;
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k = threadIdx.x; k < area; k += ZBLOCK) {
    int c[3];
    c[zdir] = z;
    c[dlo] = k % La;
    c[dhi] = k / La;
    int i = site_index(g, c[0], c[1], c[2]);
    if (h) m[0] += (double)doubletsq(ld4<R>(f.phi[0], i));
    if (tr) m[1] += (double)tripletsq(ld3(f, i));
    if (sg) {
      R s = f.sing[i];
      m[2] += (double)s;
      m[3] += (double)(s * s);
    }
  }
  __shared__ double sm[ZBLOCK / 32][4];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    double v = m[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sm[w][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0.0;
    for (int ww = 0; ww < ZBLOCK / 32; ww++) v += sm[ww][threadIdx.x];
    out[4 * (size_t)z + threadIdx.x] = v;
  }
}

// measure() (measure.c:110-233): the terms of site t (storage index) added to
// m[NSUMS]; per-site quantities in R, sums in FP64
template <typename R, int CC, typename AF>
__device__ inline void measure_site(const Fields<R>& f, const Geom& g, const CoupT<R>& cp, int t, const AF& alpha,
                                    double* m) {
  int parity = t >= g.half;
  int i = t;
  int c[3];
  site_coords(g, parity, t - parity * g.half, c);
  // local_su2wilson (su2u1.c:143-157)
  R wl = 0;
  wl += ((R)1 - (R)0.5 * ptrace(f, g, c, i, 0, 1));
  wl += ((R)1 - (R)0.5 * ptrace(f, g, c, i, 0, 2));
  wl += ((R)1 - (R)0.5 * ptrace(f, g, c, i, 1, 2));
  wl = (R)cp.beta * wl;
  // the site's action in the field precision (its terms are), summed in FP64
  R act = wl;
  m[1] += (double)wl;
  if (SU2_HAS(CC, cp.content, C_U1)) {
    R u1w = local_u1wilson(f, g, cp, c, i);
    act += u1w;
    m[2] += (double)u1w;
  }
  act += higgspotential<R, CC>(f, cp, i);
  const int nh = SU2_HAS(CC, cp.content, C_H2) ? 2 : (SU2_HAS(CC, cp.content, C_H1) ? 1 : 0);
  for (int h = 0; h < nh; h++) {
    R mod = doubletsq(ld4<R>(php(f, h), i));
    R cov = covariant_doublet<R, CC>(f, g, cp, c, i, h);
    act += cov;
    m[3 + 3 * h] += (double)cov;
    m[4 + 3 * h] += (double)mod;
    m[5 + 3 * h] += (double)(mod * mod);
  }
  if (SU2_HAS(CC, cp.content, C_T)) {
    R covt = covariant_triplet(f, g, c, i);
    act += covt;
    V3<R> tr = ld3(f, i);
    R tm = tripletsq(tr);
    if (nh > 0) m[14] += (double)(doubletsq(ld4<R>(php(f, 0), i)) * tm);
    m[12] += (double)tm;
    m[13] += (double)(tm * tm);
    R hs = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) hs += hop_triplet_fwd(f, g, c, i, d);
    m[11] += (double)hs;
    double q = magcharge_site(f, g, cp, c, i, alpha);
    m[15] += q;
    m[16] += fabs(q);
  }
  if (nh == 2) {
    Q<R> h1 = ld4<R>(php(f, 0), i), h2 = ld4<R>(php(f, 1), i);
    m[9] += (double)((R)0.5 * (h1.a * h2.a + h1.b * h2.b + h1.c * h2.c + h1.d * h2.d));
    m[10] += (double)((R)0.5 * (h1.d * h2.a + h1.c * h2.b - h1.b * h2.c - h1.a * h2.d));
  }
  if (SU2_HAS(CC, cp.content, C_S)) {
    R S = f.sing[i];
    R kin = (R)3 * S * S;
    R scov = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      R Sn = f.sing[shifted(g, c, d, 1)];
      kin -= S * Sn;
      scov += S * S - S * Sn;
    }
    act += kin;
    m[17] += (double)scov;
    m[18] += (double)S;
    m[19] += (double)(S * S);
    m[20] += (double)(S * S * S);
    m[21] += (double)(S * S * S * S);
    if (nh == 1) {
      R mod = doubletsq(ld4<R>(php(f, 0), i));
      m[22] += (double)(mod * S);
      m[23] += (double)(mod * S * S);
    }
  }
  m[0] += (double)act;
}

// sums of m[] over the block (blockDim.x == BLOCK) to partials[k * nblocks + block]
template <int CC>
__device__ inline void block_sums_out(const double* m, int content, double* partials, int nblocks, int block) {
  __shared__ double sm[BLOCK / 32][NSUMS];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NSUMS; k++) {
    if (!sum_active<CC>(k, content)) continue;
    double v = m[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sm[w][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NSUMS) {
    double v = 0.0;
    if (sum_active<CC>(threadIdx.x, content))
#pragma unroll
      for (int ww = 0; ww < BLOCK / 32; ww++) v += sm[ww][threadIdx.x];
    partials[threadIdx.x * nblocks + block] = v;
  }
}

// sites of one measurement block: MEAS_SPT per thread, BLOCK apart
constexpr int MEAS_SPT = 8;
constexpr int MEAS_TILE = BLOCK * MEAS_SPT;

// measure() over the whole lattice; alpha = the k_alpha planes (triplet
// content) or null.  gridDim.x = ceil(V / MEAS_TILE).
template <typename R, int CC>
__global__ void __launch_bounds__(BLOCK) k_measure(Fields<R> f, Geom g, CoupT<R> cp, const double* alpha,
                                                   double* partials) {
  double m[NSUMS];
#pragma unroll
  for (int k = 0; k < NSUMS; k++) m[k] = 0.0;
  const AlphaPlanes ap{alpha, g.V};
  for (int j = 0; j < MEAS_SPT; j++) {
    int t = ((int)blockIdx.x * MEAS_SPT + j) * BLOCK + threadIdx.x;
    if (t < g.V) measure_site<R, CC>(f, g, cp, t, ap, m);
  }
  block_sums_out<CC>(m, cp.content, partials, gridDim.x, blockIdx.x);
}

#ifdef SU2_WITH_GLOBAL
// fixed-order sum of partials[NSUMS][np] -> out[NSUMS]; one block per sum
__global__ void k_reduce_partials(const double* partials, int np, double* out) {
  __shared__ double red[256];
  const double* row = partials + (size_t)blockIdx.x * np;
  double v = 0.0;
  for (int b = threadIdx.x; b < np; b += blockDim.x) v += row[b];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}
#endif  // SU2_WITH_GLOBAL

// ---------------------------------------------------------------------------
// gradient flow (gradflow.c:190-414): forces from `in`, Euler step into `out`
// ---------------------------------------------------------------------------
template <typename R, int CC>
__global__ void __launch_bounds__(BLOCK) k_flow(Fields<R> in, Fields<R> out, Geom g, CoupT<R> cp, R dt,
                                                unsigned long long* first_zero) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.V) return;
  int parity = t >= g.half;
  int i = t;
  int c[3];
  site_coords(g, parity, t - parity * g.half, c);
#pragma unroll
  for (int mu = 0; mu < 3; mu++) {
    // grad_force_link (gradflow.c:190-258)
    Q<R> s = qscale(wilson_staple(in, g, c, i, mu), -cp.beta / (R)8);
    Q<R> U = ld4<R>(lk(in, mu), i);
    if (HAS(C_T)) {
      V3<R> a1 = ld3(in, i), a2 = ld3(in, shifted(g, c, mu, 1));
      Q<R> r = qmul(qmul(Q<R>{(R)0, a2.x, a2.y, a2.z}, qdag(U)), Q<R>{(R)0, a1.x, a1.y, a1.z});
      s.a -= (-r.a) / (R)4;
      s.b -= (-r.b) / (R)4;
      s.c -= (-r.c) / (R)4;
      s.d -= (-r.d) / (R)4;
    }
    Q<R> m = qmul(U, s);
    R fz[3] = {(R)2 * m.b, (R)2 * m.c, (R)2 * m.d};
    R z[3], mod = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      fz[a] *= (R)4 / cp.beta;
      z[a] = dt * fz[a];
      mod += z[a] * z[a];
    }
    // flow_gauge (gradflow.c:361-401)
    if (mod <= (R)0) {
      atomicMin(first_zero, (unsigned long long)(i * 3 + mu));
      st4<R>(lk(out, mu), i, U);
      continue;
    }
    mod = msqrt(mod);
    R sm = msin(mod);
    Q<R> u{mcos(mod), sm * z[0] / mod, sm * z[1] / mod, sm * z[2] / mod};
    st4<R>(lk(out, mu), i, qmul(u, U));
  }
  if (HAS(C_T)) {
    // grad_force_triplet (gradflow.c:267-330) and flow_triplet (405-414)
    R res[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      V3<R> r = qrot(ld4<R>(lk(in, d), i), ld3(in, shifted(g, c, d, 1)));
      res[0] -= r.x; res[1] -= r.y; res[2] -= r.z;
      int xm = shifted(g, c, d, -1);
      r = qrot(qdag(ld4<R>(lk(in, d), xm)), ld3(in, xm));
      res[0] -= r.x; res[1] -= r.y; res[2] -= r.z;
    }
    V3<R> tr = ld3(in, i);
    R tv[3] = {tr.x, tr.y, tr.z};
    R ts = tripletsq(tr);
    R hm = NHIGGS > 0 ? doubletsq(ld4<R>(php(in, 0), i)) : (R)0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      res[a] += ((R)6 + (R)cp.msqT + (R)2 * (R)cp.b4 * ts) * tv[a];
      if (NHIGGS > 0) res[a] += (R)cp.a2 * hm * tv[a];
    }
    st3(out, i, V3<R>{tv[0] + dt * (-res[0]), tv[1] + dt * (-res[1]), tv[2] + dt * (-res[2])});
  }
}

// links at or after the first zero-force link keep their value (the
// reference's early return in flow_gauge)
template <typename R>
__global__ void k_flow_fixup(Fields<R> in, Fields<R> out, Geom g, const unsigned long long* first_zero) {
  unsigned long long fz = *first_zero;
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.V * 3 || (unsigned long long)t < fz) return;
  int i = t / 3;
  int mu = (int)(t - i * 3);
  lk(out, mu)[i] = lk(in, mu)[i];
}

// ---------------------------------------------------------------------------
// transfers, tables, reunitarisation
// ---------------------------------------------------------------------------
// host AoS FP64 (lattice-file order) <-> device SoA
template <typename R>
__global__ void k_import(Fields<R> f, int V, int kind, int h, const double* src) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  switch (kind) {
    case 0:  // links [V][3][4]
      if (t < V * 3) {
        int i = t / 3;
        int d = (int)(t - i * 3);
        const double* s = src + t * 4;
        st4<R>(lk(f, d), i, Q<R>{(R)s[0], (R)s[1], (R)s[2], (R)s[3]});
      }
      break;
    case 1:  // u1 [V][3]
      if (t < V * 3) {
        int i = t / 3;
        a1p(f, t - i * 3)[i] = (R)src[t];
      }
      break;
    case 2:  // doublet [V][4]
      if (t < V) {
        const double* s = src + t * 4;
        st4<R>(php(f, h), t, Q<R>{(R)s[0], (R)s[1], (R)s[2], (R)s[3]});
      }
      break;
    case 3:  // triplet [V][3]
      if (t < V) st3(f, t, V3<R>{(R)src[3 * t], (R)src[3 * t + 1], (R)src[3 * t + 2]});
      break;
    case 4:  // singlet [V]
      if (t < V) f.sing[t] = (R)src[t];
      break;
  }
}
template <typename R>
__global__ void k_export(Fields<R> f, int V, int kind, int h, double* dst) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  switch (kind) {
    case 0:
      if (t < V * 3) {
        int i = t / 3;
        int d = (int)(t - i * 3);
        Q<R> q = ld4<R>(lk(f, d), i);
        double* s = dst + t * 4;
        s[0] = q.a; s[1] = q.b; s[2] = q.c; s[3] = q.d;
      }
      break;
    case 1:
      if (t < V * 3) {
        int i = t / 3;
        dst[t] = a1p(f, t - i * 3)[i];
      }
      break;
    case 2:
      if (t < V) {
        Q<R> q = ld4<R>(php(f, h), t);
        double* s = dst + t * 4;
        s[0] = q.a; s[1] = q.b; s[2] = q.c; s[3] = q.d;
      }
      break;
    case 3:
      if (t < V) {
        V3<R> v = ld3(f, t);
        dst[3 * t] = v.x; dst[3 * t + 1] = v.y; dst[3 * t + 2] = v.z;
      }
      break;
    case 4:
      if (t < V) dst[t] = f.sing[t];
      break;
  }
}

// renormalise every link to unit norm (FP32 form, every `interval` sweeps)
template <typename R>
__global__ void k_reunitarize(Fields<R> f, int V, const uint32_t* sweep, int interval) {
  if (interval <= 0 || (*sweep % (uint32_t)interval) != (uint32_t)(interval - 1)) return;
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= V * 3) return;
  int i = t / 3;
  int d = (int)(t - i * 3);
  Q<R> q = ld4<R>(lk(f, d), i);
  R n = (R)1 / msqrt(qsq(q));
  st4<R>(lk(f, d), i, qscale(q, n));
}

#undef HAS
#undef NHIGGS

}  // namespace su2
