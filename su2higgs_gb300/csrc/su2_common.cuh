// su2_common.cuh -- device building blocks of libsu2gpu: lattice geometry in
// the reference's EVEN-first site order, the Philox4x32-10 stream, quaternion
// algebra and the parity-split structure-of-arrays field views.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace su2 {

// ---------------------------------------------------------------------------
// field content bits (same values as SU2GPU_* in include/su2gpu.h)
// ---------------------------------------------------------------------------
enum : int { C_H1 = 0x01, C_H2 = 0x02, C_T = 0x04, C_S = 0x08, C_U1 = 0x10 };
constexpr int C_GENERIC = -1;  // content read from the runtime mask
enum : int { ALG_METRO = 1, ALG_HEATBATH = 2, ALG_OR = 3 };

#define SU2_HAS(CC, rt, bit) (((CC) == ::su2::C_GENERIC) ? (((rt) & (bit)) != 0) : (((CC) & (bit)) != 0))

// ---------------------------------------------------------------------------
// geometry.  Site index of (x,y,z): the reference orders sites
// lexicographically (x fastest, layout.c:945-972) and then moves EVEN sites
// first, keeping the order inside each parity (paritymap, layout.c:826-851).
// With L0 even this is  idx = parity*V/2 + n/2,  n = x + L0*(y + L1*z).
// ---------------------------------------------------------------------------
struct Geom {
  int L[3];
  int hL0;   // L0 / 2
  int V;     // sites (< 2^31)
  int half;  // sites per parity
  // division by hL0 and by L1 as a multiply and shift (div30)
  unsigned m_hl0, m_l1;
  int s_hl0, s_l1;
};

// floor(n / d) for 0 <= n < 2^30 as (n * m) >> s with l = ceil(log2 d),
// s = 30 + l, m = floor(2^s / d) + 1 < 2^31: then 2^s <= m d <= 2^s + 2^l,
// which makes the quotient exact (Granlund & Montgomery, PLDI 1994, thm 4.2)
inline void div30_magic(unsigned d, unsigned* m, int* s) {
  int l = 0;
  while ((1ull << l) < d) l++;
  *s = 30 + l;
  *m = (unsigned)((1ull << *s) / d + 1);
}
__host__ __device__ inline unsigned div30(unsigned n, unsigned m, int s) {
  return (unsigned)(((unsigned long long)n * m) >> s);
}

inline Geom make_geom(int L0, int L1, int L2) {
  Geom g;
  g.L[0] = L0; g.L[1] = L1; g.L[2] = L2;
  g.hL0 = L0 / 2;
  g.V = L0 * L1 * L2;
  g.half = g.V / 2;
  div30_magic((unsigned)g.hL0, &g.m_hl0, &g.s_hl0);
  div30_magic((unsigned)L1, &g.m_l1, &g.s_l1);
  return g;
}

__host__ __device__ inline int site_index(const Geom& g, int x, int y, int z) {
  int n = x + g.L[0] * (y + g.L[1] * z);
  return ((x + y + z) & 1) * g.half + (n >> 1);
}

// coordinates of the t-th site of a parity
__host__ __device__ inline void site_coords(const Geom& g, int parity, int t, int* c) {
  unsigned r = div30((unsigned)t, g.m_hl0, g.s_hl0);
  int k = t - (int)r * g.hL0;
  unsigned z = div30(r, g.m_l1, g.s_l1);
  int y = (int)(r - z * (unsigned)g.L[1]);
  c[0] = 2 * k + ((parity + y + (int)z) & 1);
  c[1] = y;
  c[2] = (int)z;
}

__host__ __device__ inline int wrap(int v, int L) { return v >= L ? v - L : (v < 0 ? v + L : v); }

// lexicographic step from c to c + s*e_d (s in {-1, 0, 1}), periodic
__host__ __device__ inline int lex_step(const Geom& g, const int* c, int d, int s) {
  const int st = d == 0 ? 1 : (d == 1 ? g.L[0] : g.L[0] * g.L[1]);
  const int cd = d == 0 ? c[0] : (d == 1 ? c[1] : c[2]);
  const int lm = (d == 0 ? g.L[0] : (d == 1 ? g.L[1] : g.L[2])) - 1;
  return s > 0 ? (cd == lm ? -lm * st : st) : (s < 0 ? (cd == 0 ? lm * st : -st) : 0);
}

// index of the site at c + s1*e_d1 + s2*e_d2 (periodic, |s| <= 1): the
// lexicographic index of c (shared by every neighbour of the site) plus the
// steps, and the parity, which every unit step flips (even sides); written
// with selects so that runtime directions never index an array
__host__ __device__ inline int shifted(const Geom& g, const int* c, int d1, int s1, int d2 = 0, int s2 = 0) {
  int n = c[0] + g.L[0] * (c[1] + g.L[1] * c[2]) + lex_step(g, c, d1, s1) + lex_step(g, c, d2, s2);
  int par = (c[0] + c[1] + c[2] + s1 + s2) & 1;
  return par * g.half + (n >> 1);
}
// coordinates of c + s*e_d
__host__ __device__ inline void shift_coords(const Geom& g, const int* c, int d, int s, int* o) {
  o[0] = wrap(c[0] + (d == 0 ? s : 0), g.L[0]);
  o[1] = wrap(c[1] + (d == 1 ? s : 0), g.L[1]);
  o[2] = wrap(c[2] + (d == 2 ? s : 0), g.L[2]);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11).  key = seed, counter =
// (site, pass<<16 | block, sweep, chain); draw 2b / 2b+1 are the two 64-bit
// halves of block b, converted as (x >> 11) * 2^-53 for FP64 (the conversion
// of the reference's dran(), generic/mersenne.c:147-150) or (x >> 40) * 2^-24
// for FP32.
// ---------------------------------------------------------------------------
constexpr uint32_t GLOBAL_SITE = 0xffffffffu;

__host__ __device__ inline uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

__host__ __device__ inline void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0,
                                              uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
}

struct RngKey {
  uint32_t k0, k1;
  uint32_t chain;
  const uint32_t* sweep;  // device word holding the current sweep number
};

template <typename R>
__host__ __device__ inline R u64_to_uniform(uint64_t x);
template <>
__host__ __device__ inline double u64_to_uniform<double>(uint64_t x) {
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}
template <>
__host__ __device__ inline float u64_to_uniform<float>(uint64_t x) {
  return (float)(uint32_t)(x >> 40) * (1.0f / 16777216.0f);
}

// per-site stream: uniforms are consumed strictly in order
template <typename R>
struct SiteRng {
  uint32_t k0, k1, site, pass_hi, sweep, chain, draw;
  uint64_t w1;
  __device__ SiteRng(const RngKey& k, uint32_t sweep_, uint32_t site_, uint32_t pass)
      : k0(k.k0), k1(k.k1), site(site_), pass_hi(pass << 16), sweep(sweep_), chain(k.chain), draw(0), w1(0) {}
  __device__ inline R uni() {
    uint32_t d = draw++;
    if (d & 1u) return u64_to_uniform<R>(w1);
    uint32_t c0 = site, c1 = pass_hi | ((d >> 1) & 0xffffu), c2 = sweep, c3 = chain;
    philox4x32_10(c0, c1, c2, c3, k0, k1);
    w1 = ((uint64_t)c2 << 32) | c3;
    return u64_to_uniform<R>(((uint64_t)c0 << 32) | c1);
  }
};

// FP32 form: four 24-bit uniforms per Philox block, (w >> 8) * 2^-24; draw k
// is word k & 3 of block k >> 2.  Statistically the same stream quality, half
// the generator work per uniform; not the FP64 form's stream.
template <>
struct SiteRng<float> {
  uint32_t k0, k1, site, pass_hi, sweep, chain, draw;
  uint32_t q1, q2, q3;  // the unread words of the current block, in order
  __device__ SiteRng(const RngKey& k, uint32_t sweep_, uint32_t site_, uint32_t pass)
      : k0(k.k0), k1(k.k1), site(site_), pass_hi(pass << 16), sweep(sweep_), chain(k.chain), draw(0), q1(0), q2(0),
        q3(0) {}
  __device__ inline float uni() {
    uint32_t d = draw++;
    uint32_t w;
    if ((d & 3u) == 0) {
      uint32_t c0 = site, c1 = pass_hi | ((d >> 2) & 0xffffu), c2 = sweep, c3 = chain;
      philox4x32_10(c0, c1, c2, c3, k0, k1);
      w = c0;
      q1 = c1;
      q2 = c2;
      q3 = c3;
    } else {
      w = q1;
      q1 = q2;
      q2 = q3;
    }
    return (float)(w >> 8) * (1.0f / 16777216.0f);
  }
};

// first uniform of block `block` of a stream position (host and device)
__host__ __device__ inline double philox_uniform53(uint32_t k0, uint32_t k1, uint32_t site, uint32_t pass,
                                                   uint32_t block, uint32_t sweep, uint32_t chain, int half) {
  uint32_t c0 = site, c1 = (pass << 16) | (block & 0xffffu), c2 = sweep, c3 = chain;
  philox4x32_10(c0, c1, c2, c3, k0, k1);
  uint64_t x = half ? (((uint64_t)c2 << 32) | c3) : (((uint64_t)c0 << 32) | c1);
  return u64_to_uniform<double>(x);
}

// ---------------------------------------------------------------------------
// math overloads
// ---------------------------------------------------------------------------
__device__ inline double msqrt(double x) { return sqrt(x); }
__device__ inline float msqrt(float x) { return sqrtf(x); }
__device__ inline double mlog(double x) { return log(x); }
__device__ inline float mlog(float x) { return logf(x); }
__device__ inline double mexp(double x) { return exp(x); }
__device__ inline float mexp(float x) { return expf(x); }
__device__ inline double mcos(double x) { return cos(x); }
__device__ inline float mcos(float x) { return cosf(x); }
// cos(2 pi u) for u in [0,1): FP64 keeps the reference's cos(2*M_PI*u)
// (heatbath.c:56); FP32 uses cospi, which needs no argument reduction
__device__ inline double mcos2pi(double u) { return cos(2 * 3.14159265358979323846 * u); }
__device__ inline float mcos2pi(float u) { return cospif(2.0f * u); }
__device__ inline double msin(double x) { return sin(x); }
__device__ inline float msin(float x) { return sinf(x); }
__device__ inline double mcbrt(double x) { return cbrt(x); }
__device__ inline float mcbrt(float x) { return cbrtf(x); }
__device__ inline double matan2(double y, double x) { return atan2(y, x); }
__device__ inline float matan2(float y, float x) { return atan2f(y, x); }
__device__ inline double mabs(double x) { return fabs(x); }
__device__ inline float mabs(float x) { return fabsf(x); }

// ---------------------------------------------------------------------------
// storage types and quaternions.  q = (a, b, c, d) is a + i(b s1 + c s2 + d s3)
// (su2u1.c:7-31); qmul is the product of the reference's su2rot().
// ---------------------------------------------------------------------------
struct __align__(32) D4 { double x, y, z, w; };
struct __align__(16) F4 { float x, y, z, w; };
template <typename R> struct V4T;
template <> struct V4T<double> { using T = D4; };
template <> struct V4T<float> { using T = F4; };
template <typename R> using V4 = typename V4T<R>::T;

template <typename R>
struct Q {
  R a, b, c, d;
};

template <typename R>
__device__ inline Q<R> ld4(const V4<R>* p, int i) {
  V4<R> v = p[i];
  return Q<R>{v.x, v.y, v.z, v.w};
}
// A load through the read-only data path, for values no thread writes during
// the launch (a pass's neighbours of the other parity, the fields it does not
// update); FP32 4-vectors as one 16-byte load, FP64 through the plain path.
// Units that define SU2_COHERENT_LOADS (the persistent sweep kernel, whose
// later passes read what its earlier passes wrote) use the plain path, since
// the read-only path is not coherent with writes made during the launch.
template <typename R>
__device__ inline Q<R> ldro4(const V4<R>* p, int i) {
#ifdef SU2_COHERENT_LOADS
  return ld4<R>(p, i);
#else
  if constexpr (sizeof(R) == 4) {
    float4 v = __ldg((const float4*)p + i);
    return Q<R>{v.x, v.y, v.z, v.w};
  } else {
    return ld4<R>(p, i);
  }
#endif
}
template <typename R>
__device__ inline void st4(V4<R>* p, int i, const Q<R>& q) {
  V4<R> v;
  v.x = q.a;
  v.y = q.b;
  v.z = q.c;
  v.w = q.d;
  p[i] = v;
}

__device__ inline float fmaR(float a, float b, float c) { return fmaf(a, b, c); }
__device__ inline double fmaR(double a, double b, double c) { return fma(a, b, c); }
// quaternion product x y (the SU(2) product in the reference's 4-real
// parametrisation, su2rot su2u1.c:60-71) with explicit fused multiply-adds,
// which fixes the rounding of every step in the source
template <typename R>
__device__ inline Q<R> qmul(const Q<R>& x, const Q<R>& y) {
  Q<R> r;
  r.a = fmaR(x.a, y.a, -fmaR(x.b, y.b, fmaR(x.c, y.c, x.d * y.d)));
  r.b = fmaR(x.a, y.b, fmaR(y.a, x.b, -fmaR(x.c, y.d, -(x.d * y.c))));
  r.c = fmaR(x.a, y.c, fmaR(y.a, x.c, -fmaR(x.d, y.b, -(x.b * y.d))));
  r.d = fmaR(x.a, y.d, fmaR(y.a, x.d, -fmaR(x.b, y.c, -(x.c * y.b))));
  return r;
}
template <typename R>
__device__ inline Q<R> qdag(const Q<R>& x) {
  return Q<R>{x.a, -x.b, -x.c, -x.d};
}
template <typename R>
__device__ inline Q<R> qadd(const Q<R>& x, const Q<R>& y) {
  return Q<R>{x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d};
}
template <typename R>
__device__ inline Q<R> qscale(const Q<R>& x, R s) {
  return Q<R>{x.a * s, x.b * s, x.c * s, x.d * s};
}
template <typename R>
__device__ inline R qsq(const Q<R>& x) {
  return x.a * x.a + x.b * x.b + x.c * x.c + x.d * x.d;
}
// scalar part of x*y
template <typename R>
__device__ inline R qdot0(const Q<R>& x, const Q<R>& y) {
  return x.a * y.a - x.b * y.b - x.c * y.c - x.d * y.d;
}
// e^{-i alpha sigma_3}
template <typename R>
__device__ inline Q<R> u1phase(R alpha) {
  return Q<R>{mcos(alpha), (R)0, (R)0, -msin(alpha)};
}

template <typename R>
struct V3 {
  R x, y, z;
};
// vec(u (0,b) u^dagger): the adjoint rotation of a triplet by a link.
// Written out with explicit fused multiply-adds: the zero real part of (0, b)
// and the real part of the result are never formed, and the rounding of every
// step is fixed by the source, so every kernel that rotates -- whatever it
// computes around the rotation -- gets the same bits.
template <typename R>
__device__ inline V3<R> qrot(const Q<R>& u, const V3<R>& b) {
  const R na = fmaR(u.d, b.z, fmaR(u.c, b.y, u.b * b.x));  // -(real part of u (0, b))
  const R px = fmaR(u.a, b.x, -fmaR(u.c, b.z, -(u.d * b.y)));
  const R py = fmaR(u.a, b.y, -fmaR(u.d, b.x, -(u.b * b.z)));
  const R pz = fmaR(u.a, b.z, -fmaR(u.b, b.y, -(u.c * b.x)));
  return V3<R>{fmaR(u.a, px, fmaR(na, u.b, fmaR(py, u.d, -(pz * u.c)))),
               fmaR(u.a, py, fmaR(na, u.c, fmaR(pz, u.b, -(px * u.d)))),
               fmaR(u.a, pz, fmaR(na, u.d, fmaR(px, u.c, -(py * u.b))))};
}
template <typename R>
__device__ inline R dot3(const V3<R>& a, const V3<R>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// ---------------------------------------------------------------------------
// device field views: parity-split SoA.  link[d][i], u1[d][i], phi[h][i],
// trip[k][i] (three planes), sing[i]; i is the EVEN-first site index.
// ---------------------------------------------------------------------------
template <typename R>
struct Fields {
  V4<R>* link[3];
  R* u1[3];
  V4<R>* phi[2];
  R* trip[3];
  R* sing;
};

// field pointers by a runtime direction / doublet index, chosen with selects
template <typename R>
__device__ inline V4<R>* lk(const Fields<R>& f, int d) {
  return d == 0 ? f.link[0] : (d == 1 ? f.link[1] : f.link[2]);
}
template <typename R>
__device__ inline R* a1p(const Fields<R>& f, int d) {
  return d == 0 ? f.u1[0] : (d == 1 ? f.u1[1] : f.u1[2]);
}
template <typename R>
__device__ inline V4<R>* php(const Fields<R>& f, int h) {
  return h == 0 ? f.phi[0] : f.phi[1];
}

template <typename R>
__device__ inline V3<R> ld3(const Fields<R>& f, int i) {
  return V3<R>{f.trip[0][i], f.trip[1][i], f.trip[2][i]};
}
// the triplet of a site no thread writes during the launch (see ldro4)
template <typename R>
__device__ inline V3<R> ldro3(const Fields<R>& f, int i) {
#ifdef SU2_COHERENT_LOADS
  return ld3(f, i);
#else
  return V3<R>{__ldg(f.trip[0] + i), __ldg(f.trip[1] + i), __ldg(f.trip[2] + i)};
#endif
}
template <typename R>
__device__ inline void st3(const Fields<R>& f, int i, const V3<R>& v) {
  f.trip[0][i] = v.x;
  f.trip[1][i] = v.y;
  f.trip[2][i] = v.z;
}

// couplings (reference params, su2.h:76-181), kept in double on the host
struct Coup {
  double beta, msq, lam;
  double msqT, a2, b4;
  double betau1, r_u1;
  double b1s, msqs, b3s, b4s, a1s, a2s;
  double msq2, m12re, m12im, lam2, lam3, lam4, lam5re, lam5im, lam6re, lam6im, lam7re, lam7im;
  int content;
  int alg_link, alg_u1, alg_d, alg_t, alg_s;
};

// the couplings in the kernels' working precision, converted once on the
// host (a double-to-float conversion per use would run on the FP64 pipe)
template <typename R>
struct CoupT {
  R beta, msq, lam;
  R msqT, a2, b4;
  R betau1, r_u1;
  R b1s, msqs, b3s, b4s, a1s, a2s;
  R msq2, m12re, m12im, lam2, lam3, lam4, lam5re, lam5im, lam6re, lam6im, lam7re, lam7im;
  int content;
  int alg_link, alg_u1, alg_d, alg_t, alg_s;
};

template <typename R>
__host__ __device__ inline CoupT<R> coup_as(const Coup& c) {
  CoupT<R> r;
  r.beta = (R)c.beta; r.msq = (R)c.msq; r.lam = (R)c.lam;
  r.msqT = (R)c.msqT; r.a2 = (R)c.a2; r.b4 = (R)c.b4;
  r.betau1 = (R)c.betau1; r.r_u1 = (R)c.r_u1;
  r.b1s = (R)c.b1s; r.msqs = (R)c.msqs; r.b3s = (R)c.b3s; r.b4s = (R)c.b4s; r.a1s = (R)c.a1s; r.a2s = (R)c.a2s;
  r.msq2 = (R)c.msq2; r.m12re = (R)c.m12re; r.m12im = (R)c.m12im;
  r.lam2 = (R)c.lam2; r.lam3 = (R)c.lam3; r.lam4 = (R)c.lam4; r.lam5re = (R)c.lam5re; r.lam5im = (R)c.lam5im;
  r.lam6re = (R)c.lam6re; r.lam6im = (R)c.lam6im; r.lam7re = (R)c.lam7re; r.lam7im = (R)c.lam7im;
  r.content = c.content;
  r.alg_link = c.alg_link; r.alg_u1 = c.alg_u1; r.alg_d = c.alg_d; r.alg_t = c.alg_t; r.alg_s = c.alg_s;
  return r;
}

// device multicanonical state (weight struct, su2.h:235-274)
struct MucaDev {
  int orderparam, mode, do_acceptance, checks_per_sweep, bins, muca_count, update_interval, last_max;
  double param_value[2];
  double min, max, wrk_min, wrk_max, delta;
  double* pos;
  double* W;
  double* slope;
  double* b;
  int* hits;
  long long* gsum;
  long long* nsum;
  double* hgram;
  double* wold;  // scratch of the slow recursion
  int last_accept;
  int weight_updates;  // number of weight recursions done (host saves the file)
};

}  // namespace su2
