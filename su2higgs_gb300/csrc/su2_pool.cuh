// su2_pool.cuh -- kernels of a pool of independent chains (the batched form):
// one launch per half-sweep covers every chain of the pool.  Block b works on
// the tile (slot, t0) of its block table; the chain's descriptor (field
// pointers, geometry, couplings, random key, sweep counter, counters) is staged
// in shared memory once per block and the per-site update is the same device
// code as the single-chain kernels.  Chains may differ in lattice size and
// couplings; they share field content, precision and update recipe.
#pragma once

#include "su2_kernels.cuh"

namespace su2 {

template <typename R>
struct __align__(16) ChainDesc {
  Fields<R> f;
  Geom g;
  CoupT<R> cp;
  uint32_t k0, k1, chain;
  uint32_t* sweep;          // this chain's sweep counter (device word)
  unsigned long long* ctr;  // this chain's counters [24]
};

struct PoolArgs {
  const void* descs;  // ChainDesc<R>[nslots]
  const int2* tiles;  // (slot, first site of the tile inside the parity / lattice)
  int nslots;
  int parity, sub, alg;
  uint32_t pass;
  int* err;
};

// a tile whose slot lies outside the descriptor table (a corrupted table)
// is reported through the error flag and skipped by the whole block
__device__ inline bool bad_tile(const PoolArgs& a, int2 tile) {
  if ((unsigned)tile.x < (unsigned)a.nslots && tile.y >= 0) return false;
  if (threadIdx.x == 0) atomicOr(a.err, 2);
  return true;
}

template <typename R>
__device__ inline const ChainDesc<R>& stage_desc(const PoolArgs& a, int slot) {
  __shared__ __align__(16) unsigned char buf[sizeof(ChainDesc<R>)];
  const uint4* src = (const uint4*)((const ChainDesc<R>*)a.descs + slot);
  uint4* dst = (uint4*)buf;
  constexpr int N = (int)(sizeof(ChainDesc<R>) / sizeof(uint4));
  static_assert(sizeof(ChainDesc<R>) % sizeof(uint4) == 0, "descriptor must be a multiple of 16 bytes");
  for (int k = threadIdx.x; k < N; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  return *(const ChainDesc<R>*)buf;
}

template <typename R, int CC, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_link(PoolArgs a) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  const CoupT<R>& cp = d.cp;
  int t = tile.y + threadIdx.x;
  int acc = 0, cap = 0, err = 0;
  if (t < d.g.half) {
    int c[3];
    site_coords(d.g, a.parity, t, c);
    int i = a.parity * d.g.half + t;
    SiteRng<R> rng(RngKey{d.k0, d.k1, d.chain, d.sweep}, *d.sweep, (uint32_t)i, a.pass);
    if (a.alg == ALG_HEATBATH) acc = heatbath<R, CC>(d.f, d.g, cp, c, i, a.sub, rng, &cap, &err);
    else acc = metro_link<R, CC>(d.f, d.g, cp, c, i, a.sub, rng);
  }
  warp_count(d.ctr + 1, acc);
  warp_count(d.ctr + 22, cap);
  if (err) atomicOr(a.err, 1);
}

template <typename R, int CC, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_u1(PoolArgs a) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  int t = tile.y + threadIdx.x;
  int acc = 0;
  if (t < d.g.half) {
    int c[3];
    site_coords(d.g, a.parity, t, c);
    int i = a.parity * d.g.half + t;
    SiteRng<R> rng(RngKey{d.k0, d.k1, d.chain, d.sweep}, *d.sweep, (uint32_t)i, a.pass);
    acc = metro_u1<R, CC>(d.f, d.g, d.cp, c, i, a.sub, rng);
  }
  warp_count(d.ctr + 3, acc);
}

template <typename R, int CC, int FIELD, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_scalar(PoolArgs a) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  const CoupT<R>& cp = d.cp;
  int t = tile.y + threadIdx.x;
  int acc = 0, fb = 0;
  if (t < d.g.half) {
    int c[3];
    site_coords(d.g, a.parity, t, c);
    int i = a.parity * d.g.half + t;
    SiteRng<R> rng(RngKey{d.k0, d.k1, d.chain, d.sweep}, *d.sweep, (uint32_t)i, a.pass);
    constexpr int CCx = CC;
    if (FIELD == 0) {
      const bool orr = cp.alg_d == ALG_OR && !a.alg;
      if (orr) acc = SU2_HAS(CCx, cp.content, C_H2) ? overrelax_higgs2<R, CC>(d.f, d.g, cp, c, i, a.sub, rng, &fb)
                                                    : overrelax_doublet<R, CC>(d.f, d.g, cp, c, i, rng, &fb);
      else acc = metro_doublet<R, CC>(d.f, d.g, cp, c, i, a.sub, rng);
    } else if (FIELD == 1) {
      if (cp.alg_t == ALG_OR && !a.alg) acc = overrelax_triplet<R, CC>(d.f, d.g, cp, c, i, rng, &fb);
      else acc = metro_triplet<R, CC>(d.f, d.g, cp, c, i, rng);
    } else {
      if (cp.alg_s == ALG_OR && !a.alg) acc = overrelax_singlet<R, CC>(d.f, d.g, cp, c, i, rng, &fb);
      else acc = metro_singlet<R, CC>(d.f, d.g, cp, c, i, rng);
    }
  }
  int base_or = FIELD == 0 ? 10 + a.sub : (FIELD == 1 ? 15 : 19);
  int base_mt = FIELD == 0 ? 6 + a.sub : (FIELD == 1 ? 13 : 17);
  bool any_or = (FIELD == 0 ? cp.alg_d : (FIELD == 1 ? cp.alg_t : cp.alg_s)) == ALG_OR && !a.alg;
  warp_count(d.ctr + (any_or ? base_or : base_mt), acc);
  warp_count(d.ctr + 23, fb);
}

#ifdef SU2_WITH_GLOBAL
// every active chain's sweep counter + 1
__global__ void k_pool_next_sweep(uint32_t* const* sweeps, int n) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) *sweeps[k] += 1u;
}
#endif

// measurement over every chain: tiles over all V sites of each chain; the
// block sums go to partials[k][block] and are then reduced per chain
template <typename R, int CC>
__global__ void __launch_bounds__(BLOCK) k_pool_measure(PoolArgs a, const double* alpha_unused, double* partials) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  const CoupT<R>& cp = d.cp;
  const Fields<R>& f = d.f;
  const Geom& g = d.g;
  int t = tile.y + threadIdx.x;
  double m[NSUMS];
#pragma unroll
  for (int k = 0; k < NSUMS; k++) m[k] = 0.0;
  if (t < g.V) {
    int parity = t >= g.half;
    int i = t;
    int c[3];
    site_coords(g, parity, t - parity * g.half, c);
    R wl = 0;
    wl += ((R)1 - (R)0.5 * ptrace(f, g, c, i, 0, 1));
    wl += ((R)1 - (R)0.5 * ptrace(f, g, c, i, 0, 2));
    wl += ((R)1 - (R)0.5 * ptrace(f, g, c, i, 1, 2));
    wl = cp.beta * wl;
    double act = (double)wl;
    m[1] = (double)wl;
    if (SU2_HAS(CC, cp.content, C_U1)) {
      R u1w = local_u1wilson(f, g, cp, c, i);
      act += (double)u1w;
      m[2] = (double)u1w;
    }
    act += (double)higgspotential<R, CC>(f, cp, i);
    const int nh = SU2_HAS(CC, cp.content, C_H2) ? 2 : (SU2_HAS(CC, cp.content, C_H1) ? 1 : 0);
    for (int h = 0; h < nh; h++) {
      R mod = doubletsq(ld4<R>(php(f, h), i));
      R cov = covariant_doublet<R, CC>(f, g, cp, c, i, h);
      act += (double)cov;
      m[3 + 3 * h] = (double)cov;
      m[4 + 3 * h] = (double)mod;
      m[5 + 3 * h] = (double)(mod * mod);
    }
    if (SU2_HAS(CC, cp.content, C_T)) {
      R covt = covariant_triplet(f, g, c, i);
      act += (double)covt;
      V3<R> tr = ld3(f, i);
      R tm = tripletsq(tr);
      if (nh > 0) m[14] = (double)(doubletsq(ld4<R>(php(f, 0), i)) * tm);
      m[12] = (double)tm;
      m[13] = (double)(tm * tm);
      R hs = 0;
#pragma unroll
      for (int dd = 0; dd < 3; dd++) hs += hop_triplet_fwd(f, g, c, i, dd);
      m[11] = (double)hs;
      int c0[3], c1[3], c2[3];
      shift_coords(g, c, 0, 1, c0);
      shift_coords(g, c, 1, 1, c1);
      shift_coords(g, c, 2, 1, c2);
      int n0 = shifted(g, c, 0, 1), n1 = shifted(g, c, 1, 1), n2 = shifted(g, c, 2, 1);
      double q = 0.0;
      double B1 = (double)alpha_proj(f, g, cp, c, i, 1, 2), B2 = (double)alpha_proj(f, g, cp, c0, n0, 1, 2);
      q += B2 - B1;
      B1 = -(double)alpha_proj(f, g, cp, c, i, 0, 2);
      B2 = -(double)alpha_proj(f, g, cp, c1, n1, 0, 2);
      q += B2 - B1;
      B1 = (double)alpha_proj(f, g, cp, c, i, 0, 1);
      B2 = (double)alpha_proj(f, g, cp, c2, n2, 0, 1);
      q += B2 - B1;
      m[15] = q;
      m[16] = fabs(q);
    }
    if (nh == 2) {
      Q<R> h1 = ld4<R>(php(f, 0), i), h2 = ld4<R>(php(f, 1), i);
      m[9] = (double)((R)0.5 * (h1.a * h2.a + h1.b * h2.b + h1.c * h2.c + h1.d * h2.d));
      m[10] = (double)((R)0.5 * (h1.d * h2.a + h1.c * h2.b - h1.b * h2.c - h1.a * h2.d));
    }
    if (SU2_HAS(CC, cp.content, C_S)) {
      R S = f.sing[i];
      R kin = (R)3 * S * S;
      R scov = 0;
#pragma unroll
      for (int dd = 0; dd < 3; dd++) {
        R Sn = f.sing[shifted(g, c, dd, 1)];
        kin -= S * Sn;
        scov += S * S - S * Sn;
      }
      act += (double)kin;
      m[17] = (double)scov;
      m[18] = (double)S;
      m[19] = (double)(S * S);
      m[20] = (double)(S * S * S);
      m[21] = (double)(S * S * S * S);
      if (nh == 1) {
        R mod = doubletsq(ld4<R>(php(f, 0), i));
        m[22] = (double)(mod * S);
        m[23] = (double)(mod * S * S);
      }
    }
    m[0] = act;
  }
  __shared__ double sm[BLOCK / 32][NSUMS];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NSUMS; k++) {
    if (!sum_active<CC>(k, cp.content)) continue;
    double v = m[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sm[w][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NSUMS) {
    double v = 0.0;
    if (sum_active<CC>(threadIdx.x, cp.content))
#pragma unroll
      for (int ww = 0; ww < BLOCK / 32; ww++) v += sm[ww][threadIdx.x];
    partials[threadIdx.x * gridDim.x + blockIdx.x] = v;
  }
}

#ifdef SU2_WITH_GLOBAL
// per-chain sums: chain k owns blocks [first[k], first[k+1]) of the measure
// tiles; one block per chain, fixed summation order
__global__ void k_pool_reduce(const double* partials, int nblocks, const int* first, double* out) {
  __shared__ double red[128];
  int k = blockIdx.x;
  int b0 = first[k], b1 = first[k + 1];
  for (int s = 0; s < NSUMS; s++) {
    const double* row = partials + (size_t)s * nblocks;
    double v = 0.0;
    for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) v += row[b];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
      if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)k * NSUMS + s] = red[0];
    __syncthreads();
  }
}

#endif  // SU2_WITH_GLOBAL

}  // namespace su2
