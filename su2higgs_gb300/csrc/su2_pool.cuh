// su2_pool.cuh -- kernels of a pool of independent chains (the batched form).
// Two ways to sweep: one launch per half-sweep covering every chain (block b
// works on the tile (slot, t0) of its block table), or the persistent
// work-list kernel k_pool_persist running whole sweeps of every chain in one
// launch.  Either way a block stages its chain's descriptor (field pointers,
// geometry, couplings, random key, sweep counter, counters) in shared memory
// and runs the same per-tile functions, whose per-site update is the device
// code of the single-chain kernels.  Chains may differ in lattice size and
// couplings; they share field content, precision and update recipe.
#pragma once

#include "su2_kernels.cuh"
#include "su2_ops.h"

namespace su2 {

template <typename R>
struct __align__(16) ChainDesc {
  Fields<R> f;
  Geom g;
  CoupT<R> cp;
  uint32_t k0, k1, chain;
  uint32_t* sweep;          // this chain's sweep counter (device word)
  unsigned long long* ctr;  // this chain's counters [24]
  // multicanonical chains: the weight, the backup of the updated field
  // (indexed like the field), the order parameter's sums over the 32-site
  // warps of a checked half-sweep, the order parameter (0: no weight in
  // this chain, or none checked in these passes)
  MucaDev* muca;
  void* mbackup;
  double* mpart;
  int mop;
  int mpad[3];
};

// whether a half-sweep of `field` (0 doublet `h`, 1 triplet) ends with a
// global multicanonical check of order parameter op (update.c:82-229)
__device__ inline bool muca_checked(int field, int h, int op) {
  if (field == 0) return (h == 0 && (op == 1 || op == 3)) || (h == 1 && op == 4);
  if (field == 1) return op == 2 || op == 3;
  return false;
}

// a chain-wide quantity read while other blocks of the launch write: past L1
template <typename R>
__device__ inline Q<R> ldcg4(const V4<R>* p, int i) {
  if constexpr (sizeof(R) == 4) {
    const float4 v = __ldcg((const float4*)p + i);
    return Q<R>{v.x, v.y, v.z, v.w};
  } else {
    const double2 a = __ldcg((const double2*)p + 2 * i), b = __ldcg((const double2*)p + 2 * i + 1);
    return Q<R>{a.x, a.y, b.x, b.y};
  }
}
// The multicanonical check of a pool chain's checked half-sweep
// (muca_check, update.c:13-30, with one check per half-sweep) takes three
// steps.  The update tiles keep the old values in the backup and leave the
// order parameter's sum over each warp's 32 sites in mpart (a fixed-order
// warp sum: the same values whatever the launch shape), with no barrier or
// fence.  The decide pass sums the warp sums in a fixed order (fixed_sum64)
// and decides (muca_decide_block), once per chain.  The restore pass puts a
// rejected half back.
template <typename R>
__device__ inline void muca_warp_partial(const ChainDesc<R>& d, int t0, double opv) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) opv += __shfl_down_sync(0xffffffffu, opv, o);
  const int w0 = t0 + (int)(threadIdx.x & ~31u);
  if ((threadIdx.x & 31) == 0 && w0 < d.g.half) d.mpart[w0 >> 5] = opv;
}

// the decision of a chain's checked half-sweep, made by the block that has
// the chain's first tile (t0 == 0); fields, partial sums and weight are
// read past L1
template <typename R, int BS>
__device__ __noinline__ void tile_decide(const ChainDesc<R>& d, int field, int h, int parity, uint32_t pass,
                                         uint32_t sweep, int t0) {
  if (t0 != 0 || !d.mop || !muca_checked(field, h, d.mop)) return;
  const MucaPre pre = muca_preload(d.muca);
  const double tot = fixed_sum64(d.mpart, (d.g.half + 31) / 32) / (double)d.g.V;
  const RngKey rk{d.k0, d.k1, d.chain, nullptr};
  muca_decide_block(d.muca, pre, tot, parity, rk, pass, 0u, sweep, d.ctr);
}

// site t of the parity back from the backup
template <typename R>
__device__ inline void restore_site(const ChainDesc<R>& d, int field, int h, int parity, int t) {
  const int i = parity * d.g.half + t;
  if (field == 0) {
    st4<R>(php(d.f, h), i, ldcg4<R>((const V4<R>*)d.mbackup, i));
  } else {
    const R* b = (const R*)d.mbackup;
    st3(d.f, i, V3<R>{__ldcg(b + 3 * i), __ldcg(b + 3 * i + 1), __ldcg(b + 3 * i + 2)});
  }
}

// whether chain d's check of this half-sweep rejected (the flag is read
// past L1: the decide pass wrote it)
template <typename R>
__device__ inline bool muca_rejected(const ChainDesc<R>& d, int field, int h) {
  return d.mop && muca_checked(field, h, d.mop) && !*(volatile const int*)&d.muca->last_accept;
}

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
__device__ inline const ChainDesc<R>& stage_desc_slot(const void* descs, int slot) {
  __shared__ __align__(16) unsigned char buf[sizeof(ChainDesc<R>)];
  const uint4* src = (const uint4*)((const ChainDesc<R>*)descs + slot);
  uint4* dst = (uint4*)buf;
  constexpr int N = (int)(sizeof(ChainDesc<R>) / sizeof(uint4));
  static_assert(sizeof(ChainDesc<R>) % sizeof(uint4) == 0, "descriptor must be a multiple of 16 bytes");
  for (int k = threadIdx.x; k < N; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  return *(const ChainDesc<R>*)buf;
}
template <typename R>
__device__ inline const ChainDesc<R>& stage_desc(const PoolArgs& a, int slot) {
  return stage_desc_slot<R>(a.descs, slot);
}

// the restore pass's tile in the persistent sweep
template <typename R, int BS>
__device__ __noinline__ void tile_restore(const ChainDesc<R>& d, int field, int h, int parity, int t0) {
  if (!muca_rejected(d, field, h)) return;
  const int t = t0 + threadIdx.x;
  if (t < d.g.half) restore_site(d, field, h, parity, t);
}

// The per-tile work of the update passes: the sites [t0, t0 + blockDim.x)
// of one parity of the chain d, with the chain's random stream at sweep
// `sweep` and pass `pass`.  Every thread of the block calls these (the
// counters are reduced per warp).  They are functions of their own, not
// inlined, with one instance per launch shape (BS, MINB): the one-launch-
// per-pass kernels and the persistent kernel then run the same compiled
// arithmetic (the compiler cannot fuse multiply-adds differently in the
// two contexts) and give the same fields bit for bit.
template <typename R, int CC, int MU, int BS, int MINB>
__device__ __noinline__ void tile_link(const ChainDesc<R>& d, int parity, int alg, uint32_t pass, uint32_t sweep, int t0,
                                 int* errp) {
  int t = t0 + threadIdx.x;
  int acc = 0, cap = 0, err = 0;
  if (t < d.g.half) {
    int c[3];
    site_coords(d.g, parity, t, c);
    int i = parity * d.g.half + t;
    SiteRng<R> rng(RngKey{d.k0, d.k1, d.chain, d.sweep}, sweep, (uint32_t)i, pass);
    if (alg == ALG_HEATBATH) acc = heatbath<R, CC>(d.f, d.g, d.cp, c, i, MU, rng, &cap, &err);
    else acc = metro_link<R, CC>(d.f, d.g, d.cp, c, i, MU, rng);
  }
  warp_count(d.ctr + 1, acc);
  warp_count(d.ctr + 22, cap);
  if (err) atomicOr(errp, 1);
}

template <typename R, int CC, int MU, int BS, int MINB>
__device__ __noinline__ void tile_u1(const ChainDesc<R>& d, int parity, uint32_t pass, uint32_t sweep, int t0) {
  int t = t0 + threadIdx.x;
  int acc = 0;
  if (t < d.g.half) {
    int c[3];
    site_coords(d.g, parity, t, c);
    int i = parity * d.g.half + t;
    SiteRng<R> rng(RngKey{d.k0, d.k1, d.chain, d.sweep}, sweep, (uint32_t)i, pass);
    acc = metro_u1<R, CC>(d.f, d.g, d.cp, c, i, MU, rng);
  }
  warp_count(d.ctr + 3, acc);
}

// FIELD 0 doublet `sub`, 1 triplet, 2 singlet; force: the pass's forced
// Metropolis flag (the last scalar sweep of an overrelaxation field).
// CHECKED: a multicanonical chain's checked half-sweep, which keeps the old
// values in the backup and sums the order parameter over the new ones (an
// instance of its own, so the plain update carries none of it)
template <typename R, int CC, int FIELD, int BS, int MINB, bool CHECKED>
__device__ __noinline__ void tile_scalar(const ChainDesc<R>& d, int parity, int sub, int force, uint32_t pass,
                                   uint32_t sweep, int t0) {
  const CoupT<R>& cp = d.cp;
  int t = t0 + threadIdx.x;
  int acc = 0, fb = 0;
  constexpr bool checked = CHECKED && FIELD != 2;
  double opv = 0.0;
  if (t < d.g.half) {
    int c[3];
    site_coords(d.g, parity, t, c);
    int i = parity * d.g.half + t;
    if (checked) {
      if (FIELD == 0) {
        ((V4<R>*)d.mbackup)[i] = php(d.f, sub)[i];
      } else {
        R* b = (R*)d.mbackup;
        b[3 * i] = d.f.trip[0][i]; b[3 * i + 1] = d.f.trip[1][i]; b[3 * i + 2] = d.f.trip[2][i];
      }
    }
    SiteRng<R> rng(RngKey{d.k0, d.k1, d.chain, d.sweep}, sweep, (uint32_t)i, pass);
    constexpr int CCx = CC;
    if (FIELD == 0) {
      const bool orr = cp.alg_d == ALG_OR && !force;
      if (orr) acc = SU2_HAS(CCx, cp.content, C_H2) ? overrelax_higgs2<R, CC>(d.f, d.g, cp, c, i, sub, rng, &fb)
                                                    : overrelax_doublet<R, CC>(d.f, d.g, cp, c, i, rng, &fb);
      else acc = metro_doublet<R, CC>(d.f, d.g, cp, c, i, sub, rng);
    } else if (FIELD == 1) {
      if (cp.alg_t == ALG_OR && !force) acc = overrelax_triplet<R, CC>(d.f, d.g, cp, c, i, rng, &fb);
      else acc = metro_triplet<R, CC>(d.f, d.g, cp, c, i, rng);
    } else {
      if (cp.alg_s == ALG_OR && !force) acc = overrelax_singlet<R, CC>(d.f, d.g, cp, c, i, rng, &fb);
      else acc = metro_singlet<R, CC>(d.f, d.g, cp, c, i, rng);
    }
    if (checked) opv = orderparam_site<R>(d.f, d.mop, i);
  }
  if (checked) muca_warp_partial(d, t0, opv);
  int base_or = FIELD == 0 ? 10 + sub : (FIELD == 1 ? 15 : 19);
  int base_mt = FIELD == 0 ? 6 + sub : (FIELD == 1 ? 13 : 17);
  bool any_or = (FIELD == 0 ? cp.alg_d : (FIELD == 1 ? cp.alg_t : cp.alg_s)) == ALG_OR && !force;
  warp_count(d.ctr + (any_or ? base_or : base_mt), acc);
  warp_count(d.ctr + 23, fb);
}

template <typename R, int CC, int FIELD, int BS, int MINB>
__device__ __noinline__ void tile_scalar_any(const ChainDesc<R>& d, int parity, int sub, int force, uint32_t pass,
                                       uint32_t sweep, int t0) {
  if (FIELD != 2 && d.mop != 0 && muca_checked(FIELD, sub, d.mop))
    tile_scalar<R, CC, FIELD, BS, MINB, FIELD != 2>(d, parity, sub, force, pass, sweep, t0);
  else
    tile_scalar<R, CC, FIELD, BS, MINB, false>(d, parity, sub, force, pass, sweep, t0);
}

// one launch per pass: block b works on tile b of the table
template <typename R, int CC, int MU, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_link(PoolArgs a) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  tile_link<R, CC, MU, BS, MINB>(d, a.parity, a.alg, a.pass, *d.sweep, tile.y, a.err);
}

template <typename R, int CC, int MU, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_u1(PoolArgs a) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  tile_u1<R, CC, MU, BS, MINB>(d, a.parity, a.pass, *d.sweep, tile.y);
}

template <typename R, int CC, int FIELD, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_scalar(PoolArgs a) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  tile_scalar_any<R, CC, FIELD, BS, MINB>(d, a.parity, a.sub, a.alg, a.pass, *d.sweep, tile.y);
}

// The decide and restore passes with one launch per pass, over the pool's
// multicanonical chains (mslots, nmuca of them): sub = the doublet, alg = the
// field (0 doublet, 1 triplet) of the checked half-sweep before them.
// Decide: one block per chain.  Restore: `kb` blocks per chain, which read
// the chain's flag in place and leave at once where the check accepted.
template <typename R, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_decide(PoolArgs a, const int* mslots) {
  const int slot = mslots[blockIdx.x];
  if ((unsigned)slot >= (unsigned)a.nslots) {
    if (threadIdx.x == 0) atomicOr(a.err, 2);
    return;
  }
  const ChainDesc<R>& d = stage_desc<R>(a, slot);
  tile_decide<R, BS>(d, a.alg, a.sub, a.parity, a.pass, *d.sweep, 0);
}

template <typename R, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_pool_restore(PoolArgs a, const int* mslots, int kb) {
  const int c = blockIdx.x / kb, b = blockIdx.x - c * kb;
  const int slot = mslots[c];
  if ((unsigned)slot >= (unsigned)a.nslots) {
    if (threadIdx.x == 0 && b == 0) atomicOr(a.err, 2);
    return;
  }
  const ChainDesc<R>& d = ((const ChainDesc<R>*)a.descs)[slot];
  if (!muca_rejected(d, a.alg, a.sub)) return;
  for (int t = b * BS + threadIdx.x; t < d.g.half; t += kb * BS) restore_site(d, a.alg, a.sub, a.parity, t);
}

// ---------------------------------------------------------------------------
// The persistent sweep: one launch runs `nsweeps` sweeps of every chain of
// the segment table.  A segment is up to `seg` consecutive 128-site tiles of
// one parity of one chain.  The work list is (sweep, pass, segment) in that
// order; each block takes the next item from an atomic counter until the
// list is done, and runs the segment's tiles one after the other.  A segment
// of pass g of chain c needs pass g-1 of chain c finished, which a per-chain
// count of finished segments says (chain c has passed g-1 when the count
// reaches g x its segments; a segment of pass g cannot finish before that,
// so the count is exact).  Chains do not wait for each other, so the passes
// of different chains overlap and no pass drains the GPU before the next.
// An item depends only on items earlier in the list, which blocks already
// running hold, so the launch needs no co-residency: the earliest unfinished
// item always has its inputs.  The wait is bounded: after spin_limit polls
// (or at once once another block has given up) the block records error bit
// 4, skips the item's work (its fields stay as they were) and counts it as
// finished; from then on every item is skipped, so the launch ends within
// about one wait and no item runs on inputs of the wrong pass.
// Fields are read with coherent loads (SU2_COHERENT_LOADS): later passes read
// what earlier passes of the same launch wrote.
// ---------------------------------------------------------------------------
constexpr int PERSIST_MAX_PASSES = 64;

// one pass of the sweep recipe: kind 0 links, 1 U(1), 2 doublet, 3 triplet,
// 4 singlet; in pools with multicanonical chains a doublet / triplet pass is
// followed by 6, the multicanonical decision, and 5, the restore; sub: the
// direction (links, U(1)) or the doublet; alg: the link algorithm of a link
// pass, the forced Metropolis flag of a scalar pass (as PoolArgs.alg), the
// field (0 doublet, 1 triplet) of a decide / restore pass; pass: the pass
// number within the sweep (that of the checked pass, for decide / restore)
struct PassDesc {
  uint8_t kind, parity, sub, alg;
  uint32_t pass;
};

struct PersistArgs {
  const void* descs;   // ChainDesc<R>[nslots]
  const int4* tiles;   // (slot, t0, the chain's segment count, 0) of every segment of one parity of
                       // every chain, chain by chain
  int ntiles, nslots;  // ntiles: segments in the table
  int seg;             // tiles per segment (the last segment of a chain may have fewer)
  int npasses, nsweeps;
  unsigned first_item;  // the work list starts here (0 in a sweep)
  int spin_limit;       // polls of a dependency before giving up
  unsigned* head;       // the work counter, 0 at launch
  unsigned* done;       // finished tiles per slot, 0 at launch
  int* err;
  PassDesc passes[PERSIST_MAX_PASSES];
};

#ifdef SU2_COHERENT_LOADS
__device__ inline unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// one tile of pass p (the tile functions are not inlined: each keeps the
// kernel's register budget to itself).  MUCA: the instance for pools with
// multicanonical chains (checked half-sweeps and restore passes); the other
// carries none of that code.
template <typename R, int CC, int BS, int MINB, bool MUCA>
__device__ inline void persist_tile(const ChainDesc<R>& d, PassDesc p, uint32_t sweep, int t0, int* errp) {
  switch (p.kind) {
    case 0:
      if (p.sub == 0) tile_link<R, CC, 0, BS, MINB>(d, p.parity, p.alg, p.pass, sweep, t0, errp);
      else if (p.sub == 1) tile_link<R, CC, 1, BS, MINB>(d, p.parity, p.alg, p.pass, sweep, t0, errp);
      else tile_link<R, CC, 2, BS, MINB>(d, p.parity, p.alg, p.pass, sweep, t0, errp);
      break;
    case 1:
      if (SU2_HAS(CC, d.cp.content, C_U1)) {
        if (p.sub == 0) tile_u1<R, CC, 0, BS, MINB>(d, p.parity, p.pass, sweep, t0);
        else if (p.sub == 1) tile_u1<R, CC, 1, BS, MINB>(d, p.parity, p.pass, sweep, t0);
        else tile_u1<R, CC, 2, BS, MINB>(d, p.parity, p.pass, sweep, t0);
      }
      break;
    case 2:
      if (SU2_HAS(CC, d.cp.content, C_H1 | C_H2)) {
        if (MUCA) tile_scalar_any<R, CC, 0, BS, MINB>(d, p.parity, p.sub, p.alg, p.pass, sweep, t0);
        else tile_scalar<R, CC, 0, BS, MINB, false>(d, p.parity, p.sub, p.alg, p.pass, sweep, t0);
      }
      break;
    case 3:
      if (SU2_HAS(CC, d.cp.content, C_T)) {
        if (MUCA) tile_scalar_any<R, CC, 1, BS, MINB>(d, p.parity, 0, p.alg, p.pass, sweep, t0);
        else tile_scalar<R, CC, 1, BS, MINB, false>(d, p.parity, 0, p.alg, p.pass, sweep, t0);
      }
      break;
    case 5:
      if (MUCA) tile_restore<R, BS>(d, p.alg, p.sub, p.parity, t0);
      break;
    case 6:
      if (MUCA) tile_decide<R, BS>(d, p.alg, p.sub, p.parity, p.pass, sweep, t0);
      break;
    default:
      if (SU2_HAS(CC, d.cp.content, C_S)) tile_scalar<R, CC, 2, BS, MINB, false>(d, p.parity, 0, p.alg, p.pass, sweep, t0);
  }
}

template <typename R, int CC, int BS, int MINB, bool MUCA>
__global__ void __launch_bounds__(BS, MINB) k_pool_persist(PersistArgs a) {
  __shared__ unsigned s_item;
  __shared__ int4 s_tile, s_next;
  __shared__ int s_go;
  __shared__ __align__(16) unsigned char dbuf[sizeof(ChainDesc<R>)];
  constexpr int NDESC = (int)(sizeof(ChainDesc<R>) / sizeof(uint4));
  static_assert(sizeof(ChainDesc<R>) % sizeof(uint4) == 0, "descriptor must be a multiple of 16 bytes");
  const unsigned nt = (unsigned)a.ntiles;
  const unsigned total = nt * (unsigned)(a.npasses * a.nsweeps);
  // thread 0 keeps the next item (and its table entry in s_next), fetched
  // while the current item runs
  unsigned next = 0;
  if (threadIdx.x == 0) {
    next = atomicAdd(a.head, 1u) + a.first_item;
    if (next < total) s_next = a.tiles[next % nt];
  }
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = next;
      s_tile = s_next;
      if (next < total) next = atomicAdd(a.head, 1u) + a.first_item;
    }
    __syncthreads();
    const unsigned q = s_item;
    if (q >= total) break;
    const int4 tile = s_tile;
    const unsigned g = q / nt;
    const unsigned s = g / (unsigned)a.npasses, k = g - s * (unsigned)a.npasses;
    const bool bad = (unsigned)tile.x >= (unsigned)a.nslots || tile.y < 0;
    if (!bad) {
      // the chain's descriptor, copied by the block while thread 0 checks
      // that the chain has finished pass g-1 (g x its segments done)
      const uint4* src = (const uint4*)((const ChainDesc<R>*)a.descs + tile.x);
      for (int i = threadIdx.x; i < NDESC; i += BS) ((uint4*)dbuf)[i] = src[i];
      if (threadIdx.x == 0) {
        const unsigned need = g * (unsigned)tile.z;
        int go = 1;
        if (need) {
          int polls = 0;
          while (ld_acquire_gpu(a.done + tile.x) < need) {
            // give up after spin_limit polls, or at once when another block
            // already gave up (the launch then ends within one wait)
            if (++polls > a.spin_limit || (*(volatile int*)a.err & 4)) {
              atomicOr(a.err, 4);
              go = 0;
              break;
            }
            __nanosleep(64);
          }
        }
        // once any wait has given up, no item runs: the counts of skipped
        // items would otherwise satisfy later dependencies out of order
        if (*(volatile int*)a.err & 4) go = 0;
        s_go = go;
      }
    } else if (threadIdx.x == 0) {
      atomicOr(a.err, 2);  // a corrupted table: the item is dropped (dependants time out)
      s_go = 0;
    }
    if (threadIdx.x == 0 && next < total) s_next = a.tiles[next % nt];
    __syncthreads();
    if (s_go) {
      const ChainDesc<R>& d = *(const ChainDesc<R>*)dbuf;
      const PassDesc p = a.passes[k];
      const uint32_t sweep = *d.sweep + s;
      for (int j = 0, t0 = tile.y; j < a.seg && t0 < d.g.half; j++, t0 += BS)
        persist_tile<R, CC, BS, MINB, MUCA>(d, p, sweep, t0, a.err);
    }
    __syncthreads();
    if (threadIdx.x == 0 && !bad) {
      __threadfence();
      atomicAdd(a.done + tile.x, 1u);
    }
  }
}
#endif  // SU2_COHERENT_LOADS

#ifdef SU2_WITH_GLOBAL
// every active chain's sweep counter + inc
__global__ void k_pool_next_sweep(uint32_t* const* sweeps, int n, uint32_t inc) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) *sweeps[k] += inc;
}
#endif

// measurement over every chain: tiles of MEAS_TILE sites of each chain
// (MEAS_SPT per thread); the block sums go to partials[k][block] and are then
// reduced per chain.  The magnetic charge's projections are computed where
// they are needed (no per-chain scratch planes).
template <typename R, int CC>
__global__ void __launch_bounds__(BLOCK) k_pool_measure(PoolArgs a, double* partials) {
  int2 tile = a.tiles[blockIdx.x];
  if (bad_tile(a, tile)) return;
  const ChainDesc<R>& d = stage_desc<R>(a, tile.x);
  double m[NSUMS];
#pragma unroll
  for (int k = 0; k < NSUMS; k++) m[k] = 0.0;
  for (int j = 0; j < MEAS_SPT; j++) {
    int t = tile.y + j * BLOCK + threadIdx.x;
    if (t < d.g.V) measure_site<R, CC>(d.f, d.g, d.cp, t, AlphaOnTheFly{}, m);
  }
  block_sums_out<CC>(m, d.cp.content, partials, gridDim.x, blockIdx.x);
}

// Field conversion of many chains in one launch: block row blockIdx.y is
// chain item y, its blocks stride over the chain's sites; each site moves all
// the chain's fields between the host layout (FP64, [V][components] per field
// in staging memory) and the device fields, with the conversions of
// k_import / k_export.
template <typename R>
__global__ void __launch_bounds__(256) k_pool_convert(const void* descs, const ConvItem* items, double* stg,
                                                      int to_device) {
  const ConvItem it = items[blockIdx.y];
  const ChainDesc<R>& d = ((const ChainDesc<R>*)descs)[it.slot];
  const Fields<R> f = d.f;
  const long long V = d.g.V;
  long long o = it.off;
  const long long o_link = o;
  if (it.mask & 1) o += 12 * V;
  const long long o_u1 = o;
  if (it.mask & 2) o += 3 * V;
  const long long o_d0 = o;
  if (it.mask & 4) o += 4 * V;
  const long long o_d1 = o;
  if (it.mask & 8) o += 4 * V;
  const long long o_tr = o;
  if (it.mask & 16) o += 3 * V;
  const long long o_s = o;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < V; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)t;
    if (it.mask & 1)
#pragma unroll
      for (int dd = 0; dd < 3; dd++) {
        double* s = stg + o_link + (t * 3 + dd) * 4;
        if (to_device) {
          st4<R>(f.link[dd], i, Q<R>{(R)s[0], (R)s[1], (R)s[2], (R)s[3]});
        } else {
          Q<R> q = ld4<R>(f.link[dd], i);
          s[0] = q.a; s[1] = q.b; s[2] = q.c; s[3] = q.d;
        }
      }
    if (it.mask & 2)
#pragma unroll
      for (int dd = 0; dd < 3; dd++) {
        double* s = stg + o_u1 + t * 3 + dd;
        if (to_device) f.u1[dd][i] = (R)*s;
        else *s = f.u1[dd][i];
      }
#pragma unroll
    for (int h = 0; h < 2; h++)
      if (it.mask & (4 << h)) {
        double* s = stg + (h ? o_d1 : o_d0) + t * 4;
        if (to_device) {
          st4<R>(f.phi[h], i, Q<R>{(R)s[0], (R)s[1], (R)s[2], (R)s[3]});
        } else {
          Q<R> q = ld4<R>(f.phi[h], i);
          s[0] = q.a; s[1] = q.b; s[2] = q.c; s[3] = q.d;
        }
      }
    if (it.mask & 16) {
      double* s = stg + o_tr + t * 3;
      if (to_device) {
        st3(f, i, V3<R>{(R)s[0], (R)s[1], (R)s[2]});
      } else {
        V3<R> v = ld3(f, i);
        s[0] = v.x; s[1] = v.y; s[2] = v.z;
      }
    }
    if (it.mask & 32) {
      double* s = stg + o_s + t;
      if (to_device) f.sing[i] = (R)*s;
      else *s = f.sing[i];
    }
  }
}

#ifdef SU2_WITH_GLOBAL
// per-chain sums: chain k owns blocks [first[k], first[k+1]) - base of the
// measure tiles (base: the first block of a group of chains); one block per
// chain, fixed summation order
__global__ void k_pool_reduce(const double* partials, int nblocks, const int* first, int base, double* out) {
  __shared__ double red[128];
  int k = blockIdx.x;
  int b0 = first[k] - base, b1 = first[k + 1] - base;
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
