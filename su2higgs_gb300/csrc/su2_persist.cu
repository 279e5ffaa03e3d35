// su2_persist.cu -- the update kernels of pools (su2_pool.cuh) for one
// (precision, content): the one-launch-per-pass kernels of every launch
// shape and the persistent sweep kernel.  Compiled like su2_inst.cu with
// -DSU2_R / -DSU2_CC / -DSU2_PERSIST=<table name>.  Fields are read with
// coherent loads here (SU2_COHERENT_LOADS), which the persistent kernel
// needs; the per-pass kernels live in the same unit so that both modes call
// the same compiled per-tile functions and give the same fields bit for bit.
#define SU2_COHERENT_LOADS 1
#include "su2_pool.cuh"

namespace su2 {

using R = SU2_R;
constexpr int CCI = SU2_CC;
// the persistent kernel's shapes: those of launch variants 0 (128 threads,
// 8 (FP32) / 4 (FP64) resident blocks per SM asked of the compiler) and 1
// (128 threads, 5 / 3 blocks: more registers, fewer warps)
constexpr int PBS = Variant<R, 0>::BS, PMB = Variant<R, 0>::MINB;
constexpr int PMB1 = Variant<R, 1>::MINB;
static_assert(Variant<R, 1>::BS == PBS, "persistent shapes share the tile size");

template <int V>
static void lp_link_v(const PoolArgs& a, unsigned nb, cudaStream_t st) {
  constexpr int BS = Variant<R, V>::BS, MB = Variant<R, V>::MINB;
  if (!nb) return;
  if (a.sub == 0) k_pool_link<R, CCI, 0, BS, MB><<<nb, BS, 0, st>>>(a);
  else if (a.sub == 1) k_pool_link<R, CCI, 1, BS, MB><<<nb, BS, 0, st>>>(a);
  else k_pool_link<R, CCI, 2, BS, MB><<<nb, BS, 0, st>>>(a);
}
template <int V>
static void lp_u1_v(const PoolArgs& a, unsigned nb, cudaStream_t st) {
  constexpr int BS = Variant<R, V>::BS, MB = Variant<R, V>::MINB;
  if (!nb) return;
  if (a.sub == 0) k_pool_u1<R, CCI, 0, BS, MB><<<nb, BS, 0, st>>>(a);
  else if (a.sub == 1) k_pool_u1<R, CCI, 1, BS, MB><<<nb, BS, 0, st>>>(a);
  else k_pool_u1<R, CCI, 2, BS, MB><<<nb, BS, 0, st>>>(a);
}
template <int V>
static void lp_scalar_v(int field, const PoolArgs& a, unsigned nb, cudaStream_t st) {
  constexpr int BS = Variant<R, V>::BS, MB = Variant<R, V>::MINB;
  if (!nb) return;
  if (field == 0) k_pool_scalar<R, CCI, 0, BS, MB><<<nb, BS, 0, st>>>(a);
  else if (field == 1) k_pool_scalar<R, CCI, 1, BS, MB><<<nb, BS, 0, st>>>(a);
  else k_pool_scalar<R, CCI, 2, BS, MB><<<nb, BS, 0, st>>>(a);
}
static void lp_link(int v, const PoolArgs& a, unsigned nb, cudaStream_t st) {
  switch (v) {
    case 1: lp_link_v<1>(a, nb, st); break;
    case 2: lp_link_v<2>(a, nb, st); break;
    case 3: lp_link_v<3>(a, nb, st); break;
    default: lp_link_v<0>(a, nb, st);
  }
}
static void lp_u1(int v, const PoolArgs& a, unsigned nb, cudaStream_t st) {
  switch (v) {
    case 1: lp_u1_v<1>(a, nb, st); break;
    case 2: lp_u1_v<2>(a, nb, st); break;
    case 3: lp_u1_v<3>(a, nb, st); break;
    default: lp_u1_v<0>(a, nb, st);
  }
}
static void lp_scalar(int v, int field, const PoolArgs& a, unsigned nb, cudaStream_t st) {
  switch (v) {
    case 1: lp_scalar_v<1>(field, a, nb, st); break;
    case 2: lp_scalar_v<2>(field, a, nb, st); break;
    case 3: lp_scalar_v<3>(field, a, nb, st); break;
    default: lp_scalar_v<0>(field, a, nb, st);
  }
}
static void lp_restore(const PoolArgs& a, const int* mslots, int n, int kb, cudaStream_t st) {
  if (n > 0) k_pool_restore<R, PBS, PMB><<<(unsigned)(n * kb), PBS, 0, st>>>(a, mslots, kb);
}
static void lp_decide(const PoolArgs& a, const int* mslots, int n, cudaStream_t st) {
  if (n > 0) k_pool_decide<R, PBS, PMB><<<(unsigned)n, PBS, 0, st>>>(a, mslots);
}
static void persist_launch(int shape, bool muca, const void* args, unsigned grid, cudaStream_t st) {
  if (!grid) return;
  const PersistArgs& a = *(const PersistArgs*)args;
  if (shape == 1) {
    if (muca) k_pool_persist<R, CCI, PBS, PMB1, true><<<grid, PBS, 0, st>>>(a);
    else k_pool_persist<R, CCI, PBS, PMB1, false><<<grid, PBS, 0, st>>>(a);
  } else {
    if (muca) k_pool_persist<R, CCI, PBS, PMB, true><<<grid, PBS, 0, st>>>(a);
    else k_pool_persist<R, CCI, PBS, PMB, false><<<grid, PBS, 0, st>>>(a);
  }
}

// resident blocks per SM of a shape: the smaller of its two instances
static int persist_blocks_per_sm(int shape) {
  int n0 = 0, n1 = 0;
  cudaError_t e0, e1;
  if (shape == 1) {
    e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, k_pool_persist<R, CCI, PBS, PMB1, false>, PBS, 0);
    e1 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_pool_persist<R, CCI, PBS, PMB1, true>, PBS, 0);
  } else {
    e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, k_pool_persist<R, CCI, PBS, PMB, false>, PBS, 0);
    e1 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_pool_persist<R, CCI, PBS, PMB, true>, PBS, 0);
  }
  return e0 == cudaSuccess && e1 == cudaSuccess ? (n0 < n1 ? n0 : n1) : 0;
}

const PoolOps SU2_PERSIST = {PBS, persist_launch, persist_blocks_per_sm, lp_link, lp_u1, lp_scalar, lp_restore,
                               lp_decide};

}  // namespace su2
