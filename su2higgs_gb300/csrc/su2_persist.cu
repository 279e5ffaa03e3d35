// su2_persist.cu -- the persistent sweep kernel of pools (k_pool_persist in
// su2_pool.cuh) for one (precision, content): compiled like su2_inst.cu with
// -DSU2_R / -DSU2_CC / -DSU2_PERSIST=<table name>.  Its own unit because the
// per-site routines must read fields with coherent loads here
// (SU2_COHERENT_LOADS), while the one-launch-per-pass kernels keep the
// read-only data path.
#define SU2_COHERENT_LOADS 1
#include "su2_pool.cuh"

namespace su2 {

using R = SU2_R;
constexpr int CCI = SU2_CC;
// the shape of launch variant 0: 128 threads, 8 (FP32) / 4 (FP64) resident
// blocks per SM asked of the compiler
constexpr int PBS = Variant<R, 0>::BS, PMB = Variant<R, 0>::MINB;

static void persist_launch(const void* args, unsigned grid, cudaStream_t st) {
  if (grid) k_pool_persist<R, CCI, PBS, PMB><<<grid, PBS, 0, st>>>(*(const PersistArgs*)args);
}

static int persist_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pool_persist<R, CCI, PBS, PMB>, PBS, 0) != cudaSuccess)
    return 0;
  return n;
}

const PersistOps SU2_PERSIST = {PBS, persist_launch, persist_blocks_per_sm};

}  // namespace su2
