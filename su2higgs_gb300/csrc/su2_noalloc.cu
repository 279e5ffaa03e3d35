// su2_noalloc.cu -- su2gpu_measure_noalloc: the volume sums of measure() for
// callers that cannot allocate device memory.
//
// Who needs it: code that must not call cudaMalloc/cudaFree -- for example a
// host framework whose own allocator owns all device memory, or a service
// loop that may not risk the device-wide synchronisation an allocation can
// cause.  Such a caller keeps the fields in its own device buffers (the
// library's parity-split layout) and passes them in, with a device buffer for
// the result.  This entry point then allocates nothing: its only scratch, the
// per-block partial sums, lives in the file-scope array below, which every
// GPU that loads the library holds until the process exits.
//
// Limits and rules:
//  * the scratch holds partial sums for NOALLOC_MAX_BLOCKS blocks of
//    su2::BLOCK sites, i.e. at most 2,097,152 sites (128^3); larger lattices
//    are rejected with SU2GPU_ERR_CAPACITY before anything is launched;
//  * every call overwrites the partial sums it reads (no entry has to start
//    at zero), and all calls share the one array: calls whose kernels overlap
//    on the GPU (different streams, several threads) race and must be
//    serialised by the caller;
//  * the first call on a device looks up the array's device address for that
//    device (cudaGetSymbolAddress); make that first call before any stream
//    capture.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/su2gpu.h"
#include "su2_kernels.cuh"
#include "su2_ops.h"

namespace su2 {

constexpr int NOALLOC_MAX_BLOCKS = 16384;
constexpr int NOALLOC_MAX_SITES = NOALLOC_MAX_BLOCKS * BLOCK;  // 2,097,152

static __device__ __align__(256) double g_noalloc_partials[NSUMS * NOALLOC_MAX_BLOCKS];

// The per-site terms of measure(), one site per thread, with the projected-U(1)
// field strengths of the magnetic charge computed where they are needed instead
// of being read from a scratch plane of 3 V doubles.
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_measure_noalloc(Fields<R> f, Geom g, CoupT<R> cp, double* partials) {
  constexpr int CC = C_GENERIC;
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  double m[NSUMS];
#pragma unroll
  for (int k = 0; k < NSUMS; k++) m[k] = 0.0;
  if (t < g.V) measure_site<R, CC>(f, g, cp, t, AlphaOnTheFly{}, m);
  block_sums_out<CC>(m, cp.content, partials, gridDim.x, blockIdx.x);
}

// device address of g_noalloc_partials, looked up once per device
static std::mutex g_noalloc_mutex;
static double* g_noalloc_addr[128];

static double* noalloc_scratch(int dev, cudaError_t* err) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (dev < 0 || dev >= 128) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  if (!g_noalloc_addr[dev]) {
    double* p = nullptr;
    *err = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
    if (*err != cudaSuccess) return nullptr;
    g_noalloc_addr[dev] = p;
  }
  *err = cudaSuccess;
  return g_noalloc_addr[dev];
}

}  // namespace su2

using namespace su2;

// the library's error text (read back with su2gpu_last_error)
__attribute__((visibility("hidden"))) void su2gpu_record_error(const char* msg);
static int noalloc_fail(int code, const char* msg) {
  su2gpu_record_error(msg);
  return code;
}

template <typename R>
static bool aligned_ok(const void* p, size_t a) {
  return p && ((uintptr_t)p % a) == 0;
}

extern "C" int su2gpu_measure_noalloc(const su2gpu_params* p, const su2gpu_device_fields* df, double* device_sums,
                                      void* cuda_stream) {
  if (!p || !df || !device_sums) return noalloc_fail(SU2GPU_ERR_INVALID, "null argument");
  if (p->dim != 3) return noalloc_fail(SU2GPU_ERR_INVALID, "only dim 3 is supported");
  for (int d = 0; d < 3; d++)
    if (p->L[d] < 2 || (p->L[d] & 1)) return noalloc_fail(SU2GPU_ERR_INVALID, "side lengths must be even and >= 2");
  double vol = (double)p->L[0] * p->L[1] * p->L[2];
  if (vol > (double)NOALLOC_MAX_SITES) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "lattice of %.0f sites exceeds the allocation-free scratch: at most %d sites (%d blocks of %d)", vol,
             NOALLOC_MAX_SITES, NOALLOC_MAX_BLOCKS, BLOCK);
    return noalloc_fail(SU2GPU_ERR_CAPACITY, msg);
  }
  if (p->precision != 64 && p->precision != 32) return noalloc_fail(SU2GPU_ERR_INVALID, "precision must be 64 or 32");
  const int c = p->content & 0x1f;
  const int nh = (c & SU2GPU_HIGGS2) ? 2 : ((c & SU2GPU_HIGGS1) ? 1 : 0);
  const size_t va = p->precision == 64 ? 32 : 16, ra = p->precision == 64 ? 8 : 4;
  for (int d = 0; d < 3; d++) {
    if (!aligned_ok<void>(df->link[d], va)) return noalloc_fail(SU2GPU_ERR_INVALID, "link arrays: null or misaligned");
    if ((c & SU2GPU_U1) && !aligned_ok<void>(df->u1[d], ra))
      return noalloc_fail(SU2GPU_ERR_INVALID, "u1 arrays: null or misaligned");
    if ((c & SU2GPU_TRIPLET) && !aligned_ok<void>(df->triplet[d], ra))
      return noalloc_fail(SU2GPU_ERR_INVALID, "triplet planes: null or misaligned");
  }
  for (int h = 0; h < nh; h++)
    if (!aligned_ok<void>(df->doublet[h], va)) return noalloc_fail(SU2GPU_ERR_INVALID, "doublet arrays: null or misaligned");
  if ((c & SU2GPU_SINGLET) && !aligned_ok<void>(df->singlet, ra))
    return noalloc_fail(SU2GPU_ERR_INVALID, "singlet array: null or misaligned");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return noalloc_fail(SU2GPU_ERR_CUDA, "cudaGetDevice failed");
  cudaError_t e;
  double* scratch = noalloc_scratch(dev, &e);
  if (!scratch) return noalloc_fail(SU2GPU_ERR_CUDA, cudaGetErrorString(e));

  Geom g = make_geom(p->L[0], p->L[1], p->L[2]);
  Coup cp;
  memset(&cp, 0, sizeof(cp));
  cp.beta = p->betasu2; cp.msq = p->msq_phi; cp.lam = p->lambda_phi;
  cp.msqT = p->msq_triplet; cp.a2 = p->a2; cp.b4 = p->b4;
  cp.betau1 = p->betau1; cp.r_u1 = p->r_u1;
  cp.b1s = p->b1_s; cp.msqs = p->msq_s; cp.b3s = p->b3_s; cp.b4s = p->b4_s; cp.a1s = p->a1_s; cp.a2s = p->a2_s;
  cp.msq2 = p->msq_phi2; cp.m12re = p->m12sq_re; cp.m12im = p->m12sq_im;
  cp.lam2 = p->lam2; cp.lam3 = p->lam3; cp.lam4 = p->lam4; cp.lam5re = p->lam5_re; cp.lam5im = p->lam5_im;
  cp.lam6re = p->lam6_re; cp.lam6im = p->lam6_im; cp.lam7re = p->lam7_re; cp.lam7im = p->lam7_im;
  cp.content = c;

  cudaStream_t st = (cudaStream_t)cuda_stream;
  unsigned nb = (unsigned)((g.V + BLOCK - 1) / BLOCK);
  if (p->precision == 64) {
    Fields<double> f;
    memset(&f, 0, sizeof(f));
    for (int d = 0; d < 3; d++) {
      f.link[d] = (D4*)df->link[d];
      f.u1[d] = (double*)df->u1[d];
      f.trip[d] = (double*)df->triplet[d];
    }
    f.phi[0] = (D4*)df->doublet[0];
    f.phi[1] = (D4*)df->doublet[1];
    f.sing = (double*)df->singlet;
    k_measure_noalloc<double><<<nb, BLOCK, 0, st>>>(f, g, coup_as<double>(cp), scratch);
  } else {
    Fields<float> f;
    memset(&f, 0, sizeof(f));
    for (int d = 0; d < 3; d++) {
      f.link[d] = (F4*)df->link[d];
      f.u1[d] = (float*)df->u1[d];
      f.trip[d] = (float*)df->triplet[d];
    }
    f.phi[0] = (F4*)df->doublet[0];
    f.phi[1] = (F4*)df->doublet[1];
    f.sing = (float*)df->singlet;
    k_measure_noalloc<float><<<nb, BLOCK, 0, st>>>(f, g, coup_as<float>(cp), scratch);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return noalloc_fail(SU2GPU_ERR_CUDA, cudaGetErrorString(e));
  launch_reduce_partials(scratch, (int)nb, device_sums, st);
  if ((e = cudaGetLastError()) != cudaSuccess) return noalloc_fail(SU2GPU_ERR_CUDA, cudaGetErrorString(e));
  return SU2GPU_OK;
}
