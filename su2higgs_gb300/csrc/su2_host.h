// su2_host.h -- host helpers shared by the units of libsu2gpu (not part of the
// C ABI): the field arena layout of one lattice, coupling conversion, kernel
// table selection and contexts over fields that live in another allocation.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include "../../include/su2gpu.h"
#include "su2_ops.h"

#define SU2_HIDDEN __attribute__((visibility("hidden")))

namespace su2 {

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

inline int nhiggs_of(int content) {
  return (content & SU2GPU_HIGGS2) ? 2 : ((content & SU2GPU_HIGGS1) ? 1 : 0);
}

// bytes of one lattice's fields: links, U(1) links, doublets, triplet planes,
// singlet, each array starting on a 256-byte boundary
inline size_t field_bytes(const su2gpu_params* p, int64_t V) {
  size_t r = p->precision == 64 ? 8 : 4, v4 = 4 * r;
  size_t b = 3 * align256(V * v4);
  if (p->content & SU2GPU_U1) b += 3 * align256(V * r);
  b += nhiggs_of(p->content) * align256(V * v4);
  if (p->content & SU2GPU_TRIPLET) b += 3 * align256(V * r);
  if (p->content & SU2GPU_SINGLET) b += align256(V * r);
  return b;
}

template <typename R>
inline void carve(Fields<R>& f, char* base, const su2gpu_params* p, int64_t V) {
  size_t r = sizeof(R), v4 = 4 * r, off = 0;
  memset(&f, 0, sizeof(f));
  for (int d = 0; d < 3; d++) { f.link[d] = (V4<R>*)(base + off); off += align256(V * v4); }
  if (p->content & SU2GPU_U1)
    for (int d = 0; d < 3; d++) { f.u1[d] = (R*)(base + off); off += align256(V * r); }
  for (int h = 0; h < nhiggs_of(p->content); h++) { f.phi[h] = (V4<R>*)(base + off); off += align256(V * v4); }
  if (p->content & SU2GPU_TRIPLET)
    for (int k = 0; k < 3; k++) { f.trip[k] = (R*)(base + off); off += align256(V * r); }
  if (p->content & SU2GPU_SINGLET) { f.sing = (R*)(base + off); off += align256(V * r); }
}

// Device address through which kernels can read or write the host buffer
// [p, p + bytes) directly: page-locked memory registered with (or allocated
// by) CUDA, which on a unified-address system is mapped into the device's
// address space.  Null for pageable memory or a buffer only partly
// registered; the caller then stages through device memory.
inline void* host_device_view(const void* p, size_t bytes) {
  if (!p || !bytes) return nullptr;
  cudaPointerAttributes a0, a1;
  const char* last = (const char*)p + bytes - 1;
  if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  if ((const char*)a1.devicePointer - (const char*)a0.devicePointer != (ptrdiff_t)(bytes - 1)) return nullptr;
  return a0.devicePointer;
}

SU2_HIDDEN Coup make_coup(const su2gpu_params* p);
SU2_HIDDEN const Ops* pick_ops(int prec, int content);

}  // namespace su2

// the text returned by su2gpu_last_error
SU2_HIDDEN void su2gpu_record_error(const char* msg);

// A context over fields of field_bytes() bytes at `fields` (device memory owned
// by the caller, laid out by carve()): nothing is copied or cold-started, and
// su2gpu_destroy leaves the fields alone.  Used for per-chain operations of a
// pool (gradient flow).
SU2_HIDDEN int su2gpu_attach(const su2gpu_params* p, void* fields, su2gpu_ctx** out);

// A context with its own copy of the fields at `fields` (device memory laid out
// by carve() for p), seeded with (seed, chain); no cold start.
SU2_HIDDEN int su2gpu_create_copy(const su2gpu_params* p, const void* fields, uint64_t seed, uint32_t chain,
                                  su2gpu_ctx** out);
