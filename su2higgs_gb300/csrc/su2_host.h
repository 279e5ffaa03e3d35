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

// Sweep order of the reference's random_sweeps mode (update.c:278-300,
// 338-344): per update_links repetition two independent Fisher-Yates
// shuffles (shuffle, update.c:461-468) of the parity array [E,O,E,O,E,O] and
// of the direction array [0,0,1,1,2,2] -- so a (direction, parity) pair may
// repeat and another be skipped, as there -- then per scalar sweep the parity
// updated first, EVEN when the uniform is below 0.5.  The random numbers come
// from the order stream: Philox with counter (ORDER_SITE, block, sweep, chain),
// 64-bit draw k = half k&1 of block k>>1; iran() is the draw itself, dran()
// its top 53 bits.
constexpr uint32_t ORDER_SITE = 0xfffffffeu;
inline void sweep_order(uint64_t seed, uint32_t chain, uint32_t sweep, int update_links, int scalar_sweeps,
                        int32_t* link_dirs, int32_t* link_pars, int32_t* scalar_first) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  uint32_t draw = 0;
  auto next64 = [&]() -> uint64_t {
    uint32_t b = draw >> 1, h = draw & 1;
    draw++;
    uint32_t c0 = ORDER_SITE, c1 = b & 0xffffu, c2 = sweep, c3 = chain;
    philox4x32_10(c0, c1, c2, c3, k0, k1);
    return h ? (((uint64_t)c2 << 32) | c3) : (((uint64_t)c0 << 32) | c1);
  };
  for (int k = 0; k < update_links; k++) {
    int32_t* par = link_pars + 6 * k;
    int32_t* dir = link_dirs + 6 * k;
    for (int j = 0; j < 6; j++) {
      par[j] = j & 1;
      dir[j] = j >> 1;
    }
    for (int i = 5; i > 0; i--) {
      int j = (int)(next64() % (uint64_t)(i + 1));
      int t = par[i]; par[i] = par[j]; par[j] = t;
    }
    for (int i = 5; i > 0; i--) {
      int j = (int)(next64() % (uint64_t)(i + 1));
      int t = dir[i]; dir[i] = dir[j]; dir[j] = t;
    }
  }
  for (int s = 0; s <= scalar_sweeps; s++) {
    double u = (double)(next64() >> 11) * (1.0 / 9007199254740992.0);
    scalar_first[s] = u < 0.5 ? 0 : 1;
  }
}

SU2_HIDDEN Coup make_coup(const su2gpu_params* p);
SU2_HIDDEN const Ops* pick_ops(int prec, int content);
SU2_HIDDEN const PoolOps* pick_persist(int prec, int content);

}  // namespace su2

// the text returned by su2gpu_last_error
SU2_HIDDEN void su2gpu_record_error(const char* msg);

// A context over fields of field_bytes() bytes at `fields` (device memory owned
// by the caller, laid out by carve()): nothing is copied or cold-started, and
// su2gpu_destroy leaves the fields alone.  Used for per-chain operations of a
// pool (gradient flow).
SU2_HIDDEN int su2gpu_attach(const su2gpu_params* p, void* fields, su2gpu_ctx** out);

// The device state a context keeps for a multicanonical weight
// (su2gpu_muca_set): its weight struct, the backup of the checked field, the
// order parameter and the checks per sweep; *muca is null without a weight.
SU2_HIDDEN int su2gpu_muca_device_state(su2gpu_ctx* c, void** muca, void** backup, int* orderparam, int* cps,
                                        int* do_acceptance);

// A context with its own copy of the fields at `fields` (device memory laid out
// by carve() for p), seeded with (seed, chain); no cold start.
SU2_HIDDEN int su2gpu_create_copy(const su2gpu_params* p, const void* fields, uint64_t seed, uint32_t chain,
                                  su2gpu_ctx** out);
