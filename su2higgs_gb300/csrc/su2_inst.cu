// su2_inst.cu -- one instantiation of the sweep kernels.  Compiled several
// times with -DSU2_R=<double|float> -DSU2_CC=<content mask or -1>
// -DSU2_OPS=<table name>; the generic units also carry the content-free
// kernels (-DSU2_WITH_PREC=<table name>) and, for FP64, the non-template ones.
#include <algorithm>

#include "su2_kernels.cuh"
#include "su2_pool.cuh"
#include "su2_ops.h"

namespace su2 {

using R = SU2_R;
constexpr int CCI = SU2_CC;

template <int V>
static unsigned l_link_v(const void* f, const PassArgs& a, cudaStream_t st) {
  constexpr int BS = Variant<R, V>::BS, MB = Variant<R, V>::MINB;
  unsigned nb = (unsigned)((a.t_hi - a.t_lo + BS - 1) / BS);
  if (!nb) return 0;
  const Fields<R>& F = *(const Fields<R>*)f;
  if (a.sub == 0) k_link<R, CCI, 0, BS, MB><<<nb, BS, 0, st>>>(F, a);
  else if (a.sub == 1) k_link<R, CCI, 1, BS, MB><<<nb, BS, 0, st>>>(F, a);
  else k_link<R, CCI, 2, BS, MB><<<nb, BS, 0, st>>>(F, a);
  return nb;
}
template <int V>
static unsigned l_u1_v(const void* f, const PassArgs& a, cudaStream_t st) {
  constexpr int BS = Variant<R, V>::BS, MB = Variant<R, V>::MINB;
  unsigned nb = (unsigned)((a.t_hi - a.t_lo + BS - 1) / BS);
  if (!nb) return 0;
  const Fields<R>& F = *(const Fields<R>*)f;
  if (a.sub == 0) k_u1<R, CCI, 0, BS, MB><<<nb, BS, 0, st>>>(F, a);
  else if (a.sub == 1) k_u1<R, CCI, 1, BS, MB><<<nb, BS, 0, st>>>(F, a);
  else k_u1<R, CCI, 2, BS, MB><<<nb, BS, 0, st>>>(F, a);
  return nb;
}
template <int V>
static unsigned l_scalar_v(int field, const void* f, const PassArgs& a, cudaStream_t st) {
  constexpr int BS = Variant<R, V>::BS, MB = Variant<R, V>::MINB;
  unsigned nb = (unsigned)((a.t_hi - a.t_lo + BS - 1) / BS);
  if (!nb) return 0;
  const Fields<R>& F = *(const Fields<R>*)f;
  if (field == 0) k_scalar<R, CCI, 0, BS, MB><<<nb, BS, 0, st>>>(F, a);
  else if (field == 1) k_scalar<R, CCI, 1, BS, MB><<<nb, BS, 0, st>>>(F, a);
  else k_scalar<R, CCI, 2, BS, MB><<<nb, BS, 0, st>>>(F, a);
  return nb;
}
static unsigned l_link(int v, const void* f, const PassArgs& a, cudaStream_t st) {
  switch (v) {
    case 1: return l_link_v<1>(f, a, st);
    case 2: return l_link_v<2>(f, a, st);
    case 3: return l_link_v<3>(f, a, st);
    default: return l_link_v<0>(f, a, st);
  }
}
static unsigned l_u1(int v, const void* f, const PassArgs& a, cudaStream_t st) {
  switch (v) {
    case 1: return l_u1_v<1>(f, a, st);
    case 2: return l_u1_v<2>(f, a, st);
    case 3: return l_u1_v<3>(f, a, st);
    default: return l_u1_v<0>(f, a, st);
  }
}
static unsigned l_scalar(int v, int field, const void* f, const PassArgs& a, cudaStream_t st) {
  switch (v) {
    case 1: return l_scalar_v<1>(field, f, a, st);
    case 2: return l_scalar_v<2>(field, f, a, st);
    case 3: return l_scalar_v<3>(field, f, a, st);
    default: return l_scalar_v<0>(field, f, a, st);
  }
}
static void l_measure(const void* f, const Geom& g, const Coup& cp, const double* alpha, double* partials,
                      unsigned nb, cudaStream_t st) {
  k_measure<R, CCI><<<nb, BLOCK, 0, st>>>(*(const Fields<R>*)f, g, coup_as<R>(cp), alpha, partials);
}
static void l_flow(const void* fin, const void* fout, const Geom& g, const Coup& cp, double dt,
                   unsigned long long* fz, unsigned nb, cudaStream_t st) {
  k_flow<R, CCI><<<nb, BLOCK, 0, st>>>(*(const Fields<R>*)fin, *(const Fields<R>*)fout, g, coup_as<R>(cp), (R)dt, fz);
}

static void lp_measure(const PoolArgs& a, double* partials, unsigned nb, cudaStream_t st) {
  if (nb) k_pool_measure<R, CCI><<<nb, BLOCK, 0, st>>>(a, partials);
}

const Ops SU2_OPS = {sizeof(R) == 8 ? 64 : 32, CCI, l_link, l_u1, l_scalar, l_measure, l_flow, lp_measure};

#ifdef SU2_WITH_PREC
static unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }
static void p_orderparam(const void* f, const Geom& g, int parity, int op, double* partials, unsigned nb,
                         cudaStream_t st) {
  k_orderparam<R><<<nb, BLOCK, 0, st>>>(*(const Fields<R>*)f, g, parity, op, partials);
}
static void p_restore(int field, const void* f, const MucaDev* m, const void* backup, int h, int64_t lo, int64_t hi,
                      cudaStream_t st) {
  if (hi <= lo) return;
  unsigned nb = std::min<unsigned>(nblk(hi - lo, 256), 304);
  if (field == 0) k_muca_restore<R, 0><<<nb, 256, 0, st>>>(*(const Fields<R>*)f, m, backup, h, lo, hi);
  else k_muca_restore<R, 1><<<nb, 256, 0, st>>>(*(const Fields<R>*)f, m, backup, h, lo, hi);
}
static void p_alpha(const void* f, const Geom& g, const Coup& cp, double* alpha, cudaStream_t st) {
  k_alpha<R><<<nblk(g.V, BLOCK), BLOCK, 0, st>>>(*(const Fields<R>*)f, g, coup_as<R>(cp), alpha);
}
static void p_import(const void* f, int64_t V, int kind, int h, const double* src, cudaStream_t st) {
  k_import<R><<<nblk(V * 3, 256), 256, 0, st>>>(*(const Fields<R>*)f, V, kind, h, src);
}
static void p_export(const void* f, int64_t V, int kind, int h, double* dst, cudaStream_t st) {
  k_export<R><<<nblk(V * 3, 256), 256, 0, st>>>(*(const Fields<R>*)f, V, kind, h, dst);
}
static void p_reunit(const void* f, int64_t V, const uint32_t* sweep, int interval, cudaStream_t st) {
  k_reunitarize<R><<<nblk(V * 3, 256), 256, 0, st>>>(*(const Fields<R>*)f, V, sweep, interval);
}
static void p_fixup(const void* fin, const void* fout, const Geom& g, const unsigned long long* fz, cudaStream_t st) {
  k_flow_fixup<R><<<nblk(g.V * 3, 256), 256, 0, st>>>(*(const Fields<R>*)fin, *(const Fields<R>*)fout, g, fz);
}
static void p_measure_local(const void* f, const Geom& g, const Coup& cp, double denom, double* out,
                            cudaStream_t st) {
  k_measure_local<R><<<nblk(g.V, BLOCK), BLOCK, 0, st>>>(*(const Fields<R>*)f, g, coup_as<R>(cp), denom, out);
}
static void p_measure_z(const void* f, const Geom& g, int content, int zdir, double* out, cudaStream_t st) {
  k_measure_z<R><<<g.L[zdir], ZBLOCK, 0, st>>>(*(const Fields<R>*)f, g, content, zdir, out);
}
static void p_pool_convert(const void* descs, const ConvItem* items, int n, int vmax, double* staging, int to_device,
                           cudaStream_t st) {
  if (n <= 0 || vmax <= 0) return;
  dim3 grid(std::min(nblk(vmax, 256), 128u), (unsigned)n);
  k_pool_convert<R><<<grid, 256, 0, st>>>(descs, items, staging, to_device);
}
const PrecOps SU2_WITH_PREC = {p_orderparam, p_restore, p_alpha, p_import, p_export, p_reunit, p_fixup,
                               p_measure_local, p_measure_z, p_pool_convert};
#endif

#ifdef SU2_WITH_GLOBAL
void launch_muca_decide(MucaDev* w, const double* partials, int np, double vol, int parity, const RngKey& rk,
                        uint32_t pass, uint32_t check, unsigned long long* ctr, cudaStream_t st) {
  k_muca_decide<<<1, 256, 0, st>>>(w, partials, np, vol, parity, rk, pass, check, ctr);
}
void launch_muca_set_param(MucaDev* w, const double* partials, int np, double vol, int parity, cudaStream_t st) {
  k_muca_set_param<<<1, 256, 0, st>>>(w, partials, np, vol, parity);
}
void launch_reduce_partials(const double* partials, int np, double* out, cudaStream_t st) {
  k_reduce_partials<<<NSUMS, 256, 0, st>>>(partials, np, out);
}
void launch_pool_reduce(const double* partials, int nblocks, const int* first, int base, int nchains, double* out,
                        cudaStream_t st) {
  if (nchains) k_pool_reduce<<<nchains, 128, 0, st>>>(partials, nblocks, first, base, out);
}
void launch_pool_next_sweep(uint32_t* const* sweeps, int n, cudaStream_t st, uint32_t inc) {
  if (n) k_pool_next_sweep<<<(n + 255) / 256, 256, 0, st>>>(sweeps, n, inc);
}
#endif

}  // namespace su2
