// su2_ops.h -- host-visible launcher tables of the kernel instantiations.
// Each (precision, content) instantiation unit (su2_inst.cu compiled with
// SU2_R / SU2_CC) fills one Ops table; the per-precision kernels that do not
// depend on the content live in a PrecOps table.
#pragma once

#include "su2_common.cuh"

namespace su2 {

struct PassArgs;
struct PoolArgs;

// The update launchers take a launch-shape variant (0..NVARIANTS-1, see
// Variant in su2_kernels.cuh) and the site range in the PassArgs; they return
// the number of blocks launched (the length of any per-block partial sums).
struct Ops {
  int prec;     // 64 or 32
  int content;  // C_GENERIC or a content mask
  unsigned (*link)(int variant, const void* f, const PassArgs& a, cudaStream_t st);
  unsigned (*u1)(int variant, const void* f, const PassArgs& a, cudaStream_t st);
  unsigned (*scalar)(int variant, int field, const void* f, const PassArgs& a, cudaStream_t st);
  void (*measure)(const void* f, const Geom& g, const Coup& cp, const double* alpha, double* partials,
                  unsigned nblocks, cudaStream_t st);
  void (*flow)(const void* fin, const void* fout, const Geom& g, const Coup& cp, double dt,
               unsigned long long* first_zero, unsigned nblocks, cudaStream_t st);
  // measurement of pools of chains (su2_pool.cuh): nblocks = length of the
  // measurement tile table
  void (*pool_measure)(const PoolArgs& a, double* partials, unsigned nblocks, cudaStream_t st);
};

// one chain of a multi-chain field conversion: its pool slot, the fields it
// carries (bit 1 links, 2 U(1), 4 doublet 0, 8 doublet 1, 16 triplet, 32
// singlet) and the offset, in doubles, of its host-layout block in staging
// memory (fields one after another in that order, each [V][components])
struct ConvItem {
  int slot, mask;
  long long off;
};

struct PrecOps {
  void (*orderparam)(const void* f, const Geom& g, int parity, int op, double* partials, unsigned nblocks,
                     cudaStream_t st);
  void (*restore)(int field, const void* f, const MucaDev* m, const void* backup, int h, int64_t lo, int64_t hi,
                  cudaStream_t st);
  void (*alpha)(const void* f, const Geom& g, const Coup& cp, double* alpha, cudaStream_t st);
  void (*import)(const void* f, int64_t V, int kind, int h, const double* src, cudaStream_t st);
  void (*exportf)(const void* f, int64_t V, int kind, int h, double* dst, cudaStream_t st);
  void (*reunitarize)(const void* f, int64_t V, const uint32_t* sweep, int interval, cudaStream_t st);
  void (*flow_fixup)(const void* fin, const void* fout, const Geom& g, const unsigned long long* fz,
                     cudaStream_t st);
  // per-site Tr Sigma^2 and magnetic charge / denom, out[2 V] (storage order)
  void (*measure_local)(const void* f, const Geom& g, const Coup& cp, double denom, double* out, cudaStream_t st);
  // plane sums along direction zdir: out[L[zdir]][4] (phi^2, Tr Sigma^2, S, S^2)
  void (*measure_z)(const void* f, const Geom& g, int content, int zdir, double* out, cudaStream_t st);
  // the host-layout FP64 blocks of `n` pool chains in staging memory <-> their
  // device fields (to_device 1: import, 0: export); vmax = the largest V
  void (*pool_convert)(const void* descs, const ConvItem* items, int n, int vmax, double* staging, int to_device,
                       cudaStream_t st);
};

// per-site values of su2gpu_site_values (su2_probe.cu): `what` is one of
// SITE_*; out holds V rows of the value's width, in layout order
enum : int {
  SITE_LINK_STAPLE = 1, SITE_WILSON_STAPLE = 2, SITE_LOCALACT_SU2LINK = 3, SITE_LOCALACT_U1LINK = 4,
  SITE_STAPLE_DOUBLET = 5, SITE_LOCALACT_DOUBLET = 6, SITE_LOCALACT_SINGLET = 7, SITE_OR_DOUBLET = 8,
  SITE_OR_DOUBLET1 = 9, SITE_OR_TRIPLET = 10, SITE_OR_SINGLET = 11
};
void launch_site_probe(int what, int parity, const Fields<double>& f, const Geom& g, const Coup& cp, double* out,
                       cudaStream_t st);

// instantiations (su2_inst.cu)
extern const Ops ops_f64_generic, ops_f64_fund, ops_f64_adj, ops_f64_su2u1s;
extern const Ops ops_f32_generic, ops_f32_fund, ops_f32_adj, ops_f32_su2u1s;
extern const PrecOps precops_f64, precops_f32;

// non-template kernels (su2_inst.cu, generic FP64 unit)
void launch_muca_decide(MucaDev* w, const double* partials, int np, double vol, int parity, const RngKey& rk,
                        uint32_t pass, uint32_t check, unsigned long long* ctr, cudaStream_t st);
void launch_muca_set_param(MucaDev* w, const double* partials, int np, double vol, int parity, cudaStream_t st);
void launch_reduce_partials(const double* partials, int np, double* out, cudaStream_t st);
void launch_pool_reduce(const double* partials, int nblocks, const int* first, int base, int nchains, double* out,
                        cudaStream_t st);
void launch_pool_next_sweep(uint32_t* const* sweeps, int n, cudaStream_t st, uint32_t inc = 1);

// the update kernels of pools of one (precision, content) instantiation
// (su2_persist.cu).  launch: the persistent sweep, the work list of `args`
// (a PersistArgs) on `grid` blocks of `threads`; blocks_per_sm: its resident
// blocks per SM.  pool_*: one pass over the tile table (nblocks tiles, built
// for the variant's block size).
// The persistent kernel comes in PERSIST_SHAPES launch shapes of `threads`
// threads (shape 0: the register budget of launch variant 0, shape 1: that
// of variant 1), which call the same per-tile functions as those variants.
constexpr int PERSIST_SHAPES = 2;
struct PoolOps {
  int threads;
  // muca: the instance for pools with multicanonical chains
  void (*launch)(int shape, bool muca, const void* args, unsigned grid, cudaStream_t st);
  int (*blocks_per_sm)(int shape);
  void (*pool_link)(int variant, const PoolArgs& a, unsigned nblocks, cudaStream_t st);
  void (*pool_u1)(int variant, const PoolArgs& a, unsigned nblocks, cudaStream_t st);
  void (*pool_scalar)(int variant, int field, const PoolArgs& a, unsigned nblocks, cudaStream_t st);
  // the multicanonical decide and restore passes over the chains mslots[0..n)
  void (*pool_restore)(const PoolArgs& a, const int* mslots, int n, int kb, cudaStream_t st);
  void (*pool_decide)(const PoolArgs& a, const int* mslots, int n, cudaStream_t st);
};
extern const PoolOps persist_f64_generic, persist_f64_fund, persist_f64_adj, persist_f64_su2u1s;
extern const PoolOps persist_f32_generic, persist_f32_fund, persist_f32_adj, persist_f32_su2u1s;

}  // namespace su2
