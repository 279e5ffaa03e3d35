// su2_pool.cu -- pools of independent chains (the batched and served forms):
// chains of one field content, precision and update recipe with their own
// lattice sizes, couplings, seeds and sweep counters, resident in one device
// arena.  Every half-sweep of update_lattice() (update.c:270-430) is a single
// launch over all chains; a sweep of the whole pool is replayed as one CUDA
// graph until the membership changes.  Admission is by device footprint: a
// chain is accepted when its fields fit in the arena.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "su2_host.h"
#include "su2_pool.cuh"

using namespace su2;

namespace {

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  su2gpu_record_error(buf);
  return code;
}

#define PCK(call)                                                                               \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

struct Buf {
  void* p = nullptr;
  size_t n = 0;
  int ensure(size_t bytes) {
    if (bytes <= n) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(SU2GPU_ERR_NOMEM, "cudaMalloc(%zu) failed", bytes);
    n = bytes;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

__global__ void k_cold_links4f(F4* p, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = F4{1.f, 0.f, 0.f, 0.f};
}
__global__ void k_cold_links4d(D4* p, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = D4{1.0, 0.0, 0.0, 0.0};
}

// doubles per site of one chain's host arrays (links 12, U(1) 3, two doublets
// 8, triplet 3, singlet 1)
constexpr int STAGE_REALS = 27;

struct Slot {
  bool active = false;
  su2gpu_params p;
  Geom g;
  Coup cp;
  size_t off = 0, bytes = 0;
  uint64_t seed = 0;
  uint32_t chain = 0;
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  // a multicanonical weight: a context attached to the chain's fields keeps
  // its device state (su2gpu_pool_muca_set)
  su2gpu_ctx* mctx = nullptr;
  void* mdev = nullptr;
  void* mbackup = nullptr;
  double* mpart = nullptr;  // the order parameter's 32-site warp sums (cudaMalloc)
  int mop = 0;
};

}  // namespace

struct su2gpu_pool {
  su2gpu_params recipe;
  int prec, content;
  const Ops* ops;
  const PrecOps* pops;
  cudaStream_t st = nullptr;      // execution stream (the caller's, or own_st)
  cudaStream_t own_st = nullptr;  // the pool's own stream; graphs are captured on it
  std::vector<cudaEvent_t>* prof = nullptr;  // per-pass events while profiling
  std::vector<int>* prof_kind = nullptr;
  Buf arena;
  std::vector<std::pair<size_t, size_t>> free_list;  // (offset, length), sorted by offset
  std::vector<Slot> slots;
  int max_slots;
  Buf slotmem;   // per slot: sweep counter word + 24 counters
  Buf descs;     // ChainDesc<R>[max_slots]
  Buf tiles[NVARIANTS], mtiles, mfirst, sweepptrs, partials, sums, stage, err;
  // the active chains with a multicanonical weight (their slots), the
  // restore launch's blocks per chain, and the half-sweeps that any of them
  // checks (bit 0 / 1: doublet 0 / 1, bit 2: triplet)
  Buf mslots;
  int restore_kb = 1, mucamask = 0;
  int64_t stage_sites = 0;          // sites each staging half holds (STAGE_REALS doubles per site)
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  // batch transfers (upload_many / download_many): a ring of staging memory
  // that the copy engines fill or drain on copy_st while the conversion
  // kernels run on st, each chain's region guarded by device-side events
  Buf ring;
  cudaStream_t copy_st = nullptr;
  std::vector<cudaEvent_t> ring_ev;  // two per chain of a batch: copied, converted
  int ntiles[NVARIANTS] = {0, 0, 0, 0}, nmtiles = 0;
  std::vector<int> active;  // active slots in slot order
  bool dirty = true;
  cudaGraphExec_t gexec = nullptr;
  // the persistent sweep (k_pool_persist): on by default; its work counter
  // and per-slot finished-tile counts, its resident grid, and the graph of
  // one launch of gexec_p_n sweeps
  const PoolOps* pers = nullptr;
  int persist_mode = -1;    // 1 on, 0 off (one launch per pass), -1 automatic
  bool persistent = false;  // the mode in effect for the current membership
  Buf qstate;
  // its work items: segments of seg_tiles 128-site tiles of one chain, and
  // the first segment of each active chain (+ the end)
  int seg_tiles = 8, seg_env = 0, seg_tuned = 0;  // seg_tuned: the autotuner's pick (0: none)
  int npasses = 0;  // passes per sweep of the recipe (set at the rebuild)
  int nmuca = 0;    // active chains with a multicanonical weight (set at the rebuild)
  Buf segs;
  std::vector<int4> h_segs;  // (slot, t0, the chain's segment count, 0)
  std::vector<int> h_sfirst;
  unsigned persist_grid = 0;      // resident blocks of the persistent kernel in its current shape
  int persist_shape = 0;          // launch shape of the persistent kernel (PERSIST_SHAPES)
  unsigned persist_grids[PERSIST_SHAPES] = {0, 0};
  cudaGraphExec_t gexec_p = nullptr;
  int gexec_p_n = 0;
  int var[5] = {0, 0, 0, 0, 0};
  int64_t sweep_passes[SU2GPU_NCOUNTERS] = {0};  // half-sweeps of each kind in one sweep (graph replay)
  // host images of the descriptor and tile tables; members, so that they
  // outlive every asynchronous copy from them
  std::vector<unsigned char> h_desc;
  std::vector<int2> h_tiles[NVARIANTS], h_mtiles;
  std::vector<int> h_first;
  std::vector<int> h_tfirst[NVARIANTS];  // first update tile of each active chain (+ the end)
  // pipelined cycles (su2gpu_pool_cycle): a second ring for the downloads,
  // the download copy stream, and one sweep graph per group of chains
  Buf ring_down;
  cudaStream_t down_st = nullptr;
  // update streams of the grouped sweep and the cycle, forked from and
  // joined back into st: the sweeps of consecutive groups run side by side
  // (highest priority, as own_st, whatever the caller's stream)
  static constexpr int CYCLE_SWEEP_STREAMS = 8;
  cudaStream_t sweep_st[CYCLE_SWEEP_STREAMS] = {};
  std::vector<cudaEvent_t> grp_ev;
  // the grouped sweep mode (one launch per pass, the chains split into
  // grp_G groups of about equal sites whose sweeps run on grp_NS streams in
  // turn; grp_G <= 1: off), its groups (active-chain ranges) and whether it
  // is in effect for the current membership
  int grp_G = 0, grp_NS = 1;
  std::vector<int> h_groups;
  bool grouped = false;
  std::vector<cudaEvent_t> cyc_ev;
  // n: sweeps per replay; per_pass: one launch per pass even where the group
  // would sweep persistently
  struct GroupGraph { int a0, a1, n; bool per_pass; cudaGraphExec_t exec; };
  std::vector<GroupGraph> ggraphs;
  ConvItem* h_items = nullptr;  // page-locked conversion items of a cycle (2 per chain)
  size_t h_items_n = 0;
  Buf d_items;
  std::vector<uint32_t*> h_sweeps;
  size_t rsize() const { return prec == 64 ? 8 : 4; }
};

// group helpers (defined with the C entry points below)
extern "C" {
static int group_graph(su2gpu_pool* P, int a0, int a1, int n, cudaGraphExec_t* out, bool per_pass);
static int enqueue_group_sweep(su2gpu_pool* P, int a0, int a1, int n, int64_t* tot, bool per_pass);
static std::vector<int> make_groups(const su2gpu_pool* P, int G, bool light_ends);
static int sweep_streams(su2gpu_pool* P, int NS, std::vector<cudaStream_t>& ss);
}

namespace {

int arena_alloc(su2gpu_pool* P, size_t bytes, size_t* off) {
  for (size_t k = 0; k < P->free_list.size(); k++) {
    auto& fr = P->free_list[k];
    if (fr.second >= bytes) {
      *off = fr.first;
      fr.first += bytes;
      fr.second -= bytes;
      if (!fr.second) P->free_list.erase(P->free_list.begin() + k);
      return 0;
    }
  }
  return -1;
}

void arena_free(su2gpu_pool* P, size_t off, size_t bytes) {
  P->free_list.push_back({off, bytes});
  std::sort(P->free_list.begin(), P->free_list.end());
  std::vector<std::pair<size_t, size_t>> merged;
  for (auto& fr : P->free_list) {
    if (!merged.empty() && merged.back().first + merged.back().second == fr.first) merged.back().second += fr.second;
    else merged.push_back(fr);
  }
  P->free_list.swap(merged);
}

// the captured graphs of the current membership, launch shapes and mode
void drop_graphs(su2gpu_pool* P) {
  if (P->gexec) cudaGraphExecDestroy(P->gexec);
  P->gexec = nullptr;
  if (P->gexec_p) cudaGraphExecDestroy(P->gexec_p);
  P->gexec_p = nullptr;
  P->gexec_p_n = 0;
  for (auto& gg : P->ggraphs) cudaGraphExecDestroy(gg.exec);
  P->ggraphs.clear();
}

template <typename R>
ChainDesc<R> make_desc(su2gpu_pool* P, int s, char* arena_base, char* slot_base) {
  const Slot& sl = P->slots[s];
  ChainDesc<R> d;
  memset(&d, 0, sizeof(d));
  carve(d.f, arena_base + sl.off, &sl.p, sl.g.V);
  d.g = sl.g;
  d.cp = coup_as<R>(sl.cp);
  d.k0 = (uint32_t)sl.seed;
  d.k1 = (uint32_t)(sl.seed >> 32);
  d.chain = sl.chain;
  d.sweep = (uint32_t*)(slot_base + (size_t)s * 256);
  d.ctr = (unsigned long long*)(slot_base + (size_t)s * 256 + 32);
  // the weight only on the pool's own fields: the autotuner's scratch copy
  // sweeps without checks, leaving the chain's multicanonical state alone
  if (sl.mdev && arena_base == (char*)P->arena.p) {
    d.muca = (MucaDev*)sl.mdev;
    d.mbackup = sl.mbackup;
    d.mpart = sl.mpart;
    d.mop = sl.mop;
  }
  return d;
}

void sweep_recipe(const su2gpu_params& p, std::vector<PassDesc>& out, int64_t* tot, int mucamask = 0);

// the work-list segments of slot s: (slot, t0, the chain's segment count, 0)
// for every `seg` tiles of 128 sites of one parity
void append_segments(const su2gpu_pool* P, int s, int seg, std::vector<int4>& out) {
  const int step = kVariantBS[0] * seg;
  const int half = (int)P->slots[s].g.half, nseg = (half + step - 1) / step;
  for (int t0 = 0; t0 < half; t0 += step) out.push_back(int4{s, t0, nseg, 0});
}

// descriptors and tile tables for the current membership
int rebuild(su2gpu_pool* P, void* arena_base = nullptr, void* slot_base = nullptr, void* descs = nullptr) {
  char* ab = (char*)(arena_base ? arena_base : P->arena.p);
  char* sb = (char*)(slot_base ? slot_base : P->slotmem.p);
  void* dd = descs ? descs : P->descs.p;
  P->active.clear();
  for (int s = 0; s < (int)P->slots.size(); s++)
    if (P->slots[s].active) P->active.push_back(s);
  size_t dsz = P->prec == 64 ? sizeof(ChainDesc<double>) : sizeof(ChainDesc<float>);
  PCK(cudaStreamSynchronize(P->st));  // no copy from the host images is in flight
  std::vector<unsigned char>& hd = P->h_desc;
  hd.assign(dsz * P->max_slots, 0);
  for (int s : P->active) {
    if (P->prec == 64) {
      ChainDesc<double> d = make_desc<double>(P, s, ab, sb);
      memcpy(hd.data() + dsz * s, &d, dsz);
    } else {
      ChainDesc<float> d = make_desc<float>(P, s, ab, sb);
      memcpy(hd.data() + dsz * s, &d, dsz);
    }
  }
  PCK(cudaMemcpyAsync(dd, hd.data(), hd.size(), cudaMemcpyHostToDevice, P->st));
  if (!descs) {
    for (int v = 0; v < NVARIANTS; v++) {
      std::vector<int2>& t = P->h_tiles[v];
      t.clear();
      P->h_tfirst[v].clear();
      int bs = kVariantBS[v];
      for (int s : P->active) {
        P->h_tfirst[v].push_back((int)t.size());
        for (int t0 = 0; t0 < P->slots[s].g.half; t0 += bs) t.push_back(int2{s, t0});
      }
      P->h_tfirst[v].push_back((int)t.size());
      P->ntiles[v] = (int)t.size();
      if (int rc = P->tiles[v].ensure(std::max<size_t>(t.size(), 1) * sizeof(int2))) return rc;
      if (!t.empty()) PCK(cudaMemcpyAsync(P->tiles[v].p, t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice, P->st));
    }
    // the persistent mode and its segment size: at least 4 work items per
    // resident block in a pass, at most 8 tiles per item.  Each item pays a
    // dependency check and a completion signal (about 1.5 us of latency);
    // the automatic mode uses the persistent sweep where that is spread over
    // 4 tiles or more and there are 8 chains or more whose passes can
    // overlap (the passes of one chain follow one another in either mode):
    // measured on GB300, the 384-chain ensemble (8-tile segments) runs 4 %
    // faster than with one launch per pass, pools of 16^3 chains (1-tile
    // segments) 25-30 % slower
    int64_t ntiles_all = 0;
    for (int s : P->active) ntiles_all += (P->slots[s].g.half + kVariantBS[0] - 1) / kVariantBS[0];
    const int64_t grid = std::max<int64_t>(1, P->persist_grid);
    const int seg_auto = (int)std::max<int64_t>(1, std::min<int64_t>(8, ntiles_all / (4 * grid)));
    P->seg_tiles = P->seg_env ? P->seg_env : (P->seg_tuned ? P->seg_tuned : seg_auto);
    std::vector<PassDesc> rec;
    int64_t counts[SU2GPU_NCOUNTERS] = {0};
    std::vector<int> ms;
    int64_t mhalf = 1;
    P->mucamask = 0;
    for (int s : P->active)
      if (P->slots[s].mdev && P->slots[s].mop) {
        const int op = P->slots[s].mop;
        ms.push_back(s);
        mhalf = std::max<int64_t>(mhalf, P->slots[s].g.half);
        P->mucamask |= (op == SU2GPU_PHISQ || op == SU2GPU_PHI2MINUSSIGMA2 ? 1 : 0) |
                       (op == SU2GPU_PHI2SQ ? 2 : 0) | (op == SU2GPU_SIGMASQ || op == SU2GPU_PHI2MINUSSIGMA2 ? 4 : 0);
      }
    P->nmuca = (int)ms.size();
    // restore blocks per chain: up to 8 sites per thread
    P->restore_kb = (int)std::max<int64_t>(1, (mhalf + 8 * 128 - 1) / (8 * 128));
    if (int rc = P->mslots.ensure(std::max<size_t>(ms.size(), 1) * sizeof(int))) return rc;
    if (!ms.empty()) PCK(cudaMemcpyAsync(P->mslots.p, ms.data(), ms.size() * sizeof(int), cudaMemcpyHostToDevice, P->st));
    sweep_recipe(P->recipe, rec, counts, P->mucamask);
    P->npasses = (int)rec.size();
    // a recipe of more passes than the work list holds always sweeps one
    // launch per pass (forcing the persistent mode on is refused for it)
    const bool fits = P->npasses <= PERSIST_MAX_PASSES;
    P->persistent = fits && (P->persist_mode == 1 ||
                             (P->persist_mode < 0 && P->active.size() >= 8 && seg_auto >= 4));
    // the grouped mode (set by the autotuner or su2gpu_pool_set_sweep_groups)
    // takes precedence over the automatic choice, not over a forced one
    P->grouped = P->grp_G > 1 && (int)P->active.size() > 1 && P->persist_mode != 1 && P->nmuca == 0;
    if (P->grouped) {
      P->persistent = false;
      P->h_groups = make_groups(P, P->grp_G, false);
    } else {
      P->h_groups.clear();
    }
    P->h_segs.clear();
    P->h_sfirst.clear();
    for (int s : P->active) {
      P->h_sfirst.push_back((int)P->h_segs.size());
      append_segments(P, s, P->seg_tiles, P->h_segs);
    }
    P->h_sfirst.push_back((int)P->h_segs.size());
    if (int rc = P->segs.ensure(std::max<size_t>(P->h_segs.size(), 1) * sizeof(int4))) return rc;
    if (!P->h_segs.empty())
      PCK(cudaMemcpyAsync(P->segs.p, P->h_segs.data(), P->h_segs.size() * sizeof(int4), cudaMemcpyHostToDevice,
                          P->st));
    std::vector<int2>& mt = P->h_mtiles;
    std::vector<int>& first = P->h_first;
    std::vector<uint32_t*>& sp = P->h_sweeps;
    mt.clear();
    first.clear();
    sp.clear();
    for (int s : P->active) {
      first.push_back((int)mt.size());
      for (int t0 = 0; t0 < P->slots[s].g.V; t0 += MEAS_TILE) mt.push_back(int2{s, t0});
      sp.push_back((uint32_t*)(sb + (size_t)s * 256));
    }
    first.push_back((int)mt.size());
    P->nmtiles = (int)mt.size();
    int rc;
    if ((rc = P->mtiles.ensure(std::max<size_t>(mt.size(), 1) * sizeof(int2))) ||
        (rc = P->mfirst.ensure(first.size() * sizeof(int))) ||
        (rc = P->sweepptrs.ensure(std::max<size_t>(sp.size(), 1) * sizeof(void*))) ||
        (rc = P->partials.ensure(std::max<size_t>(mt.size(), 1) * NSUMS * 8)) ||
        (rc = P->sums.ensure(std::max<size_t>(P->active.size(), 1) * NSUMS * 8)))
      return rc;
    if (!mt.empty()) PCK(cudaMemcpyAsync(P->mtiles.p, mt.data(), mt.size() * sizeof(int2), cudaMemcpyHostToDevice, P->st));
    PCK(cudaMemcpyAsync(P->mfirst.p, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice, P->st));
    if (!sp.empty()) PCK(cudaMemcpyAsync(P->sweepptrs.p, sp.data(), sp.size() * sizeof(void*), cudaMemcpyHostToDevice, P->st));
    drop_graphs(P);
    P->dirty = false;
  }
  PCK(cudaStreamSynchronize(P->st));
  return SU2GPU_OK;
}

void mark(su2gpu_pool* P, int kind) {
  if (!P->prof) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, P->st);
  P->prof->push_back(e);
  P->prof_kind->push_back(kind);
}

// the passes of one sweep (update.c:270-430 order); `tot` receives the
// per-chain half-site totals of one sweep
void sweep_recipe(const su2gpu_params& p, std::vector<PassDesc>& out, int64_t* tot, int mucamask) {
  out.clear();
  uint32_t pass = 0;
  const int nh = nhiggs_of(p.content);
  for (int k = 0; k < p.update_links; k++) {
    for (int mu = 0; mu < 3; mu++)
      for (int par = 0; par <= 1; par++) {
        out.push_back(PassDesc{0, (uint8_t)par, (uint8_t)mu, (uint8_t)p.algorithm_su2link, pass++});
        tot[SU2GPU_C_TOTAL_SU2LINK] += 1;
      }
    if (p.content & SU2GPU_U1)
      for (int mu = 0; mu < 3; mu++)
        for (int par = 0; par <= 1; par++) {
          out.push_back(PassDesc{1, (uint8_t)par, (uint8_t)mu, 0, pass++});
          tot[SU2GPU_C_TOTAL_U1LINK] += 1;
        }
  }
  int nsweeps = p.scalar_sweeps + 1;
  for (int s = 0; s < nsweeps; s++) {
    struct F { int field, count, alg; };
    F fields[3] = {{0, nh > 0 ? p.update_su2doublet : 0, p.algorithm_su2doublet},
                   {1, (p.content & SU2GPU_TRIPLET) ? p.update_su2triplet : 0, p.algorithm_su2triplet},
                   {2, (p.content & SU2GPU_SINGLET) ? p.update_singlet : 0, p.algorithm_singlet}};
    for (const F& fd : fields)
      for (int k = 0; k < fd.count; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (fd.alg == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        int nrep = fd.field == 0 ? nh : 1;
        for (int h = 0; h < nrep; h++)
          for (int par = 0; par <= 1; par++) {
            out.push_back(PassDesc{(uint8_t)(2 + fd.field), (uint8_t)par, (uint8_t)h, (uint8_t)force, pass});
            // a half-sweep that a multicanonical chain of the pool checks is
            // followed by the decision and the restore (with its pass number)
            if (fd.field < 2 && (mucamask >> (fd.field == 0 ? h : 2) & 1)) {
              out.push_back(PassDesc{6, (uint8_t)par, (uint8_t)h, (uint8_t)fd.field, pass});
              out.push_back(PassDesc{5, (uint8_t)par, (uint8_t)h, (uint8_t)fd.field, pass});
            }
            pass++;
            bool orr = fd.alg == SU2GPU_OVERRELAX && !force;
            int idx = fd.field == 0 ? (orr ? SU2GPU_C_TOTAL_OR_DOUBLET : SU2GPU_C_TOTAL_DOUBLET) + h
                                    : (fd.field == 1 ? (orr ? SU2GPU_C_TOTAL_OR_TRIPLET : SU2GPU_C_TOTAL_TRIPLET)
                                                     : (orr ? SU2GPU_C_TOTAL_OR_SINGLET : SU2GPU_C_TOTAL_SINGLET));
            tot[idx] += 1;
          }
      }
  }
}

// one sweep of every chain of the tile tables, one launch per pass
int enqueue_pool_sweep(su2gpu_pool* P, const void* descs, const int2* const* tiles, const int* nt,
                       int64_t* tot) {
  if (!nt) nt = P->ntiles;
  std::vector<PassDesc> passes;
  sweep_recipe(P->recipe, passes, tot, P->mucamask);
  PoolArgs a;
  memset(&a, 0, sizeof(a));
  a.descs = descs;
  a.nslots = P->max_slots;
  a.err = (int*)P->err.p;
  for (const PassDesc& q : passes) {
    const int kind = q.kind, v = kind >= 5 ? 0 : P->var[kind];
    a.parity = q.parity; a.sub = q.sub; a.alg = q.alg; a.pass = q.pass;
    a.tiles = tiles[v];
    mark(P, kind);
    if (kind == 0) P->pers->pool_link(v, a, nt[v], P->st);
    else if (kind == 1) P->pers->pool_u1(v, a, nt[v], P->st);
    else if (kind == 5) P->pers->pool_restore(a, (const int*)P->mslots.p, P->nmuca, P->restore_kb, P->st);
    else if (kind == 6) P->pers->pool_decide(a, (const int*)P->mslots.p, P->nmuca, P->st);
    else P->pers->pool_scalar(v, kind - 2, a, nt[v], P->st);
  }
  mark(P, -1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "pool sweep launch: %s", cudaGetErrorString(e));
  return SU2GPU_OK;
}

// `nsweeps` sweeps of the chains of a range of the segment table in one
// launch of the persistent kernel, then their sweep counters + nsweeps.
// first_item / spin_limit: see PersistArgs.
int enqueue_persist(su2gpu_pool* P, const int4* tiles, int nt, uint32_t* const* sweeps, int nchains, int nsweeps,
                    int64_t* tot, unsigned first_item = 0, int spin_limit = 1 << 18, const void* descs = nullptr,
                    int seg = 0) {
  std::vector<PassDesc> passes;
  sweep_recipe(P->recipe, passes, tot, P->mucamask);
  if ((int)passes.size() > PERSIST_MAX_PASSES)
    return fail(SU2GPU_ERR_INVALID, "%d passes per sweep: the persistent sweep takes at most %d", (int)passes.size(),
                PERSIST_MAX_PASSES);
  if (kVariantBS[0] != P->pers->threads) return fail(SU2GPU_ERR_INVALID, "persistent sweep: tile size mismatch");
  if (!P->persist_grid) return fail(SU2GPU_ERR_CUDA, "persistent sweep: no resident blocks per SM");
  PersistArgs A;
  memset(&A, 0, sizeof(A));
  A.descs = descs ? descs : P->descs.p;
  A.tiles = tiles;
  A.ntiles = nt;
  A.seg = seg ? seg : P->seg_tiles;
  A.nslots = P->max_slots;
  A.npasses = (int)passes.size();
  A.first_item = first_item;
  A.spin_limit = spin_limit;
  A.head = (unsigned*)P->qstate.p;
  A.done = (unsigned*)P->qstate.p + 1;
  A.err = (int*)P->err.p;
  for (size_t k = 0; k < passes.size(); k++) A.passes[k] = passes[k];
  // the work counter is 32 bits: at most 2^31 items per launch, more sweeps
  // in several launches (each after the previous one's counter increment)
  const int64_t per_sweep = (int64_t)nt * (int64_t)passes.size();
  const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(nsweeps, (1LL << 31) / std::max<int64_t>(1, per_sweep)));
  for (int s0 = 0; s0 < std::max(nsweeps, 1); s0 += chunk) {
    const int n = std::min(chunk, std::max(nsweeps - s0, 1));
    A.nsweeps = nsweeps > 0 ? n : 0;
    PCK(cudaMemsetAsync(P->qstate.p, 0, P->qstate.n, P->st));
    const unsigned grid = (unsigned)std::min<int64_t>(P->persist_grid, per_sweep * std::max(n, 1));
    P->pers->launch(P->persist_shape, P->nmuca > 0, &A, grid, P->st);
    PCK(cudaGetLastError());
    if (nsweeps > 0 && first_item == 0 && sweeps) launch_pool_next_sweep(sweeps, nchains, P->st, (uint32_t)n);
    PCK(cudaGetLastError());
  }
  return SU2GPU_OK;
}

bool same_recipe(const su2gpu_params* a, const su2gpu_params* b) {
  return a->content == b->content && a->precision == b->precision && a->algorithm_su2link == b->algorithm_su2link &&
         a->algorithm_u1link == b->algorithm_u1link && a->algorithm_su2doublet == b->algorithm_su2doublet &&
         a->algorithm_su2triplet == b->algorithm_su2triplet && a->algorithm_singlet == b->algorithm_singlet &&
         a->update_links == b->update_links && a->scalar_sweeps == b->scalar_sweeps &&
         a->update_su2doublet == b->update_su2doublet && a->update_su2triplet == b->update_su2triplet &&
         a->update_singlet == b->update_singlet;
}

}  // namespace

extern "C" {

int64_t su2gpu_pool_chain_bytes(const su2gpu_params* p) {
  if (!p || p->dim != 3) return -1;
  for (int d = 0; d < 3; d++)
    if (p->L[d] < 2 || (p->L[d] & 1)) return -1;
  return (int64_t)field_bytes(p, (int64_t)p->L[0] * p->L[1] * p->L[2]);
}

int su2gpu_pool_create(const su2gpu_params* recipe, int64_t arena_bytes, int32_t max_chains, su2gpu_pool** out) {
  if (!recipe || !out || arena_bytes <= 0 || max_chains <= 0) return fail(SU2GPU_ERR_INVALID, "bad pool arguments");
  if (recipe->precision != 64 && recipe->precision != 32) return fail(SU2GPU_ERR_INVALID, "precision must be 64 or 32");
  if ((recipe->content & SU2GPU_HIGGS1) && (recipe->content & SU2GPU_HIGGS2))
    return fail(SU2GPU_ERR_INVALID, "HIGGS1 and HIGGS2 are exclusive");
  if (recipe->algorithm_su2link != SU2GPU_HEATBATH && recipe->algorithm_su2link != SU2GPU_METROPOLIS)
    return fail(SU2GPU_ERR_INVALID, "algorithm_su2link must be heatbath or metropolis");
  su2gpu_pool* P = new su2gpu_pool();
  P->recipe = *recipe;
  P->prec = recipe->precision;
  P->content = recipe->content & 0x1f;
  P->ops = pick_ops(P->prec, P->content);
  P->pops = P->prec == 64 ? &precops_f64 : &precops_f32;
  P->pers = pick_persist(P->prec, P->content);
  if (const char* e = getenv("SU2GPU_PERSIST_TILES")) P->seg_env = std::max(1, atoi(e));
  P->max_slots = max_chains;
  P->slots.resize(max_chains);
  int rc;
  // the update stream at the highest priority: the transfer streams' kernels
  // (field conversions) fill in around the sweeps instead of displacing them
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (cudaStreamCreateWithPriority(&P->own_st, cudaStreamNonBlocking, greatest) != cudaSuccess) {
    delete P;
    return fail(SU2GPU_ERR_CUDA, "cudaStreamCreate failed");
  }
  P->st = P->own_st;
  if (cudaEventCreateWithFlags(&P->stage_ev[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&P->stage_ev[1], cudaEventDisableTiming) != cudaSuccess) {
    su2gpu_pool_destroy(P);
    return fail(SU2GPU_ERR_CUDA, "cudaEventCreate failed");
  }
  size_t dsz = P->prec == 64 ? sizeof(ChainDesc<double>) : sizeof(ChainDesc<float>);
  if ((rc = P->arena.ensure((size_t)arena_bytes)) || (rc = P->slotmem.ensure((size_t)max_chains * 256)) ||
      (rc = P->descs.ensure(dsz * max_chains)) || (rc = P->err.ensure(256)) ||
      (rc = P->qstate.ensure(((size_t)max_chains + 1) * sizeof(unsigned)))) {
    su2gpu_pool_destroy(P);
    return rc;
  }
  P->free_list.push_back({0, (size_t)arena_bytes});
  {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int k = 0; k < PERSIST_SHAPES; k++)
      P->persist_grids[k] = (unsigned)std::max(0, sms * P->pers->blocks_per_sm(k));
    P->persist_grid = P->persist_grids[0];
  }
  cudaMemsetAsync(P->slotmem.p, 0, P->slotmem.n, P->st);
  cudaMemsetAsync(P->err.p, 0, P->err.n, P->st);
  if (cudaStreamSynchronize(P->st) != cudaSuccess) {
    su2gpu_pool_destroy(P);
    return fail(SU2GPU_ERR_CUDA, "pool initialisation failed");
  }
  *out = P;
  return SU2GPU_OK;
}

int su2gpu_pool_destroy(su2gpu_pool* P) {
  if (!P) return SU2GPU_OK;
  if (P->st) cudaStreamSynchronize(P->st);
  if (P->own_st) cudaStreamSynchronize(P->own_st);
  drop_graphs(P);
  for (Slot& sl : P->slots) {
    if (sl.mctx) su2gpu_destroy(sl.mctx);
    if (sl.mpart) cudaFree(sl.mpart);
  }
  P->qstate.release();
  P->segs.release();
  P->arena.release(); P->slotmem.release(); P->descs.release(); P->mtiles.release(); P->mfirst.release();
  P->sweepptrs.release(); P->partials.release(); P->sums.release(); P->stage.release(); P->err.release();
  P->mslots.release();
  for (int v = 0; v < NVARIANTS; v++) P->tiles[v].release();
  for (int k = 0; k < 2; k++)
    if (P->stage_ev[k]) cudaEventDestroy(P->stage_ev[k]);
  if (P->copy_st) cudaStreamSynchronize(P->copy_st);
  if (P->down_st) cudaStreamSynchronize(P->down_st);
  for (cudaStream_t x : P->sweep_st)
    if (x) cudaStreamSynchronize(x);
  P->ring.release();
  P->ring_down.release();
  for (cudaEvent_t e : P->ring_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : P->cyc_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : P->grp_ev) cudaEventDestroy(e);
  if (P->h_items) cudaFreeHost(P->h_items);
  P->d_items.release();
  if (P->copy_st) cudaStreamDestroy(P->copy_st);
  if (P->down_st) cudaStreamDestroy(P->down_st);
  for (cudaStream_t x : P->sweep_st)
    if (x) cudaStreamDestroy(x);
  if (P->own_st) cudaStreamDestroy(P->own_st);
  delete P;
  return SU2GPU_OK;
}

int su2gpu_pool_add(su2gpu_pool* P, const su2gpu_params* p, uint64_t seed, uint32_t chain, int32_t* slot_out) {
  if (!P || !p || !slot_out) return fail(SU2GPU_ERR_INVALID, "null argument");
  if (!same_recipe(&P->recipe, p)) return fail(SU2GPU_ERR_INVALID, "chain recipe (content, precision, algorithms, update counts) differs from the pool's");
  if (p->dim != 3) return fail(SU2GPU_ERR_INVALID, "only dim 3 is supported");
  for (int d = 0; d < 3; d++)
    if (p->L[d] < 2 || (p->L[d] & 1)) return fail(SU2GPU_ERR_INVALID, "side lengths must be even and >= 2");
  int64_t V = (int64_t)p->L[0] * p->L[1] * p->L[2];
  if (V * 3 >= 2147483647LL) return fail(SU2GPU_ERR_INVALID, "lattice too large");
  int s = -1;
  for (int k = 0; k < P->max_slots; k++)
    if (!P->slots[k].active) { s = k; break; }
  if (s < 0) return fail(SU2GPU_ERR_CAPACITY, "pool has no free chain slot (%d)", P->max_slots);
  size_t bytes = field_bytes(p, V), off = 0;
  if (arena_alloc(P, bytes, &off)) return fail(SU2GPU_ERR_CAPACITY, "chain of %zu bytes does not fit in the arena", bytes);
  Slot& sl = P->slots[s];
  sl = Slot();
  sl.active = true;
  sl.p = *p;
  sl.g = make_geom(p->L[0], p->L[1], p->L[2]);
  sl.cp = make_coup(p);
  sl.off = off;
  sl.bytes = bytes;
  sl.seed = seed;
  sl.chain = chain;
  char* base = (char*)P->arena.p + off;
  PCK(cudaMemsetAsync(base, 0, bytes, P->st));
  PCK(cudaMemsetAsync((char*)P->slotmem.p + (size_t)s * 256, 0, 256, P->st));
  // cold links (setsu2, init.c:18-28): the three link arrays lead the chain's block
  size_t lbytes = align256((size_t)V * 4 * P->rsize());
  for (int d = 0; d < 3; d++) {
    if (P->prec == 64) k_cold_links4d<<<(unsigned)((V + 255) / 256), 256, 0, P->st>>>((D4*)(base + d * lbytes), V);
    else k_cold_links4f<<<(unsigned)((V + 255) / 256), 256, 0, P->st>>>((F4*)(base + d * lbytes), V);
  }
  PCK(cudaGetLastError());
  PCK(cudaStreamSynchronize(P->st));
  P->dirty = true;
  P->seg_tuned = 0;  // a tuned work-item size holds for the membership it was tuned on
  *slot_out = s;
  return SU2GPU_OK;
}

int su2gpu_pool_remove(su2gpu_pool* P, int32_t s) {
  if (!P || s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
  PCK(cudaStreamSynchronize(P->st));
  arena_free(P, P->slots[s].off, P->slots[s].bytes);
  if (P->slots[s].mctx) su2gpu_destroy(P->slots[s].mctx);
  if (P->slots[s].mpart) cudaFree(P->slots[s].mpart);
  P->slots[s] = Slot();
  P->dirty = true;
  P->seg_tuned = 0;
  return SU2GPU_OK;
}

int su2gpu_pool_info(su2gpu_pool* P, int32_t* nactive, int64_t* used_bytes, int64_t* free_bytes, int64_t* largest_free) {
  if (!P) return SU2GPU_ERR_INVALID;
  int n = 0;
  int64_t used = 0;
  for (auto& sl : P->slots)
    if (sl.active) { n++; used += sl.bytes; }
  int64_t fr = 0, big = 0;
  for (auto& f : P->free_list) { fr += f.second; big = std::max<int64_t>(big, f.second); }
  if (nactive) *nactive = n;
  if (used_bytes) *used_bytes = used;
  if (free_bytes) *free_bytes = fr;
  if (largest_free) *largest_free = big;
  return SU2GPU_OK;
}

// one chain's fields to / from FP64 AoS host arrays.  Uploads from
// page-locked arrays are read by the conversion kernel in place; other
// uploads and every download go through staging memory: the chain's arrays
// at their own offsets in one of two staging halves (`half`), so that one
// chain's copies overlap the next chain's conversion.  The caller waits on
// P->stage_ev[half] before reusing a half.
static int slot_transfer(su2gpu_pool* P, int32_t s, int upload, double* const* h, int half) {
  if (!P || s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
  const Slot& sl = P->slots[s];
  int64_t V = sl.g.V;
  Fields<double> f64;
  Fields<float> f32;
  char* base = (char*)P->arena.p + sl.off;
  if (P->prec == 64) carve(f64, base, &sl.p, V);
  else carve(f32, base, &sl.p, V);
  const void* F = P->prec == 64 ? (const void*)&f64 : (const void*)&f32;
  int nh = nhiggs_of(P->content);
  struct Item { int kind, hid; size_t n; bool present; };
  const Item items[6] = {{0, 0, (size_t)V * 12, true},
                         {1, 0, (size_t)V * 3, (bool)(P->content & SU2GPU_U1)},
                         {2, 0, (size_t)V * 4, nh > 0},
                         {2, 1, (size_t)V * 4, nh > 1},
                         {3, 0, (size_t)V * 3, (bool)(P->content & SU2GPU_TRIPLET)},
                         {4, 0, (size_t)V, (bool)(P->content & SU2GPU_SINGLET)}};
  if ((size_t)V > (size_t)P->stage_sites) {
    // staging for a chain this large: both halves grow (waits for all copies)
    PCK(cudaStreamSynchronize(P->st));
    P->stage_sites = V;
    int rc = P->stage.ensure(2 * (size_t)V * STAGE_REALS * 8);
    if (rc) return rc;
  }
  double* st = (double*)((char*)P->stage.p + (size_t)half * (size_t)P->stage_sites * STAGE_REALS * 8);
  size_t off = 0;
  for (int k = 0; k < 6; k++) {
    const Item& it = items[k];
    if (!it.present || !h[k]) continue;
    if (upload) {
      double* direct = (double*)host_device_view(h[k], it.n * 8);
      if (direct) {
        P->pops->import(F, V, it.kind, it.hid, direct, P->st);
        continue;
      }
      PCK(cudaMemcpyAsync(st + off, h[k], it.n * 8, cudaMemcpyHostToDevice, P->st));
      P->pops->import(F, V, it.kind, it.hid, st + off, P->st);
    } else {
      P->pops->exportf(F, V, it.kind, it.hid, st + off, P->st);
      PCK(cudaMemcpyAsync(h[k], st + off, it.n * 8, cudaMemcpyDeviceToHost, P->st));
    }
    off += it.n;
  }
  PCK(cudaEventRecord(P->stage_ev[half], P->st));
  PCK(cudaGetLastError());
  return SU2GPU_OK;
}

int su2gpu_pool_upload(su2gpu_pool* P, int32_t s, const double* link, const double* u1, const double* d0,
                       const double* d1, const double* trip, const double* sing) {
  double* h[6] = {(double*)link, (double*)u1, (double*)d0, (double*)d1, (double*)trip, (double*)sing};
  int rc = slot_transfer(P, s, 1, h, 0);
  if (rc) return rc;
  PCK(cudaStreamSynchronize(P->st));
  // a multicanonical chain takes the order parameter of its new fields
  if (P->slots[s].mctx)
    for (int par = 0; par < 2; par++)
      if ((rc = su2gpu_calc_orderparam(P->slots[s].mctx, par, nullptr))) return rc;
  return SU2GPU_OK;
}

int su2gpu_pool_download(su2gpu_pool* P, int32_t s, double* link, double* u1, double* d0, double* d1, double* trip,
                         double* sing) {
  double* h[6] = {link, u1, d0, d1, trip, sing};
  int rc = slot_transfer(P, s, 0, h, 0);
  if (rc) return rc;
  PCK(cudaStreamSynchronize(P->st));
  return SU2GPU_OK;
}

// many chains in one call: fields[k][j] is field k (link, u1, doublet0,
// doublet1, triplet, singlet) of slots[j]; a null fields[k] skips field k
// Field arrays of one chain and their FP64 element counts, in transfer order
struct ChainIo {
  int kind[6], hid[6];
  size_t n[6];
  int count = 0;
  size_t total = 0;
};
static ChainIo chain_io(const su2gpu_pool* P, int64_t V, double* const* h, double** hp) {
  ChainIo c;
  const int nh = nhiggs_of(P->content);
  const struct { int kind, hid; size_t n; bool present; } items[6] = {
      {0, 0, (size_t)V * 12, true},
      {1, 0, (size_t)V * 3, (bool)(P->content & SU2GPU_U1)},
      {2, 0, (size_t)V * 4, nh > 0},
      {2, 1, (size_t)V * 4, nh > 1},
      {3, 0, (size_t)V * 3, (bool)(P->content & SU2GPU_TRIPLET)},
      {4, 0, (size_t)V, (bool)(P->content & SU2GPU_SINGLET)}};
  for (int k = 0; k < 6; k++) {
    if (!items[k].present || !h[k]) continue;
    c.kind[c.count] = items[k].kind;
    c.hid[c.count] = items[k].hid;
    c.n[c.count] = items[k].n;
    hp[c.count] = h[k];
    c.total += items[k].n;
    c.count++;
  }
  return c;
}

// staging ring of batch transfers: 2 GiB (or the batch, if smaller; at least
// the largest chain), or SU2GPU_RING_BYTES bytes when that is set
static size_t ring_bytes() {
  const char* e = getenv("SU2GPU_RING_BYTES");
  if (e && *e) return (size_t)strtoull(e, nullptr, 10);
  return (size_t)1 << 31;
}

// A staging ring of host transfers: chain regions are placed one after
// another and wrap to the start; a region is reused only after every earlier
// chain placed over it was consumed, which the producer of the new chain
// waits for on the device.
struct Ring {
  char* base = nullptr;
  size_t cap = 0, head = 0;
  struct Placed { size_t lo, hi; cudaEvent_t consumed; };
  std::vector<Placed> live;
};
static int ring_take(Ring& R, size_t bytes, cudaStream_t producer, size_t* lo) {
  if (R.head + bytes > R.cap) R.head = 0;
  *lo = R.head;
  const size_t hi = R.head + bytes;
  R.head = hi;
  for (size_t q = 0; q < R.live.size();) {
    if (R.live[q].lo < hi && *lo < R.live[q].hi) {
      PCK(cudaStreamWaitEvent(producer, R.live[q].consumed, 0));
      R.live.erase(R.live.begin() + q);
    } else {
      q++;
    }
  }
  return SU2GPU_OK;
}

// one chain's host arrays into its fields: copies on `copy`, conversion
// kernels on `comp` once the copies are done (events `ready`, `consumed`)
static int chain_up(su2gpu_pool* P, Ring& R, int32_t s, double* const* h, cudaEvent_t ready, cudaEvent_t consumed,
                    cudaStream_t copy, cudaStream_t comp) {
  const Slot& sl = P->slots[s];
  const int64_t V = sl.g.V;
  double* hp[6];
  const ChainIo io = chain_io(P, V, h, hp);
  size_t lo;
  int rc = ring_take(R, io.total * 8, copy, &lo);
  if (rc) return rc;
  double* st = (double*)(R.base + lo);
  Fields<double> f64;
  Fields<float> f32;
  char* base = (char*)P->arena.p + sl.off;
  if (P->prec == 64) carve(f64, base, &sl.p, V);
  else carve(f32, base, &sl.p, V);
  const void* F = P->prec == 64 ? (const void*)&f64 : (const void*)&f32;
  size_t off = 0;
  for (int k = 0; k < io.count; k++) {
    PCK(cudaMemcpyAsync(st + off, hp[k], io.n[k] * 8, cudaMemcpyHostToDevice, copy));
    off += io.n[k];
  }
  PCK(cudaEventRecord(ready, copy));
  PCK(cudaStreamWaitEvent(comp, ready, 0));
  off = 0;
  for (int k = 0; k < io.count; k++) {
    P->pops->import(F, V, io.kind[k], io.hid[k], st + off, comp);
    off += io.n[k];
  }
  PCK(cudaEventRecord(consumed, comp));
  PCK(cudaGetLastError());
  R.live.push_back({lo, lo + io.total * 8, consumed});
  return SU2GPU_OK;
}

// one chain's fields into its host arrays: conversion kernels on `comp`,
// copies on `copy` once they are done
static int chain_down(su2gpu_pool* P, Ring& R, int32_t s, double* const* h, cudaEvent_t ready, cudaEvent_t consumed,
                      cudaStream_t comp, cudaStream_t copy) {
  const Slot& sl = P->slots[s];
  const int64_t V = sl.g.V;
  double* hp[6];
  const ChainIo io = chain_io(P, V, h, hp);
  size_t lo;
  int rc = ring_take(R, io.total * 8, comp, &lo);
  if (rc) return rc;
  double* st = (double*)(R.base + lo);
  Fields<double> f64;
  Fields<float> f32;
  char* base = (char*)P->arena.p + sl.off;
  if (P->prec == 64) carve(f64, base, &sl.p, V);
  else carve(f32, base, &sl.p, V);
  const void* F = P->prec == 64 ? (const void*)&f64 : (const void*)&f32;
  size_t off = 0;
  for (int k = 0; k < io.count; k++) {
    P->pops->exportf(F, V, io.kind[k], io.hid[k], st + off, comp);
    off += io.n[k];
  }
  PCK(cudaEventRecord(ready, comp));
  PCK(cudaStreamWaitEvent(copy, ready, 0));
  off = 0;
  for (int k = 0; k < io.count; k++) {
    PCK(cudaMemcpyAsync(hp[k], st + off, io.n[k] * 8, cudaMemcpyDeviceToHost, copy));
    off += io.n[k];
  }
  PCK(cudaEventRecord(consumed, copy));
  PCK(cudaGetLastError());
  R.live.push_back({lo, lo + io.total * 8, consumed});
  return SU2GPU_OK;
}

static int ensure_events(std::vector<cudaEvent_t>& v, size_t n) {
  while (v.size() < n) {
    cudaEvent_t e;
    PCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    v.push_back(e);
  }
  return SU2GPU_OK;
}

// a transfer stream, at the lowest priority
static int ensure_stream(cudaStream_t* st) {
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (!*st && cudaStreamCreateWithPriority(st, cudaStreamNonBlocking, least) != cudaSuccess)
    return fail(SU2GPU_ERR_CUDA, "cudaStreamCreate failed");
  return SU2GPU_OK;
}

// a ring buffer for a batch of `total` staged bytes whose largest chain
// needs `largest`
static int ensure_ring(su2gpu_pool* P, Buf& buf, size_t total, size_t largest, Ring* R) {
  const size_t want = std::max(largest, std::min(total, ring_bytes()));
  if (buf.n < want) {
    if (P->copy_st) PCK(cudaStreamSynchronize(P->copy_st));
    if (P->down_st) PCK(cudaStreamSynchronize(P->down_st));
    PCK(cudaStreamSynchronize(P->st));
    int rc = buf.ensure(want);
    if (rc) return rc;
  }
  R->base = (char*)buf.p;
  R->cap = want;
  return SU2GPU_OK;
}

// upload_many / download_many.  The batch goes through a staging ring: chain
// j's host arrays are copied by the copy engines on copy_st and converted by
// the kernels on st, with device-side events between the two streams per
// chain (copied -> convert for uploads, converted -> copy for downloads), so
// copies and conversions overlap and the host never waits inside the batch.
static int many_transfer(su2gpu_pool* P, int32_t n, const int32_t* slots, int upload, double* const* const* fields) {
  if (!P || n < 0 || (n && !slots) || !fields) return fail(SU2GPU_ERR_INVALID, "bad arguments");
  if (!n) return SU2GPU_OK;
  size_t total = 0, largest = 0;
  for (int32_t j = 0; j < n; j++) {
    const int32_t s = slots[j];
    if (s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
    const size_t b = (size_t)P->slots[s].g.V * STAGE_REALS * 8;
    total += b;
    largest = std::max(largest, b);
  }
  int rc;
  Ring R;
  if ((rc = ensure_stream(&P->copy_st)) || (rc = ensure_ring(P, P->ring, total, largest, &R)) ||
      (rc = ensure_events(P->ring_ev, 2 * (size_t)n + 1)))
    return rc;
  // the fields may still be in use by earlier work on st
  PCK(cudaEventRecord(P->ring_ev[2 * n], P->st));
  PCK(cudaStreamWaitEvent(P->copy_st, P->ring_ev[2 * n], 0));
  for (int32_t j = 0; j < n; j++) {
    double* h[6];
    for (int k = 0; k < 6; k++) h[k] = fields[k] ? fields[k][j] : nullptr;
    rc = upload ? chain_up(P, R, slots[j], h, P->ring_ev[2 * j], P->ring_ev[2 * j + 1], P->copy_st, P->st)
                : chain_down(P, R, slots[j], h, P->ring_ev[2 * j], P->ring_ev[2 * j + 1], P->st, P->copy_st);
    if (rc) return rc;
  }
  PCK(cudaStreamSynchronize(P->copy_st));
  PCK(cudaStreamSynchronize(P->st));
  return SU2GPU_OK;
}

// batch uploads leave a multicanonical chain's order parameter behind its
// fields: they are refused for such chains (su2gpu_pool_upload recomputes it)
static int refuse_muca_batch(const su2gpu_pool* P, int32_t n, const int32_t* slots) {
  for (int j = 0; j < n; j++)
    if (slots && slots[j] >= 0 && slots[j] < P->max_slots && P->slots[slots[j]].mctx)
      return fail(SU2GPU_ERR_UNSUPPORTED, "chain slot %d has a multicanonical weight: upload it with "
                  "su2gpu_pool_upload, which recomputes its order parameter", slots[j]);
  return SU2GPU_OK;
}

int su2gpu_pool_upload_many(su2gpu_pool* P, int32_t n, const int32_t* slots, const double* const* const* fields) {
  if (!P) return SU2GPU_ERR_INVALID;
  if (int rc = refuse_muca_batch(P, n, slots)) return rc;
  return many_transfer(P, n, slots, 1, (double* const* const*)fields);
}

int su2gpu_pool_download_many(su2gpu_pool* P, int32_t n, const int32_t* slots, double* const* const* fields) {
  return many_transfer(P, n, slots, 0, fields);
}

int su2gpu_pool_set_sweep(su2gpu_pool* P, int32_t s, uint32_t sweep) {
  if (!P || s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
  PCK(cudaMemcpyAsync((char*)P->slotmem.p + (size_t)s * 256, &sweep, 4, cudaMemcpyHostToDevice, P->st));
  PCK(cudaStreamSynchronize(P->st));
  return SU2GPU_OK;
}


static int pool_enqueue(su2gpu_pool* P, int32_t nsweeps, int32_t use_graph) {
  if (!P || nsweeps < 0) return fail(SU2GPU_ERR_INVALID, "bad pool run arguments");
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  if (P->active.empty() || !nsweeps) return SU2GPU_OK;
  const int2* tiles[NVARIANTS];
  for (int v = 0; v < NVARIANTS; v++) tiles[v] = (const int2*)P->tiles[v].p;
  uint32_t* const* sweeps = (uint32_t* const*)P->sweepptrs.p;
  const int na = (int)P->active.size();
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  if (P->persistent) {
    // one launch of the persistent kernel for all nsweeps sweeps (in a graph
    // captured for this number of sweeps)
    if (use_graph) {
      if (!P->gexec_p || P->gexec_p_n != nsweeps) {
        if (P->gexec_p) cudaGraphExecDestroy(P->gexec_p);
        P->gexec_p = nullptr;
        cudaGraph_t graph;
        cudaStream_t exec = P->st;
        PCK(cudaStreamSynchronize(exec));
        P->st = P->own_st;
        PCK(cudaStreamBeginCapture(P->st, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_persist(P, (const int4*)P->segs.p, (int)P->h_segs.size(), sweeps, na, nsweeps, tot);
        cudaError_t e = cudaStreamEndCapture(P->st, &graph);
        P->st = exec;
        if (rc) return rc;
        if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "pool graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&P->gexec_p, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "pool graph instantiate: %s", cudaGetErrorString(e));
        P->gexec_p_n = nsweeps;
      } else {
        std::vector<PassDesc> passes;
        sweep_recipe(P->recipe, passes, tot);
      }
      PCK(cudaGraphLaunch(P->gexec_p, P->st));
    } else if ((rc = enqueue_persist(P, (const int4*)P->segs.p, (int)P->h_segs.size(), sweeps, na, nsweeps,
                                     tot))) {
      return rc;
    }
  } else if (P->grouped) {
    // the groups' sweeps on grp_NS streams in turn, forked from and joined
    // back into the pool's stream
    const int Gn = (int)P->h_groups.size() - 1;
    std::vector<cudaStream_t> ss;
    if ((rc = sweep_streams(P, P->grp_NS, ss)) || (rc = ensure_events(P->grp_ev, ss.size() + 1))) return rc;
    const int NS = (int)ss.size();
    std::vector<cudaGraphExec_t> gex(Gn, nullptr);
    if (use_graph)
      for (int g = 0; g < Gn; g++)
        if ((rc = group_graph(P, P->h_groups[g], P->h_groups[g + 1], nsweeps, &gex[g], true))) return rc;
    PCK(cudaEventRecord(P->grp_ev[0], P->st));
    for (int k = 0; k < NS; k++) PCK(cudaStreamWaitEvent(ss[k], P->grp_ev[0], 0));
    for (int g = 0; g < Gn; g++) {
      if (use_graph) {
        PCK(cudaGraphLaunch(gex[g], ss[g % NS]));
      } else {
        cudaStream_t home = P->st;
        P->st = ss[g % NS];
        int64_t t1[SU2GPU_NCOUNTERS] = {0};
        rc = enqueue_group_sweep(P, P->h_groups[g], P->h_groups[g + 1], nsweeps, t1, true);
        P->st = home;
        if (rc) return rc;
      }
    }
    for (int k = 0; k < NS; k++) {
      PCK(cudaEventRecord(P->grp_ev[k + 1], ss[k]));
      PCK(cudaStreamWaitEvent(P->st, P->grp_ev[k + 1], 0));
    }
    std::vector<PassDesc> passes;
    sweep_recipe(P->recipe, passes, tot);
  } else if (use_graph) {
    if (!P->gexec) {
      cudaGraph_t graph;
      cudaStream_t exec = P->st;
      PCK(cudaStreamSynchronize(exec));
      P->st = P->own_st;
      PCK(cudaStreamBeginCapture(P->st, cudaStreamCaptureModeThreadLocal));
      rc = enqueue_pool_sweep(P, P->descs.p, tiles, nullptr, tot);
      launch_pool_next_sweep(sweeps, na, P->st);
      cudaError_t e = cudaStreamEndCapture(P->st, &graph);
      P->st = exec;
      if (rc) return rc;
      if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "pool graph capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&P->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "pool graph instantiate: %s", cudaGetErrorString(e));
      memcpy(P->sweep_passes, tot, sizeof(tot));
    }
    for (int k = 0; k < nsweeps; k++) PCK(cudaGraphLaunch(P->gexec, P->st));
    memcpy(tot, P->sweep_passes, sizeof(tot));
  } else {
    for (int k = 0; k < nsweeps; k++) {
      int64_t t1[SU2GPU_NCOUNTERS] = {0};
      if ((rc = enqueue_pool_sweep(P, P->descs.p, tiles, nullptr, t1))) return rc;
      launch_pool_next_sweep(sweeps, na, P->st);
      if (k == 0) memcpy(tot, t1, sizeof(t1));
    }
  }
  for (int s : P->active)
    for (int k = 0; k < SU2GPU_NCOUNTERS; k++) P->slots[s].tot[k] += tot[k] * (int64_t)P->slots[s].g.half * nsweeps;
  return SU2GPU_OK;
}

static int pool_check(su2gpu_pool* P) {
  PCK(cudaStreamSynchronize(P->st));
  int herr = 0;
  PCK(cudaMemcpyAsync(&herr, P->err.p, sizeof(int), cudaMemcpyDeviceToHost, P->st));
  PCK(cudaStreamSynchronize(P->st));
  if (herr) {
    // the flags are reported once: cleared here, so that the next call on
    // the pool runs again (the chains of a failed call are left partly
    // swept: their fields hold whatever passes completed)
    PCK(cudaMemsetAsync(P->err.p, 0, sizeof(int), P->st));
    PCK(cudaStreamSynchronize(P->st));
    return fail(SU2GPU_ERR_KERNEL, "a pool kernel reported an invalid state (flags %d: 1 NaN fields, 2 bad tile, "
                "4 persistent sweep dependency wait timed out)", herr);
  }
  return SU2GPU_OK;
}

int su2gpu_pool_run(su2gpu_pool* P, int32_t nsweeps, int32_t use_graph) {
  int rc = pool_enqueue(P, nsweeps, use_graph);
  if (rc) return rc;
  return pool_check(P);
}

// ---------------------------------------------------------------------------
// pipelined cycle: upload, sweeps, measurement and download of the whole pool
// with the host transfers of some groups of chains under the sweeps of others
// ---------------------------------------------------------------------------
// whether the sweeps of the group [a0, a1) run as one persistent launch:
// when forced, or in the automatic mode by the pool's rule applied to the
// group alone (8 chains or more, 16 tiles or more per resident block)
static bool group_persistent(const su2gpu_pool* P, int a0, int a1) {
  if (P->npasses > PERSIST_MAX_PASSES) return false;
  if (P->persist_mode != -1) return P->persist_mode == 1;
  const int64_t tiles = P->h_tfirst[0][a1] - P->h_tfirst[0][a0];
  return a1 - a0 >= 8 && tiles >= 16 * (int64_t)std::max(1u, P->persist_grid);
}

// `n` sweeps of the active chains [a0, a1): their tile ranges and sweep
// counters (persistent: one launch; otherwise one launch per pass and sweep)
static int enqueue_group_sweep(su2gpu_pool* P, int a0, int a1, int n, int64_t* tot, bool per_pass) {
  uint32_t* const* sweeps = (uint32_t* const*)P->sweepptrs.p + a0;
  if (!per_pass && group_persistent(P, a0, a1)) {
    const int4* sg = (const int4*)P->segs.p + P->h_sfirst[a0];
    return enqueue_persist(P, sg, P->h_sfirst[a1] - P->h_sfirst[a0], sweeps, a1 - a0, n, tot);
  }
  const int2* tiles[NVARIANTS];
  int nt[NVARIANTS];
  for (int v = 0; v < NVARIANTS; v++) {
    tiles[v] = (const int2*)P->tiles[v].p + P->h_tfirst[v][a0];
    nt[v] = P->h_tfirst[v][a1] - P->h_tfirst[v][a0];
  }
  for (int k = 0; k < n; k++) {
    int64_t t1[SU2GPU_NCOUNTERS] = {0};
    int rc = enqueue_pool_sweep(P, P->descs.p, tiles, nt, k ? t1 : tot);
    if (rc) return rc;
    launch_pool_next_sweep(sweeps, a1 - a0, P->st);
  }
  PCK(cudaGetLastError());
  return SU2GPU_OK;
}

// the sweep graph of the group [a0, a1) (n sweeps per replay), captured on
// the pool's own stream
static int group_graph(su2gpu_pool* P, int a0, int a1, int n, cudaGraphExec_t* out, bool per_pass) {
  for (auto& gg : P->ggraphs)
    if (gg.a0 == a0 && gg.a1 == a1 && gg.n == n && gg.per_pass == per_pass) {
      *out = gg.exec;
      return SU2GPU_OK;
    }
  cudaStream_t exec = P->st;
  PCK(cudaStreamSynchronize(exec));
  PCK(cudaStreamSynchronize(P->own_st));
  P->st = P->own_st;
  cudaGraph_t graph;
  PCK(cudaStreamBeginCapture(P->st, cudaStreamCaptureModeThreadLocal));
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  int rc = enqueue_group_sweep(P, a0, a1, n, tot, per_pass);
  cudaError_t e = cudaStreamEndCapture(P->st, &graph);
  P->st = exec;
  if (rc) return rc;
  if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "group graph capture: %s", cudaGetErrorString(e));
  cudaGraphExec_t ge;
  e = cudaGraphInstantiate(&ge, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(SU2GPU_ERR_CUDA, "group graph instantiate: %s", cudaGetErrorString(e));
  P->ggraphs.push_back({a0, a1, n, per_pass, ge});
  *out = ge;
  return SU2GPU_OK;
}

// measure() sums of the active chains [a0, a1) into sums[a][NSUMS]
static void enqueue_group_measure(su2gpu_pool* P, int a0, int a1, double* sums) {
  const int b0 = P->h_first[a0], b1 = P->h_first[a1];
  PoolArgs a;
  memset(&a, 0, sizeof(a));
  a.descs = P->descs.p;
  a.nslots = P->max_slots;
  a.tiles = (const int2*)P->mtiles.p + b0;
  a.err = (int*)P->err.p;
  double* part = (double*)P->partials.p + (size_t)b0 * NSUMS;
  P->ops->pool_measure(a, part, b1 - b0, P->st);
  launch_pool_reduce(part, b1 - b0, (const int*)P->mfirst.p + a0, b0, a1 - a0, sums + (size_t)a0 * NSUMS, P->st);
}

// groups of consecutive active chains, G of them with about equal numbers of
// sites; light_ends: the first and the last a quarter of the others (the
// first group's upload and the last one's download in a cycle are not hidden
// under sweeps)
static std::vector<int> make_groups(const su2gpu_pool* P, int G, bool light_ends) {
  const int na = (int)P->active.size();
  int64_t total = 0;
  for (int s : P->active) total += P->slots[s].g.V;
  G = std::max(1, std::min(G, na));
  std::vector<double> edge(G + 1, 0.0);  // cumulative weight at each group's end
  for (int g = 0; g < G; g++) edge[g + 1] = edge[g] + ((light_ends && G > 2 && (g == 0 || g == G - 1)) ? 0.25 : 1.0);
  std::vector<int> b(1, 0);
  int64_t acc = 0;
  for (int a = 0; a < na; a++) {
    acc += P->slots[P->active[a]].g.V;
    const int k = (int)b.size();
    if (k < G && a + 1 < na && (double)acc >= (double)total * edge[k] / edge[G]) b.push_back(a + 1);
  }
  b.push_back(na);
  return b;
}

// the cycle's groups: about 64 MB of host arrays each, at most 32
static std::vector<int> cycle_groups(const su2gpu_pool* P) {
  int64_t total = 0;
  for (int s : P->active) total += P->slots[s].g.V;
  const int64_t bytes = total * STAGE_REALS * 8;
  int G = (int)std::min<int64_t>(32, std::max<int64_t>(1, bytes / (64ll << 20)));
  const char* e = getenv("SU2GPU_CYCLE_GROUPS");
  if (e && *e) G = std::max(1, atoi(e));
  return make_groups(P, G, true);
}

// NS of the pool's update streams (highest priority), created on first use
static int sweep_streams(su2gpu_pool* P, int NS, std::vector<cudaStream_t>& ss) {
  NS = std::max(1, std::min(NS, su2gpu_pool::CYCLE_SWEEP_STREAMS));
  ss.assign(NS, nullptr);
  for (int k = 0; k < NS; k++) {
    if (!P->sweep_st[k]) {
      int least = 0, greatest = 0;
      cudaDeviceGetStreamPriorityRange(&least, &greatest);
      PCK(cudaStreamCreateWithPriority(&P->sweep_st[k], cudaStreamNonBlocking, greatest));
    }
    ss[k] = P->sweep_st[k];
  }
  return SU2GPU_OK;
}

int su2gpu_pool_cycle(su2gpu_pool* P, int32_t n, const int32_t* slots, const double* const* const* in, int32_t nsweeps,
                      int32_t use_graph, double* sums, double* const* const* out) {
  if (!P || n < 0 || (n && !slots) || !in || !out || nsweeps < 0) return fail(SU2GPU_ERR_INVALID, "bad arguments");
  int rc;
  if ((rc = refuse_muca_batch(P, n, slots))) return rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  const int na = (int)P->active.size();
  if (n != na) return fail(SU2GPU_ERR_INVALID, "a cycle lists every active chain once (%d listed, %d active)", n, na);
  if (!na) return SU2GPU_OK;
  // position in the caller's lists of every active chain
  std::vector<int> pos(na, -1), act_of(P->max_slots, -1);
  for (int a = 0; a < na; a++) act_of[P->active[a]] = a;
  size_t total = 0, largest = 0;
  for (int j = 0; j < n; j++) {
    const int s = slots[j];
    if (s < 0 || s >= P->max_slots || act_of[s] < 0 || pos[act_of[s]] >= 0)
      return fail(SU2GPU_ERR_INVALID, "slot %d is not an active chain listed once", s);
    pos[act_of[s]] = j;
    const size_t b = (size_t)P->slots[s].g.V * STAGE_REALS * 8;
    total += b;
    largest = std::max(largest, b);
  }
  const std::vector<int> groups = cycle_groups(P);
  const int G = (int)groups.size() - 1;
  std::vector<cudaGraphExec_t> gex(G, nullptr);
  // sweeps per graph replay: all of them in one persistent launch, else one
  std::vector<int> per_replay(G, 1);
  bool any_persistent = false;
  for (int g = 0; g < G; g++)
    if (group_persistent(P, groups[g], groups[g + 1])) {
      per_replay[g] = std::max(1, (int)nsweeps);
      any_persistent = true;
    }
  // the groups' sweeps (one launch per pass: a group is a few waves of
  // blocks, each pass with its ramp and tail) run on NS streams in turn, so
  // that consecutive groups fill each other's gaps; persistent groups share
  // the work counters and stay on one stream
  int NS = any_persistent ? 1 : std::min(G, 3);
  if (const char* e = getenv("SU2GPU_CYCLE_STREAMS"); e && *e && !any_persistent)
    NS = std::max(1, std::min(std::min(G, su2gpu_pool::CYCLE_SWEEP_STREAMS), atoi(e)));
  std::vector<cudaStream_t> ss;
  if ((rc = sweep_streams(P, NS, ss))) return rc;
  if (use_graph && nsweeps > 0)
    for (int g = 0; g < G; g++)
      if ((rc = group_graph(P, groups[g], groups[g + 1], per_replay[g], &gex[g], false))) return rc;
  // staging bytes of every group; a group's chains sit side by side in the
  // rings (a ring holds the largest group at least), so a chain only ever
  // overlaps chains of earlier groups, whose release events are recorded
  std::vector<size_t> gbytes(G, 0);
  for (int g = 0; g < G; g++)
    for (int a = groups[g]; a < groups[g + 1]; a++) gbytes[g] += (size_t)P->slots[P->active[a]].g.V * STAGE_REALS * 8;
  const size_t gmax = *std::max_element(gbytes.begin(), gbytes.end());
  Ring up, down;
  if ((rc = ensure_stream(&P->copy_st)) || (rc = ensure_stream(&P->down_st)) ||
      (rc = ensure_ring(P, P->ring, total, gmax, &up)) || (rc = ensure_ring(P, P->ring_down, total, gmax, &down)) ||
      (rc = ensure_events(P->cyc_ev, 4 * (size_t)G + 1 + NS)) || (rc = P->d_items.ensure(2 * (size_t)na * sizeof(ConvItem))))
    return rc;
  if (P->h_items_n < 2 * (size_t)na) {
    if (P->h_items) cudaFreeHost(P->h_items);
    P->h_items = nullptr;
    P->h_items_n = 0;
    PCK(cudaMallocHost((void**)&P->h_items, 2 * (size_t)na * sizeof(ConvItem)));
    P->h_items_n = 2 * (size_t)na;
  }
  std::vector<cudaEvent_t>& ev = P->cyc_ev;
  ConvItem* dit = (ConvItem*)P->d_items.p;
  // the fields may still be in use by earlier work on st
  PCK(cudaEventRecord(ev[4 * G], P->st));
  PCK(cudaStreamWaitEvent(P->copy_st, ev[4 * G], 0));
  PCK(cudaStreamWaitEvent(P->down_st, ev[4 * G], 0));
  for (int k = 0; k < NS; k++) PCK(cudaStreamWaitEvent(ss[k], ev[4 * G], 0));
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  // one chain's host arrays and their staging layout
  auto layout = [&](int a, const double* const* const* tab, double** hp, ConvItem* it, size_t* bytes) {
    const Slot& sl = P->slots[P->active[a]];
    const int64_t V = sl.g.V;
    double* h[6];
    for (int k = 0; k < 6; k++) h[k] = tab[k] ? (double*)tab[k][pos[a]] : nullptr;
    const ChainIo io = chain_io(P, V, h, hp);
    int mask = 0;
    for (int k = 0; k < io.count; k++) {
      const int kind = io.kind[k];
      mask |= kind == 0 ? 1 : kind == 1 ? 2 : kind == 2 ? (4 << io.hid[k]) : kind == 3 ? 16 : 32;
    }
    it->slot = P->active[a];
    it->mask = mask;
    *bytes = io.total * 8;
    return io;
  };
  for (int g = 0; g < G; g++) {
    const int a0 = groups[g], a1 = groups[g + 1];
    int vmax = 0;
    for (int a = a0; a < a1; a++) vmax = std::max(vmax, (int)P->slots[P->active[a]].g.V);
    if (up.head + gbytes[g] > up.cap) up.head = 0;
    if (down.head + gbytes[g] > down.cap) down.head = 0;
    // upload stream: the group's host arrays -> staging (copy engine), then
    // one conversion launch into the fields
    for (int a = a0; a < a1; a++) {
      double* hp[6];
      size_t bytes, lo;
      ConvItem& it = P->h_items[a];
      const ChainIo io = layout(a, in, hp, &it, &bytes);
      if ((rc = ring_take(up, bytes, P->copy_st, &lo))) return rc;
      it.off = (long long)(lo / 8);
      size_t off = 0;
      for (int k = 0; k < io.count; k++) {
        PCK(cudaMemcpyAsync((double*)(up.base + lo) + off, hp[k], io.n[k] * 8, cudaMemcpyHostToDevice, P->copy_st));
        off += io.n[k];
      }
      up.live.push_back({lo, lo + bytes, ev[4 * g + 1]});
    }
    PCK(cudaMemcpyAsync(dit + a0, P->h_items + a0, (a1 - a0) * sizeof(ConvItem), cudaMemcpyHostToDevice, P->copy_st));
    P->pops->pool_convert(P->descs.p, dit + a0, a1 - a0, vmax, (double*)up.base, 1, P->copy_st);
    PCK(cudaEventRecord(ev[4 * g + 1], P->copy_st));
    // update stream of the group: its sweeps and measurement (the enqueue
    // helpers launch on P->st, pointed at that stream meanwhile)
    {
      cudaStream_t home = P->st;
      P->st = ss[g % NS];
      auto group_work = [&]() -> int {
        PCK(cudaStreamWaitEvent(P->st, ev[4 * g + 1], 0));
        if (nsweeps > 0) {
          if (use_graph) {
            for (int k = 0; k < nsweeps; k += per_replay[g]) PCK(cudaGraphLaunch(gex[g], P->st));
          } else {
            int64_t t1[SU2GPU_NCOUNTERS] = {0};
            if (int r = enqueue_group_sweep(P, a0, a1, nsweeps, t1, false)) return r;
          }
        }
        if (sums) enqueue_group_measure(P, a0, a1, (double*)P->sums.p);
        PCK(cudaEventRecord(ev[4 * g + 2], P->st));
        return SU2GPU_OK;
      };
      rc = group_work();
      P->st = home;
      if (rc) return rc;
    }
    // download stream: one conversion launch into staging, then the copies
    // to the host arrays
    PCK(cudaStreamWaitEvent(P->down_st, ev[4 * g + 2], 0));
    std::vector<std::pair<ChainIo, size_t>> outs;
    std::vector<std::array<double*, 6>> outp;
    for (int a = a0; a < a1; a++) {
      std::array<double*, 6> hp;
      size_t bytes, lo;
      ConvItem& it = P->h_items[na + a];
      const ChainIo io = layout(a, out, hp.data(), &it, &bytes);
      if ((rc = ring_take(down, bytes, P->down_st, &lo))) return rc;
      it.off = (long long)(lo / 8);
      outs.push_back({io, lo});
      outp.push_back(hp);
      down.live.push_back({lo, lo + bytes, ev[4 * g + 3]});
    }
    PCK(cudaMemcpyAsync(dit + na + a0, P->h_items + na + a0, (a1 - a0) * sizeof(ConvItem), cudaMemcpyHostToDevice,
                        P->down_st));
    P->pops->pool_convert(P->descs.p, dit + na + a0, a1 - a0, vmax, (double*)down.base, 0, P->down_st);
    for (size_t q = 0; q < outs.size(); q++) {
      const ChainIo& io = outs[q].first;
      size_t off = 0;
      for (int k = 0; k < io.count; k++) {
        PCK(cudaMemcpyAsync(outp[q][k], (double*)(down.base + outs[q].second) + off, io.n[k] * 8,
                            cudaMemcpyDeviceToHost, P->down_st));
        off += io.n[k];
      }
    }
    PCK(cudaEventRecord(ev[4 * g + 3], P->down_st));
    PCK(cudaGetLastError());
  }
  // half-sweeps of each kind in one sweep of a chain
  {
    std::vector<PassDesc> passes;
    sweep_recipe(P->recipe, passes, tot);
  }
  // the pool's stream follows the other update streams
  for (int k = 0; k < NS; k++) {
    PCK(cudaEventRecord(ev[4 * G + 1 + k], ss[k]));
    PCK(cudaStreamWaitEvent(P->st, ev[4 * G + 1 + k], 0));
  }
  std::vector<double> hs;
  if (sums) {
    hs.resize((size_t)na * NSUMS);
    PCK(cudaMemcpyAsync(hs.data(), P->sums.p, hs.size() * 8, cudaMemcpyDeviceToHost, P->st));
  }
  PCK(cudaStreamSynchronize(P->copy_st));
  PCK(cudaStreamSynchronize(P->down_st));
  if ((rc = pool_check(P))) return rc;
  if (sums)
    for (int a = 0; a < na; a++) memcpy(sums + (size_t)pos[a] * NSUMS, hs.data() + (size_t)a * NSUMS, NSUMS * 8);
  for (int a = 0; a < na; a++) {
    Slot& sl = P->slots[P->active[a]];
    for (int k = 0; k < SU2GPU_NCOUNTERS; k++) sl.tot[k] += tot[k] * (int64_t)sl.g.half * nsweeps;
  }
  return SU2GPU_OK;
}

int su2gpu_pool_enqueue(su2gpu_pool* P, int32_t nsweeps, int32_t use_graph) {
  return pool_enqueue(P, nsweeps, use_graph);
}

int su2gpu_pool_set_persistent(su2gpu_pool* P, int32_t on) {
  if (!P) return SU2GPU_ERR_INVALID;
  if (on > 0) {
    std::vector<PassDesc> passes;
    int64_t counts[SU2GPU_NCOUNTERS] = {0};
    sweep_recipe(P->recipe, passes, counts, P->mucamask);
    if ((int)passes.size() > PERSIST_MAX_PASSES)
      return fail(SU2GPU_ERR_INVALID, "the recipe has %d passes per sweep: the persistent sweep takes at most %d",
                  (int)passes.size(), PERSIST_MAX_PASSES);
  }
  PCK(cudaStreamSynchronize(P->st));
  P->persist_mode = on < 0 ? -1 : (on ? 1 : 0);
  P->dirty = true;  // the mode in effect and the segments are set at the rebuild
  drop_graphs(P);
  return SU2GPU_OK;
}

int su2gpu_pool_get_persist_tiles(su2gpu_pool* P, int32_t* tiles) {
  if (!P || !tiles) return SU2GPU_ERR_INVALID;
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  *tiles = P->seg_tiles;
  return SU2GPU_OK;
}

int su2gpu_pool_set_persist_shape(su2gpu_pool* P, int32_t shape) {
  if (!P || shape < 0 || shape >= PERSIST_SHAPES || !P->persist_grids[shape])
    return fail(SU2GPU_ERR_INVALID, "no such persistent launch shape");
  PCK(cudaStreamSynchronize(P->st));
  P->persist_shape = shape;
  P->persist_grid = P->persist_grids[shape];
  P->seg_tuned = 0;  // a tuned item size belongs to the shape it was timed with
  P->dirty = true;
  drop_graphs(P);
  return SU2GPU_OK;
}

int su2gpu_pool_get_persist_shape(su2gpu_pool* P, int32_t* shape, int32_t* threads, int32_t* blocks_per_sm) {
  if (!P || !shape) return SU2GPU_ERR_INVALID;
  *shape = P->persist_shape;
  if (threads) *threads = P->pers->threads;
  if (blocks_per_sm) *blocks_per_sm = P->pers->blocks_per_sm(P->persist_shape);
  return SU2GPU_OK;
}

int su2gpu_pool_get_persistent(su2gpu_pool* P, int32_t* on) {
  if (!P || !on) return SU2GPU_ERR_INVALID;
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  *on = P->persistent ? 1 : 0;
  return SU2GPU_OK;
}

// the persistent kernel on a work list whose dependencies never finish: the
// list starts at pass 1 of the chains' first sweep, and pass 0 is never run,
// so every item's wait runs out after spin_limit polls.  Fields and sweep
// counters stay as they were; *flags receives the kernel's error flags
// (4 = a wait timed out), which are cleared afterwards.
int su2gpu_pool_check_wait_timeout(su2gpu_pool* P, int32_t spin_limit, int32_t* flags) {
  if (!P || !flags || spin_limit < 1) return fail(SU2GPU_ERR_INVALID, "bad wait-timeout check arguments");
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  if (P->active.empty()) return fail(SU2GPU_ERR_INVALID, "the pool has no chains");
  PCK(cudaStreamSynchronize(P->st));
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  const int nt = (int)P->h_segs.size();
  if ((rc = enqueue_persist(P, (const int4*)P->segs.p, nt, (uint32_t* const*)P->sweepptrs.p,
                            (int)P->active.size(), 1, tot, (unsigned)nt, spin_limit)))
    return rc;
  PCK(cudaStreamSynchronize(P->st));
  int herr = 0;
  PCK(cudaMemcpy(&herr, P->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  PCK(cudaMemset(P->err.p, 0, sizeof(int)));
  *flags = herr;
  return SU2GPU_OK;
}

int su2gpu_pool_muca_set(su2gpu_pool* P, int32_t s, const su2gpu_weight* w) {
  if (!P || !w || s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
  if (w->checks_per_sweep != 1)
    return fail(SU2GPU_ERR_UNSUPPORTED, "pool chains take one multicanonical check per half-sweep (checks_per_sweep 1)");
  const int op = w->orderparam, content = P->content;
  const bool ok = (op == SU2GPU_PHISQ && (content & (SU2GPU_HIGGS1 | SU2GPU_HIGGS2))) ||
                  (op == SU2GPU_SIGMASQ && (content & SU2GPU_TRIPLET)) ||
                  (op == SU2GPU_PHI2MINUSSIGMA2 && (content & SU2GPU_HIGGS1) && (content & SU2GPU_TRIPLET)) ||
                  (op == SU2GPU_PHI2SQ && (content & SU2GPU_HIGGS2));
  if (!ok) return fail(SU2GPU_ERR_INVALID, "order parameter %d does not fit the pool's field content", op);
  PCK(cudaStreamSynchronize(P->st));
  Slot& sl = P->slots[s];
  int rc;
  if (!sl.mctx && (rc = su2gpu_attach(&sl.p, (char*)P->arena.p + sl.off, &sl.mctx))) return rc;
  if ((rc = su2gpu_muca_set(sl.mctx, w))) return rc;
  // the order parameter of both parities from the chain's current fields
  for (int par = 0; par < 2; par++)
    if ((rc = su2gpu_calc_orderparam(sl.mctx, par, nullptr))) return rc;
  int mop = 0, cps = 0, acc = 0;
  if ((rc = su2gpu_muca_device_state(sl.mctx, &sl.mdev, &sl.mbackup, &mop, &cps, &acc))) return rc;
  if (!sl.mpart && cudaMalloc((void**)&sl.mpart, (size_t)((sl.g.half + 31) / 32) * sizeof(double)) != cudaSuccess) {
    sl.mpart = nullptr;
    return fail(SU2GPU_ERR_NOMEM, "cudaMalloc of the order parameter's partial sums failed");
  }
  sl.mop = acc ? mop : 0;
  P->dirty = true;
  drop_graphs(P);
  return SU2GPU_OK;
}

int su2gpu_pool_muca_get(su2gpu_pool* P, int32_t s, su2gpu_weight* w) {
  if (!P || !w || s < 0 || s >= P->max_slots || !P->slots[s].active || !P->slots[s].mctx)
    return fail(SU2GPU_ERR_INVALID, "no multicanonical chain in that slot");
  PCK(cudaStreamSynchronize(P->st));
  return su2gpu_muca_get(P->slots[s].mctx, w);
}

int su2gpu_pool_calc_orderparam(su2gpu_pool* P, int32_t s, int32_t parity, double* value) {
  if (!P || s < 0 || s >= P->max_slots || !P->slots[s].active || !P->slots[s].mctx || parity < 0 || parity > 1)
    return fail(SU2GPU_ERR_INVALID, "no multicanonical chain in that slot");
  PCK(cudaStreamSynchronize(P->st));
  return su2gpu_calc_orderparam(P->slots[s].mctx, parity, value);
}

int su2gpu_pool_raise_error(su2gpu_pool* P, int32_t flags) {
  if (!P || flags <= 0) return fail(SU2GPU_ERR_INVALID, "bad error flags");
  PCK(cudaStreamSynchronize(P->st));
  int herr = 0;
  PCK(cudaMemcpy(&herr, P->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  herr |= flags;
  PCK(cudaMemcpy(P->err.p, &herr, sizeof(int), cudaMemcpyHostToDevice));
  return SU2GPU_OK;
}

int su2gpu_pool_set_stream(su2gpu_pool* P, void* stream) {
  if (!P) return SU2GPU_ERR_INVALID;
  PCK(cudaStreamSynchronize(P->st));
  P->st = stream ? (cudaStream_t)stream : P->own_st;
  return SU2GPU_OK;
}

int su2gpu_pool_launches_per_sweep(su2gpu_pool* P, int32_t* n) {
  if (!P || !n) return SU2GPU_ERR_INVALID;
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  if (P->persistent) {
    *n = 2;
    return SU2GPU_OK;
  }
  const int ngroups = P->grouped ? (int)P->h_groups.size() - 1 : 1;
  // the recipe's passes per sweep, in the order of enqueue_pool_sweep
  const su2gpu_params& p = P->recipe;
  const int nh = nhiggs_of(p.content);
  int passes = p.update_links * 6 * (1 + ((p.content & SU2GPU_U1) ? 1 : 0));
  int nsw = p.scalar_sweeps + 1;
  auto count = [&](int upd, int alg, int rep) {
    int c = 0;
    for (int s = 0; s < nsw; s++)
      for (int k = 0; k < upd; k++) {
        if (s >= nsw - 1 && alg != SU2GPU_OVERRELAX) continue;
        c += 2 * rep;
      }
    return c;
  };
  if (nh) passes += count(p.update_su2doublet, p.algorithm_su2doublet, nh);
  if (p.content & SU2GPU_TRIPLET) passes += count(p.update_su2triplet, p.algorithm_su2triplet, 1);
  if (p.content & SU2GPU_SINGLET) passes += count(p.update_singlet, p.algorithm_singlet, 1);
  // a decide and a restore pass after every checked half-sweep
  for (int h = 0; h < nh; h++)
    if (P->mucamask >> h & 1) passes += 2 * count(p.update_su2doublet, p.algorithm_su2doublet, 1);
  if ((p.content & SU2GPU_TRIPLET) && (P->mucamask & 4)) passes += 2 * count(p.update_su2triplet, p.algorithm_su2triplet, 1);
  *n = ngroups * (passes + 1);  // + the sweep-counter increment (per group)
  return SU2GPU_OK;
}

int su2gpu_pool_set_sweep_groups(su2gpu_pool* P, int32_t groups, int32_t streams) {
  if (!P || streams < 1 || streams > su2gpu_pool::CYCLE_SWEEP_STREAMS)
    return fail(SU2GPU_ERR_INVALID, "sweep groups: 1 to %d streams", su2gpu_pool::CYCLE_SWEEP_STREAMS);
  PCK(cudaStreamSynchronize(P->st));
  P->grp_G = groups > 1 ? groups : 0;
  P->grp_NS = groups > 1 ? streams : 1;
  P->dirty = true;
  drop_graphs(P);
  return SU2GPU_OK;
}

int su2gpu_pool_get_sweep_groups(su2gpu_pool* P, int32_t* groups, int32_t* streams) {
  if (!P || !groups || !streams) return SU2GPU_ERR_INVALID;
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  *groups = P->grouped ? (int)P->h_groups.size() - 1 : 0;
  *streams = P->grouped ? std::min(P->grp_NS, su2gpu_pool::CYCLE_SWEEP_STREAMS) : 1;
  return SU2GPU_OK;
}

// one sweep of every chain with CUDA events around every pass (the chains advance)
int su2gpu_pool_profile_sweep(su2gpu_pool* P, int32_t maxp, int32_t* kinds, float* ms, int32_t* npasses) {
  if (!P || !kinds || !ms || !npasses) return SU2GPU_ERR_INVALID;
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  *npasses = 0;
  if (P->active.empty()) return SU2GPU_OK;
  const int2* tiles[NVARIANTS];
  for (int v = 0; v < NVARIANTS; v++) tiles[v] = (const int2*)P->tiles[v].p;
  std::vector<cudaEvent_t> ev;
  std::vector<int> kd;
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  P->prof = &ev;
  P->prof_kind = &kd;
  rc = enqueue_pool_sweep(P, P->descs.p, tiles, nullptr, tot);
  P->prof = nullptr;
  P->prof_kind = nullptr;
  if (!rc) launch_pool_next_sweep((uint32_t* const*)P->sweepptrs.p, (int)P->active.size(), P->st);
  for (int s : P->active)
    for (int k = 0; k < SU2GPU_NCOUNTERS; k++) P->slots[s].tot[k] += tot[k] * (int64_t)P->slots[s].g.half;
  if (!rc) rc = pool_check(P);
  int n = 0;
  for (size_t k = 0; !rc && k + 1 < ev.size() && n < maxp; k++, n++) {
    kinds[n] = kd[k];
    cudaEventElapsedTime(&ms[n], ev[k], ev[k + 1]);
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  *npasses = n;
  return rc;
}

int su2gpu_pool_active(su2gpu_pool* P, int32_t* slots, int32_t max, int32_t* n) {
  if (!P || !n) return SU2GPU_ERR_INVALID;
  int k = 0;
  for (int s = 0; s < P->max_slots; s++)
    if (P->slots[s].active) {
      if (slots && k < max) slots[k] = s;
      k++;
    }
  *n = k;
  return SU2GPU_OK;
}

// measure() sums of every active chain, in slot order: sums[k*NMEAS + m]
static int pool_enqueue_measure(su2gpu_pool* P, double* dev_out, int32_t max_chains, int32_t* nchains) {
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  int n = (int)P->active.size();
  *nchains = n;
  if (!n) return SU2GPU_OK;
  if (n > max_chains) return fail(SU2GPU_ERR_INVALID, "output holds %d chains, pool has %d", max_chains, n);
  PoolArgs a;
  memset(&a, 0, sizeof(a));
  a.descs = P->descs.p;
  a.nslots = P->max_slots;
  a.tiles = (const int2*)P->mtiles.p;
  a.err = (int*)P->err.p;
  P->ops->pool_measure(a, (double*)P->partials.p, P->nmtiles, P->st);
  launch_pool_reduce((const double*)P->partials.p, P->nmtiles, (const int*)P->mfirst.p, 0, n, dev_out, P->st);
  PCK(cudaGetLastError());
  return SU2GPU_OK;
}

int su2gpu_pool_measure(su2gpu_pool* P, double* sums, int32_t max_chains, int32_t* nchains) {
  if (!P || !sums || !nchains) return SU2GPU_ERR_INVALID;
  int rc = pool_enqueue_measure(P, (double*)P->sums.p, max_chains, nchains);
  if (rc || !*nchains) return rc;
  PCK(cudaMemcpyAsync(sums, P->sums.p, (size_t)*nchains * NSUMS * 8, cudaMemcpyDeviceToHost, P->st));
  PCK(cudaStreamSynchronize(P->st));
  return SU2GPU_OK;
}

int su2gpu_pool_enqueue_measure(su2gpu_pool* P, double* device_sums, int32_t max_chains, int32_t* nchains) {
  if (!P || !device_sums || !nchains) return SU2GPU_ERR_INVALID;
  return pool_enqueue_measure(P, device_sums, max_chains, nchains);
}

int su2gpu_pool_counters(su2gpu_pool* P, int32_t s, int64_t* out) {
  if (!P || !out || s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
  unsigned long long d[SU2GPU_NCOUNTERS];
  PCK(cudaMemcpyAsync(d, (char*)P->slotmem.p + (size_t)s * 256 + 32, sizeof(d), cudaMemcpyDeviceToHost, P->st));
  PCK(cudaStreamSynchronize(P->st));
  for (int k = 0; k < SU2GPU_NCOUNTERS; k++) out[k] = (int64_t)d[k] + P->slots[s].tot[k];
  return SU2GPU_OK;
}

// launch shapes for the pool's kernels, timed on a scratch copy of the arena
// sweeps per timed launch when the autotuner compares sweep modes: several,
// so that ramps, tails and the streams' drift weigh as in a run
constexpr int TUNE_SWEEPS = 3;

// mean time of one sweep of every chain (no sweep-counter increment) with
// the chains in G groups whose TUNE_SWEEPS sweeps (one launch per pass, a
// graph per group) run on NS streams in turn; G = 1: one stream, one graph
static int time_grouped(su2gpu_pool* P, void* descs, int G, int NS, int reps, float* ms_out) {
  const std::vector<int> groups = make_groups(P, G, false);
  const int Gn = (int)groups.size() - 1;
  std::vector<cudaGraphExec_t> gex(Gn, nullptr);
  std::vector<cudaStream_t> ss;
  int rc;
  if ((rc = sweep_streams(P, NS, ss)) || (rc = ensure_events(P->grp_ev, ss.size() + 1))) return rc;
  cudaStream_t exec = P->st;
  PCK(cudaStreamSynchronize(exec));
  PCK(cudaStreamSynchronize(P->own_st));
  cudaEvent_t e0, e1;  // timing events (the pool's join events record no time)
  PCK(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(SU2GPU_ERR_CUDA, "cudaEventCreate failed");
  }
  for (int g = 0; g < Gn && !rc; g++) {
    const int2* tiles[NVARIANTS];
    int nt[NVARIANTS];
    for (int v = 0; v < NVARIANTS; v++) {
      tiles[v] = (const int2*)P->tiles[v].p + P->h_tfirst[v][groups[g]];
      nt[v] = P->h_tfirst[v][groups[g + 1]] - P->h_tfirst[v][groups[g]];
    }
    P->st = P->own_st;
    cudaGraph_t graph;
    int64_t t1[SU2GPU_NCOUNTERS] = {0};
    cudaError_t e = cudaStreamBeginCapture(P->st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      for (int k = 0; k < TUNE_SWEEPS && !rc; k++) rc = enqueue_pool_sweep(P, descs, tiles, nt, t1);
      e = cudaStreamEndCapture(P->st, &graph);
      if (e == cudaSuccess) {
        e = cudaGraphInstantiate(&gex[g], graph, 0);
        cudaGraphDestroy(graph);
      }
    }
    P->st = exec;
    if (!rc && e != cudaSuccess) rc = fail(SU2GPU_ERR_CUDA, "grouped sweep timing: %s", cudaGetErrorString(e));
  }
  float ms = 0.f;
  for (int r = -1; r < reps && !rc; r++) {
    cudaEventRecord(e0, P->st);
    for (int k = 0; k < (int)ss.size(); k++) cudaStreamWaitEvent(ss[k], e0, 0);
    for (int g = 0; g < Gn; g++) cudaGraphLaunch(gex[g], ss[g % ss.size()]);
    for (int k = 0; k < (int)ss.size(); k++) {
      cudaEventRecord(P->grp_ev[k + 1], ss[k]);
      cudaStreamWaitEvent(P->st, P->grp_ev[k + 1], 0);
    }
    cudaEventRecord(e1, P->st);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = fail(SU2GPU_ERR_CUDA, "grouped sweep timing: %s", cudaGetErrorString(e));
      break;
    }
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (r >= 0) ms += t;
  }
  for (cudaGraphExec_t g : gex)
    if (g) cudaGraphExecDestroy(g);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_out = ms / reps / TUNE_SWEEPS;
  return rc;
}

int su2gpu_pool_autotune(su2gpu_pool* P, int32_t* choices, float* best_ms) {
  if (!P) return SU2GPU_ERR_INVALID;
  int rc;
  if (P->dirty && (rc = rebuild(P))) return rc;
  if (P->active.empty()) return SU2GPU_OK;
  size_t used = 0;
  for (int s : P->active) used = std::max(used, P->slots[s].off + P->slots[s].bytes);
  Buf arena2, slot2, desc2;
  if ((rc = arena2.ensure(used)) || (rc = slot2.ensure(P->slotmem.n)) || (rc = desc2.ensure(P->descs.n))) return rc;
  PCK(cudaMemcpyAsync(arena2.p, P->arena.p, used, cudaMemcpyDeviceToDevice, P->st));
  PCK(cudaMemcpyAsync(slot2.p, P->slotmem.p, P->slotmem.n, cudaMemcpyDeviceToDevice, P->st));
  if ((rc = rebuild(P, arena2.p, slot2.p, desc2.p))) return rc;
  const int nh = nhiggs_of(P->content);
  bool present[5] = {true, (bool)(P->content & SU2GPU_U1), nh > 0, (bool)(P->content & SU2GPU_TRIPLET),
                     (bool)(P->content & SU2GPU_SINGLET)};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  PoolArgs a;
  memset(&a, 0, sizeof(a));
  a.descs = desc2.p;
  a.nslots = P->max_slots;
  a.err = (int*)P->err.p;
  const int reps = 3;
  float base_ms = 0.f;  // one sweep in the mode the pool would use without groups
  for (int kind = 0; kind < 5; kind++) {
    if (!present[kind]) continue;
    float best = 1e30f;
    int bestv = 0;
    for (int v = 0; v < NVARIANTS; v++) {
      float ms = 0.f;
      for (int r = -1; r < reps; r++) {
        a.parity = r & 1;
        a.sub = kind <= 1 ? (r + 3) % 3 : 0;
        a.alg = kind == 0 ? P->recipe.algorithm_su2link : 0;
        a.pass = 60000 + r;
        a.tiles = (const int2*)P->tiles[v].p;
        cudaEventRecord(e0, P->st);
        if (kind == 0) P->pers->pool_link(v, a, P->ntiles[v], P->st);
        else if (kind == 1) P->pers->pool_u1(v, a, P->ntiles[v], P->st);
        else P->pers->pool_scalar(v, kind - 2, a, P->ntiles[v], P->st);
        cudaEventRecord(e1, P->st);
        PCK(cudaEventSynchronize(e1));
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r >= 0) ms += t;
      }
      if (ms < best) { best = ms; bestv = v; }
    }
    P->var[kind] = bestv;
    if (best_ms) best_ms[kind] = best / reps;
  }
  // the persistent sweep's work-item size (tiles per segment), when the pool
  // sweeps persistently: one sweep of every chain per candidate, timed on
  // the scratch copy, the fastest kept (unless SU2GPU_PERSIST_TILES fixes it)
  if (P->persistent && !P->seg_env) {
    int64_t ntiles_all = 0;
    for (int s : P->active) ntiles_all += (P->slots[s].g.half + kVariantBS[0] - 1) / kVariantBS[0];
    const int cand[7] = {4, 6, 8, 12, 16, 24, 32};
    float best = 1e30f;
    int bestseg = P->seg_tiles, bestshape = P->persist_shape;
    Buf segbuf;
    std::vector<int4> tab;
    // every launch shape of the persistent kernel with every item size
    for (int shape = 0; shape < PERSIST_SHAPES && !rc; shape++)
    for (int seg : cand) {
      if (!P->persist_grids[shape]) break;
      P->persist_shape = shape;
      P->persist_grid = P->persist_grids[shape];
      if (ntiles_all / seg < (int64_t)P->persist_grid) continue;  // at least one item per resident block and pass
      tab.clear();
      for (int s : P->active) append_segments(P, s, seg, tab);
      if ((rc = segbuf.ensure(tab.size() * sizeof(int4)))) break;
      PCK(cudaMemcpyAsync(segbuf.p, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice, P->st));
      float ms = 0.f;
      for (int r = -1; r < reps; r++) {
        int64_t t1[SU2GPU_NCOUNTERS] = {0};
        cudaEventRecord(e0, P->st);
        rc = enqueue_persist(P, (const int4*)segbuf.p, (int)tab.size(), nullptr, (int)P->active.size(), 1, t1, 0,
                             1 << 18, desc2.p, seg);
        cudaEventRecord(e1, P->st);
        if (rc) break;
        PCK(cudaEventSynchronize(e1));
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r >= 0) ms += t;
      }
      if (rc) break;
      // a candidate whose dependency wait gave up skipped its remaining
      // items (and so finished early): its flags are cleared and it is not kept
      int herr = 0;
      PCK(cudaMemcpyAsync(&herr, P->err.p, sizeof(int), cudaMemcpyDeviceToHost, P->st));
      PCK(cudaStreamSynchronize(P->st));
      if (herr) {
        PCK(cudaMemsetAsync(P->err.p, 0, sizeof(int), P->st));
        continue;
      }
      if (ms < best) { best = ms; bestseg = seg; bestshape = shape; }
    }
    P->persist_shape = bestshape;
    P->persist_grid = P->persist_grids[bestshape];
    if (!rc) {
      P->seg_tuned = bestseg;
      P->dirty = true;  // the segment table is rebuilt with the pick
      // the pick with TUNE_SWEEPS sweeps per launch: the baseline of the
      // grouped mode below
      tab.clear();
      for (int s : P->active) append_segments(P, s, bestseg, tab);
      if (!(rc = segbuf.ensure(tab.size() * sizeof(int4)))) {
        PCK(cudaMemcpyAsync(segbuf.p, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice, P->st));
        float ms = 0.f;
        for (int r = -1; r < reps && !rc; r++) {
          int64_t t1[SU2GPU_NCOUNTERS] = {0};
          cudaEventRecord(e0, P->st);
          rc = enqueue_persist(P, (const int4*)segbuf.p, (int)tab.size(), nullptr, (int)P->active.size(),
                               TUNE_SWEEPS, t1, 0, 1 << 18, desc2.p, bestseg);
          cudaEventRecord(e1, P->st);
          if (rc) break;
          PCK(cudaEventSynchronize(e1));
          float t = 0.f;
          cudaEventElapsedTime(&t, e0, e1);
          if (r >= 0) ms += t;
        }
        int herr = 0;
        PCK(cudaMemcpyAsync(&herr, P->err.p, sizeof(int), cudaMemcpyDeviceToHost, P->st));
        PCK(cudaStreamSynchronize(P->st));
        if (herr) PCK(cudaMemsetAsync(P->err.p, 0, sizeof(int), P->st));
        // a baseline whose wait gave up is not trusted: the grouped mode is
        // then compared with one launch per pass
        if (!rc && !herr) base_ms = ms / reps / TUNE_SWEEPS;
      }
    }
    segbuf.release();
  }
  // the grouped mode against the mode the pool would otherwise use (one
  // persistent launch, or one launch per pass on one stream): TUNE_SWEEPS
  // sweeps of every chain per candidate (groups x streams), on the scratch copy
  // SU2GPU_SWEEP_GROUPS="G,NS" fixes the pick (a profiler that serialises
  // kernels cannot time the overlap the grouped mode is for)
  const char* fixg = getenv("SU2GPU_SWEEP_GROUPS");
  if (!rc && fixg && *fixg) {
    int g = 0, ns = 1;
    if (sscanf(fixg, "%d,%d", &g, &ns) >= 1) {
      P->grp_G = g > 1 ? g : 0;
      P->grp_NS = std::max(1, std::min(ns, su2gpu_pool::CYCLE_SWEEP_STREAMS));
      P->dirty = true;
    }
  } else if (!rc && P->persist_mode == -1 && P->nmuca == 0 && P->active.size() >= 8) {
    const int na = (int)P->active.size();
    if (base_ms <= 0.f && (rc = time_grouped(P, desc2.p, 1, 1, reps, &base_ms))) {
      // base_ms stays unset; rc is returned below
    }
    // (groups, streams): on the 384-chain ensemble (11 M sites) groups of
    // about 0.23 M sites on 4 streams were fastest (48 groups); the
    // candidates are around that group size, on 3 and 4 streams
    std::vector<std::pair<int, int>> cand;
    auto add = [&](int g, int ns) {
      if (g < 3 || g > na) return;
      for (auto& c : cand)
        if (c.first == g && c.second == ns) return;
      cand.push_back({g, ns});
    };
    int64_t total_sites = 0;
    for (int s : P->active) total_sites += P->slots[s].g.V;
    const int gt = (int)std::max<int64_t>(3, (total_sites + 115000) / 230000);
    for (int ns : {4, 3}) {
      add(gt, ns);
      add(gt * 2 / 3, ns);
      add(gt * 4 / 3, ns);
    }
    add(gt / 2, 3);
    add(gt * 2, 4);
    float bestg = base_ms;
    int bg = 0, bns = 1;
    for (size_t c = 0; c < cand.size() && !rc; c++) {
      float ms = 0.f;
      if ((rc = time_grouped(P, desc2.p, cand[c].first, cand[c].second, reps, &ms))) break;
      if (ms < bestg) { bestg = ms; bg = cand[c].first; bns = cand[c].second; }
    }
    // the grouped mode only where it wins clearly (2 %): a near tie is left to
    // the mode the pool would use anyway
    if (bg && !(bestg < 0.98f * base_ms)) bg = 0;
    if (!rc) {
      P->grp_G = bg;
      P->grp_NS = bg ? bns : 1;
      P->dirty = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  PCK(cudaStreamSynchronize(P->st));
  arena2.release(); slot2.release(); desc2.release();
  drop_graphs(P);
  if (choices)
    for (int k = 0; k < 5; k++) choices[k] = P->var[k];
  return SU2GPU_OK;
}

int su2gpu_pool_set_variants(su2gpu_pool* P, const int32_t* choices) {
  if (!P || !choices) return SU2GPU_ERR_INVALID;
  for (int k = 0; k < 5; k++) {
    if (choices[k] < 0 || choices[k] >= NVARIANTS) return SU2GPU_ERR_INVALID;
    P->var[k] = choices[k];
  }
  drop_graphs(P);
  return SU2GPU_OK;
}

}  // extern "C"

// a chain copied out of the pool into a single-lattice context of its own
// (same parameters, seed and chain id; the chain stays in the pool)
extern "C" int su2gpu_pool_extract(su2gpu_pool* P, int32_t s, su2gpu_ctx** out) {
  if (!P || !out || s < 0 || s >= P->max_slots || !P->slots[s].active) return fail(SU2GPU_ERR_INVALID, "no such chain slot");
  PCK(cudaStreamSynchronize(P->st));
  const Slot& sl = P->slots[s];
  return su2gpu_create_copy(&sl.p, (const char*)P->arena.p + sl.off, sl.seed, sl.chain, out);
}

// gradient flow of one chain (gradflow.c:46-173): a context over the chain's
// fields in the arena runs the single-lattice flow on its own copies
extern "C" int su2gpu_pool_grad_flow(su2gpu_pool* P, int32_t s, double t_max, double dt, int32_t meas_interval,
                                     double* rows, int32_t maxrows, int32_t* nrows) {
  if (!P || !rows || !nrows || meas_interval <= 0 || dt <= 0 || s < 0 || s >= P->max_slots || !P->slots[s].active)
    return fail(SU2GPU_ERR_INVALID, "bad flow arguments");
  PCK(cudaStreamSynchronize(P->st));
  su2gpu_ctx* c = nullptr;
  int rc = su2gpu_attach(&P->slots[s].p, (char*)P->arena.p + P->slots[s].off, &c);
  if (rc) return rc;
  rc = su2gpu_grad_flow(c, t_max, dt, meas_interval, rows, maxrows, nrows);
  su2gpu_destroy(c);
  return rc;
}
