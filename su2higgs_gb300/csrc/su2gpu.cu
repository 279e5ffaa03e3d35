// su2gpu.cu -- the C ABI of libsu2gpu (include/su2gpu.h): device-resident
// lattice contexts, the half-sweep sequence of the reference's
// update_lattice() (update.c:270-430), multicanonical global checks decided
// on the device, measurements, gradient flow and CUDA-graph replay.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/su2gpu.h"
#include "su2_correl.h"
#include "su2_host.h"
#include "su2_kernels.cuh"
#include "su2_ops.h"

using namespace su2;

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";
static void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
// C++ linkage, not part of the ABI: lets other units of the library set the
// text returned by su2gpu_last_error
void su2gpu_record_error(const char* msg) { set_err("%s", msg); }

#define CK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return SU2GPU_ERR_CUDA;                                                        \
    }                                                                                \
  } while (0)
#define CKL()                                                                        \
  do {                                                                               \
    cudaError_t e_ = cudaGetLastError();                                             \
    if (e_ != cudaSuccess) {                                                         \
      set_err("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return SU2GPU_ERR_CUDA;                                                        \
    }                                                                                \
  } while (0)

static unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

__global__ void k_set_u32(uint32_t* p, uint32_t v) { *p = v; }
__global__ void k_inc_u32(uint32_t* p) { *p += 1u; }
__global__ void k_fill_u64(unsigned long long* p, unsigned long long v) { *p = v; }

// layout tables (layout.c:657-756 serial order) from the closed form
__global__ void k_layout_tables(Geom g, int64_t* next, int64_t* prev, int64_t* coords, int32_t* parity) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.V) return;
  int par = i >= g.half;
  int c[3];
  site_coords(g, par, i - par * g.half, c);
  for (int d = 0; d < 3; d++) {
    next[i * 3 + d] = shifted(g, c, d, 1);
    prev[i * 3 + d] = shifted(g, c, d, -1);
    coords[i * 3 + d] = c[d];
  }
  parity[i] = par;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  int ensure(size_t bytes) {
    if (bytes <= n) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      set_err("cudaMalloc(%zu) failed", bytes);
      return SU2GPU_ERR_NOMEM;
    }
    n = bytes;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// device words of a context: counters, error flag, sweep number, flow
// marker, and from byte 4096 the arrival counts of a multicanonical check
// decided inside its update launch (1 + MUCA_MAX_CHUNKS words)
constexpr size_t CTRBUF_BYTES = 4096 + 4 * (1 + MUCA_MAX_CHUNKS) + 4;

struct su2gpu_ctx {
  su2gpu_params p;
  int prec, nh, has_t, has_s, has_u1;
  Geom g;
  Coup cp;
  const Ops* ops;
  const PrecOps* pops;
  cudaStream_t st = nullptr;      // execution stream (the caller's, or own_st)
  cudaStream_t own_st = nullptr;  // the context's own stream; graphs are captured on it
  int launches = 0;               // kernel launches enqueued by the last sweep
  std::vector<cudaEvent_t>* prof = nullptr;  // per-pass events while profiling
  std::vector<int>* prof_kind = nullptr;
  DevBuf fields, stage, ctrbuf, partials, sums, alpha, backup, muca, flow, rows, local, correl;
  bool borrowed = false;  // fields belong to another allocation (su2gpu_attach)
  Fields<double> f64{};
  Fields<float> f32{};
  unsigned long long* d_ctr = nullptr;  // [24] counters (accepted + muca)
  int* d_err = nullptr;
  uint32_t* d_sweep = nullptr;
  unsigned long long* d_fz = nullptr;
  unsigned* d_arrive = nullptr;  // arrival counts of the multicanonical check decided in the pass
  int64_t host_tot[SU2GPU_NCOUNTERS] = {0};
  int var[5] = {0, 0, 0, 0, 0};  // launch-shape variant per kernel kind (link, U(1), doublet, triplet, singlet)
  int random_sweeps = 0;         // the reference's random_sweeps mode: the order changes every sweep
  uint64_t seed = 0;
  uint32_t chain = 0;
  // multicanonical
  bool muca_on = false;
  int muca_bins = 0;
  MucaDev* d_muca = nullptr;
  int muca_orderparam = 0, muca_cps = 1, muca_do_acc = 0;
  // graph of one sweep
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_tot[SU2GPU_NCOUNTERS] = {0};

  const void* F() const { return prec == 64 ? (const void*)&f64 : (const void*)&f32; }
  size_t rsize() const { return prec == 64 ? 8 : 4; }
  size_t v4size() const { return prec == 64 ? 32 : 16; }
};

static int valid_params(const su2gpu_params* p) {
  if (!p) return 0;
  if (p->dim != 3) { set_err("only dim 3 is supported on the GPU (got %d)", p->dim); return 0; }
  for (int d = 0; d < 3; d++)
    if (p->L[d] < 2 || (p->L[d] & 1)) { set_err("L%d = %d: side lengths must be even and >= 2", d + 1, p->L[d]); return 0; }
  if ((double)p->L[0] * p->L[1] * p->L[2] * 3.0 >= 2147483647.0) { set_err("lattice too large (3 V must fit in 31 bits)"); return 0; }
  if (p->precision != 64 && p->precision != 32) { set_err("precision must be 64 or 32"); return 0; }
  int c = p->content;
  if ((c & SU2GPU_HIGGS1) && (c & SU2GPU_HIGGS2)) { set_err("HIGGS1 and HIGGS2 are exclusive"); return 0; }
  if ((c & SU2GPU_HIGGS2) && (c & (SU2GPU_TRIPLET | SU2GPU_SINGLET))) {
    set_err("two doublets with a triplet or singlet are not implemented (as in the reference)");
    return 0;
  }
  if (p->algorithm_su2link != SU2GPU_HEATBATH && p->algorithm_su2link != SU2GPU_METROPOLIS) {
    set_err("algorithm_su2link must be heatbath or metropolis"); return 0;
  }
  return 1;
}

Coup su2::make_coup(const su2gpu_params* p) {
  Coup c;
  c.beta = p->betasu2; c.msq = p->msq_phi; c.lam = p->lambda_phi;
  c.msqT = p->msq_triplet; c.a2 = p->a2; c.b4 = p->b4;
  c.betau1 = p->betau1; c.r_u1 = p->r_u1;
  c.b1s = p->b1_s; c.msqs = p->msq_s; c.b3s = p->b3_s; c.b4s = p->b4_s; c.a1s = p->a1_s; c.a2s = p->a2_s;
  c.msq2 = p->msq_phi2; c.m12re = p->m12sq_re; c.m12im = p->m12sq_im;
  c.lam2 = p->lam2; c.lam3 = p->lam3; c.lam4 = p->lam4; c.lam5re = p->lam5_re; c.lam5im = p->lam5_im;
  c.lam6re = p->lam6_re; c.lam6im = p->lam6_im; c.lam7re = p->lam7_re; c.lam7im = p->lam7_im;
  c.content = p->content & 0x1f;
  c.alg_link = p->algorithm_su2link; c.alg_u1 = p->algorithm_u1link; c.alg_d = p->algorithm_su2doublet;
  c.alg_t = p->algorithm_su2triplet; c.alg_s = p->algorithm_singlet;
  return c;
}

const Ops* su2::pick_ops(int prec, int content) {
  int c = content & 0x1f;
  if (prec == 64) {
    if (c == C_H1) return &ops_f64_fund;
    if (c == C_T) return &ops_f64_adj;
    if (c == (C_H1 | C_S | C_U1)) return &ops_f64_su2u1s;
    return &ops_f64_generic;
  }
  if (c == C_H1) return &ops_f32_fund;
  if (c == C_T) return &ops_f32_adj;
  if (c == (C_H1 | C_S | C_U1)) return &ops_f32_su2u1s;
  return &ops_f32_generic;
}

// the pool update kernels of the same instantiation as pick_ops
const PoolOps* su2::pick_persist(int prec, int content) {
  int c = content & 0x1f;
  if (prec == 64) {
    if (c == C_H1) return &persist_f64_fund;
    if (c == C_T) return &persist_f64_adj;
    if (c == (C_H1 | C_S | C_U1)) return &persist_f64_su2u1s;
    return &persist_f64_generic;
  }
  if (c == C_H1) return &persist_f32_fund;
  if (c == C_T) return &persist_f32_adj;
  if (c == (C_H1 | C_S | C_U1)) return &persist_f32_su2u1s;
  return &persist_f32_generic;
}

extern "C" {

int su2gpu_version(void) { return 10000; }

const char* su2gpu_last_error(void) { return g_err; }

int su2gpu_device_info(int* sm_count, int* cc_major, int* cc_minor, int64_t* free_bytes) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  cudaDeviceProp pr;
  CK(cudaGetDeviceProperties(&pr, dev));
  if (sm_count) *sm_count = pr.multiProcessorCount;
  if (cc_major) *cc_major = pr.major;
  if (cc_minor) *cc_minor = pr.minor;
  if (free_bytes) {
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    *free_bytes = (int64_t)fr;
  }
  return SU2GPU_OK;
}

int64_t su2gpu_footprint_bytes(const su2gpu_params* p) {
  if (!valid_params(p)) return -1;
  int64_t V = (int64_t)p->L[0] * p->L[1] * p->L[2];
  size_t b = field_bytes(p, V);
  b += align256((size_t)(V / BLOCK + 2) * NSUMS * 8);        // partials
  b += 4096;                                                 // counters, flags, sums
  if (p->content & SU2GPU_TRIPLET) b += align256(3 * V * 8);  // alpha planes
  return (int64_t)b;
}

static int create_ctx(const su2gpu_params* p, void* borrowed, const void* copy_from, su2gpu_ctx** out) {
  if (!out) return SU2GPU_ERR_INVALID;
  *out = nullptr;
  if (!valid_params(p)) return SU2GPU_ERR_INVALID;
  su2gpu_ctx* c = new su2gpu_ctx();
  c->p = *p;
  c->prec = p->precision;
  c->nh = (p->content & SU2GPU_HIGGS2) ? 2 : ((p->content & SU2GPU_HIGGS1) ? 1 : 0);
  c->has_t = !!(p->content & SU2GPU_TRIPLET);
  c->has_s = !!(p->content & SU2GPU_SINGLET);
  c->has_u1 = !!(p->content & SU2GPU_U1);
  c->g = make_geom(p->L[0], p->L[1], p->L[2]);
  c->cp = make_coup(p);
  c->ops = pick_ops(c->prec, p->content);
  c->pops = c->prec == 64 ? &precops_f64 : &precops_f32;
  int rc;
  if (cudaStreamCreateWithFlags(&c->own_st, cudaStreamNonBlocking) != cudaSuccess) {
    set_err("cudaStreamCreate failed");
    delete c;
    return SU2GPU_ERR_CUDA;
  }
  c->st = c->own_st;
  int64_t V = c->g.V;
  if (borrowed) {
    c->fields.p = borrowed;
    c->fields.n = field_bytes(p, V);
    c->borrowed = true;
  }
  if ((!borrowed && (rc = c->fields.ensure(field_bytes(p, V)))) ||
      (rc = c->ctrbuf.ensure(CTRBUF_BYTES)) ||
      (rc = c->partials.ensure((size_t)(nblk(V, BLOCK) + 2) * NSUMS * 8)) ||
      (rc = c->sums.ensure(NSUMS * 8))) {
    su2gpu_destroy(c);
    return rc;
  }
  if (c->prec == 64) carve(c->f64, (char*)c->fields.p, p, V);
  else carve(c->f32, (char*)c->fields.p, p, V);
  c->d_ctr = (unsigned long long*)c->ctrbuf.p;
  c->d_err = (int*)((char*)c->ctrbuf.p + 512);
  c->d_sweep = (uint32_t*)((char*)c->ctrbuf.p + 1024);
  c->d_fz = (unsigned long long*)((char*)c->ctrbuf.p + 1536);
  c->d_arrive = (unsigned*)((char*)c->ctrbuf.p + 4096);
  if ((!borrowed && !copy_from && cudaMemsetAsync(c->fields.p, 0, c->fields.n, c->st) != cudaSuccess) ||
      (copy_from && cudaMemcpyAsync(c->fields.p, copy_from, c->fields.n, cudaMemcpyDeviceToDevice, c->st) != cudaSuccess) ||
      cudaMemsetAsync(c->ctrbuf.p, 0, c->ctrbuf.n, c->st) != cudaSuccess) {
    set_err("cudaMemset failed");
    su2gpu_destroy(c);
    return SU2GPU_ERR_CUDA;
  }
  // cold links: unit quaternions (setsu2, init.c:18-28)
  if (!borrowed && !copy_from) {
    std::vector<double> one((size_t)V * 12, 0.0);
    for (int64_t k = 0; k < V * 3; k++) one[(size_t)k * 4] = 1.0;
    if ((rc = c->stage.ensure((size_t)V * 12 * 8))) { su2gpu_destroy(c); return rc; }
    if (cudaMemcpyAsync(c->stage.p, one.data(), (size_t)V * 12 * 8, cudaMemcpyHostToDevice, c->st) != cudaSuccess) {
      set_err("cold-start upload failed");
      su2gpu_destroy(c);
      return SU2GPU_ERR_CUDA;
    }
    c->pops->import(c->F(), V, 0, 0, (const double*)c->stage.p, c->st);
    if (cudaStreamSynchronize(c->st) != cudaSuccess) {
      set_err("cold start failed: %s", cudaGetErrorString(cudaGetLastError()));
      su2gpu_destroy(c);
      return SU2GPU_ERR_CUDA;
    }
  }
  if ((borrowed || copy_from) && cudaStreamSynchronize(c->st) != cudaSuccess) {
    set_err("context set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
    su2gpu_destroy(c);
    return SU2GPU_ERR_CUDA;
  }
  *out = c;
  return SU2GPU_OK;
}

int su2gpu_create(const su2gpu_params* p, su2gpu_ctx** out) { return create_ctx(p, nullptr, nullptr, out); }

int su2gpu_destroy(su2gpu_ctx* c) {
  if (!c) return SU2GPU_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->own_st) cudaStreamSynchronize(c->own_st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->borrowed) c->fields.p = nullptr;
  c->fields.release(); c->stage.release(); c->ctrbuf.release(); c->partials.release(); c->sums.release();
  c->alpha.release(); c->backup.release(); c->muca.release(); c->flow.release(); c->rows.release();
  c->local.release(); c->correl.release();
  if (c->own_st) cudaStreamDestroy(c->own_st);
  delete c;
  return SU2GPU_OK;
}

int su2gpu_layout_tables(su2gpu_ctx* c, int64_t* next, int64_t* prev, int64_t* coords, int32_t* parity) {
  if (!c) return SU2GPU_ERR_INVALID;
  int64_t V = c->g.V;
  DevBuf t;
  int rc = t.ensure((size_t)V * (3 * 8 * 3 + 4));
  if (rc) return rc;
  int64_t* dn = (int64_t*)t.p;
  int64_t* dp = dn + V * 3;
  int64_t* dc = dp + V * 3;
  int32_t* dpar = (int32_t*)(dc + V * 3);
  k_layout_tables<<<nblk(V, 256), 256, 0, c->st>>>(c->g, dn, dp, dc, dpar);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && next) e = cudaMemcpyAsync(next, dn, V * 24, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess && prev) e = cudaMemcpyAsync(prev, dp, V * 24, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess && coords) e = cudaMemcpyAsync(coords, dc, V * 24, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess && parity) e = cudaMemcpyAsync(parity, dpar, V * 4, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  t.release();
  if (e != cudaSuccess) { set_err("layout tables: %s", cudaGetErrorString(e)); return SU2GPU_ERR_CUDA; }
  return SU2GPU_OK;
}

// ---------------------------------------------------------------------------
// field transfer
// ---------------------------------------------------------------------------
int su2gpu_site_values(su2gpu_ctx* c, int32_t what, double* out) {
  if (!c || !out) return SU2GPU_ERR_INVALID;
  if (c->prec != 64) {
    set_err("per-site values are computed on FP64 contexts only");
    return SU2GPU_ERR_UNSUPPORTED;
  }
  static_assert(SITE_OR_SINGLET == SU2GPU_SITE_OR_SINGLET, "site value codes differ");
  int width = 0;
  bool present = true;
  switch (what) {
    case SU2GPU_SITE_LINK_STAPLE: case SU2GPU_SITE_WILSON_STAPLE: width = 12; break;
    case SU2GPU_SITE_LOCALACT_SU2LINK: width = 3; break;
    case SU2GPU_SITE_LOCALACT_U1LINK: width = 3; present = c->has_u1; break;
    case SU2GPU_SITE_STAPLE_DOUBLET: width = 4; present = c->nh > 0; break;
    case SU2GPU_SITE_LOCALACT_DOUBLET: width = 1; present = c->nh > 0; break;
    case SU2GPU_SITE_LOCALACT_SINGLET: width = 1; present = c->has_s; break;
    case SU2GPU_SITE_OR_DOUBLET: width = 4; present = c->nh > 0; break;
    case SU2GPU_SITE_OR_DOUBLET1: width = 4; present = c->nh > 1; break;
    case SU2GPU_SITE_OR_TRIPLET: width = 3; present = c->has_t; break;
    case SU2GPU_SITE_OR_SINGLET: width = 1; present = c->has_s; break;
    default: set_err("unknown per-site value %d", what); return SU2GPU_ERR_INVALID;
  }
  if (!present) {
    set_err("per-site value %d: the field content lacks its field", what);
    return SU2GPU_ERR_INVALID;
  }
  const size_t bytes = (size_t)c->g.V * width * sizeof(double);
  DevBuf buf;
  int rc = buf.ensure(bytes);
  if (rc) return rc;
  for (int par = 0; par < 2; par++) launch_site_probe(what, par, c->f64, c->g, c->cp, (double*)buf.p, c->st);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf.p, bytes, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  buf.release();
  if (e != cudaSuccess) {
    set_err("per-site values: %s", cudaGetErrorString(e));
    return SU2GPU_ERR_CUDA;
  }
  return SU2GPU_OK;
}

static int transfer(su2gpu_ctx* c, int upload, double* link, double* u1, double* d0, double* d1, double* trip,
                    double* sing) {
  int64_t V = c->g.V;
  int rc = c->stage.ensure((size_t)V * 12 * 8);
  if (rc) return rc;
  double* st = (double*)c->stage.p;
  struct Item { double* h; int kind, h_id; size_t n; bool present; };
  Item items[] = {
      {link, 0, 0, (size_t)V * 12, true},
      {u1, 1, 0, (size_t)V * 3, (bool)c->has_u1},
      {d0, 2, 0, (size_t)V * 4, c->nh > 0},
      {d1, 2, 1, (size_t)V * 4, c->nh > 1},
      {trip, 3, 0, (size_t)V * 3, (bool)c->has_t},
      {sing, 4, 0, (size_t)V, (bool)c->has_s},
  };
  // uploads from page-locked host arrays are read by the conversion kernel in
  // place (as fast as a copy, one pass); everything else goes through the
  // staging buffer, one array at a time: downloads are converted on the
  // device and copied by the copy engine, which writes host memory far faster
  // than kernel stores do
  for (const Item& it : items) {
    if (!it.present || !it.h) continue;
    if (upload) {
      double* direct = (double*)host_device_view(it.h, it.n * 8);
      if (direct) {
        c->pops->import(c->F(), V, it.kind, it.h_id, direct, c->st);
        CKL();
        continue;
      }
      CK(cudaMemcpyAsync(st, it.h, it.n * 8, cudaMemcpyHostToDevice, c->st));
      c->pops->import(c->F(), V, it.kind, it.h_id, st, c->st);
      CKL();
    } else {
      c->pops->exportf(c->F(), V, it.kind, it.h_id, st, c->st);
      CKL();
      CK(cudaMemcpyAsync(it.h, st, it.n * 8, cudaMemcpyDeviceToHost, c->st));
    }
    CK(cudaStreamSynchronize(c->st));  // the staging buffer is reused by the next array
  }
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

int su2gpu_upload_fields(su2gpu_ctx* c, const double* link, const double* u1, const double* d0, const double* d1,
                         const double* trip, const double* sing) {
  if (!c) return SU2GPU_ERR_INVALID;
  return transfer(c, 1, (double*)link, (double*)u1, (double*)d0, (double*)d1, (double*)trip, (double*)sing);
}

int su2gpu_download_fields(su2gpu_ctx* c, double* link, double* u1, double* d0, double* d1, double* trip,
                           double* sing) {
  if (!c) return SU2GPU_ERR_INVALID;
  return transfer(c, 0, link, u1, d0, d1, trip, sing);
}

int su2gpu_set_seed(su2gpu_ctx* c, uint64_t seed, uint32_t chain) {
  if (!c) return SU2GPU_ERR_INVALID;
  c->seed = seed;
  c->chain = chain;
  if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
  return SU2GPU_OK;
}

double su2gpu_stream_uniform(uint64_t seed, uint32_t site, uint32_t pass, uint32_t draw, uint32_t sweep,
                             uint32_t chain) {
  return philox_uniform53((uint32_t)seed, (uint32_t)(seed >> 32), site, pass, draw >> 1, sweep, chain, draw & 1);
}

// ---------------------------------------------------------------------------
// one sweep: update_lattice (update.c:270-430), non-random order
// ---------------------------------------------------------------------------
static void mark(su2gpu_ctx* c, int kind) {
  if (!c->prof) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, c->st);
  c->prof->push_back(e);
  c->prof_kind->push_back(kind);
}

static int scalar_pass(su2gpu_ctx* c, const PassArgs& base, int field, int h, int par, int metro, uint32_t pass,
                       int64_t* tot) {
  const int64_t N = c->g.half;
  int alg = field == 0 ? c->p.algorithm_su2doublet : (field == 1 ? c->p.algorithm_su2triplet : c->p.algorithm_singlet);
  bool orr = alg == SU2GPU_OVERRELAX && !metro;
  int tot_idx = field == 0 ? (orr ? SU2GPU_C_TOTAL_OR_DOUBLET : SU2GPU_C_TOTAL_DOUBLET) + h
                           : (field == 1 ? (orr ? SU2GPU_C_TOTAL_OR_TRIPLET : SU2GPU_C_TOTAL_TRIPLET)
                                         : (orr ? SU2GPU_C_TOTAL_OR_SINGLET : SU2GPU_C_TOTAL_SINGLET));
  tot[tot_idx] += N;
  PassArgs a = base;
  a.parity = par;
  a.sub = h;
  a.alg = metro;
  a.pass = pass;
  int op = c->muca_orderparam;
  bool do_muca = c->muca_on && c->muca_do_acc && field != 2 &&
                 ((field == 0 && ((h == 0 && (op == SU2GPU_PHISQ || op == SU2GPU_PHI2MINUSSIGMA2)) ||
                                  (h == 1 && op == SU2GPU_PHI2SQ))) ||
                  (field == 1 && (op == SU2GPU_SIGMASQ || op == SU2GPU_PHI2MINUSSIGMA2)));
  mark(c, 2 + field);
  if (!do_muca) {
    a.t_lo = 0;
    a.t_hi = N;
    c->ops->scalar(c->var[2 + field], field, c->F(), a, c->st);
    c->launches++;
    CKL();
    return SU2GPU_OK;
  }
  // checkerboard_sweep_su2doublet/_su2triplet (update.c:82-229): global
  // checks after every `interval` sites, a final one if the blocks do not
  // add up; the fields of the checked block are restored on reject
  const int cps = c->muca_cps;
  int64_t interval = N / cps;
  if (interval <= 0) interval = 1;
  int64_t m = N / interval;
  bool fused = (m == 1 && interval == N);
  double* partials = (double*)c->partials.p;
  const double vol = (double)c->g.V;
  uint32_t check = 0;
  RngKey rk = base.rk;
  a.backup = c->backup.p;
  a.op = op;
  // a check over the whole parity is decided by the update launch itself
  // (muca_fused_finish) when its blocks fit the arrival counters
  const bool in_pass = fused && (N + 63) / 64 <= (int64_t)MUCA_CHUNK * MUCA_MAX_CHUNKS;
  for (int64_t k = 0; k < m; k++) {
    a.t_lo = k * interval;
    a.t_hi = (k + 1) * interval;
    a.partials = fused ? partials : nullptr;
    if (in_pass) {
      a.muca = c->d_muca;
      a.arrive = c->d_arrive;
      a.check = check++;
      a.vol = vol;
    }
    unsigned nb = c->ops->scalar(c->var[2 + field], field, c->F(), a, c->st);
    CKL();
    unsigned np = nb;
    if (!fused) {
      np = nblk(N, BLOCK);
      c->pops->orderparam(c->F(), c->g, par, op, partials, np, c->st);
      c->launches++;
      CKL();
    }
    if (!in_pass) {
      launch_muca_decide(c->d_muca, partials, (int)np, vol, par, rk, pass, check++, c->d_ctr, c->st);
      c->launches++;
      CKL();
    }
    c->pops->restore(field, c->F(), c->d_muca, c->backup.p, h, par * N + a.t_lo, par * N + a.t_hi, c->st);
    c->launches += 2;
    CKL();
  }
  a.muca = nullptr;
  if (N % cps != 0) {
    int64_t lo = m * interval, hi = N, rlo = lo, rhi = hi;
    if (lo < hi) {
      a.t_lo = lo;
      a.t_hi = hi;
      a.partials = nullptr;
      c->ops->scalar(c->var[2 + field], field, c->F(), a, c->st);
      c->launches++;
      CKL();
    } else {
      // nothing left to update: a reject reverts the last block, whose
      // backup the reference did not refresh after its final check
      rlo = (m - 1) * interval;
      rhi = m * interval;
    }
    unsigned np = nblk(N, BLOCK);
    c->pops->orderparam(c->F(), c->g, par, op, partials, np, c->st);
    CKL();
    launch_muca_decide(c->d_muca, partials, (int)np, vol, par, rk, pass, check++, c->d_ctr, c->st);
    CKL();
    c->pops->restore(field, c->F(), c->d_muca, c->backup.p, h, par * N + rlo, par * N + rhi, c->st);
    c->launches += 3;
    CKL();
  }
  return SU2GPU_OK;
}

static int enqueue_sweep(su2gpu_ctx* c, int64_t* tot, uint32_t host_sweep) {
  const su2gpu_params& p = c->p;
  // pass order: the fixed one, or in random_sweeps mode the one drawn for
  // this sweep (sweep_order)
  std::vector<int32_t> ldir(6 * (size_t)p.update_links), lpar(6 * (size_t)p.update_links),
      sfirst((size_t)p.scalar_sweeps + 1);
  if (c->random_sweeps) {
    sweep_order(c->seed, c->chain, host_sweep, p.update_links, p.scalar_sweeps, ldir.data(), lpar.data(),
                sfirst.data());
  } else {
    for (int k = 0; k < p.update_links; k++)
      for (int j = 0; j < 6; j++) { ldir[6 * k + j] = j >> 1; lpar[6 * k + j] = j & 1; }
    for (int s = 0; s <= p.scalar_sweeps; s++) sfirst[s] = 0;
  }
  c->launches = 0;
  const int64_t N = c->g.half;
  PassArgs base;
  memset(&base, 0, sizeof(base));
  base.g = c->g;
  base.cpd = coup_as<double>(c->cp);
  base.cpf = coup_as<float>(c->cp);
  base.rk = RngKey{(uint32_t)c->seed, (uint32_t)(c->seed >> 32), c->chain, c->d_sweep};
  base.ctr = c->d_ctr;
  base.err = c->d_err;
  uint32_t pass = 0;
  int rc;
  for (int k = 0; k < p.update_links; k++) {
    for (int j = 0; j < 6; j++) {
      PassArgs a = base;
      a.parity = lpar[6 * k + j]; a.sub = ldir[6 * k + j]; a.alg = p.algorithm_su2link; a.pass = pass++;
      a.t_lo = 0; a.t_hi = N;
      mark(c, 0);
      c->ops->link(c->var[0], c->F(), a, c->st);
      c->launches++;
      CKL();
      tot[SU2GPU_C_TOTAL_SU2LINK] += N;
    }
    if (c->has_u1)
      for (int j = 0; j < 6; j++) {
        PassArgs a = base;
        a.parity = lpar[6 * k + j]; a.sub = ldir[6 * k + j]; a.pass = pass++; a.t_lo = 0; a.t_hi = N;
        mark(c, 1);
        c->ops->u1(c->var[1], c->F(), a, c->st);
        c->launches++;
        CKL();
        tot[SU2GPU_C_TOTAL_U1LINK] += N;
      }
  }
  int nsweeps = p.scalar_sweeps + 1;
  for (int s = 0; s < nsweeps; s++) {
    const int p0 = sfirst[s], pr[2] = {p0, 1 - p0};
    if (c->nh > 0)
      for (int k = 0; k < p.update_su2doublet; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (p.algorithm_su2doublet == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        for (int h = 0; h < c->nh; h++)
          for (int j = 0; j <= 1; j++)
            if ((rc = scalar_pass(c, base, 0, h, pr[j], force, pass++, tot))) return rc;
      }
    if (c->has_t)
      for (int k = 0; k < p.update_su2triplet; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (p.algorithm_su2triplet == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        for (int j = 0; j <= 1; j++)
          if ((rc = scalar_pass(c, base, 1, 0, pr[j], force, pass++, tot))) return rc;
      }
    if (c->has_s)
      for (int k = 0; k < p.update_singlet; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (p.algorithm_singlet == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        for (int j = 0; j <= 1; j++)
          if ((rc = scalar_pass(c, base, 2, 0, pr[j], force, pass++, tot))) return rc;
      }
  }
  // FP32: links are re-normalised where they are written (heatbath and
  // Metropolis kernels), which subsumes a periodic re-unitarisation pass
  mark(c, -1);
  return SU2GPU_OK;
}

static int check_device_error(su2gpu_ctx* c) {
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (herr) {
    set_err("a kernel reported an invalid state (sphere sampling did not terminate: NaN fields?)");
    return SU2GPU_ERR_KERNEL;
  }
  return SU2GPU_OK;
}

int su2gpu_update_lattice(su2gpu_ctx* c, uint32_t sweep) {
  if (!c) return SU2GPU_ERR_INVALID;
  k_set_u32<<<1, 1, 0, c->st>>>(c->d_sweep, sweep);
  CKL();
  int rc = enqueue_sweep(c, c->host_tot, sweep);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

static int enqueue_sweeps(su2gpu_ctx* c, uint32_t first_sweep, int32_t nsweeps, int32_t use_graph) {
  k_set_u32<<<1, 1, 0, c->st>>>(c->d_sweep, first_sweep);
  CKL();
  if (use_graph && !c->random_sweeps) {  // a random order differs every sweep: no replay
    if (!c->gexec) {
      int64_t tot[SU2GPU_NCOUNTERS] = {0};
      cudaGraph_t graph;
      cudaStream_t exec = c->st;
      CK(cudaStreamSynchronize(exec));
      c->st = c->own_st;
      CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_sweep(c, tot, first_sweep);
      k_inc_u32<<<1, 1, 0, c->st>>>(c->d_sweep);
      cudaError_t e = cudaStreamEndCapture(c->st, &graph);
      c->st = exec;
      if (rc) return rc;
      if (e != cudaSuccess) { set_err("graph capture: %s", cudaGetErrorString(e)); return SU2GPU_ERR_CUDA; }
      e = cudaGraphInstantiate(&c->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) { set_err("graph instantiate: %s", cudaGetErrorString(e)); return SU2GPU_ERR_CUDA; }
      memcpy(c->graph_tot, tot, sizeof(tot));
      c->launches += 1;
    }
    for (int s = 0; s < nsweeps; s++) {
      CK(cudaGraphLaunch(c->gexec, c->st));
      for (int k = 0; k < SU2GPU_NCOUNTERS; k++) c->host_tot[k] += c->graph_tot[k];
    }
  } else {
    for (int s = 0; s < nsweeps; s++) {
      int rc = enqueue_sweep(c, c->host_tot, first_sweep + (uint32_t)s);
      if (rc) return rc;
      k_inc_u32<<<1, 1, 0, c->st>>>(c->d_sweep);
      CKL();
    }
  }
  return SU2GPU_OK;
}

int su2gpu_run_sweeps(su2gpu_ctx* c, uint32_t first_sweep, int32_t nsweeps, int32_t use_graph) {
  if (!c || nsweeps < 0) return SU2GPU_ERR_INVALID;
  int rc = enqueue_sweeps(c, first_sweep, nsweeps, use_graph);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

int su2gpu_enqueue_sweeps(su2gpu_ctx* c, uint32_t first_sweep, int32_t nsweeps, int32_t use_graph) {
  if (!c || nsweeps < 0) return SU2GPU_ERR_INVALID;
  return enqueue_sweeps(c, first_sweep, nsweeps, use_graph);
}

int su2gpu_set_random_sweeps(su2gpu_ctx* c, int32_t on) {
  if (!c) return SU2GPU_ERR_INVALID;
  c->random_sweeps = on ? 1 : 0;
  if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
  return SU2GPU_OK;
}

int su2gpu_clone(su2gpu_ctx* src, uint64_t seed, uint32_t chain, su2gpu_ctx** out) {
  if (!src || !out) return SU2GPU_ERR_INVALID;
  CK(cudaStreamSynchronize(src->st));
  return su2gpu_create_copy(&src->p, src->fields.p, seed, chain, out);
}

int su2gpu_copy_fields(su2gpu_ctx* dst, su2gpu_ctx* src) {
  if (!dst || !src) return SU2GPU_ERR_INVALID;
  if (dst == src) return SU2GPU_OK;
  if (dst->prec != src->prec || dst->p.content != src->p.content || dst->fields.n != src->fields.n ||
      dst->p.L[0] != src->p.L[0] || dst->p.L[1] != src->p.L[1] || dst->p.L[2] != src->p.L[2]) {
    set_err("su2gpu_copy_fields: the contexts differ in lattice, content or precision");
    return SU2GPU_ERR_INVALID;
  }
  CK(cudaStreamSynchronize(src->st));
  CK(cudaMemcpyAsync(dst->fields.p, src->fields.p, dst->fields.n, cudaMemcpyDeviceToDevice, dst->st));
  CK(cudaStreamSynchronize(dst->st));
  return SU2GPU_OK;
}

int su2gpu_sweep_order(uint64_t seed, uint32_t chain, uint32_t sweep, int32_t update_links, int32_t scalar_sweeps,
                       int32_t* link_dirs, int32_t* link_pars, int32_t* scalar_first) {
  if (update_links < 0 || scalar_sweeps < 0 || (update_links && (!link_dirs || !link_pars)) || !scalar_first)
    return SU2GPU_ERR_INVALID;
  sweep_order(seed, chain, sweep, update_links, scalar_sweeps, link_dirs, link_pars, scalar_first);
  return SU2GPU_OK;
}

int su2gpu_set_stream(su2gpu_ctx* c, void* stream) {
  if (!c) return SU2GPU_ERR_INVALID;
  CK(cudaStreamSynchronize(c->st));
  c->st = stream ? (cudaStream_t)stream : c->own_st;
  return SU2GPU_OK;
}

int su2gpu_launches_per_sweep(su2gpu_ctx* c, int32_t* n) {
  if (!c || !n) return SU2GPU_ERR_INVALID;
  int64_t tot[SU2GPU_NCOUNTERS] = {0};
  // count by enqueueing nothing: replay the bookkeeping of one sweep on a
  // capture that is discarded
  cudaGraph_t graph;
  cudaStream_t exec = c->st;
  CK(cudaStreamSynchronize(exec));
  c->st = c->own_st;
  CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_sweep(c, tot, 0);
  cudaError_t e = cudaStreamEndCapture(c->st, &graph);
  c->st = exec;
  if (rc) return rc;
  if (e != cudaSuccess) { set_err("capture: %s", cudaGetErrorString(e)); return SU2GPU_ERR_CUDA; }
  size_t nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nodes);
  cudaGraphDestroy(graph);
  *n = (int32_t)nodes;
  return SU2GPU_OK;
}

// one sweep with an event before every pass: kinds[k] (0 link, 1 U(1),
// 2 doublet, 3 triplet, 4 singlet, 5 reunitarisation) and its duration ms[k]
int su2gpu_profile_sweep(su2gpu_ctx* c, uint32_t sweep, int32_t maxp, int32_t* kinds, float* ms, int32_t* npasses) {
  if (!c || !kinds || !ms || !npasses) return SU2GPU_ERR_INVALID;
  std::vector<cudaEvent_t> ev;
  std::vector<int> kd;
  k_set_u32<<<1, 1, 0, c->st>>>(c->d_sweep, sweep);
  c->prof = &ev;
  c->prof_kind = &kd;
  int rc = enqueue_sweep(c, c->host_tot, sweep);
  c->prof = nullptr;
  c->prof_kind = nullptr;
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->st));
  int n = 0;
  for (size_t k = 0; k + 1 < ev.size() && n < maxp; k++, n++) {
    kinds[n] = kd[k];
    cudaEventElapsedTime(&ms[n], ev[k], ev[k + 1]);
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  *npasses = n;
  return SU2GPU_OK;
}

int su2gpu_host_register(void* p, int64_t bytes) {
  if (!p || bytes <= 0) return SU2GPU_ERR_INVALID;
  CK(cudaHostRegister(p, (size_t)bytes, cudaHostRegisterDefault));
  return SU2GPU_OK;
}

int su2gpu_host_unregister(void* p) {
  if (!p) return SU2GPU_ERR_INVALID;
  CK(cudaHostUnregister(p));
  return SU2GPU_OK;
}

int su2gpu_run_halfsweep(su2gpu_ctx* c, int32_t kind, int32_t parity, int32_t sub, uint32_t pass, uint32_t sweep) {
  if (!c || kind < 0 || kind > 7 || (parity != 0 && parity != 1)) return SU2GPU_ERR_INVALID;
  int field = kind < 2 ? -1 : (kind - 2) / 2;  // 0 doublet, 1 triplet, 2 singlet
  if ((kind == 1 && !c->has_u1) || (field == 0 && sub >= c->nh) || (field == 1 && !c->has_t) ||
      (field == 2 && !c->has_s) || (kind <= 1 && (sub < 0 || sub > 2))) {
    set_err("half-sweep kind %d / index %d not present in this content", kind, sub);
    return SU2GPU_ERR_INVALID;
  }
  const int64_t N = c->g.half;
  k_set_u32<<<1, 1, 0, c->st>>>(c->d_sweep, sweep);
  CKL();
  PassArgs a;
  memset(&a, 0, sizeof(a));
  a.g = c->g;
  a.cpd = coup_as<double>(c->cp);
  a.cpf = coup_as<float>(c->cp);
  a.rk = RngKey{(uint32_t)c->seed, (uint32_t)(c->seed >> 32), c->chain, c->d_sweep};
  a.ctr = c->d_ctr;
  a.err = c->d_err;
  a.parity = parity;
  a.sub = sub;
  a.pass = pass;
  a.t_lo = 0;
  a.t_hi = (int)N;
  if (kind == 0) {
    a.alg = c->p.algorithm_su2link;
    c->ops->link(c->var[0], c->F(), a, c->st);
    c->host_tot[SU2GPU_C_TOTAL_SU2LINK] += N;
  } else if (kind == 1) {
    c->ops->u1(c->var[1], c->F(), a, c->st);
    c->host_tot[SU2GPU_C_TOTAL_U1LINK] += N;
  } else {
    int metro = (kind & 1);
    int alg = field == 0 ? c->p.algorithm_su2doublet : (field == 1 ? c->p.algorithm_su2triplet : c->p.algorithm_singlet);
    bool orr = alg == SU2GPU_OVERRELAX && !metro;
    int idx = field == 0 ? (orr ? SU2GPU_C_TOTAL_OR_DOUBLET : SU2GPU_C_TOTAL_DOUBLET) + sub
                         : (field == 1 ? (orr ? SU2GPU_C_TOTAL_OR_TRIPLET : SU2GPU_C_TOTAL_TRIPLET)
                                       : (orr ? SU2GPU_C_TOTAL_OR_SINGLET : SU2GPU_C_TOTAL_SINGLET));
    c->host_tot[idx] += N;
    a.alg = metro;
    c->ops->scalar(c->var[2 + field], field, c->F(), a, c->st);
  }
  CKL();
  CK(cudaStreamSynchronize(c->st));
  return check_device_error(c);
}

// Launch-shape autotuner: times every variant of every update kernel kind of
// this content on a scratch copy of the fields (the chain itself is not
// advanced, its counters are untouched) and keeps the fastest.
int su2gpu_autotune(su2gpu_ctx* c, int32_t* choices, float* best_ms) {
  if (!c) return SU2GPU_ERR_INVALID;
  DevBuf tmp, ctr;
  int rc = tmp.ensure(c->fields.n);
  if (rc) return rc;
  if ((rc = ctr.ensure(4096))) { tmp.release(); return rc; }
  CK(cudaMemcpyAsync(tmp.p, c->fields.p, c->fields.n, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemsetAsync(ctr.p, 0, 4096, c->st));
  Fields<double> f64;
  Fields<float> f32;
  if (c->prec == 64) carve(f64, (char*)tmp.p, &c->p, c->g.V);
  else carve(f32, (char*)tmp.p, &c->p, c->g.V);
  const void* F = c->prec == 64 ? (const void*)&f64 : (const void*)&f32;
  k_set_u32<<<1, 1, 0, c->st>>>((uint32_t*)((char*)ctr.p + 1024), 0x7fffffffu);
  PassArgs a;
  memset(&a, 0, sizeof(a));
  a.g = c->g;
  a.cpd = coup_as<double>(c->cp);
  a.cpf = coup_as<float>(c->cp);
  a.rk = RngKey{(uint32_t)c->seed ^ 0x5eedu, (uint32_t)(c->seed >> 32), c->chain, (uint32_t*)((char*)ctr.p + 1024)};
  a.ctr = (unsigned long long*)ctr.p;
  a.err = (int*)((char*)ctr.p + 512);
  a.t_lo = 0;
  a.t_hi = (int)c->g.half;
  bool present[5] = {true, (bool)c->has_u1, c->nh > 0, (bool)c->has_t, (bool)c->has_s};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int reps = 4;
  for (int kind = 0; kind < 5; kind++) {
    if (!present[kind]) continue;
    float best = 1e30f;
    int bestv = 0;
    for (int v = 0; v < NVARIANTS; v++) {
      float ms = 0.f;
      for (int r = -1; r < reps; r++) {  // r = -1: warm-up
        a.parity = r & 1;
        a.sub = (r + 3) % 3;
        a.pass = 60000 + r;
        a.alg = kind == 0 ? c->p.algorithm_su2link : 0;
        if (kind == 2) a.sub = 0;
        cudaEventRecord(e0, c->st);
        if (kind == 0) c->ops->link(v, F, a, c->st);
        else if (kind == 1) c->ops->u1(v, F, a, c->st);
        else c->ops->scalar(v, kind - 2, F, a, c->st);
        cudaEventRecord(e1, c->st);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
          set_err("autotune: %s", cudaGetErrorString(e));
          return SU2GPU_ERR_CUDA;
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r >= 0) ms += t;
      }
      if (ms < best) {
        best = ms;
        bestv = v;
      }
    }
    c->var[kind] = bestv;
    if (best_ms) best_ms[kind] = best / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaStreamSynchronize(c->st));
  tmp.release();
  ctr.release();
  if (choices)
    for (int k = 0; k < 5; k++) choices[k] = c->var[k];
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  return SU2GPU_OK;
}

int su2gpu_set_variants(su2gpu_ctx* c, const int32_t* choices) {
  if (!c || !choices) return SU2GPU_ERR_INVALID;
  for (int k = 0; k < 5; k++) {
    if (choices[k] < 0 || choices[k] >= NVARIANTS) return SU2GPU_ERR_INVALID;
    c->var[k] = choices[k];
  }
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  return SU2GPU_OK;
}

int su2gpu_get_counters(su2gpu_ctx* c, int64_t* out) {
  if (!c || !out) return SU2GPU_ERR_INVALID;
  unsigned long long d[SU2GPU_NCOUNTERS];
  CK(cudaMemcpyAsync(d, c->d_ctr, sizeof(d), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int k = 0; k < SU2GPU_NCOUNTERS; k++) out[k] = (int64_t)d[k] + c->host_tot[k];
  return check_device_error(c);
}

int su2gpu_reset_counters(su2gpu_ctx* c) {
  if (!c) return SU2GPU_ERR_INVALID;
  CK(cudaMemsetAsync(c->d_ctr, 0, SU2GPU_NCOUNTERS * 8, c->st));
  CK(cudaStreamSynchronize(c->st));
  memset(c->host_tot, 0, sizeof(c->host_tot));
  return SU2GPU_OK;
}

// ---------------------------------------------------------------------------
// measurements
// ---------------------------------------------------------------------------
static int enqueue_measure(su2gpu_ctx* c, const void* F, const Coup& cp, double* out) {
  int64_t V = c->g.V;
  if (c->has_t) {
    int rc = c->alpha.ensure((size_t)V * 3 * 8);
    if (rc) return rc;
    c->pops->alpha(F, c->g, cp, (double*)c->alpha.p, c->st);
    CKL();
  }
  unsigned nb = nblk(V, MEAS_TILE);
  c->ops->measure(F, c->g, cp, (const double*)c->alpha.p, (double*)c->partials.p, nb, c->st);
  CKL();
  launch_reduce_partials((const double*)c->partials.p, (int)nb, out, c->st);
  CKL();
  return SU2GPU_OK;
}

int su2gpu_enqueue_measure(su2gpu_ctx* c, double* dev_sums) {
  if (!c || !dev_sums) return SU2GPU_ERR_INVALID;
  return enqueue_measure(c, c->F(), c->cp, dev_sums);
}

int su2gpu_measure(su2gpu_ctx* c, double* sums) {
  if (!c || !sums) return SU2GPU_ERR_INVALID;
  int rc = enqueue_measure(c, c->F(), c->cp, (double*)c->sums.p);
  if (rc) return rc;
  CK(cudaMemcpyAsync(sums, c->sums.p, NSUMS * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

// ---------------------------------------------------------------------------
// multicanonical state
// ---------------------------------------------------------------------------
int su2gpu_muca_set(su2gpu_ctx* c, const su2gpu_weight* w) {
  if (!c || !w || w->bins <= 0) return SU2GPU_ERR_INVALID;
  if (w->checks_per_sweep <= 0 || w->update_interval <= 0) { set_err("checks_per_sweep and update_interval must be > 0"); return SU2GPU_ERR_INVALID; }
  int n = w->bins + 2;
  size_t arr = align256((size_t)n * 8);
  int rc = c->muca.ensure(align256(sizeof(MucaDev)) + 9 * arr);
  if (rc) return rc;
  char* base = (char*)c->muca.p;
  MucaDev m;
  memset(&m, 0, sizeof(m));
  m.orderparam = w->orderparam; m.mode = w->mode; m.do_acceptance = w->do_acceptance;
  m.checks_per_sweep = w->checks_per_sweep; m.bins = w->bins; m.muca_count = w->muca_count;
  m.update_interval = w->update_interval; m.last_max = w->last_max;
  m.param_value[0] = w->param_value[0]; m.param_value[1] = w->param_value[1];
  m.min = w->min; m.max = w->max; m.wrk_min = w->wrk_min; m.wrk_max = w->wrk_max; m.delta = w->delta;
  size_t off = align256(sizeof(MucaDev));
  m.pos = (double*)(base + off); off += arr;
  m.W = (double*)(base + off); off += arr;
  m.slope = (double*)(base + off); off += arr;
  m.b = (double*)(base + off); off += arr;
  m.hits = (int*)(base + off); off += arr;
  m.gsum = (long long*)(base + off); off += arr;
  m.nsum = (long long*)(base + off); off += arr;
  m.hgram = (double*)(base + off); off += arr;
  m.wold = (double*)(base + off); off += arr;
  CK(cudaMemcpyAsync(base, &m, sizeof(m), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(m.pos, w->pos, n * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(m.W, w->W, n * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(m.slope, w->slope, n * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(m.b, w->b, n * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(m.hits, w->hits, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(m.gsum, 0, arr * 3, c->st));
  if (w->gsum) CK(cudaMemcpyAsync(m.gsum, w->gsum, n * 8, cudaMemcpyHostToDevice, c->st));
  if (w->nsum) CK(cudaMemcpyAsync(m.nsum, w->nsum, n * 8, cudaMemcpyHostToDevice, c->st));
  if (w->hgram) CK(cudaMemcpyAsync(m.hgram, w->hgram, n * 8, cudaMemcpyHostToDevice, c->st));
  size_t bu = c->prec == 64 ? 32 : 16;
  if ((rc = c->backup.ensure((size_t)c->g.V * bu))) return rc;
  CK(cudaStreamSynchronize(c->st));
  c->d_muca = (MucaDev*)base;
  c->muca_on = true;
  c->muca_bins = w->bins;
  c->muca_orderparam = w->orderparam;
  c->muca_cps = w->checks_per_sweep;
  c->muca_do_acc = w->do_acceptance;
  if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
  return SU2GPU_OK;
}

int su2gpu_muca_get(su2gpu_ctx* c, su2gpu_weight* w) {
  if (!c || !w || !c->muca_on) return SU2GPU_ERR_INVALID;
  MucaDev m;
  CK(cudaMemcpyAsync(&m, c->d_muca, sizeof(m), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  int n = m.bins + 2;
  w->orderparam = m.orderparam; w->mode = m.mode; w->do_acceptance = m.do_acceptance;
  w->checks_per_sweep = m.checks_per_sweep; w->bins = m.bins; w->muca_count = m.muca_count;
  w->update_interval = m.update_interval; w->last_max = m.last_max;
  w->param_value[0] = m.param_value[0]; w->param_value[1] = m.param_value[1];
  w->min = m.min; w->max = m.max; w->wrk_min = m.wrk_min; w->wrk_max = m.wrk_max; w->delta = m.delta;
  if (w->pos) CK(cudaMemcpyAsync(w->pos, m.pos, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (w->W) CK(cudaMemcpyAsync(w->W, m.W, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (w->slope) CK(cudaMemcpyAsync(w->slope, m.slope, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (w->b) CK(cudaMemcpyAsync(w->b, m.b, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (w->hits) CK(cudaMemcpyAsync(w->hits, m.hits, n * 4, cudaMemcpyDeviceToHost, c->st));
  if (w->gsum) CK(cudaMemcpyAsync(w->gsum, m.gsum, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (w->nsum) CK(cudaMemcpyAsync(w->nsum, m.nsum, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (w->hgram) CK(cudaMemcpyAsync(w->hgram, m.hgram, n * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

// number of weight recursions done on the device so far (the host rewrites
// the weight file when it changes, as save_weight() does after each update)
int su2gpu_muca_weight_updates(su2gpu_ctx* c, int32_t* n) {
  if (!c || !n || !c->muca_on) return SU2GPU_ERR_INVALID;
  MucaDev m;
  CK(cudaMemcpyAsync(&m, c->d_muca, sizeof(m), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *n = m.weight_updates;
  return SU2GPU_OK;
}

int su2gpu_calc_orderparam(su2gpu_ctx* c, int32_t parity, double* value) {
  if (!c || !c->muca_on || (parity != 0 && parity != 1)) return SU2GPU_ERR_INVALID;
  unsigned np = nblk(c->g.half, BLOCK);
  c->pops->orderparam(c->F(), c->g, parity, c->muca_orderparam, (double*)c->partials.p, np, c->st);
  CKL();
  launch_muca_set_param(c->d_muca, (const double*)c->partials.p, (int)np, (double)c->g.V, parity, c->st);
  CKL();
  MucaDev m;
  CK(cudaMemcpyAsync(&m, c->d_muca, sizeof(m), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (value) *value = m.param_value[parity] + m.param_value[1 - parity];
  return SU2GPU_OK;
}

// init_last_max (multicanonical.c:826-831)
int su2gpu_muca_init_last_max(su2gpu_ctx* c) {
  if (!c || !c->muca_on) return SU2GPU_ERR_INVALID;
  MucaDev m;
  CK(cudaMemcpyAsync(&m, c->d_muca, sizeof(m), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  double val = m.param_value[0] + m.param_value[1];
  int lm = (fabs(val - m.wrk_min) >= fabs(val - m.wrk_max));
  CK(cudaMemcpyAsync((char*)c->d_muca + offsetof(MucaDev, last_max), &lm, sizeof(int), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

// ---------------------------------------------------------------------------
// gradient flow (gradflow.c:46-173)
// ---------------------------------------------------------------------------
}  // extern "C"

// remove_counterterms (gradflow.c:424-459): the triplet's tree-level mass
static double triplet_tree_mass(const su2gpu_params* p) {
  const double Sigma = 3.17591153625, zeta = 0.08849, delta = 1.942130, rho = -0.313964;
  const double k1 = 0.958382, k2 = 0.25 * Sigma * Sigma - 0.5 * delta - 0.25, k3 = 0.751498, k4 = 1.204295;
  double gsq = 4.0 / p->betasu2, RGscale = gsq, b4 = p->b4;
  double ct = -(4.0 * gsq + 5.0 * b4) * Sigma / (4.0 * M_PI);
  ct += -1.0 / (16.0 * M_PI * M_PI) *
        ((20.0 * b4 * gsq - 10.0 * b4 * b4) * (log(6.0 / (RGscale)) + zeta) + 20.0 * b4 * gsq * (0.25 * Sigma * Sigma - delta) +
         2.0 * gsq * gsq * (1.25 * Sigma * Sigma + M_PI / 3.0 * Sigma - 6.0 * delta - 6.0 * rho + 4.0 * k1 - k2 - k3 - 3.0 * k4));
  return p->msq_triplet - ct;
}

template <typename R>
static int flow_impl(su2gpu_ctx* c, Fields<R>& main, double t_max, double dt, int32_t mi, double* rows,
                     int32_t maxrows, int32_t* nrows, double* local, int32_t max_local) {
  int64_t V = c->g.V;
  size_t lb = align256((size_t)V * sizeof(V4<R>)), tb = align256((size_t)V * sizeof(R));
  size_t per = 3 * lb + (c->has_t ? 3 * tb : 0);
  int rc = c->flow.ensure(2 * per);
  if (rc) return rc;
  Fields<R> A = main, B = main;
  char* base = (char*)c->flow.p;
  for (int d = 0; d < 3; d++) {
    A.link[d] = (V4<R>*)(base + d * lb);
    B.link[d] = (V4<R>*)(base + per + d * lb);
    CK(cudaMemcpyAsync(A.link[d], main.link[d], V * sizeof(V4<R>), cudaMemcpyDeviceToDevice, c->st));
  }
  if (c->has_t)
    for (int k = 0; k < 3; k++) {
      A.trip[k] = (R*)(base + 3 * lb + k * tb);
      B.trip[k] = (R*)(base + per + 3 * lb + k * tb);
      CK(cudaMemcpyAsync(A.trip[k], main.trip[k], V * sizeof(R), cudaMemcpyDeviceToDevice, c->st));
    }
  Coup cp = c->cp;
  if (c->has_t) cp.msqT = triplet_tree_mass(&c->p);
  const int W = 1 + NSUMS;
  // rows buffered on the device: one copy back at the end
  int64_t cap = maxrows > 0 ? maxrows : 1;
  if ((rc = c->rows.ensure((size_t)cap * NSUMS * 8))) return rc;
  double* drows = (double*)c->rows.p;
  std::vector<double> times;
  int nr = 0;
  double t = 0.0;
  // measure_local of the flowed fields at every measurement (gradflow.c:81-86),
  // copied to the caller's host buffer, V x 2 doubles per measurement
  int nl = 0;
  const double denom = 2.0 * M_PI * sqrt(c->p.betasu2);
  if (local && max_local > 0 && (rc = c->local.ensure((size_t)V * 2 * 8))) return rc;
  auto meas = [&](double tt) -> int {
    if (nr >= maxrows) return SU2GPU_OK;
    int r = enqueue_measure(c, &A, cp, drows + (size_t)nr * NSUMS);
    if (r) return r;
    if (local && nl < max_local) {
      c->pops->measure_local(&A, c->g, cp, denom, (double*)c->local.p, c->st);
      CKL();
      CK(cudaMemcpyAsync(local + (size_t)nl * V * 2, c->local.p, (size_t)V * 2 * 8, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      nl++;
    }
    times.push_back(tt);
    nr++;
    return SU2GPU_OK;
  };
  if ((rc = meas(t))) return rc;
  int iter = 1;
  unsigned nb = nblk(V, BLOCK);
  while (t < t_max) {
    if (t + dt > t_max) dt = t_max - t;
    k_fill_u64<<<1, 1, 0, c->st>>>(c->d_fz, ~0ull);
    c->ops->flow(&A, &B, c->g, cp, dt, c->d_fz, nb, c->st);
    CKL();
    c->pops->flow_fixup(&A, &B, c->g, c->d_fz, c->st);
    CKL();
    std::swap(A, B);
    t += dt;
    if (iter % mi == 0)
      if ((rc = meas(t))) return rc;
    iter++;
  }
  if ((iter - 1) % mi != 0)
    if ((rc = meas(t))) return rc;
  std::vector<double> h((size_t)nr * NSUMS);
  if (nr) CK(cudaMemcpyAsync(h.data(), drows, (size_t)nr * NSUMS * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int r = 0; r < nr; r++) {
    rows[(size_t)r * W] = times[r];
    memcpy(rows + (size_t)r * W + 1, h.data() + (size_t)r * NSUMS, NSUMS * 8);
  }
  *nrows = nr;
  return SU2GPU_OK;
}

extern "C" {

int su2gpu_grad_flow(su2gpu_ctx* c, double t_max, double dt, int32_t meas_interval, double* rows, int32_t maxrows,
                     int32_t* nrows) {
  return su2gpu_grad_flow_local(c, t_max, dt, meas_interval, rows, maxrows, nrows, nullptr, 0);
}

int su2gpu_grad_flow_local(su2gpu_ctx* c, double t_max, double dt, int32_t meas_interval, double* rows,
                           int32_t maxrows, int32_t* nrows, double* local, int32_t max_local) {
  if (!c || !rows || !nrows || meas_interval <= 0 || dt <= 0) return SU2GPU_ERR_INVALID;
  if (local && !c->has_t) {
    set_err("local measurements need the triplet");
    return SU2GPU_ERR_INVALID;
  }
  if (c->prec == 64)
    return flow_impl<double>(c, c->f64, t_max, dt, meas_interval, rows, maxrows, nrows, local, max_local);
  return flow_impl<float>(c, c->f32, t_max, dt, meas_interval, rows, maxrows, nrows, local, max_local);
}

int su2gpu_measure_z(su2gpu_ctx* c, int32_t* z_dir, double* sums) {
  if (!c || !sums) return SU2GPU_ERR_INVALID;
  // init_z_coord (z_coord.c:18-24): the longest direction, ties to the last
  int zd = 2;
  for (int d = 2; d >= 0; d--)
    if (c->g.L[d] > c->g.L[zd]) zd = d;
  const int Lz = c->g.L[zd];
  int rc = c->local.ensure((size_t)c->g.V * 2 * 8 > (size_t)Lz * 4 * 8 ? (size_t)c->g.V * 2 * 8 : (size_t)Lz * 4 * 8);
  if (rc) return rc;
  c->pops->measure_z(c->F(), c->g, c->cp.content, zd, (double*)c->local.p, c->st);
  CKL();
  CK(cudaMemcpyAsync(sums, c->local.p, (size_t)Lz * 4 * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (z_dir) *z_dir = zd;
  return SU2GPU_OK;
}

// ---------------------------------------------------------------------------
// correlators and blocking (correlation.c, blocking.c, su2u1.c:752-905)
// ---------------------------------------------------------------------------
// max_block_level (blocking.c:17-38): how many times every blocked direction
// can be halved without making a side odd or smaller than 2 first
static int block_levels_possible(const int* L, const int* bd, int want) {
  int len[3] = {L[0], L[1], L[2]}, count = 0;
  while (count < want) {
    for (int d = 0; d < 3; d++)
      if (bd[d] && (len[d] % 2 != 0 || len[d] <= 2)) return count;
    for (int d = 0; d < 3; d++)
      if (bd[d]) len[d] /= 2;
    count++;
  }
  return count;
}

// The plain lattice of the fields, blocked `levels` times in the directions
// bd; with out, the correlators along dir of the lattice itself (levels = 0)
// or of every blocked level, one after another (L_k[dir]/2 rows each); with
// last, the plain lattice of the last level is left in c->correl for a copy
// to the host.
static int correl_run(su2gpu_ctx* c, int dir, const int* bd, int levels, double* out, PlainLat* last) {
  const int has_phi = c->nh > 0, has_trip = c->has_t;
  int dev = 0, sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  // sides of every level, then the sizes of the buffers
  std::vector<std::array<int, 3>> Ls(1, std::array<int, 3>{c->g.L[0], c->g.L[1], c->g.L[2]});
  for (int k = 1; k <= levels; k++) {
    std::array<int, 3> n = Ls.back();
    for (int d = 0; d < 3; d++)
      if (bd[d]) n[d] /= 2;
    Ls.push_back(n);
  }
  auto vol = [](const std::array<int, 3>& L) { return (int64_t)L[0] * L[1] * L[2]; };
  const size_t n0 = plain_doubles(c->g.V, has_phi, has_trip);
  const size_t n1 = levels > 0 ? plain_doubles(vol(Ls[1]), 0, has_trip) : 0;
  size_t npart = 0, ntot = 0, nout = 0;
  const int first = levels > 0 ? 1 : 0;
  for (int k = first; k <= levels; k++) {
    PlainLat q = make_plain(Ls[k].data(), nullptr, 0, 0);
    const int Lz = Ls[k][dir];
    npart = std::max(npart, (size_t)Lz * correl_chunks(q, dir, sm) * NCORR_PLANE);
    ntot = std::max(ntot, (size_t)Lz * NCORR_PLANE);
    nout += (size_t)(Lz / 2) * NCORR;
  }
  int rc = c->correl.ensure((n0 + 2 * n1 + npart + ntot + nout) * sizeof(double));
  if (rc) return rc;
  double* base = (double*)c->correl.p;
  double *ping[2] = {base + n0, base + n0 + n1}, *part = base + n0 + 2 * n1, *tot = part + npart, *dout = tot + ntot;
  PlainLat cur = make_plain(Ls[0].data(), base, has_phi, has_trip);
  launch_to_plain(c->prec, c->F(), c->g, has_phi, has_trip, cur, c->st);
  CKL();
  const double sqb = sqrt(c->p.betasu2);
  double* o = dout;
  if (out && levels == 0) {
    launch_correlators(cur, dir, has_phi, has_trip, sqb, correl_chunks(cur, dir, sm), part, tot, o, c->st);
    CKL();
    o += (size_t)(Ls[0][dir] / 2) * NCORR;
  }
  for (int k = 1; k <= levels; k++) {
    PlainLat nxt = make_plain(Ls[k].data(), ping[(k - 1) & 1], 0, has_trip);
    launch_block(cur, nxt, bd, has_trip, c->st);
    CKL();
    cur = nxt;
    if (out) {
      launch_correlators(cur, dir, 0, has_trip, sqb, correl_chunks(cur, dir, sm), part, tot, o, c->st);
      CKL();
      o += (size_t)(Ls[k][dir] / 2) * NCORR;
    }
  }
  if (out) CK(cudaMemcpyAsync(out, dout, (size_t)(o - dout) * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (last) *last = cur;
  return SU2GPU_OK;
}

static int check_block_dir(su2gpu_ctx* c, const int32_t* block_dir, int* bd) {
  int any = 0;
  for (int d = 0; d < 3; d++) {
    bd[d] = block_dir[d] ? 1 : 0;
    any |= bd[d];
  }
  if (!any) {
    set_err("no blocked direction");
    return SU2GPU_ERR_INVALID;
  }
  (void)c;
  return SU2GPU_OK;
}

int su2gpu_measure_correlators(su2gpu_ctx* c, int32_t dir, double* out) {
  if (!c || !out || dir < 0 || dir > 2) return SU2GPU_ERR_INVALID;
  return correl_run(c, dir, nullptr, 0, out, nullptr);
}

int su2gpu_measure_blocked_correlators(su2gpu_ctx* c, int32_t dir, const int32_t* block_dir, int32_t levels,
                                       double* out, int32_t* levels_done) {
  if (!c || !out || !block_dir || dir < 0 || dir > 2 || levels < 0) return SU2GPU_ERR_INVALID;
  if (c->nh > 0) {
    // measure_blocked_correlators (correlation.c:414-418) has no doublet smearing
    set_err("blocked correlators with a doublet: the reference's Higgs smearing is not implemented");
    return SU2GPU_ERR_UNSUPPORTED;
  }
  int bd[3];
  int rc = check_block_dir(c, block_dir, bd);
  if (rc) return rc;
  const int n = block_levels_possible(c->g.L, bd, levels);
  if (levels_done) *levels_done = n;
  if (n == 0) return SU2GPU_OK;
  return correl_run(c, dir, bd, n, out, nullptr);
}

int su2gpu_blocked_fields(su2gpu_ctx* c, const int32_t* block_dir, int32_t level, int32_t* Lb, double* link,
                          double* trip) {
  if (!c || !block_dir || !Lb || level < 0) return SU2GPU_ERR_INVALID;
  int bd[3];
  int rc = check_block_dir(c, block_dir, bd);
  if (rc) return rc;
  if (block_levels_possible(c->g.L, bd, level) < level) {
    set_err("the lattice cannot be blocked %d times", level);
    return SU2GPU_ERR_INVALID;
  }
  PlainLat q;
  if ((rc = correl_run(c, 0, bd, level, nullptr, &q))) return rc;
  for (int d = 0; d < 3; d++) Lb[d] = q.L[d];
  const size_t V = (size_t)q.V;
  std::vector<double> h(V * 15);
  CK(cudaMemcpy(h.data(), q.link, V * 12 * sizeof(double), cudaMemcpyDeviceToHost));
  if (trip && q.trip) CK(cudaMemcpy(h.data() + V * 12, q.trip, V * 3 * sizeof(double), cudaMemcpyDeviceToHost));
  for (size_t n = 0; n < V; n++) {
    for (int k = 0; link && k < 12; k++) link[n * 12 + k] = h[(size_t)k * V + n];
    for (int k = 0; trip && q.trip && k < 3; k++) trip[n * 3 + k] = h[(size_t)(12 + k) * V + n];
  }
  return SU2GPU_OK;
}

int su2gpu_measure_local(su2gpu_ctx* c, double* out) {
  if (!c || !out) return SU2GPU_ERR_INVALID;
  if (!c->has_t) {
    set_err("local measurements need the triplet");
    return SU2GPU_ERR_INVALID;
  }
  int64_t V = c->g.V;
  int rc = c->local.ensure((size_t)V * 2 * 8);
  if (rc) return rc;
  c->pops->measure_local(c->F(), c->g, c->cp, 2.0 * M_PI * sqrt(c->p.betasu2), (double*)c->local.p, c->st);
  CKL();
  CK(cudaMemcpyAsync(out, c->local.p, (size_t)V * 2 * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SU2GPU_OK;
}

// ---------------------------------------------------------------------------
// drop-in update_lattice with host buffers
// ---------------------------------------------------------------------------
int su2gpu_update_lattice_host(su2gpu_ctx* c, uint32_t sweep, double* link, double* u1, double* d0, double* d1,
                               double* trip, double* sing) {
  int rc = su2gpu_upload_fields(c, link, u1, d0, d1, trip, sing);
  if (rc) return rc;
  if ((rc = su2gpu_update_lattice(c, sweep))) return rc;
  return su2gpu_download_fields(c, link, u1, d0, d1, trip, sing);
}

}  // extern "C"

// C++ linkage, not part of the ABI (declared in su2_host.h)
int su2gpu_muca_device_state(su2gpu_ctx* c, void** muca, void** backup, int* orderparam, int* cps,
                             int* do_acceptance) {
  if (!c) return SU2GPU_ERR_INVALID;
  *muca = c->muca_on ? (void*)c->d_muca : nullptr;
  *backup = c->backup.p;
  *orderparam = c->muca_orderparam;
  *cps = c->muca_cps;
  *do_acceptance = c->muca_do_acc;
  return SU2GPU_OK;
}


int su2gpu_attach(const su2gpu_params* p, void* fields, su2gpu_ctx** out) {
  if (!fields) return SU2GPU_ERR_INVALID;
  return create_ctx(p, fields, nullptr, out);
}

int su2gpu_create_copy(const su2gpu_params* p, const void* fields, uint64_t seed, uint32_t chain,
                       su2gpu_ctx** out) {
  if (!fields) return SU2GPU_ERR_INVALID;
  int rc = create_ctx(p, nullptr, fields, out);
  if (rc) return rc;
  return su2gpu_set_seed(*out, seed, chain);
}
