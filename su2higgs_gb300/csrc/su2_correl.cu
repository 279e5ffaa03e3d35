// su2_correl.cu -- correlators and blocking on the device: the reference's
// measure_correlators (correlation.c:350-398) and, for coarser lattices,
// smear_fields + make_blocked_fields (su2u1.c:752-905, blocking.c:296-374).
//
// The measurement works on a "plain" lattice: FP64 structure-of-arrays in
// lexicographic site order (x fastest), filled once from the resident
// parity-split fields.  Blocked lattices halve the sides of the blocked
// directions and may have odd sides (6 -> 3), which the EVEN-first
// checkerboard layout of the update kernels cannot hold; the plain layout
// holds any side.  Kernels:
//   k_to_plain       resident fields (FP64 or FP32) -> plain FP64
//   k_block          smeared fields of the even sites of one plain lattice ->
//                    the next, coarser plain lattice
//   k_plane_ops      per plane x_dir = z the sums of |phi|^2/2, Tr Sigma^2 and
//                    the four photon operators (complex), split into chunks of
//                    the plane, each chunk reduced in a fixed order
//   k_plane_totals   chunks -> plane totals, fixed order
//   k_correl_combine per distance d the sums over z of products of plane
//                    totals at z and z + d (periodic), divided by the volume
#include <cuda_runtime.h>

#include "su2_correl.h"
#include "su2_kernels.cuh"

namespace su2 {

__device__ inline void plain_coords(const PlainLat& p, int n, int* c) {
  c[0] = n % p.L[0];
  int r = n / p.L[0];
  c[1] = r % p.L[1];
  c[2] = r / p.L[1];
}
__device__ inline int plain_index(const PlainLat& p, const int* c) {
  return c[0] + p.L[0] * (c[1] + p.L[1] * c[2]);
}
// index of c + s1 e_d1 + s2 e_d2 (periodic), |s| <= 1
__device__ inline int plain_nb(const PlainLat& p, const int* c, int d1, int s1, int d2 = 0, int s2 = 0) {
  int x[3] = {c[0], c[1], c[2]};
  x[d1] = wrap(x[d1] + s1, p.L[d1]);
  x[d2] = wrap(x[d2] + s2, p.L[d2]);
  return plain_index(p, x);
}
__device__ inline Q<double> plink(const PlainLat& p, int n, int d) {
  const double* b = p.link + (size_t)(4 * d) * p.V + n;
  return Q<double>{b[0], b[p.V], b[2 * (size_t)p.V], b[3 * (size_t)p.V]};
}
__device__ inline void st_plink(const PlainLat& p, int n, int d, const Q<double>& q) {
  double* b = p.link + (size_t)(4 * d) * p.V + n;
  b[0] = q.a;
  b[p.V] = q.b;
  b[2 * (size_t)p.V] = q.c;
  b[3 * (size_t)p.V] = q.d;
}
__device__ inline V3<double> ptrip(const PlainLat& p, int n) {
  return V3<double>{p.trip[n], p.trip[p.V + n], p.trip[2 * (size_t)p.V + n]};
}

// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_to_plain(Fields<R> f, Geom g, int has_phi, int has_trip, PlainLat p) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.V) return;
  int parity = t >= g.half;
  int c[3];
  site_coords(g, parity, t - parity * g.half, c);
  int n = plain_index(p, c);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    Q<R> u = ld4<R>(f.link[d], t);
    st_plink(p, n, d, Q<double>{(double)u.a, (double)u.b, (double)u.c, (double)u.d});
  }
  if (has_trip) {
    V3<R> a = ld3(f, t);
    p.trip[n] = (double)a.x;
    p.trip[p.V + n] = (double)a.y;
    p.trip[2 * (size_t)p.V + n] = (double)a.z;
  }
  if (has_phi) {
    Q<R> h = ld4<R>(f.phi[0], t);
    p.phi[n] = (double)h.a;
    p.phi[p.V + n] = (double)h.b;
    p.phi[2 * (size_t)p.V + n] = (double)h.c;
    p.phi[3 * (size_t)p.V + n] = (double)h.d;
  }
}

// su2staple_wilson_onedir(.., dagger = 1) (staples.c:197-232): both staples of
// U_mu(c) in the (mu, nu) plane, conjugated:
//   U_nu(c) U_mu(c+nu) U_nu(c+mu)^+  +  U_nu(c-nu)^+ U_mu(c-nu) U_nu(c+mu-nu)
__device__ inline Q<double> staple_onedir_dag(const PlainLat& p, const int* c, int mu, int nu) {
  const int n = plain_index(p, c);
  const int xp = plain_nb(p, c, mu, 1), xn = plain_nb(p, c, nu, 1), xm = plain_nb(p, c, nu, -1),
            xpm = plain_nb(p, c, mu, 1, nu, -1);
  Q<double> up = qmul(plink(p, n, nu), qmul(plink(p, xn, mu), qdag(plink(p, xp, nu))));
  Q<double> lo = qmul(qdag(plink(p, xm, nu)), qmul(plink(p, xm, mu), plink(p, xpm, nu)));
  return qadd(up, lo);
}

// smear_link (su2u1.c:752-795): V_dir(c) V_dir(c+dir), normalised, with
// V_dir(y) = (U_dir(y) + staples in the smeared directions j != dir) / paths
__device__ inline Q<double> smear_link(const PlainLat& p, const int* bd, const int* c, int dir) {
  int cp[3] = {c[0], c[1], c[2]};
  cp[dir] = wrap(cp[dir] + 1, p.L[dir]);
  Q<double> r = plink(p, plain_index(p, c), dir), v2 = plink(p, plain_index(p, cp), dir);
  int paths = 1;
  for (int j = 0; j < 3; j++) {
    if (j == dir || !bd[j]) continue;
    r = qadd(r, staple_onedir_dag(p, c, dir, j));
    v2 = qadd(v2, staple_onedir_dag(p, cp, dir, j));
    paths += 2;
  }
  r = qscale(r, 1.0 / (double)paths);
  v2 = qscale(v2, 1.0 / (double)paths);
  Q<double> res = qmul(r, v2);
  return qscale(res, 1.0 / sqrt(qsq(res)));
}

// smear_triplet (su2u1.c:805-852): (Sigma(c) + sum over smeared d of
// U_d(c) Sigma(c+d) U_d(c)^+ + U_d(c-d)^+ Sigma(c-d) U_d(c-d)) / sites
__device__ inline V3<double> smear_triplet(const PlainLat& p, const int* bd, const int* c) {
  const int n = plain_index(p, c);
  V3<double> cov{0.0, 0.0, 0.0};
  int sites = 1;
  for (int d = 0; d < 3; d++) {
    if (!bd[d]) continue;
    const int np = plain_nb(p, c, d, 1), nm = plain_nb(p, c, d, -1);
    V3<double> f = qrot(plink(p, n, d), ptrip(p, np));
    V3<double> b = qrot(qdag(plink(p, nm, d)), ptrip(p, nm));
    cov.x += f.x; cov.y += f.y; cov.z += f.z;
    cov.x += b.x; cov.y += b.y; cov.z += b.z;
    sites += 2;
  }
  V3<double> a = ptrip(p, n);
  const double s = (double)sites;
  return V3<double>{(a.x + cov.x) / s, (a.y + cov.y) / s, (a.z + cov.z) / s};
}

// one site of the coarser lattice b: the fields of the site of s at twice its
// coordinate in the blocked directions, links smeared in the blocked
// directions (copied in the others), the triplet smeared over the blocked
// directions; the doublet is not carried (the reference does not smear it)
__global__ void __launch_bounds__(BLOCK) k_block(PlainLat s, PlainLat b, int bd0, int bd1, int bd2, int has_trip) {
  int nb = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (nb >= b.V) return;
  const int bd[3] = {bd0, bd1, bd2};
  int cb[3], cs[3];
  plain_coords(b, nb, cb);
#pragma unroll
  for (int d = 0; d < 3; d++) cs[d] = bd[d] ? 2 * cb[d] : cb[d];
  const int ns = plain_index(s, cs);
#pragma unroll
  for (int d = 0; d < 3; d++) st_plink(b, nb, d, bd[d] ? smear_link(s, bd, cs, d) : plink(s, ns, d));
  if (has_trip) {
    V3<double> t = smear_triplet(s, bd, cs);
    b.trip[nb] = t.x;
    b.trip[b.V + nb] = t.y;
    b.trip[2 * (size_t)b.V + nb] = t.z;
  }
}

// clover_su2 (su2u1.c:207-274): the four plaquettes of the (d1, d2) plane
// that start at c, summed
__device__ inline Q<double> clover(const PlainLat& p, const int* c, int d1, int d2) {
  const int n = plain_index(p, c);
  const int x1 = plain_nb(p, c, d1, 1), x2 = plain_nb(p, c, d2, 1), xm1 = plain_nb(p, c, d1, -1),
            xm2 = plain_nb(p, c, d2, -1), x2m1 = plain_nb(p, c, d2, 1, d1, -1),
            xm12 = plain_nb(p, c, d1, -1, d2, -1), x1m2 = plain_nb(p, c, d1, 1, d2, -1);
  // U_1(x) U_2(x+1) U_1(x+2)^+ U_2(x)^+
  Q<double> cl = qmul(plink(p, n, d1), qmul(plink(p, x1, d2), qmul(qdag(plink(p, x2, d1)), qdag(plink(p, n, d2)))));
  // U_2(x) U_1(x+2-1)^+ U_2(x-1)^+ U_1(x-1)
  cl = qadd(cl, qmul(plink(p, n, d2),
                     qmul(qdag(plink(p, x2m1, d1)), qmul(qdag(plink(p, xm1, d2)), plink(p, xm1, d1)))));
  // U_1(x-1)^+ U_2(x-1-2)^+ U_1(x-1-2) U_2(x-2)
  cl = qadd(cl, qmul(qdag(plink(p, xm1, d1)),
                     qmul(qdag(plink(p, xm12, d2)), qmul(plink(p, xm12, d1), plink(p, xm2, d2)))));
  // U_2(x-2)^+ U_1(x-2) U_2(x+1-2) U_1(x)^+
  cl = qadd(cl, qmul(qdag(plink(p, xm2, d2)),
                     qmul(plink(p, xm2, d1), qmul(plink(p, x1m2, d2), qdag(plink(p, n, d1))))));
  return cl;
}

// alpha_proj (magfield.c:189-216) on the plain layout, from the spinors of
// the projectors and the four link overlaps (the same angle as the
// reference's product of projected link matrices; see alpha_proj)
__device__ inline double plain_alpha_proj(const PlainLat& p, const int* c, int d1, int d2, double sqrt_beta) {
  int c1[3] = {c[0], c[1], c[2]}, c2[3] = {c[0], c[1], c[2]};
  c1[d1] = wrap(c1[d1] + 1, p.L[d1]);
  c2[d2] = wrap(c2[d2] + 1, p.L[d2]);
  const int n = plain_index(p, c), n1 = plain_index(p, c1), n2 = plain_index(p, c2), n12 = plain_nb(p, c1, d2, 1);
  const Spinor<double> sx = proj_spinor(ptrip(p, n)), s1 = proj_spinor(ptrip(p, n1)), s2 = proj_spinor(ptrip(p, n2)),
                       s12 = proj_spinor(ptrip(p, n12));
  double z1r, z1i, z2r, z2i, z3r, z3i, z4r, z4i;
  link_overlap(sx, plink(p, n, d1), s1, z1r, z1i);
  link_overlap(s1, plink(p, n1, d2), s12, z2r, z2i);
  link_overlap(s2, plink(p, n2, d1), s12, z3r, z3i);
  link_overlap(sx, plink(p, n, d2), s2, z4r, z4i);
  const double pr = z1r * z2r - z1i * z2i, pi = z1r * z2i + z1i * z2r;
  const double qr = z3r * z4r - z3i * z4i, qi = z3r * z4i + z3i * z4r;
  return atan2(pi * qr - pr * qi, pr * qr + pi * qi) * sqrt_beta;
}

// Per plane z (blockIdx.y) and chunk (blockIdx.x) of its sites: q = 0 the sum
// of |phi|^2/2 (plane_sum(doubletsq), correlation.c:16-33), 1 Tr Sigma^2, then
// re/im of the photon operators for (transmom, mode) = (1,0), (2,0), (1,1),
// (2,1): mode 0 the clover field strength projected on Sigma
// (projected_photon_operator, correlation.c:99-164), mode 1 twice the
// projected alpha of the plane (photon_projection_full, correlation.c:207-253),
// times exp(2 pi i p.x) with p = (transmom, 0, 0) when dir != 0 and p = 0 when
// dir = 0 (photon_correl, correlation.c:270-274, stops its direction loop after
// the first direction).  Out: part[(z * chunks + chunk) * NCORR_PLANE + q].
__global__ void __launch_bounds__(CBLOCK) k_plane_ops(PlainLat p, int dir, int has_phi, int has_trip,
                                                      double sqrt_beta, int chunks, double* part) {
  const int z = blockIdx.y, chunk = blockIdx.x;
  const int d1 = dir == 0 ? 1 : 0, d2 = dir == 2 ? 1 : 2;
  const int area = p.V / p.L[dir];
  const int per = (area + chunks - 1) / chunks, lo = chunk * per, hi = min(area, lo + per);
  double m[NCORR_PLANE];
#pragma unroll
  for (int q = 0; q < NCORR_PLANE; q++) m[q] = 0.0;
  for (int k = lo + (int)threadIdx.x; k < hi; k += CBLOCK) {
    int c[3];
    c[dir] = z;
    c[d1] = k % p.L[d1];
    c[d2] = k / p.L[d1];
    const int n = plain_index(p, c);
    if (has_phi)
      m[0] += 0.5 * (p.phi[n] * p.phi[n] + p.phi[p.V + n] * p.phi[p.V + n] +
                     p.phi[2 * (size_t)p.V + n] * p.phi[2 * (size_t)p.V + n] +
                     p.phi[3 * (size_t)p.V + n] * p.phi[3 * (size_t)p.V + n]);
    if (has_trip) {
      V3<double> a = ptrip(p, n);
      m[1] += 0.5 * (a.x * a.x + a.y * a.y + a.z * a.z);
      Q<double> cl = clover(p, c, d1, d2);
      const double tr = a.x * (cl.b / 4.0) + a.y * (cl.c / 4.0) + a.z * (cl.d / 4.0);
      const double al = 2.0 * plain_alpha_proj(p, c, d1, d2, sqrt_beta);
#pragma unroll
      for (int tm = 1; tm <= 2; tm++) {
        double sn = 0.0, cs = 1.0;
        if (dir != 0) sincospi(2.0 * ((double)(tm * c[0]) / (double)p.L[0]), &sn, &cs);
        m[2 + 2 * (tm - 1)] += tr * cs;
        m[3 + 2 * (tm - 1)] += tr * sn;
        m[6 + 2 * (tm - 1)] += al * cs;
        m[7 + 2 * (tm - 1)] += al * sn;
      }
    }
  }
  __shared__ double sm[CBLOCK / 32][NCORR_PLANE];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NCORR_PLANE; q++) {
    double v = m[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sm[w][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < NCORR_PLANE) {
    double v = 0.0;
    for (int ww = 0; ww < CBLOCK / 32; ww++) v += sm[ww][threadIdx.x];
    part[((size_t)z * chunks + chunk) * NCORR_PLANE + threadIdx.x] = v;
  }
}

__global__ void k_plane_totals(const double* part, int Lz, int chunks, double* tot) {
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Lz * NCORR_PLANE) return;
  const int z = t / NCORR_PLANE, q = t % NCORR_PLANE;
  double v = 0.0;
  for (int k = 0; k < chunks; k++) v += part[((size_t)z * chunks + k) * NCORR_PLANE + q];
  tot[t] = v;
}

// measure_correlators' values (correlation.c:350-398) at distance d = thread:
// 4 sum_z h(z) h(z+d) / V (higgs_correlator, doubletsq is half the trace),
// sum_z s(z) s(z+d) / V, and sum_z O(z) O(z+d)^* / V for the four photon
// operators (cmult, stddefs.h:93-98); out[d][NCORR]
__global__ void k_correl_combine(const double* tot, int Lz, double vol, int has_phi, int has_trip, double* out) {
  const int d = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= Lz / 2) return;
  double hc = 0.0, sc = 0.0, pre[4] = {0, 0, 0, 0}, pim[4] = {0, 0, 0, 0};
  for (int z = 0; z < Lz; z++) {
    const int zd = (z + d) % Lz;
    const double* a = tot + (size_t)z * NCORR_PLANE;
    const double* b = tot + (size_t)zd * NCORR_PLANE;
    hc += a[0] * b[0];
    sc += a[1] * b[1];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const double ar = a[2 + 2 * k], ai = a[3 + 2 * k], br = b[2 + 2 * k], bi = -b[3 + 2 * k];
      pre[k] += ar * br - ai * bi;
      pim[k] += br * ai + ar * bi;
    }
  }
  double* r = out + (size_t)d * NCORR;
  r[0] = has_phi ? 4.0 * hc / vol : 0.0;
  r[1] = has_trip ? sc / vol : 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    r[2 + 2 * k] = has_trip ? pre[k] / vol : 0.0;
    r[3 + 2 * k] = has_trip ? pim[k] / vol : 0.0;
  }
}

// ---------------------------------------------------------------------------
void launch_to_plain(int prec, const void* f, const Geom& g, int has_phi, int has_trip, const PlainLat& p,
                     cudaStream_t st) {
  if (prec == 64)
    k_to_plain<double><<<(g.V + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(*(const Fields<double>*)f, g, has_phi, has_trip,
                                                                    p);
  else
    k_to_plain<float><<<(g.V + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(*(const Fields<float>*)f, g, has_phi, has_trip,
                                                                   p);
}

void launch_block(const PlainLat& s, const PlainLat& b, const int* bd, int has_trip, cudaStream_t st) {
  k_block<<<(b.V + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(s, b, bd[0], bd[1], bd[2], has_trip);
}

int correl_chunks(const PlainLat& p, int dir, int sm_count) {
  const int Lz = p.L[dir], area = p.V / Lz;
  int chunks = (2 * sm_count + Lz - 1) / Lz;  // about two blocks per SM over all planes
  const int most = (area + CBLOCK - 1) / CBLOCK;
  if (chunks > most) chunks = most;
  return chunks < 1 ? 1 : chunks;
}

void launch_correlators(const PlainLat& p, int dir, int has_phi, int has_trip, double sqrt_beta, int chunks,
                        double* part, double* tot, double* out, cudaStream_t st) {
  const int Lz = p.L[dir];
  k_plane_ops<<<dim3(chunks, Lz), CBLOCK, 0, st>>>(p, dir, has_phi, has_trip, sqrt_beta, chunks, part);
  k_plane_totals<<<(Lz * NCORR_PLANE + 127) / 128, 128, 0, st>>>(part, Lz, chunks, tot);
  k_correl_combine<<<(Lz / 2 + 63) / 64, 64, 0, st>>>(tot, Lz, (double)p.V, has_phi, has_trip, out);
}

}  // namespace su2
