// su2_correl.h -- launchers of the correlator and blocking kernels
// (su2_correl.cu) and the plain lattice they work on.
#pragma once

#include <cuda_runtime.h>

#include "su2_common.cuh"

namespace su2 {

// A lattice in lexicographic site order (n = x + L0 (y + L1 z)), FP64
// structure-of-arrays: component k of the link in direction d of site n at
// link[(4 d + k) V + n], triplet component k at trip[k V + n], first doublet
// component k at phi[k V + n] (null where absent).  Any side >= 1.
struct PlainLat {
  int L[3];
  int V;
  double* link;
  double* trip;
  double* phi;
};

constexpr int CBLOCK = 128;        // threads of a plane-chunk block
constexpr int NCORR_PLANE = 10;    // per plane: |phi|^2/2, Tr Sigma^2, 4 photon operators (re, im)
constexpr int NCORR = 10;          // per distance: the columns of SU2GPU_CORR_*

// doubles of a plain lattice's arrays
inline size_t plain_doubles(long long V, int has_phi, int has_trip) {
  return (size_t)V * (12 + (has_trip ? 3 : 0) + (has_phi ? 4 : 0));
}
// carve a plain lattice of sides L out of buf (plain_doubles of them)
inline PlainLat make_plain(const int* L, double* buf, int has_phi, int has_trip) {
  PlainLat p;
  p.L[0] = L[0]; p.L[1] = L[1]; p.L[2] = L[2];
  p.V = L[0] * L[1] * L[2];
  p.link = buf;
  p.trip = has_trip ? buf + (size_t)12 * p.V : nullptr;
  p.phi = has_phi ? buf + (size_t)(12 + (has_trip ? 3 : 0)) * p.V : nullptr;
  return p;
}

// fields (a Fields<double> or Fields<float>, by prec) -> plain lattice p
void launch_to_plain(int prec, const void* f, const Geom& g, int has_phi, int has_trip, const PlainLat& p,
                     cudaStream_t st);
// smear s in the directions bd[d] != 0 and move its even sites onto b
void launch_block(const PlainLat& s, const PlainLat& b, const int* bd, int has_trip, cudaStream_t st);
// chunks per plane of launch_correlators for a device with sm_count SMs
int correl_chunks(const PlainLat& p, int dir, int sm_count);
// correlators along dir: part[L[dir] chunks NCORR_PLANE], tot[L[dir] NCORR_PLANE],
// out[L[dir]/2 NCORR]
void launch_correlators(const PlainLat& p, int dir, int has_phi, int has_trip, double sqrt_beta, int chunks,
                        double* part, double* tot, double* out, cudaStream_t st);

}  // namespace su2
