// su2_probe.cu -- per-site values of the deterministic parts of the update
// sweep (staples, local actions, overrelaxation proposals) on a context's
// FP64 fields, for checking them one site at a time against the reference
// (su2gpu_site_values).  The kernel calls the device functions the sweep
// kernels call; the overrelaxation updates run with ZeroRng, whose uniforms
// are all 0, so every proposal is accepted: the thread reads the proposal
// back and restores the site's old value.  A launch covers one parity, whose
// sites read only each other's neighbours of the other parity, so the
// temporary write of a site is seen by its own thread alone.
#include "su2_kernels.cuh"
#include "su2_ops.h"

namespace su2 {

__global__ void __launch_bounds__(BLOCK) k_site_probe(Fields<double> f, Geom g, CoupT<double> cp, int what,
                                                      int parity, double* out) {
  using R = double;
  constexpr int CC = C_GENERIC;
  int t = (int)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.half) return;
  int c[3];
  site_coords(g, parity, t, c);
  const int i = parity * g.half + t;
  const size_t si = (size_t)i;
  int fb = 0;
  ZeroRng<R> zr;
  switch (what) {
    case SITE_LINK_STAPLE:
    case SITE_WILSON_STAPLE:
#pragma unroll
      for (int mu = 0; mu < 3; mu++) {
        Q<R> s = what == SITE_LINK_STAPLE ? link_staple<R, CC>(f, g, cp, c, i, mu) : wilson_staple(f, g, c, i, mu);
        double* o = out + (si * 3 + mu) * 4;
        o[0] = s.a; o[1] = s.b; o[2] = s.c; o[3] = s.d;
      }
      break;
    case SITE_LOCALACT_SU2LINK:
      for (int mu = 0; mu < 3; mu++) out[si * 3 + mu] = localact_su2link<R, CC>(f, g, cp, c, i, mu);
      break;
    case SITE_LOCALACT_U1LINK:
      for (int mu = 0; mu < 3; mu++) out[si * 3 + mu] = localact_u1link<R, CC>(f, g, cp, c, i, mu);
      break;
    case SITE_STAPLE_DOUBLET: {
      Q<R> s = staple_doublet<R, CC>(f, g, cp, c, i, 0);
      double* o = out + si * 4;
      o[0] = s.a; o[1] = s.b; o[2] = s.c; o[3] = s.d;
      break;
    }
    case SITE_LOCALACT_DOUBLET:
      out[si] = localact_doublet<R, CC>(f, g, cp, c, i, 0);
      break;
    case SITE_LOCALACT_SINGLET:
      out[si] = localact_singlet<R, CC>(f, g, cp, c, i);
      break;
    case SITE_OR_DOUBLET:
    case SITE_OR_DOUBLET1: {
      const int h = what == SITE_OR_DOUBLET ? 0 : 1;
      const Q<R> old = ld4<R>(php(f, h), i);
      if (SU2_HAS(CC, cp.content, C_H2)) overrelax_higgs2<R, CC>(f, g, cp, c, i, h, zr, &fb);
      else overrelax_doublet<R, CC>(f, g, cp, c, i, zr, &fb);
      const Q<R> nw = ld4<R>(php(f, h), i);
      st4<R>(php(f, h), i, old);
      double* o = out + si * 4;
      o[0] = nw.a; o[1] = nw.b; o[2] = nw.c; o[3] = nw.d;
      break;
    }
    case SITE_OR_TRIPLET: {
      const V3<R> old = ld3(f, i);
      overrelax_triplet<R, CC>(f, g, cp, c, i, zr, &fb);
      const V3<R> nw = ld3(f, i);
      st3(f, i, old);
      double* o = out + si * 3;
      o[0] = nw.x; o[1] = nw.y; o[2] = nw.z;
      break;
    }
    case SITE_OR_SINGLET: {
      const R old = f.sing[i];
      overrelax_singlet<R, CC>(f, g, cp, c, i, zr, &fb);
      out[si] = f.sing[i];
      f.sing[i] = old;
      break;
    }
    default:
      break;
  }
}

void launch_site_probe(int what, int parity, const Fields<double>& f, const Geom& g, const Coup& cp, double* out,
                       cudaStream_t st) {
  const unsigned nb = (unsigned)((g.half + BLOCK - 1) / BLOCK);
  if (nb) k_site_probe<<<nb, BLOCK, 0, st>>>(f, g, coup_as<double>(cp), what, parity, out);
}

}  // namespace su2
