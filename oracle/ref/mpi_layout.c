/* TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * Runs the site layout of the reference's MPI build (layout.c:16-402, built
 * with -DMPI against mpistub/mpi.h) for one rank of an N-rank run, so that
 * the order in which an N-rank run writes its lattice file (write_field,
 * checkpoint.c:226-269: rank 0's sites, then rank 1's, ... each in its local
 * storage order) can be read off the reference itself.  Only the steps of
 * layout() that exchange no message are run: make_slices, the lattice
 * tables, sitemap, set_parity and the EVEN-first paritymap. */
#include "su2.h"
#include "comms.h"

#include <stdio.h>
#include <stdlib.h>

static int stub_called(const char* what) {
  fprintf(stderr, "mpi_layout: %s called in the layout-only harness\n", what);
  return 1;
}
int MPI_Init(int* a, char*** b) { (void)a; (void)b; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
int MPI_Comm_split(MPI_Comm c, int a, int b, MPI_Comm* o) { (void)c; (void)a; (void)b; *o = 0; return stub_called("MPI_Comm_split"); }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int g, MPI_Comm c) { (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; return stub_called("MPI_Send"); }
int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Status* st) { (void)b; (void)n; (void)t; (void)s; (void)g; (void)c; (void)st; return stub_called("MPI_Recv"); }
int MPI_Isend(const void* b, int n, MPI_Datatype t, int d, int g, MPI_Comm c, MPI_Request* r) { (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; (void)r; return stub_called("MPI_Isend"); }
int MPI_Irecv(void* b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Request* r) { (void)b; (void)n; (void)t; (void)s; (void)g; (void)c; (void)r; return stub_called("MPI_Irecv"); }
int MPI_Wait(MPI_Request* r, MPI_Status* s) { (void)r; (void)s; return 0; }
int MPI_Waitall(int n, MPI_Request* r, MPI_Status* s) { (void)n; (void)r; (void)s; return 0; }
int MPI_Probe(int s, int g, MPI_Comm c, MPI_Status* st) { (void)s; (void)g; (void)c; (void)st; return stub_called("MPI_Probe"); }
int MPI_Get_count(const MPI_Status* s, MPI_Datatype t, int* n) { (void)s; (void)t; *n = 0; return stub_called("MPI_Get_count"); }
int MPI_Bcast(void* b, int n, MPI_Datatype t, int r, MPI_Comm c) { (void)b; (void)n; (void)t; (void)r; (void)c; return 0; }
int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, int x, MPI_Comm c) { (void)s; (void)r; (void)n; (void)t; (void)o; (void)x; (void)c; return stub_called("MPI_Reduce"); }
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) { (void)s; (void)r; (void)n; (void)t; (void)o; (void)c; return stub_called("MPI_Allreduce"); }
int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); }
double MPI_Wtime(void) { return 0.0; }

/* The global coordinates of rank `rank`'s sites in its storage order (the
 * order write_field writes them), sites x dim longs; returns the number of
 * sites per rank, and the slicing in nslices[dim]. */
long ref_mpi_rank_sites(int dim, const int* Lin, int size, int rank, long* coords, int* nslices) {
  lattice l;
  memset(&l, 0, sizeof(l));
  l.dim = dim;
  l.L = malloc(dim * sizeof(*l.L));
  l.vol = 1;
  for (int d = 0; d < dim; d++) { l.L[d] = Lin[d]; l.vol *= Lin[d]; }
  l.size = size;
  l.rank = rank;
  myRank = rank;
  MPISize = size;
  /* layout.c:16-65, the steps before the first message */
  l.sliceL = malloc(dim * sizeof(*l.sliceL));
  l.nslices = malloc(dim * sizeof(*l.nslices));
  l.offset = malloc(dim * sizeof(*l.offset));
  make_slices(&l, 0);
  alloc_lattice_arrays(&l, l.sites_total);
  long tot_old = l.sites_total;
  sitemap(&l);
  realloc_lattice_arrays(&l, tot_old, l.sites_total);
  set_parity(&l);
  long* newindex = malloc(l.sites_total * sizeof(long));
  paritymap(&l, newindex);
  remap_lattice_arrays(&l, newindex, l.sites_total);
  free(newindex);
  for (long i = 0; i < l.sites; i++)
    for (int d = 0; d < dim; d++) coords[i * dim + d] = l.coords[i][d];
  for (int d = 0; d < dim; d++) nslices[d] = l.nslices[d];
  return l.sites;
}
