/* su2host.h -- the C host of bin/su2: config reader, lattice/weight files,
 * labels/measure writers.  Mirrors the reference's host-side behaviour
 * (parameters.c, checkpoint.c, multicanonical.c file I/O, measure.c output)
 * so that `bin/su2 config` is a drop-in for the reference binary; all field
 * updates and volume sums run on the GPU through libsu2gpu. */
#ifndef SU2HOST_H
#define SU2HOST_H

#include <stdint.h>
#include <stdio.h>

#include "../../include/su2gpu.h"

/* run settings read from the config (params, parameters.c:157-338) */
typedef struct {
  su2gpu_params p;
  int nhiggs, triplet, singlet, u1, gradflow;
  int reset;
  long iterations, checkpoint, n_thermalize, interval;
  char resultsfile[200];
  char latticefile[200];
  int run_checks, do_local_meas, multicanonical;
  double phi0, sigma0, singlet0;
  /* gradient flow */
  int do_flow, flow_interval, flow_meas_interval;
  double flow_dt, flow_t_max;
  /* profiles along z (the reference's -DMEASURE_Z build, z_coord.c) */
  int measure_z, do_z_meas, setup_wall;
  long meas_interval_z;
  /* heatbath real-time trajectories (the reference's -DHB_TRAJECTORY build) */
  int hb_trajectory, do_trajectory;
  /* rank count of the lattice file layout: file_ranks as read (1 for a new
   * lattice), lattice_mpi_size the optional key that sets the layout written
   * (0 = as read) */
  int file_ranks, lattice_mpi_size;
  /* correlators and blocking (-DCORRELATORS, -DBLOCKING) */
  int correlators, blocking, do_correlators, correlator_interval, blocks;
  /* additions of this implementation (optional keys) */
  uint64_t seed;
  int have_seed;
  int use_graph;
} host_params;

/* multicanonical settings (get_weight_parameters, parameters.c:344-402) */
typedef struct {
  char weightfile[200];
  int mode, checks_per_sweep, bins, orderparam;
  double min, max, delta;
} host_muca;

/* settings of the heatbath trajectories, read from "realtime_config"
 * (trajectory struct, su2.h:566-575) */
typedef struct {
  int n_traj, interval, mode_interval;
  double min, max;
} host_traj;

/* config.c */
int cfg_open(const char* fname, FILE** f);
int cfg_find(FILE* f, const char* label, char* result); /* 1 found, 0 not */
int cfg_get_int(FILE* f, const char* label);
long cfg_get_long(FILE* f, const char* label);
double cfg_get_double(FILE* f, const char* label);
void cfg_get_string(FILE* f, const char* label, char* result);
int cfg_get_algorithm(FILE* f, const char* label);
int cfg_optional_string(const char* fname, const char* label, char* result);
void read_parameters(const char* fname, host_params* hp);
void read_weight_parameters(const char* fname, const host_params* hp, host_muca* hm);
void read_updated_parameters(const char* fname, host_params* hp);
void print_parameters(const host_params* hp);
void die(int code);

/* files.c */
int64_t field_count(const host_params* hp, int which); /* doubles per field array */
/* site order of the lattice file of an nranks-rank run of the reference:
 * order[k] = lexicographic index of the k-th site; 0, or -1 if the reference
 * could not lay the lattice out on that many ranks */
int mpi_file_order(int dim, const int* L, int nranks, int64_t* order);
int save_lattice(const char* fname, const host_params* hp, long iter, double total_time, double comms_time,
                 double* const* arrays);
int load_lattice(const char* fname, host_params* hp, long* iter, double* total_time, double* comms_time,
                 double** arrays);
void print_labels(const host_params* hp);
void print_labels_local(const host_params* hp, const char* fname);
void print_z_labels(const host_params* hp);
/* one measure_along_z block appended to measure_z from the plane sums
 * sums[4 z + q] (q: phi^2, Tr Sigma^2, S, S^2) along direction zdir */
void write_measure_z(const host_params* hp, int zdir, const double* sums);
/* prepare_wall (z_coord.c:304-375): two phases split at the middle of the z
 * direction, in the FP64 host arrays; seed drives the host's own stream */
void prepare_wall(const host_params* hp, double* const* arrays, uint64_t seed);
int z_direction(const host_params* hp);
/* one measure_local file: per site in storage order its coordinates and, with
 * the triplet, (Tr Sigma^2, magnetic charge) from vals[2 V] */
int write_measure_local(const char* fname, const host_params* hp, const double* vals);
void write_measure_row(FILE* f, const host_params* hp, const double* sums, const su2gpu_weight* w, int have_muca);
int load_weight(su2gpu_weight* w, host_muca* hm);
void save_weight(const su2gpu_weight* w);
void linearize_weight(su2gpu_weight* w);
double get_weight(const su2gpu_weight* w, double val);
void print_acceptance(const host_params* hp, const int64_t* c);

/* correl.c */
/* print_labels_correlators (correlation.c:320-346): labels_correl */
void print_labels_correlators(const host_params* hp);
/* one measure_correlators block (correlation.c:350-398) appended to fname:
 * the header with meas_id, then per distance d < nrows the values of
 * rows[d * SU2GPU_NCORR + col] the content has */
void write_correlators(const char* fname, const host_params* hp, int meas_id, const double* rows, int nrows);

/* trajectory.c */
void read_realtime_config(const char* fname, host_traj* t);
void print_realtime_params(const host_params* hp, const host_traj* t);
/* one set of trajectories from the configuration in `ctx` (the fields are
 * not changed); `w` is the run's weight, used read-only for the order
 * parameter; sweeps run on a second context seeded by (seed, chain
 * 0x40000000 + id) */
int make_realtime_trajectories(su2gpu_ctx* ctx, const host_params* hp, const su2gpu_weight* w,
                               const host_traj* t, int id, uint64_t seed, int64_t* counters);

#endif
