/* su2_main.c -- bin/su2, the drop-in for the reference's program (main.c):
 *
 *   bin/su2 [--content NAME] [--precision 64|32] [--seed N] [--files-only] <config>
 *
 * --files-only runs the host side of a run of 0 iterations without touching
 * the GPU: read the config, the lattice file and (multicanonical runs) the
 * weight file, and write labels, lattice and weight back as the reference
 * does; a check of file compatibility that needs no device.
 *
 * Same config keys, same outputs (labels, measure, measure_flow, lattice,
 * weight) and the same iteration structure as main.c:10-421: thermalise with
 * the weight read-only after a reset, then per iteration measure (every
 * `interval`), flow (every `flow_interval`), heatbath trajectories (every
 * `mode_interval` of realtime_config, -DHB_TRAJECTORY builds: content
 * modifier +hb_trajectory), correlators (every `correlator_interval`,
 * -DCORRELATORS / -DBLOCKING: modifiers +correlators, +blocking), update,
 * checkpoint.  All field
 * updates, measurements and flows run on the GPU through libsu2gpu; runs of
 * iterations without host work in between are replayed as one CUDA graph.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <time.h>
#include <unistd.h>

#include "su2host.h"

static double wall(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

#define GPU(call)                                                              \
  do {                                                                         \
    int rc_ = (call);                                                          \
    if (rc_ != SU2GPU_OK) {                                                    \
      fprintf(stderr, "GPU error %d in %s: %s\n", rc_, #call, su2gpu_last_error()); \
      exit(600 - rc_);                                                         \
    }                                                                          \
  } while (0)

/* the file side of a run of 0 iterations (main.c:200-290, 395-401) */
static int files_roundtrip(host_params* hp, host_muca* hm) {
  int64_t V = 1;
  for (int d = 0; d < hp->p.dim; d++) V *= hp->p.L[d];
  double* arrays[6] = {0};
  for (int k = 0; k < 6; k++) {
    int64_t n = field_count(hp, k);
    if (n) arrays[k] = (double*)calloc((size_t)(V * n), sizeof(double));
  }
  long citer = 0;
  double total_time = 0.0, comms_time = 0.0;
  if (access(hp->latticefile, R_OK) == 0) {
    load_lattice(hp->latticefile, hp, &citer, &total_time, &comms_time, arrays);
  } else {
    for (int64_t k = 0; k < V * hp->p.dim; k++) arrays[0][4 * k] = 1.0;
    for (int h = 0; h < hp->nhiggs; h++)
      for (int64_t i = 0; i < V; i++) arrays[2 + h][4 * i] = hp->phi0;
    if (hp->triplet)
      for (int64_t i = 0; i < V; i++) arrays[4][3 * i] = hp->sigma0;
    if (hp->singlet)
      for (int64_t i = 0; i < V; i++) arrays[5][i] = hp->singlet0;
    hp->reset = 1;
  }
  if (hp->measure_z && hp->do_z_meas) print_z_labels(hp);
  print_labels(hp);
  if (hp->do_local_meas) print_labels_local(hp, "labels_local");
  if (hp->multicanonical) {
    su2gpu_weight w;
    load_weight(&w, hm); /* writes the weight back, as load_weight() does */
  }
  save_lattice(hp->latticefile, hp, hp->reset ? 1 : citer + 1, 0.0, 0.0, arrays);
  for (int k = 0; k < 6; k++) free(arrays[k]);
  return 0;
}

int main(int argc, char** argv) {
  const char* content = NULL;
  const char* precision = NULL;
  const char* seed_arg = NULL;
  int files_only = 0;
  int a = 1;
  while (a < argc && !strncmp(argv[a], "--", 2)) {
    if (!strcmp(argv[a], "--content") && a + 1 < argc) content = argv[++a];
    else if (!strcmp(argv[a], "--precision") && a + 1 < argc) precision = argv[++a];
    else if (!strcmp(argv[a], "--seed") && a + 1 < argc) seed_arg = argv[++a];
    else if (!strcmp(argv[a], "--files-only")) files_only = 1;
    else break;
    a++;
  }
  if (argc - a != 1) {
    printf("Usage: ./<program name> <config file>\n");
    die(0);
  }
  const char* cfg = argv[a];
  if (content) setenv("SU2_CONTENT", content, 1);

  host_params hp;
  read_parameters(cfg, &hp);
  if (precision) hp.p.precision = atoi(precision);
  uint64_t seed;
  if (seed_arg) seed = strtoull(seed_arg, NULL, 10);
  else if (hp.have_seed) seed = hp.seed;
  else {
    long s = time(NULL);
    s = s ^ (s << 26) ^ (s << 9);
    seed = (uint64_t)s;
  }
  printf("Seed in root node: %ld\n", (long)seed);
  print_parameters(&hp);

  host_muca hm;
  read_weight_parameters(cfg, &hp, &hm);

  /* main.c:98-157: correlators along the longest direction (ties to the
   * last, make_misc_tables layout.c:773-777); blocking in all the others */
  int corr_dir = hp.p.dim - 1;
  for (int d = hp.p.dim - 1; d >= 0; d--)
    if (hp.p.L[d] > hp.p.L[corr_dir]) corr_dir = d;
  const int docorr = hp.correlators && hp.do_correlators && hp.correlator_interval > 0;
  if (hp.correlators && hp.do_correlators) {
    print_labels_correlators(&hp);
    printf("\nMeasuring correlation functions along direction %d every %d iterations\n", corr_dir + 1,
           hp.correlator_interval);
  }
  int32_t block_dir[3] = {0, 0, 0};
  int block_levels = 0;
  if (hp.blocking) {
    block_levels = hp.blocks;
    printf("\n--- Using blocking in directions: ");
    for (int d = 0; d < hp.p.dim; d++)
      if (d != corr_dir) {
        block_dir[d] = 1;
        printf("%d ", d);
      }
    printf(", up to %d levels ---\n", block_levels);
    /* max_block_level (blocking.c:17-38) */
    int len[3] = {hp.p.L[0], hp.p.L[1], hp.p.L[2]}, mx = 0, ok = 1;
    while (ok && mx < 64) {
      for (int d = 0; d < 3 && ok; d++)
        if (block_dir[d] && (len[d] % 2 != 0 || len[d] <= 2)) ok = 0;
      if (!ok) break;
      for (int d = 0; d < 3; d++)
        if (block_dir[d]) len[d] /= 2;
      mx++;
    }
    if (mx < block_levels) {
      printf("Warning: unable to block to %d levels; max is %d. Using %d levels instead.\n", block_levels, mx, mx);
      block_levels = mx;
    }
    int bl[3] = {hp.p.L[0], hp.p.L[1], hp.p.L[2]};
    for (int k = 0; k < block_levels; k++) {
      for (int d = 0; d < 3; d++)
        if (block_dir[d]) bl[d] /= 2;
      printf("Initializing blocked lattice of volume: %d x %d x %d (MPI size = 1)\n", bl[0], bl[1], bl[2]);
    }
    printf("--- Blocking structs ready ---\n\n");
    fflush(stdout);
  }

  if (files_only) return files_roundtrip(&hp, &hm);

  double t0 = wall();
  su2gpu_ctx* ctx = NULL;
  GPU(su2gpu_create(&hp.p, &ctx));
  GPU(su2gpu_set_seed(ctx, seed, 0));
  printf("Initialization done! Took %lf seconds.\n", wall() - t0);
  fflush(stdout);

  int64_t V = 1;
  for (int d = 0; d < hp.p.dim; d++) V *= hp.p.L[d];
  double* arrays[6] = {0};
  for (int k = 0; k < 6; k++) {
    int64_t n = field_count(&hp, k);
    if (n) arrays[k] = (double*)calloc((size_t)(V * n), sizeof(double));
  }
  printf("Allocated memory for fields.\n");

  long citer = 1;
  double total_time = 0.0, comms_time = 0.0;
  if (access(hp.latticefile, R_OK) == 0) {
    printf("\nLoading latticefile: %s\n", hp.latticefile);
    load_lattice(hp.latticefile, &hp, &citer, &total_time, &comms_time, arrays);
    printf("Fields loaded succesfully.\n");
  } else {
    /* setfields (init.c:92-112): cold start */
    printf("No latticefile found; starting with cold configuration.\n");
    for (int64_t k = 0; k < V * hp.p.dim; k++) arrays[0][4 * k] = 1.0;
    for (int h = 0; h < hp.nhiggs; h++)
      for (int64_t i = 0; i < V; i++) arrays[2 + h][4 * i] = hp.phi0;
    if (hp.triplet)
      for (int64_t i = 0; i < V; i++) arrays[4][3 * i] = hp.sigma0;
    if (hp.singlet)
      for (int64_t i = 0; i < V; i++) arrays[5][i] = hp.singlet0;
    hp.reset = 1;
  }
  /* main.c:189-199: a phase-interface start overrides the field initialisation */
  if (hp.measure_z && hp.reset && hp.setup_wall) prepare_wall(&hp, arrays, seed);
  GPU(su2gpu_upload_fields(ctx, arrays[0], arrays[1], arrays[2], arrays[3], arrays[4], arrays[5]));

  if (hp.measure_z && hp.do_z_meas) {
    print_z_labels(&hp);
    printf("Measuring profiles along direction %d every %ld iterations\n", z_direction(&hp) + 1, hp.meas_interval_z);
  }
  print_labels(&hp);
  if (hp.do_local_meas) print_labels_local(&hp, "labels_local");

  FILE* results = fopen(hp.resultsfile, "a");
  su2gpu_weight w;
  memset(&w, 0, sizeof(w));
  int weight_updates = 0;
  if (hp.multicanonical) {
    load_weight(&w, &hm);
    GPU(su2gpu_muca_set(ctx, &w));
    GPU(su2gpu_calc_orderparam(ctx, 0, NULL));
    GPU(su2gpu_calc_orderparam(ctx, 1, NULL));
    GPU(su2gpu_muca_get(ctx, &w));
    if (w.mode == SU2GPU_MUCA_READONLY) printf("Read-only run, will not modify weight. \n");
  }
  /* main.c:223-240 */
  host_traj traj;
  memset(&traj, 0, sizeof(traj));
  const int dotraj = hp.hb_trajectory && hp.do_trajectory;
  if (dotraj) {
    printf("\nReal time simulation: reading file \"realtime_config\"\n");
    read_realtime_config("realtime_config", &traj);
    print_realtime_params(&hp, &traj);
    if (!hp.multicanonical) {
      printf("\nError: Need multicanonical for heatbath trajectories!! Exiting...\n");
      die(-44);
    }
    FILE* tf = fopen("trajectory", "a");
    fprintf(tf, "===== Realtime trajectories: min=%g, max=%g, n_traj=%d ===== \n", traj.min, traj.max, traj.n_traj);
    fclose(tf);
  }
  if (hp.gradflow && hp.do_flow) {
    printf("\n----- Gradient flow every %d iterations -----\n", hp.flow_interval);
    printf("dt %lf\tt_max %lf\t\tmeas_interval %d \n", hp.flow_dt, hp.flow_t_max, hp.flow_meas_interval);
  }

  uint32_t sweep = 0; /* counter word of the random stream: one per sweep of this run */
  long iter = 1;
  if (hp.reset) {
    int mode = w.mode;
    if (hp.multicanonical && mode != SU2GPU_MUCA_READONLY) {
      GPU(su2gpu_muca_get(ctx, &w));
      w.mode = SU2GPU_MUCA_READONLY;
      GPU(su2gpu_muca_set(ctx, &w));
    }
    printf("\nThermalizing %ld iterations\n", hp.n_thermalize);
    fflush(stdout);
    double ts = wall();
    if (hp.n_thermalize > 0) GPU(su2gpu_run_sweeps(ctx, sweep, (int32_t)hp.n_thermalize, hp.use_graph));
    sweep += (uint32_t)hp.n_thermalize;
    printf("Thermalization done, took %lf seconds.\n", wall() - ts);
    GPU(su2gpu_reset_counters(ctx));
    if (hp.multicanonical && mode != SU2GPU_MUCA_READONLY) {
      GPU(su2gpu_muca_get(ctx, &w));
      w.mode = mode;
      GPU(su2gpu_muca_set(ctx, &w));
      GPU(su2gpu_muca_init_last_max(ctx));
    }
    printf("\nStarting new simulation!\n");
  } else {
    iter = citer + 1;
    printf("\nContinuing from iteration %ld!\n", iter - 1);
  }
  if (hp.multicanonical) GPU(su2gpu_muca_weight_updates(ctx, &weight_updates));

  total_time = 0.0;
  comms_time = 0.0;
  double tstart = wall();
  int flow_id = 1;
  int traj_id = 1;
  int correlator_id = 1;
  int nmeas = 1 + SU2GPU_NMEAS;
  while (iter <= hp.iterations) {
    if (hp.interval > 0 && iter % hp.interval == 0) {
      double m[SU2GPU_NMEAS];
      GPU(su2gpu_measure(ctx, m));
      if (hp.multicanonical) GPU(su2gpu_muca_get(ctx, &w));
      write_measure_row(results, &hp, m, &w, hp.multicanonical);
    }
    const int zmeas = hp.measure_z && hp.do_z_meas && hp.meas_interval_z > 0;
    if (zmeas && iter % hp.meas_interval_z == 0) {
      double* zs = (double*)malloc(sizeof(double) * 4 * (size_t)hp.p.L[z_direction(&hp)]);
      int32_t zd = 0;
      GPU(su2gpu_measure_z(ctx, &zd, zs));
      write_measure_z(&hp, zd, zs);
      free(zs);
    }
    if (hp.gradflow && hp.do_flow && hp.flow_interval > 0 && iter % hp.flow_interval == 0) {
      int maxrows = (int)(hp.flow_t_max / hp.flow_dt) / (hp.flow_meas_interval > 0 ? hp.flow_meas_interval : 1) + 4;
      double* rows = (double*)malloc(sizeof(double) * maxrows * nmeas);
      int32_t nr = 0;
      double* local = NULL;
      if (hp.do_local_meas && hp.triplet) {
        local = (double*)malloc(sizeof(double) * (size_t)maxrows * (size_t)V * 2);
        GPU(su2gpu_grad_flow_local(ctx, hp.flow_t_max, hp.flow_dt, hp.flow_meas_interval, rows, maxrows, &nr, local,
                                   maxrows));
      } else {
        GPU(su2gpu_grad_flow(ctx, hp.flow_t_max, hp.flow_dt, hp.flow_meas_interval, rows, maxrows, &nr));
      }
      /* measure_local files of the flow (gradflow.c:81-86, 124-129, 151-156) */
      for (int r = 0; hp.do_local_meas && r < nr; r++) {
        char fname[200];
        snprintf(fname, sizeof(fname), "measure_local_%d_%d", flow_id, r + 1);
        write_measure_local(fname, &hp, local ? local + (size_t)r * V * 2 : NULL);
      }
      free(local);
      if (hp.multicanonical) GPU(su2gpu_muca_get(ctx, &w));
      FILE* ff = fopen("measure_flow", "a");
      fprintf(ff, "\n =========== Flow id: %d ===========\n", flow_id);
      /* step count of the flow's time loop (gradflow.c:91-141), same double
       * arithmetic as the library's loop */
      long steps = 0;
      double tt = 0.0, dtt = hp.flow_dt;
      while (tt < hp.flow_t_max) {
        if (tt + dtt > hp.flow_t_max) dtt = hp.flow_t_max - tt;
        tt += dtt;
        steps++;
      }
      int extra_row = (steps % hp.flow_meas_interval) != 0;
      for (int r = 0; r < nr; r++) {
        /* gradflow.c:78,120 print "%.6lf "; the closing row of a flow whose
         * measurement interval does not divide the step count uses "%g "
         * (gradflow.c:148) */
        int last_extra = extra_row && (r == nr - 1);
        fprintf(ff, last_extra ? "%g " : "%.6lf ", rows[r * nmeas]);
        write_measure_row(ff, &hp, rows + r * nmeas + 1, &w, hp.multicanonical);
      }
      fclose(ff);
      free(rows);
      flow_id++;
    }
    if (dotraj && iter % traj.mode_interval == 0) {
      GPU(su2gpu_muca_get(ctx, &w));
      GPU(make_realtime_trajectories(ctx, &hp, &w, &traj, traj_id, seed, NULL));
      traj_id++;
    }
    /* main.c:330-349 */
    if (docorr && iter % hp.correlator_interval == 0) {
      const int nr = hp.p.L[corr_dir] / 2;
      double* crows = (double*)malloc(sizeof(double) * (size_t)(nr > 0 ? nr : 1) * SU2GPU_NCORR *
                                      (size_t)(block_levels + 1));
      GPU(su2gpu_measure_correlators(ctx, corr_dir, crows));
      write_correlators("correl0", &hp, correlator_id, crows, nr);
      if (block_levels > 0) {
        if (hp.nhiggs > 0) {
          /* measure_blocked_correlators (correlation.c:414-418) */
          for (int k = 0; k < block_levels; k++) printf("Error in correlation.c: Higgs smearing not yet implemented!!!\n");
        } else {
          int32_t done = 0;
          GPU(su2gpu_measure_blocked_correlators(ctx, corr_dir, block_dir, block_levels, crows, &done));
          for (int k = 0; k < done; k++) {
            char fname[100];
            snprintf(fname, sizeof(fname), "correl%d", k + 1);
            write_correlators(fname, &hp, correlator_id, crows + (size_t)k * nr * SU2GPU_NCORR, nr);
          }
        }
      }
      free(crows);
      correlator_id++;
    }
    /* iterations up to the next host event run back to back */
    long n = 1;
    while (iter + n <= hp.iterations && (hp.interval <= 0 || (iter + n) % hp.interval != 0) &&
           !(hp.gradflow && hp.do_flow && hp.flow_interval > 0 && (iter + n) % hp.flow_interval == 0) &&
           !(zmeas && (iter + n) % hp.meas_interval_z == 0) &&
           !(dotraj && (iter + n) % traj.mode_interval == 0) &&
           !(docorr && (iter + n) % hp.correlator_interval == 0) &&
           (hp.checkpoint <= 0 || (iter + n - 1) % hp.checkpoint != 0) && n < 1000000)
      n++;
    GPU(su2gpu_run_sweeps(ctx, sweep, (int32_t)n, hp.use_graph));
    sweep += (uint32_t)n;
    iter += n - 1;
    if (hp.multicanonical && w.mode != SU2GPU_MUCA_READONLY) {
      int32_t nu = 0;
      GPU(su2gpu_muca_weight_updates(ctx, &nu));
      if (nu != weight_updates) {
        GPU(su2gpu_muca_get(ctx, &w));
        save_weight(&w);
        weight_updates = nu;
      }
    }
    if (hp.checkpoint > 0 && iter % hp.checkpoint == 0) {
      double now = wall();
      total_time += now - tstart;
      tstart = now;
      int64_t cnt[SU2GPU_NCOUNTERS];
      GPU(su2gpu_get_counters(ctx, cnt));
      printf("\nCheckpointing at iteration %lu. Total time: %.1lfs, %.2lf%% comms.\n", iter, total_time,
             100.0 * comms_time / (total_time > 0 ? total_time : 1));
      print_acceptance(&hp, cnt);
      fflush(stdout);
      GPU(su2gpu_download_fields(ctx, arrays[0], arrays[1], arrays[2], arrays[3], arrays[4], arrays[5]));
      save_lattice(hp.latticefile, &hp, iter, total_time, comms_time, arrays);
      read_updated_parameters(cfg, &hp);
    }
    iter++;
  }
  if (results) fclose(results);
  total_time += wall() - tstart;
  GPU(su2gpu_download_fields(ctx, arrays[0], arrays[1], arrays[2], arrays[3], arrays[4], arrays[5]));
  save_lattice(hp.latticefile, &hp, iter, total_time, comms_time, arrays);
  if (hp.multicanonical && w.mode != SU2GPU_MUCA_READONLY) {
    GPU(su2gpu_muca_get(ctx, &w));
    save_weight(&w);
  }
  su2gpu_destroy(ctx);
  for (int k = 0; k < 6; k++) free(arrays[k]);
  printf("Freed memory allocated for fields.\n");
  printf("\nReached end! Total time taken: %.1lfs, of which %.2lf%% comms. time per iteration: %.6lfs \n", total_time,
         0.0, hp.iterations > 0 ? total_time / hp.iterations : 0.0);
  return 0;
}
