/* pfmd.h -- C ABI of the GB300 (sm_103a) implementation of PFMDS's MD
 * force-and-integration hot path.
 *
 * PFMDS (Fortran 90 + OpenMP) has no plugin or FFI layer: its hot path is the
 * body of md() in code_source/MOLECULAR_DYNAMICS/md_simulation.f90, reached from
 * the run_md_simulation command line.  Each entry point below names the reference
 * subroutine or program it replaces; a Fortran md() calls them through an
 * ISO_C_BINDING interface module (one bind(C) interface per entry point, with
 * the same argument order), a C or C++ host calls them directly, and
 * run_md_simulation (built from this library) is the drop-in executable.
 *
 * Conventions: plain C types only.  Per-atom arrays are xyz-interleaved doubles
 * (3*N), i.e. the Fortran (3,N) column-major layout of particles%positions.
 * Neighbour-list and atom indexes are 0-based.  Every call returns PFMD_OK (0) or
 * one of the PFMD_E_* codes and keeps a message for pfmd_errmsg().  The caller owns
 * every host array; the library copies in and out and keeps no host pointer after
 * a call returns.  The library owns its device buffers and one CUDA stream.  One
 * host thread per context.
 */
#ifndef PFMD_H
#define PFMD_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PFMD_OK 0
#define PFMD_E_NLIST_OVERFLOW 1 /* 'error: too many neighbours' (md_neighbours.f90:80,151) */
#define PFMD_E_OUT_OF_CELL 2    /* 'particle out of cell' (md_general.f90:342-364) */
#define PFMD_E_GR_NN 3          /* graphene nearest neighbours != 3 (graphenenorm.f90:26,30) */
#define PFMD_E_PARAM 4          /* bad settings / parameters ('wrong nhc parameters', ...) */
#define PFMD_E_CUDA 5           /* CUDA runtime error, or the library built without a device */
#define PFMD_E_TIMEOUT 6        /* a bounded device wait gave up */
#define PFMD_E_IO 7             /* unreadable or malformed input file, unwritable output */
#define PFMD_E_STATE 8          /* call not valid in the context's current state */

/* ---- arithmetic forms -------------------------------------------------- */
#define PFMD_FORM_PLAIN 0     /* FP64 throughout, as the reference (-fdefault-real-8) */
#define PFMD_FORM_PRECISION 1 /* FP32 forces with compensated per-atom sums; FP64
                                 positions, velocities, Nose-Hoover chain, energies */

typedef struct pfmd_ctx pfmd_ctx;

typedef struct pfmd_options {
  int form;                  /* PFMD_FORM_* */
  int rand_seed;             /* md()'s rand_seed; run_md_simulation passes 1 */
  int out_period;            /* -op: period of the output-unit block (default 1) */
  int out_fd;                /* output unit as a POSIX file descriptor, -1 = none */
  int all_out_fd;            /* unit for the closing all_out record, -1 = out_fd */
  int write_files;           /* log, snapshot_*.xyz, traj_*.xyz, final_* files */
  const char* output_prefix; /* -p / list prefix, prepended to every output file */
  int num_threads;           /* echoed in 'RUNNING ON n OPENMP THREADS' */
  int device;                /* CUDA device ordinal */
  int use_graphs;            /* capture repeated step segments in CUDA graphs */
  int threads_per_row;       /* force-kernel threads per list row: 1,2,4,...,32, 0 = automatic */
  int async_io;              /* 1: snapshot and trajectory files are formatted and written by a
                                background thread while the next steps run (complete when
                                pfmd_finish / pfmd_md / pfmd_destroy returns); 0: at the event */
  int skin_lists;            /* precision form, 1: at its update step a list is rebuilt only when
                                an atom of its groups moved, since the build plus over the last
                                period, more than half of (r_cut - the interaction's cut-off);
                                0: at every update step, as the reference (the plain form always) */
  int fuse_steps;            /* precision form, nve with one rjl interaction over all atoms, 1: a
                                step's force kernel also runs the next step's first half-kick and
                                drift (the same arithmetic, one launch less per step); 0: separate */
} pfmd_options;

/* Defaults of run_md_simulation.f90:10-24 (out_period 1, seed 1, no prefix),
 * plain form, device 0, graphs on, background file writing on, skin-triggered
 * list rebuilds on (precision form). */
void pfmd_default_options(pfmd_options* opt);

/* ---- set-up and teardown ----------------------------------------------- */

/* md() set-up, md_simulation.f90:44-113: reads the fixed-order settings file
 * input_path+settings_filename, the .xyz file and parameter files it names
 * (read_box_size/read_particles md_read_write.f90:22-61, create_groups and
 * create_interactions md_interactions.f90:38-136, set_nose_hoover_chain
 * md_integrators.f90:182, set_new_temperature md_general.f90:328), echoes what md()
 * echoes to the output unit, and uploads the system to the device.  opt may be
 * NULL (pfmd_default_options).  *ctx is set even on failure, for pfmd_errmsg; the
 * caller destroys it. */
int pfmd_create_from_files(const char* input_path, const char* settings_filename,
                           const pfmd_options* opt, pfmd_ctx** ctx);

/* Releases the device buffers, stream and graphs (md() returning). */
void pfmd_destroy(pfmd_ctx* ctx);

/* Message of the last failing call on ctx (the reference's stop message). */
const char* pfmd_errmsg(const pfmd_ctx* ctx);
/* Name of a status code, e.g. "PFMD_E_NLIST_OVERFLOW". */
const char* pfmd_strerror(int code);

/* ---- the step loop ----------------------------------------------------- */

/* Runs up to max_steps passes of md()'s loop body (md_simulation.f90:116-241:
 * group changes, integrator switches, check_positions, Nose-Hoover chain,
 * velocity-Verlet, neighbour lists, forces, molecular statics, energies, log /
 * output block / snapshot / trajectory) on the device.  Host work happens only at
 * output events.  *finished is set to 1 once the loop has exited (md_step_limit
 * passed, no more integrators, or nvms converged). */
int pfmd_advance(pfmd_ctx* ctx, long long max_steps, int* finished);

/* The lines after the loop, md_simulation.f90:245-272: 'steps number', the
 * PERFOMANCE block, the all_out and final log records and final_<xyz>. */
int pfmd_finish(pfmd_ctx* ctx);

/* Whole md() call (md_simulation.f90:19): create, advance to the end, finish,
 * destroy. */
int pfmd_md(const char* input_path, const char* settings_filename, const pfmd_options* opt);

/* The run_md_simulation program (runners/run_md_simulation.f90:1-77): options
 * -i -p -op -omp_n -ipath -ilist -opath -ofile, plus -form plain|precision. */
int pfmd_run_md_simulation(int argc, const char* const* argv);

/* ---- analysis and fitting programs -------------------------------------------
 * gr_on_cu_analysis (graphene_on_surface_analysis.f90:8-29): arr1 = mean, minimum
 * and maximum z of the atoms of types C, C_a, C_b above height z; arr2 the same for
 * CU, CU_fixed (position_analysis, md_general.f90:400-421).  Host-only. */
int pfmd_gr_on_cu_analysis(const char* xyz_path, double z, double* arr1, double* arr2);
/* The run_gr_analysis program (runners/run_gr_analysis.f90): -path -fl -o -z. */
int pfmd_run_gr_analysis(int argc, const char* const* argv);
/* The run_gr_moire_fitting program (runners/run_gr_moire_fitting.f90 with
 * fit_gr_moire.f90): -fpfn -op -omp_n -delta_error_gold -delta_error_fit, plus
 * -form plain|precision and -device n.  md() runs that do not depend on each
 * other run concurrently on the GPU; files and fit_out.txt are the reference's,
 * except that the original parameter file stays in place (the reference moves
 * it to the first evaluation's numbered name, which is also written). */
int pfmd_run_gr_moire_fitting(int argc, const char* const* argv);

/* ---- state access -------------------------------------------------------- */

int pfmd_natoms(const pfmd_ctx* ctx, int* n);
/* The md_step the loop will run next, and dt%simulation_time. */
int pfmd_md_step(const pfmd_ctx* ctx, long long* md_step, double* simulation_time);

/* particles%positions / velocities / forces (md_general.f90:11-16); any pointer
 * may be NULL.  Arrays are 3*N doubles, xyz per atom.  Page-locked arrays
 * (cudaHostAlloc, cudaHostRegister) are written in place by the device; others
 * through a staging copy.  Returns when the arrays are filled. */
int pfmd_get_state(pfmd_ctx* ctx, double* pos, double* vel, double* frc);
/* Overwrites positions and/or velocities (NULL leaves them); the next step checks
 * the positions as check_positions does and puts every list through its update
 * (a skin-triggered list is rebuilt if the new positions moved too far).
 * Page-locked arrays are read in place by the device.  Returns when the arrays
 * may be reused. */
int pfmd_set_state(pfmd_ctx* ctx, const double* pos, const double* vel);

/* Energies of the last energy step: interactions%energy (one per interaction),
 * potential, kinetic, temperature, Nose-Hoover chain sum, conserved
 * (md_simulation.f90:190-201).  Any pointer may be NULL. */
int pfmd_energies(pfmd_ctx* ctx, double* e_inter, double* pe, double* ke, double* temperature,
                  double* e_nhc, double* e_conserved);

/* update_interactions_neighbour_lists + zero_forces + calculate_forces +
 * calculate_potential_energies (md_interactions.f90:138,210,263; md_integrators.f90:147)
 * outside the step loop, with every list rebuilt (rebuild=1) or only refreshed
 * (rebuild=0).  e_inter may be NULL. */
int pfmd_compute(pfmd_ctx* ctx, int rebuild, double* e_inter);

/* Number of interactions and the shape of list `list` of interaction `inter`
 * (interactions(i)%nl(j), md_interactions.f90:26-34). */
int pfmd_ninteractions(const pfmd_ctx* ctx, int* n);
int pfmd_nlist_shape(const pfmd_ctx* ctx, int inter, int list, int* n_rows, int* nmax);
/* The list arrays as the reference holds them (md_general.f90:34-39): nnum,
 * lessnnum, particle_index and nlist[row*nmax+slot] (group-2 indexes, ascending
 * within a row).  Any pointer may be NULL. */
int pfmd_get_nlist(pfmd_ctx* ctx, int inter, int list, int* nnum, int* lessnnum, int* pidx,
                   int* nlist);
/* Largest neighbour count of every list, in nlists_load order
 * (md_interactions.f90:427-444); maxnnum holds one int per list. */
int pfmd_nlist_load(pfmd_ctx* ctx, int* maxnnum, int* count);
/* Rebuilds so far of every list, in nlists_load order: for a skin-triggered list
 * (pfmd_options.skin_lists) the rebuilds done, -1 for a list rebuilt at every
 * update step.  builds holds one long long per list. */
int pfmd_nlist_builds(pfmd_ctx* ctx, long long* builds, int* count);
/* gr_norm of an ljc / morsec interaction (graphenenorm.f90:38-56), 3 per row. */
int pfmd_get_gr_norm(pfmd_ctx* ctx, int inter, double* norm);

/* change_particle_group_N's effect (md_general.f90:82-95): sets the current size
 * of group `group` (1-based) to n, clamped to the group's capacity. */
int pfmd_set_group_n(pfmd_ctx* ctx, int group, int n);

/* Test hook for the bounded device waits; it has no counterpart in the
 * reference, which stops on errors and never waits on the device.  The waits
 * are the batched kernel's grid barrier and the tensor-core network kernels'
 * mbarrier waits; each gives up after a poll limit and the call then returns
 * PFMD_E_TIMEOUT.  spin_limit != 0 replaces the built-in limits (0 restores
 * them); stall = 1 makes every wait launched from then on impossible (the
 * barrier expects one arrival more than the grid has; the network kernels wait
 * for an mbarrier phase that no MMA completes), so the timeout path runs.
 * Process-wide, read at each launch; batched runs launch directly (no CUDA
 * graph) while it is set.  For tests of the timeout path only. */
int pfmd_debug_waits(unsigned int spin_limit, int stall);

/* The CUDA stream every kernel of ctx is launched on (a cudaStream_t). */
int pfmd_get_stream(pfmd_ctx* ctx, void** stream);
/* Number of kernels the library has launched on ctx so far (graph nodes count
 * once per replay). */
int pfmd_kernel_launches(const pfmd_ctx* ctx, long long* n);

/* ---- measurement ----------------------------------------------------------
 * No reference counterpart (PFMDS times phases with omp_get_wtime,
 * md_simulation.f90:104-202); these support the benchmark. */

/* pfmd_advance with CUDA events recorded on the context's stream right before
 * the first and right after the last kernel of the call; *device_ms is the
 * elapsed device time between them. */
int pfmd_advance_timed(pfmd_ctx* ctx, long long max_steps, int* finished, double* device_ms);

/* Times `reps` back-to-back launches of one kernel group on the context's
 * stream with CUDA events and restores the forces afterwards.  name: "forces"
 * (zero_forces + every interaction's force kernels), "lists" (every list
 * rebuild), or one kernel: "lj", "lj1g", "rjl_density", "rjl_force",
 * "tb_bond", "tb_force", "cos_graphene", "cos_metal" (first interaction of that
 * kind).  *ms = average per launch; *bytes = the kernel's algorithmic HBM bytes
 * per launch (list entries, per-row data and force updates; neighbour positions
 * counted as cache-resident). */
int pfmd_time_kernel(pfmd_ctx* ctx, const char* name, int reps, double* ms, double* bytes);

/* Writes `bytes` bytes of a scratch buffer on the context's stream, evicting the
 * step's working set from L2 between timed runs.  The buffer is allocated on the
 * first call and kept. */
int pfmd_flush_l2(pfmd_ctx* ctx, long long bytes);

/* ---- learned form ----------------------------------------------------------
 * No reference counterpart: a per-atom network potential (32 radial + 16 angular
 * Behler-Parrinello symmetry functions, 48-64-64-1 with SiLU) standing in for the
 * tb and rjl interactions, trained on what the plain kernels compute; the
 * classical kernels remain its fallback and the check on its error. */

/* Trains on frames of this context's own run (plain form only): `frames` times it
 * advances `stride` steps (md()'s loop), takes the per-atom tb and rjl energies and
 * the forces the plain kernels give for the configuration, and takes `iters` Adam
 * steps (learning rate lr) on mean squared per-atom energy error plus
 * force_weight times the mean squared force error (0: energies only).
 * model_in: a model file to continue from, or NULL for new networks
 * (normalisation from the first frame); model_out: file to write (may be NULL).
 * rmse (per interaction, NaN where no network; may be NULL): per-atom energy RMSE
 * (eV) on the last frame; force_rmse (may be NULL): learned against plain force
 * RMSE (eV/A) over all atoms on the last frame. */
int pfmd_learned_train(pfmd_ctx* ctx, const char* model_in, const char* model_out, int frames, int stride,
                       int iters, double lr, double force_weight, int flags, double* rmse, double* force_rmse);
/* flags of pfmd_learned_train / pfmd_learned_gradient / pfmd_learned_use:
 * PFMD_LEARNED_TENSOR_CORES runs the networks (training: forward, tangent, backward
 * and the weight-gradient sums) on the tensor cores, BF16 operands with FP32
 * accumulation; otherwise FP32 on the CUDA cores. */
#define PFMD_LEARNED_TENSOR_CORES 1
/* Floats per network in a gradient (and in a model file's weight block). */
#define PFMD_LEARNED_NET_FLOATS 7361
/* The training-loss gradient of the networks in model_in (NULL: new networks,
 * normalised on this configuration) at the current configuration, with the
 * loss of pfmd_learned_train, and no update: grad receives PFMD_LEARNED_NET_FLOATS
 * floats per network (in interaction order: W1, b1, W2, b2, w3, b3), loss (may be
 * NULL) the sum of squared per-atom energy errors of each network, device_ms (may
 * be NULL) the device time of the gradient kernels. */
int pfmd_learned_gradient(pfmd_ctx* ctx, const char* model_in, double force_weight, int flags, float* grad,
                          double* loss, double* device_ms);
/* Switches the context's tb and rjl interactions to the networks in model_path.
 * Every check_period steps (0: never) the classical kernels recompute the forces
 * of the same configuration; if the RMSE between the two exceeds max_rmse (eV/A)
 * the run falls back to the classical kernels for good.  flags as above. */
int pfmd_learned_use(pfmd_ctx* ctx, const char* model_path, long long check_period, double max_rmse, int flags);
/* RMSE (eV/A) between learned and classical forces at the current positions;
 * leaves the forces of the active form. */
int pfmd_learned_check(pfmd_ctx* ctx, double* rmse);
/* Learned kernels active, checks done, last check's RMSE (-1: none), fell back. */
int pfmd_learned_status(const pfmd_ctx* ctx, int* active, int* checks, double* last_rmse, int* fallen_back);

/* ---- batched form: many independent replicas -----------------------------
 * PFMDS runs independent systems one per MPI rank, each rank calling md() on one
 * entry of a settings list (runners/run_md_simulation_mpi.f90:68-88, the -ilist
 * format: a count, then settings-file / output-prefix pairs).  These entry points
 * load every entry of such a list into one device state and advance all replicas
 * together in one persistent cooperative kernel (precision form).  A replica is a
 * binary LJ gas (lj1g, lj1g, lj) or an rjl slab integrated with nve, or with nvt
 * under one Nose-Hoover chain; all replicas share one list period. */
typedef struct pfmd_batch pfmd_batch;

/* Reads input_path+list_file and every settings file it names (as md() reads
 * them, md_simulation.f90:44-113) and uploads the replicas.  opt may be NULL.
 * *batch is set even on failure, for pfmd_batch_errmsg; destroy it. */
int pfmd_batch_create(const char* input_path, const char* list_file, const pfmd_options* opt,
                      pfmd_batch** batch);
/* The same from the list's entries given directly: n settings files and their
 * output prefixes (the pairs of an -ilist file, run_md_simulation.f90:56-70). */
int pfmd_batch_create_entries(const char* input_path, int n, const char* const* settings,
                              const char* const* prefixes, const pfmd_options* opt, pfmd_batch** batch);
/* Whether the batched kernel takes the settings file (PFMD_OK) or not (the code
 * and, in why, the reason).  On PFMD_OK: its step count, list update period and
 * zero_momentum_period, which every replica of one batch must share.  Host only;
 * run_md_simulation -ilist -batch runs the entries it refuses one by one. */
int pfmd_batch_accepts(const char* input_path, const char* settings, long long* steps, int* list_period,
                       long long* zero_momentum_period, char* why, int why_len);
void pfmd_batch_destroy(pfmd_batch* batch);
const char* pfmd_batch_errmsg(const pfmd_batch* batch);
/* Number of replicas, total atoms, MD steps done. */
int pfmd_batch_info(const pfmd_batch* batch, int* n_replicas, long long* n_atoms, long long* md_step);
/* Replica r (0-based, list order): first atom in the concatenated state, atom
 * count, kind (0 LJ gas, 1 rjl slab). */
int pfmd_batch_replica(const pfmd_batch* batch, int r, int* atom0, int* n, int* kind);
/* Advances every replica by nsteps MD steps (md()'s loop body for nve: kick,
 * drift, lists at the list period, forces, kick; energies at the log period);
 * *device_ms (may be NULL) is the device time of the launches. */
int pfmd_batch_run(pfmd_batch* batch, long long nsteps, double* device_ms);
/* Runs are captured as CUDA graphs (one per run length) and replayed: *n is the
 * number held now, -1 if the driver could not capture the cooperative launch
 * (runs then launch directly). */
int pfmd_batch_graphs(const pfmd_batch* batch, int* n);
/* Autotuner: times `steps` MD steps with threads per list row 1, 2, 4 and 8 for
 * each size bucket (kind x {<2,000, <8,000, larger} atoms) on a saved copy of the
 * state, keeps the fastest and restores the state; only at a list-period boundary.
 * tpa (may be NULL) receives the 6 choices. */
int pfmd_batch_tune(pfmd_batch* batch, int steps, int* tpa);
/* Sets the 6 bucket choices directly (1, 2, 4 or 8). */
int pfmd_batch_set_tpa(pfmd_batch* batch, const int* tpa);
/* Positions, velocities, forces of replica r (3*n doubles each; NULL skips). */
int pfmd_batch_get_state(pfmd_batch* batch, int r, double* pos, double* vel, double* frc);
/* Potential and kinetic energy of every replica at the last energy step. */
int pfmd_batch_energies(pfmd_batch* batch, double* e_pot, double* e_kin);
/* A settings-list run (run_md_simulation -ilist, run_md_simulation.f90:40-66) on
 * the batched kernel: every entry advanced from step 0 to the end of its nve or
 * nvt stage together, and for each entry the files its own run writes, with prefix =
 * out_path + the entry's prefix -- the log (lines at the log period, then the
 * closing record), snapshot_<step>.xyz, traj_<group>.xyz and final_<xyz> -- plus
 * its closing record as one line to all_out_fd when that is >= 0 (list order).
 * Every entry must run the same number of steps (PFMD_E_PARAM otherwise); the
 * batch must be at step 0 (PFMD_E_STATE).  No per-step output block is written. */
int pfmd_batch_run_list(pfmd_batch* b, const char* out_path, int all_out_fd, double* device_ms);

/* Energy history: rows x replicas x 5 (the potential energies of the replica's
 * interactions -- LJ gas: lj1g A-A, lj1g B-B, lj A-B; rjl slab: rjl, 0, 0 --
 * the kinetic energy and the Nose-Hoover chain's energy, 0 under nve), one row
 * per energy step from step 0; *rows and *period (steps between rows) are
 * returned; hist may be NULL to query the size. */
int pfmd_batch_energy_history(pfmd_batch* batch, double* hist, long long* rows, int* period);

/* ---- rjl forces without device allocation ----------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * host codes whose device memory is all reserved up front by their own pool
 * allocator, and loops that cannot take the device-wide synchronisation that
 * cudaMalloc and cudaFree imply.  It allocates nothing; the caller passes every
 * input and output as device memory it owns.
 *
 * Computes the plain (FP64) rjl forces and total energy of n_atoms atoms that
 * all belong to one rjl interaction (rows = atoms 0..n_atoms-1, a full list):
 *   pos     device, n_atoms x 3 doubles (x, y, z of atom i at pos[3i..3i+2]),
 *           each coordinate wrapped into [0, box): the minimum image is the
 *           reference's single shift (md_general.f90:423-441), exact only for
 *           separations within one box length
 *   box     host, the three periodic box lengths
 *   params  host, the parameter file's seven values: A0 xi p q r0 R1 R2
 *   nnum    device, n_atoms ints: entries of each row
 *   nbr     device, n_atoms x max_nbr ints, row i at nbr[i*max_nbr]: 0-based
 *           partner atoms; entries outside 0..n_atoms-1 are skipped, and a row
 *           whose count exceeds max_nbr (the reference stops with 'too many
 *           neighbours') gets NaN forces and a NaN energy, which its partners'
 *           forces then carry too
 *   frc     device, n_atoms x 3 doubles, written (not added to)
 *   energy  device, one double, or NULL to skip the energy
 *   stream  cudaStream_t to launch on (NULL: the default stream); the call
 *           returns once its three kernels are queued
 *   err     optional host buffer of err_len bytes for a message on failure
 * Returns PFMD_OK, PFMD_E_PARAM (sizes or parameters out of range, including
 * n_atoms above 1048576, the capacity of its fixed scratch) or PFMD_E_CUDA.
 *
 * Its scratch (1/Eb per atom, per-block energy partials; about 8 MiB) is a
 * fixed array inside the library, held by every device that loads it until the
 * process exits.  The first call on each device (and again after a device reset
 * or in another CUDA context) looks up that array's device address with that
 * device current; make that first call before any stream capture.  A CUDA error
 * pending from the caller's earlier work is reported (PFMD_E_CUDA) and left
 * pending.  All calls share the one array, so calls whose kernels overlap on
 * the GPU (other streams, other host threads) race: order them on one stream
 * or with events. */
int pfmd_rjl_forces_noalloc(int n_atoms, const double* pos, const double box[3], const double params[7],
                            const int* nnum, const int* nbr, int max_nbr, double* frc, double* energy,
                            void* stream, char* err, int err_len);

#ifdef __cplusplus
}
#endif
#endif /* PFMD_H */
