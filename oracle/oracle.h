/* CPU oracle for the PFMDS MD hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A C++ FP64 restatement of PFMDS's run_md_simulation -> md() step loop (Fortran 90
 * with OpenMP).  It exists to check the CUDA library against, and to time the
 * reference algorithm on the host cores: only the tests, the smoke entry point and
 * the benchmark's CPU-baseline leg load it.  The product library never links it.
 *
 * PARITY UNPINNED: the reference is Fortran, no Fortran compiler is available to
 * build it, and the reference ships no tests, fixtures or example inputs.  The
 * restatement is therefore checked against physics invariants (finite-difference
 * forces, zero force sum, NVE energy conservation, the Nose-Hoover conserved
 * quantity) and hand-derived known answers instead of reference outputs.
 *
 * All entry points return 0 on success or a PFMD_E_* code (values as in
 * include/pfmd.h) and keep the message in orc_errmsg().
 */
#ifndef PFMD_ORACLE_H
#define PFMD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* md() set-up, md_simulation.f90:44-113.  write_files=0 keeps the log, snapshot,
 * trajectory and final files in memory-less mode (nothing written). */
int orc_create(const char* input_path, const char* settings_filename, const char* output_prefix,
               int out_period, int num_threads, int rand_seed, int write_files, orc_sim** out);
/* One pass of the loop body for the next md_step (md_simulation.f90:116-241).
 * *finished is set to 1 when the loop has exited (no more integrators, nvms
 * converged, or md_step_limit passed). */
int orc_step(orc_sim* s, int* finished);
/* Up to nsteps passes of the loop body; stops early when the loop exits. */
int orc_run(orc_sim* s, long long nsteps, int* finished);
/* The lines after the loop (md_simulation.f90:245-272). */
int orc_finish(orc_sim* s);
void orc_destroy(orc_sim* s);

long long orc_md_step(const orc_sim* s); /* the next md_step the loop will run */
int orc_natoms(const orc_sim* s);
void orc_get_state(const orc_sim* s, double* pos, double* vel, double* frc); /* 3N each, xyz */
void orc_set_state(orc_sim* s, const double* pos, const double* vel);
double orc_sim_time(const orc_sim* s);
int orc_ninteractions(const orc_sim* s);
int orc_nl_shape(const orc_sim* s, int inter, int list, int* n_rows, int* nmax);
/* Neighbour-list arrays of interaction `inter`, list `list` (0-based): row-major
 * [row][slot]; nlist holds 0-based group-2 indexes, pidx 0-based atom indexes. */
int orc_get_nl(const orc_sim* s, int inter, int list, int* nnum, int* lessnnum, int* pidx,
               int* nlist, double* moddr);
/* Graphene normals of an ljc/morsec interaction (3 x rows of its third list). */
int orc_get_gr_norm(const orc_sim* s, int inter, double* norm);
/* Last energies computed by the loop: per interaction, potential, kinetic,
 * temperature, Nose-Hoover chain total, conserved. */
int orc_energies(const orc_sim* s, double* e_inter, double* pe, double* ke, double* temp,
                 double* e_nhc, double* e_conserved);
/* Outside the loop: update every neighbour list as at a rebuild step (rebuild=1) or a
 * distance-refresh step (rebuild=0), zero the forces of the all-atoms group,
 * compute all forces and all interaction energies.  Used by gradient tests. */
int orc_eval(orc_sim* s, int rebuild, double* e_inter);
const char* orc_errmsg(const orc_sim* s);
const char* orc_output(const orc_sim* s); /* text written to the output unit so far */

/* Whole run_md_simulation (single settings file or -ilist), run_md_simulation.f90. */
int orc_run_md_simulation(int argc, const char* const* argv);

/* Scalar kernels for known-answer tests. */
double orc_f_cut_cos(double r, double R1, double R2);
double orc_df_cut_cos(double r, double R1, double R2);
double orc_f_cut_poly(double r, double R1, double R2);
void orc_f_dfr_cut(double r, double R1, double R2, double* f, double* dfr);
void orc_find_distance(const double* v1, const double* v2, const double* box, double* dr,
                       double* dr2);

#ifdef __cplusplus
}
#endif
#endif
