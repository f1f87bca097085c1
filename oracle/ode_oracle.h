/*
 * ode_oracle.h -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of ODE 0.12's contact generation + dWorldQuickStep path,
 * in the precision chosen by ORACLE_REAL (double by default). Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * Every function cites the reference file:line whose behaviour it restates.
 */
#ifndef ODE_ORACLE_H
#define ODE_ORACLE_H
#include "odegpu_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_BODY_REC 13     /* pos[3] q[4] lvel[3] avel[3]               */
#define ORACLE_CONTACT_REC 9   /* pos[3] normal[3] depth gi gj              */

/* Same contract as ref_run_world in oracle/ref_harness.cpp. */
int oracle_run_world(const odegpuScene* sc, int w, int n_steps, double* state,
                     int* ncontacts, double* contacts, int max_rec, double* feedback,
                     unsigned int* seed_out);

/* dCollide(heightfield H placed at H->pos / H->R, geom of class t2 with
 * parameters p2 at pos2 / R2 (row-major 3x3)); out: [n][9] pos, normal,
 * depth, 0, 0. Returns the contact count. */
int oracle_collide_hf(const odegpuHeightfield* H, int t2, const double* p2, const double* pos2,
                      const double* R2, int flags, double* out);

/* World w built from the scene, then every body's state replaced by
 * init_state ([nb][13], quaternion used as given), stepped n_steps times;
 * final_state receives [nb][13]. For finite differences of the step with
 * respect to the state it starts from. */
int oracle_run_world_from(const odegpuScene* sc, int w, int n_steps, const double* init_state,
                          double* final_state);

/* Run worlds [w_begin, w_end) for n_steps on n_threads host threads; writes the
 * final state [nb_total_in_range][13]. Returns total contacts created. */
long long oracle_run_worlds(const odegpuScene* sc, int w_begin, int w_end, int n_steps,
                            int n_threads, double* final_state);

/* Worlds [w_begin, w_end), each built from the scene with its body state
 * replaced by state_in (the range's bodies, [nb][13]; NULL: the scene's
 * initial state) and its dRand seed by seed_in[w - w_begin] (NULL: the
 * scene's), stepped n_steps times as steps step0, step0 + 1, ... (the step
 * index selects the per-step controls), on n_threads host threads.
 * state_out receives the final states, seed_out the seeds after the last
 * step, counts [w][n_steps][3] each step's contacts, constraint rows and
 * islands with rows (any output may be NULL). Returns 0 or -1. */
int oracle_step_worlds_from(const odegpuScene* sc, int w_begin, int w_end, int step0, int n_steps,
                            int n_threads, const double* state_in, const unsigned int* seed_in,
                            double* state_out, unsigned int* seed_out, int* counts);

/* One step (step index `step`) of world w from state_in ([nb][13]; NULL: the
 * scene's initial state) with dRand seed `seed`; contacts receives up to
 * max_rec records [9] (pos, normal, depth, geom i, geom k) in creation order,
 * state_out (may be NULL) the state after the step. Returns the contact
 * count or -1. */
int oracle_step_world_contacts(const odegpuScene* sc, int w, int step, const double* state_in,
                               unsigned int seed, double* contacts, int max_rec, double* state_out);

/* Stage taps for per-kernel parity. For world w, run `pre_steps` full steps,
 * then for the next step record, in ODE's island/row order:
 *   n_islands, island_rows[i] (rows per island), island_bodies[i],
 *   rows: J[m][12] (as passed to SOR_LCP, unscaled), rhs[m], cfm[m] (already
 *         divided by h), lo[m], hi[m], findex[m] (island-local row index or -1),
 *         jb[m][2] (island-local body index or -1), body_of[island_body] ->
 *         world-local body index,
 *   lambda[m] and cforce[nb][6] returned by SOR_LCP,
 *   seed_before (dRand seed entering the step).
 * Arrays must hold cap_rows / cap_bodies entries. Returns total rows or -1. */
typedef struct oracleTap {
  int n_islands;
  int* island_rows;     /* [cap_islands] */
  int* island_bodies;   /* [cap_islands] */
  int cap_islands;
  double* J; double* rhs; double* cfm; double* lo; double* hi;
  int* findex; int* jb; int cap_rows;
  int* body_of; int cap_bodies;
  double* lambda; double* cforce;
  int* joint_of_row;    /* [cap_rows] joint ordinal in creation order: persistent
                           joints 0..nj-1 then contacts nj.. in creation order */
  unsigned int seed_before;
} oracleTap;
int oracle_tap_step(const odegpuScene* sc, int w, int pre_steps, oracleTap* tap);

/* Solve one island with the oracle's SOR_LCP (ode/src/quickstep.cpp:342-584)
 * on given inputs: J is modified in place as the reference does. */
void oracle_sor_lcp(int m, int nb, double* J, const int* jb, const double* invMass,
                    const double* invI /*[nb][12] world frame*/, double* lambda,
                    double* fc, double* b, const double* lo, const double* hi,
                    const double* cfm, const int* findex, int iterations, double sor_w,
                    unsigned int* seed);

/* One dCollide call on standalone geoms (same contract as ref_collide). */
int oracle_collide(int t1, const double* p1, const double* pos1, const double* R1, int t2,
                   const double* p2, const double* pos2, const double* R2, int flags,
                   double* out);

/* RNG (ode/src/misc.cpp:33-117). */
/* 1: worlds step with dWorldStep (ode/src/step.cpp + lcp.cpp) instead of
 * dWorldQuickStep; process-wide. */
void oracle_set_stepper(int exact);
/* LCP solves that stopped early on a non-positive step (s <= 0) so far. */
int oracle_lcp_errors(void);
void oracle_rand_set_seed(unsigned int s);
unsigned int oracle_rand_get_seed(void);
int oracle_rand_int(int n);
int oracle_test_rand(void);

#ifdef __cplusplus
}
#endif
#endif
