/*
 * nlm_oracle.h -- CPU ORACLE for the peridynamics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++/OpenMP restatement of the
 * reference NLMech algorithms (cited file:line in nlm_oracle.cpp).  It is the
 * checker the CUDA library is compared against and the CPU baseline that
 * bench.py times.  Nothing in the product library (nlmech_gb300/, libnlmgpu)
 * may link, load or call it.
 *
 * The description structs are the ones of include/nlmgpu.h so that a test
 * feeds both sides the same inputs.
 */
#ifndef NLM_ORACLE_H
#define NLM_ORACLE_H

#include <stdint.h>

#include "../include/nlmgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

const char *orc_last_error(void);
int orc_num_threads(void);
void orc_set_num_threads(int n);

/* util::compare (compare.cpp:25-33) exposed for tests. */
int orc_definitely_less_than(double a, double b);
int orc_definitely_greater_than(double a, double b);

/* geometry::Neighbor brute force (neighbor.cpp:69-89).  counts[i] = row
 * length; call with cols == NULL first, then with rowptr filled. */
int orc_neighbors_brute(int64_t n, const double *x, double horizon,
                        int64_t *rowptr, int32_t *cols);
/* Same predicate with a cell list (identical sets, ascending rows). */
int orc_neighbors_grid(int dim, int64_t n, const double *x, double horizon,
                       int64_t *rowptr, int32_t *cols);

/* RNPBond material parameters (rnpBond.cpp:23-189): out = {C, beta, rbar,
 * invFactor, influence moment M, nu, lambda}. */
int orc_rnp_params(const nlm_material *m, int dim, double horizon,
                   double *out7);

/* ---- explicit model --------------------------------------------------- */
typedef struct orc_fd orc_fd;
int orc_fd_create(const nlm_fd_desc *d, int use_grid_neighbors, orc_fd **out);
int orc_fd_destroy(orc_fd *h);
int orc_fd_num_bonds(const orc_fd *h, int64_t *nnz);
int orc_fd_get_neighbors(const orc_fd *h, int64_t *rowptr, int32_t *cols);
int orc_fd_run(orc_fd *h, int64_t nsteps);
int orc_fd_get_state(const orc_fd *h, double *u, double *v, double *f);
int orc_fd_set_state(orc_fd *h, const double *u, const double *v);
int orc_fd_get_time(const orc_fd *h, double *t, int64_t *n);
int orc_fd_get_bond_state(const orc_fd *h, uint8_t *broken);
int orc_fd_set_bond_state(orc_fd *h, const uint8_t *broken);
int orc_fd_damage(orc_fd *h, float *phi, float *Z);
/* Energies of computePostProcFields (RNPBond): strain, work done, kinetic,
 * fracture, per node, and their sums. */
int orc_fd_energies(orc_fd *h, float *strain, float *work, float *kinetic, float *fracture,
                    double *totals);
/* Reaction force of FDModel::computeForce (2-D RNPBond). */
int orc_fd_reaction_force(orc_fd *h, double *R, double *total, double *sum);
/* Fixity bits per node as set by ULoading (uLoading.cpp:99-102). */
int orc_fd_get_fixity(const orc_fd *h, uint8_t *fix);
/* ElasticState helpers (volumeCorrection.cpp:25-67,
 * stateBasedHelperFunctions.cpp:26-83): omega per bond, m per node and the
 * dilatation of the current state. */
int orc_fd_es_fields(orc_fd *h, double *omega, double *m, double *theta);
/* One internal force evaluation at the current u without advancing time
 * and without updating bond state: f_int only (3n). */
int orc_fd_eval_force(orc_fd *h, double *f);

/* ---- quasi-static model (QuasiStaticModel.cpp) -------------------------- */
typedef struct orc_qs_params {
  int jacobian;      /* 0: reference FD, component-diagonal (QuasiStatic-
                        Model.cpp:361-454); 1: full FD blocks (dense)      */
  int solver;        /* 0: CG, 1: BiCGSTAB                                 */
  int max_iters;     /* Newton iterations (Solver.Max_Iteration)           */
  double tol;        /* Solver.Tolerance                                   */
  int tol_relative;  /* 0: absolute ||r|| (reference), 1: ||r||/||r0||     */
  double perturbation; /* Solver.Perturbation, eps = perturbation * h     */
  int lin_max_iters; /* linear solver iteration cap                        */
  double lin_tol;    /* linear solver relative tolerance                   */
  double dt;         /* load-step "time" increment                         */
} orc_qs_params;

typedef struct orc_qs orc_qs;
/* Material must be ElasticState (the reference's only QS instantiation,
 * QuasiStaticModel.cpp:648). */
int orc_qs_create(const nlm_fd_desc *d, const orc_qs_params *p, orc_qs **out);
int orc_qs_destroy(orc_qs *h);
/* Solve load steps; iters[k] = Newton iterations of step k (may be NULL). */
int orc_qs_solve(orc_qs *h, int nsteps, int *iters, double *final_res);
/* u: 3n displacement; fout: 3n force (f_int * V_i as written to "Force",
 * model/util.cpp:49-59) after the final computeForces(true). */
int orc_qs_get(const orc_qs *h, double *u, double *fout, int64_t *nnz);

/* ---- quasi-static RNPBond (build definition; see nlm_oracle.cpp) ------- */
typedef struct orc_qsr orc_qsr;
typedef struct orc_qsr_stats {
  int newton_iters, lin_iters, break_rounds, used_guess;
  int64_t broken;
  double res_plain, res_start, res_final;
} orc_qsr_stats;
int orc_qsr_create(const nlm_fd_desc *d, int max_newton, double tol, int lin_max_iters,
                   double lin_tol, int break_bonds, int max_break_rounds, orc_qsr **out);
int orc_qsr_destroy(orc_qsr *h);
int orc_qsr_load_step(orc_qsr *h, const double *guess, orc_qsr_stats *st);
int orc_qsr_get_state(const orc_qsr *h, double *u);
int orc_qsr_get_bond_state(const orc_qsr *h, uint8_t *broken);

#ifdef __cplusplus
}
#endif

#endif
