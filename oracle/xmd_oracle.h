/*
 * xmd_oracle.h - CPU restatement of XMD's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU engine is compared
 * against (and the timed CPU baseline); the engine never links or calls it.
 * Each function cites the reference file:line it restates.  The restatement
 * is itself pinned against the reference's own kernel translation units,
 * compiled from the reference tree by oracle/ref/build_ref.sh.
 */
#ifndef XMD_ORACLE_H
#define XMD_ORACLE_H
#include <stdint.h>
#include "../include/xmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xo_sys xo_sys;

xo_sys *xo_create(const xmd_params *p, int32_t n, const int32_t *chain_idx,
                  const int32_t *seq_idx, const uint8_t *atype, const double cell[3],
                  double temperature, uint64_t seed);
void xo_destroy(xo_sys *s);
int xo_set_tethers(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                   const double *nat_dist);
int xo_set_angles(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                  const int32_t *i3, const double *nat_theta);
int xo_set_dihedrals(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                     const int32_t *i3, const int32_t *i4, const double *nat_phi);
int xo_set_chirals(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                   const int32_t *i4, const double *nat_factor, const double *nat_chir);
int xo_set_ssbonds(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2);
int xo_set_velocity_afm(xo_sys *s, int32_t n, const int32_t *bead, const double *orig, const double *vel);
int xo_set_force_afm(xo_sys *s, int32_t n, const int32_t *bead, const double *F);
int xo_eval_at(xo_sys *s, const double *r, double *F, double *V);
int xo_set_walls(xo_sys *s, int32_t kind, int32_t n, const double *origin, const double *normal);
int xo_set_heuristic_angles(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3);
int xo_set_heuristic_dihedrals(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                               const int32_t *i4);
int xo_set_native_contacts(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                           const double *nat_dist);
int xo_set_state(xo_sys *s, const double *r, const double *v);
int xo_set_history(xo_sys *s, const double *y, double t, uint64_t rng_state);
int xo_get_state(const xo_sys *s, double *r, double *v, double *t);
int xo_get_history(const xo_sys *s, double *y, double *t, uint64_t *rng_state);

int xo_eval_forces(xo_sys *s, double *F, double *V);
int xo_step(xo_sys *s, int32_t nsteps);
/* Same step, driven with the reference's OpenMP structure (per-thread F/V
 * buffers, omp for per term, atomic reduce, master integrates and rebuilds;
 * main.cpp:909-1077).  nthreads <= 0 uses omp_get_max_threads(). */
int xo_step_omp(xo_sys *s, int32_t nsteps, int32_t nthreads);
int xo_observables(xo_sys *s, double *E, double *K, double *Rg, double *Q);

/* Introspection for tests. counts[0..7] = go, pauli, es, free pairs (live),
 * free-pair slots, contacts (live), contact slots, nl rebuilds. */
int xo_counts(const xo_sys *s, int64_t *counts);
/* Live QA contacts in slot order: (i1, i2, type, status) and ref_time. */
int xo_qa_contacts(const xo_sys *s, int32_t cap, int32_t *out4, double *ref_time);
/* Live free pairs in slot order (i1, i2). */
int xo_free_pairs(const xo_sys *s, int32_t cap, int32_t *out2);
/* Non-native neighbour-list pairs of the last rebuild in list order. */
int xo_nl_pairs(const xo_sys *s, int64_t cap, int32_t *out2);
/* Per-bead valence counters sync[n][4]. */
int xo_sync(const xo_sys *s, int8_t *out);
/* Cutoff bookkeeping: max_cutoff, pad, req_r (legacy_update.cpp:7-8). */
int xo_cutoffs(const xo_sys *s, double *out3);
/* Reference generator helpers (rand_gen.h:22-58). */
uint64_t xo_rng_next(uint64_t *state);
double xo_rng_normal(uint64_t *state);

#ifdef __cplusplus
}
#endif
#endif
