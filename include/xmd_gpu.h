/*
 * xmd_gpu.h - C ABI of the GB300 engine for XMD's per-step hot path.
 *
 * The reference (vitreusx/xmd) exposes its hot path as C++ "term objects"
 * (public parameter fields, raw array views, operator()() / omp_async())
 * wired together by the driver in src/freeform/main.cpp:208-1077 and
 * configured by the YAML keys of src/freeform/defaults.yml.  This header is
 * the flat, FFI-friendly replacement for that wiring: one context owns the
 * device state of one or more systems ("replicas"), is configured by the same
 * YAML keys and units, and runs the same force terms and integrator.
 *
 * Conventions
 *  - Every function returns XMD_OK (0) or a negative XMD_ERR_* code; the
 *    message of the last failure on the calling thread is returned by
 *    xmd_gpu_last_error().  No C++ exception crosses this boundary (the
 *    reference reports errors only through C++ exceptions, e.g.
 *    include/xmd/store/store.h:152).
 *  - Lengths, energies and times are in the reference's internal units
 *    (include/xmd/utils/units.h:11-62: length 1 = 5 A, energy eps, time tau,
 *    kB = 1).  YAML values carry units and are converted on parsing.
 *  - Arrays of vectors are flat double[3*n] (x0,y0,z0,x1,...).  Caller
 *    arrays are copied; the context owns all device memory.
 *  - Bead indices in topology arrays are 0-based and local to the replica.
 *  - One host thread drives a context at a time (the reference's master
 *    thread, src/freeform/main.cpp:1007-1075); contexts are independent.
 */
#ifndef XMD_GPU_H
#define XMD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XMD_GPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
    XMD_OK = 0,
    XMD_ERR_ARG = -1,       /* invalid argument (null pointer, bad index, ...) */
    XMD_ERR_CONFIG = -2,    /* YAML / unit parse error or unknown key value    */
    XMD_ERR_STATE = -3,     /* call out of order (e.g. step before topology)   */
    XMD_ERR_CUDA = -4,      /* CUDA runtime error or no usable GPU             */
    XMD_ERR_CAPACITY = -5,  /* a fixed-capacity device list overflowed         */
    XMD_ERR_NUMERIC = -6,   /* non-finite force/energy detected on the device  */
    XMD_ERR_BUDGET = -7     /* request does not fit the serving memory budget  */
};

/* ---- force terms (mirrors the kernel<T> opt-in of main.cpp:29-75) ------ */
enum {
    XMD_TERM_TETHER = 0,    /* eval_tether_forces      src/forces/tether.cpp:21-36            */
    XMD_TERM_NAT_ANG = 1,   /* eval_native_angle_forces src/forces/angle/native.cpp:13-39     */
    XMD_TERM_CND = 2,       /* eval_cnd_forces  src/forces/dihedral/complex_native.cpp:13-49  */
    XMD_TERM_SND = 3,       /* eval_snd_forces  src/forces/dihedral/simple_native.cpp:13-45   */
    XMD_TERM_GO = 4,        /* eval_go_forces   src/forces/go.cpp:31-46                        */
    XMD_TERM_PAULI = 5,     /* eval_pauli_exclusion_forces src/forces/pauli.cpp:32-48         */
    XMD_TERM_CONST_ES = 6,  /* eval_const_es_forces src/forces/es/const.cpp:13-32             */
    XMD_TERM_REL_ES = 7,    /* eval_relative_es_forces src/forces/es/relative.cpp:13-32       */
    XMD_TERM_QA = 8,        /* qa::process_contacts src/forces/qa/process_contacts.cpp:13-57  */
    XMD_TERM_CHIR = 9,      /* eval_chiral_forces src/forces/chiral.cpp:15-37                 */
    XMD_TERM_NAT_SS = 10,   /* eval_nat_ssbond_forces src/forces/native_ss.cpp:27-40          */
    XMD_TERM_HEUR_ANG = 11, /* eval_heurestic_angle_forces src/forces/angle/heurestic.cpp:29-59 */
    XMD_TERM_HEUR_DIH = 12, /* eval_heurestic_dihedral_forces src/forces/dihedral/heurestic.cpp:29-70 */
    XMD_TERM_VEL_AFM = 13,  /* eval_velocity_afm_forces src/forces/velocity_afm.cpp (no energy) */
    XMD_TERM_FORCE_AFM = 14,/* eval_force_afm_forces src/forces/force_afm.cpp (no energy)       */
    XMD_TERM_SOLID_WALL = 15,  /* eval_solid_wall_forces src/forces/walls/solid.cpp:12-27      */
    XMD_TERM_LJ_WALL = 16,     /* eval_lj_attr_wall_forces src/forces/walls/lj_attr.cpp:5-43    */
    XMD_TERM_PID = 17,         /* pid::eval_pid_forces src/forces/pid/eval_forces.cpp:14-141      */
    XMD_NUM_TERMS = 18
};

#define XMD_MAX_WALLS 8   /* planes per wall kind */

enum { XMD_PREC_FP64 = 0, XMD_PREC_MIXED = 1 };

#define XMD_NUM_AA 20
#define XMD_NUM_SS (XMD_NUM_AA * XMD_NUM_AA)

/* Resolved numeric parameters, internal units.  Filled from YAML by
 * xmd_gpu_create(); field names follow the reference's params structs
 * (include/xmd/freeform/params.h) and term fields. */
typedef struct xmd_params {
    int32_t on[XMD_NUM_TERMS];          /* `enabled:` of each term section          */
    int32_t langevin_on;                /* langevin: enabled                        */
    int32_t precision;                  /* XMD_PREC_*  (engine key `precision`)     */

    /* general */
    double total_time;                  /* general: total time                      */
    uint64_t seed;                      /* general: seed                            */

    /* langevin / integrator (lang_pc.h:9-10) */
    double gamma_factor, temperature, dt;

    /* neighbor list (legacy_update.h:11); cutoff/skin are additive engine keys:
       <= 0 means "derive as the reference does" */
    double pad_factor, nl_cutoff, nl_skin;

    /* tether forces (tether.h:21-22) */
    double tether_H1, tether_H2, tether_def_length;
    /* native angles / dihedrals */
    double nat_ang_k, cnd_CDA, cnd_CDB, snd_CDH;
    /* native contacts (go.h:13; report_structure.cpp:85) */
    double go_depth, go_active_threshold;
    /* Pauli exclusion (pauli.h:24) */
    double pauli_r_excl, pauli_depth;
    /* const ES / relative ES (es/const.h:10-11, es/relative.h:10-11) */
    double const_es_screen_dist, const_es_permittivity;
    double rel_es_screen_dist, rel_es_factor;
    /* amino acid data: charge, polarization (NONE=0, POLAR=1, HYDROPHOBIC=2),
       contact limits {back, side_all, side_polar, side_hydrophobic} */
    double charge[XMD_NUM_AA];
    int32_t polarization[XMD_NUM_AA];
    int32_t limits[XMD_NUM_AA][4];
    /* quasi-adiabatic potential (process_contacts.h:15-16, sift_candidates.h:14) */
    double qa_phase_duration, qa_breaking_factor;
    double qa_min_cos_hr, qa_min_cos_hh, qa_max_cos_nr;
    /* lj force variants (lj_variants.h:13-14); ss tables indexed 20*aa1+aa2 */
    double lj_bb_r_min, lj_bb_depth, lj_bs_r_min, lj_bs_depth;
    int32_t ss_sinking;
    double ss_depth[XMD_NUM_SS], ss_r_max[XMD_NUM_SS];
    /* engine: initial Verlet row capacity per bead (entries kept by pair
       terms) and whether rows grow when a rebuild needs more (else the
       overflow is reported as XMD_ERR_CAPACITY) */
    int32_t nl_capacity;
    int32_t nl_grow;
    /* engine: CUDA device ordinal the context runs on */
    int32_t device;
    /* engine: Verlet build, XMD_NL_BUILD_* ("nl build: auto | cell | tile");
       both builds keep exactly the same pairs */
    int32_t nl_build;
    /* chirality (chiral.h: e_chi) */
    double chir_e_chi;
    /* native ssbonds (native_ss.h: H1, nat_r = `equilibrium dist`) */
    double nat_ss_H1, nat_ss_dist;
    /* heuristic angles: V(theta) = sum_d a_d theta^d, d = 0..6, per pair
       type 3 t1 + t2 of the angle's first two residues (G = 0, P = 1, other
       = 2); `heurestic angles: coefficients`, angle/heurestic.h:40-41 */
    double heur_ang_coeffs[9][7];
    /* heuristic dihedrals: V(phi) = c0 + c1 sin + c2 cos + c3 sin^2 + c4 cos^2
       + c5 sin cos, per pair type of the dihedral's middle residues;
       `heurestic dihedrals: coefficients`, dihedral/heurestic.h:37-38 */
    double heur_dih_coeffs[9][6];
    /* velocity AFM (velocity_afm.h: afm_force = harmonic(H1, H2, 0)) */
    double vel_afm_H1, vel_afm_H2;
    /* solid walls (walls/solid.h: eps = depth, cutoff) */
    double solid_wall_depth, solid_wall_cutoff;
    /* LJ attractive walls (walls/lj_attr.h: wall_min_dist, breaking_factor,
       cycle_time = phase duration; lj_depth = `depth`, which the shipped
       params never read) */
    double lj_wall_min_dist, lj_wall_breaking_factor, lj_wall_phase_duration, lj_wall_depth;
    /* pseudo-improper dihedral potential (pid/eval_forces.h, lambda.h):
       lambda version 0 = cosine, 1 = algebraic; bb+ / bb- (alpha, psi_0,
       r_min, depth) and ss (alpha, psi_0) */
    int32_t pid_lambda;
    double pid_bbp[4], pid_bbm[4], pid_ss[2];
} xmd_params;

enum { XMD_NL_BUILD_AUTO = 0, XMD_NL_BUILD_CELL = 1, XMD_NL_BUILD_TILE = 2 };

/* xmd_gpu_stats() slots */
enum {
    XMD_STAT_BEADS = 0,          /* beads of all replicas                         */
    XMD_STAT_REPLICAS = 1,
    XMD_STAT_NL_ENTRIES = 2,     /* Verlet entries kept (directed, both beads)     */
    XMD_STAT_GO_ACTIVE = 3,      /* native contacts in the Go list (directed)      */
    XMD_STAT_REBUILDS = 4,       /* list rebuilds summed over replicas             */
    XMD_STAT_LAUNCHES = 5,       /* kernels launched by this context so far        */
    XMD_STAT_QA_CONTACTS = 6,    /* live quasi-adiabatic contacts                  */
    XMD_STAT_MD_STEPS = 7,       /* steps taken                                    */
    XMD_NUM_STATS = 8
};

typedef struct xmd_gpu_ctx xmd_gpu_ctx;

/* ---- library ----------------------------------------------------------- */
int xmd_gpu_abi_version(void);
/* sizeof(xmd_params) as compiled into the library (layout check for FFI). */
int xmd_gpu_params_size(void);
const char *xmd_gpu_last_error(void);
/* Advance a reference generator state (rand_gen.h:22-28) by n draws with the
 * GF(2) jump-ahead the engine uses to give every bead its own stream slice. */
uint64_t xmd_gpu_rng_jump(uint64_t state, uint64_t n_draws);
/* Parse YAML text (merged over the built-in defaults, as main.cpp:97-106 does)
 * into resolved parameters without creating a context or touching the GPU. */
int xmd_gpu_parse_params(const char *yaml_text, xmd_params *out);

/* ---- context lifecycle -------------------------------------------------- */
/* yaml_text: YAML overrides (may be NULL or "" for pure defaults). */
int xmd_gpu_create(const char *yaml_text, xmd_gpu_ctx **out);
int xmd_gpu_create_from_file(const char *yaml_path, xmd_gpu_ctx **out);
int xmd_gpu_destroy(xmd_gpu_ctx *ctx);
int xmd_gpu_get_params(const xmd_gpu_ctx *ctx, xmd_params *out);
/* Replace all parameters (before the first add_replica). */
int xmd_gpu_set_params(xmd_gpu_ctx *ctx, const xmd_params *p);
/* Opt a term in or out (kernel<T> semantics, main.cpp:29-75). */
int xmd_gpu_enable_term(xmd_gpu_ctx *ctx, int term, int on);
int xmd_gpu_set_precision(xmd_gpu_ctx *ctx, int precision);

/* ---- topology and state (per replica) ----------------------------------- */
/* Add one system of n beads.  Beads of a chain must be contiguous and in
 * sequence order (seq_idx = 0,1,2,... within each chain), as the driver lays
 * them out (main.cpp:134-206).  cell = box edge lengths, 0 = open boundary
 * along that axis (box.h:12-22).  temperature <= 0 uses the YAML value.
 * Returns the replica id (>= 0) through *replica_id. */
int xmd_gpu_add_replica(xmd_gpu_ctx *ctx, int32_t n, const int32_t *chain_idx,
                        const int32_t *seq_idx, const uint8_t *atype,
                        const double cell[3], double temperature, uint64_t seed,
                        int32_t *replica_id);
/* Bonded lists; entries must be consecutive beads of one chain
 * (i2 = i1+1, ...), which is how main.cpp:400-479 builds them. */
int xmd_gpu_set_tethers(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                        const int32_t *i2, const double *nat_dist);
int xmd_gpu_set_angles(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                       const int32_t *i2, const int32_t *i3, const double *nat_theta);
int xmd_gpu_set_dihedrals(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                          const int32_t *i2, const int32_t *i3, const int32_t *i4,
                          const double *nat_phi);
/* Chiral quadruplets (chiral_quad{i1..i4, nat_factor, nat_chir},
 * main.cpp:372-398): consecutive beads of one chain; nat_factor = |r23|^-3
 * and nat_chir = r12 . (r23 x r34) * nat_factor of the native structure. */
int xmd_gpu_set_chirals(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                        const int32_t *i2, const int32_t *i3, const int32_t *i4,
                        const double *nat_factor, const double *nat_chir);
/* Heuristic angles heur_ang{i1, i2, i3, type} (angle/heurestic.h:27-31),
 * (k, k+1, k+2) of one chain; the type follows from the residues i1 and i2.
 * A centre has either a native or a heuristic angle. */
int xmd_gpu_set_heuristic_angles(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                                 const int32_t *i2, const int32_t *i3);
/* Heuristic dihedrals heur_dih{i1..i4, type} (dihedral/heurestic.h:27-31),
 * (k, ..., k+3) of one chain; the type follows from the residues i2 and i3. */
int xmd_gpu_set_heuristic_dihedrals(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                                    const int32_t *i2, const int32_t *i3, const int32_t *i4);
/* AFM tips (main.cpp:876-906).  Velocity tips vel_afm_tip{res_idx,
 * afm_orig, afm_vel}: orig[3k..3k+2] (NaN: the bead's position when the
 * replica is placed, as main.cpp:884 takes r[pulled_idx]) and vel[3k..];
 * at most one per bead.  Force tips force_afm_tip{res_idx, pull_force}:
 * F[3k..]; several on one bead add up. */
int xmd_gpu_set_velocity_afm(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *bead,
                             const double *orig, const double *vel);
int xmd_gpu_set_force_afm(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *bead, const double *F);
/* Wall planes plane{origin, normal} of one kind (0 = solid walls, 1 = LJ
 * attractive walls; `planes:` of their YAML sections, main.cpp:815-871),
 * at most XMD_MAX_WALLS each; they act on every replica.  Set before the
 * first replica is placed. */
int xmd_gpu_set_walls(xmd_gpu_ctx *ctx, int32_t kind, int32_t n, const double *origin, const double *normal);
/* Native disulfide bonds (model contacts of type NAT_SS, main.cpp:554-598). */
int xmd_gpu_set_ssbonds(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2);
/* All native contacts (nat_cont{i1,i2,nat_dist}, main.cpp:505-552). */
int xmd_gpu_set_native_contacts(xmd_gpu_ctx *ctx, int32_t rep, int32_t n,
                                const int32_t *i1, const int32_t *i2,
                                const double *nat_dist);
/* Positions r[3n] (and optional velocities v[3n], NULL = 0): y0 = r,
 * y1 = v*dt, y2..y5 = 0, t = 0, as main.cpp:208-253 initialises them. */
int xmd_gpu_set_state(xmd_gpu_ctx *ctx, int32_t rep, const double *r, const double *v);
/* Full predictor-corrector history y[6][3n], time and generator state. */
int xmd_gpu_set_history(xmd_gpu_ctx *ctx, int32_t rep, const double *y, double t,
                        uint64_t rng_state);
int xmd_gpu_get_state(xmd_gpu_ctx *ctx, int32_t rep, double *r, double *v, double *t);
int xmd_gpu_get_history(xmd_gpu_ctx *ctx, int32_t rep, double *y, double *t,
                        uint64_t *rng_state);
/* Snapshot of the replica's whole mutable state (positions, history, time,
 * per-bead generators, Verlet rows, Go/disulfide activity, quasi-adiabatic
 * contacts, free pairs and valences): the store of main.cpp's make_saved
 * items (include/xmd/store/store.h), with the generator, so that a restored
 * run continues bit for bit.  Restore into the same replica slot of a context
 * built the same way (same parameters, systems added in the same order);
 * another layout is XMD_ERR_ARG. */
int xmd_gpu_snapshot_size(xmd_gpu_ctx *ctx, int32_t rep, int64_t *bytes);
int xmd_gpu_snapshot(xmd_gpu_ctx *ctx, int32_t rep, void *buf, int64_t bytes);
int xmd_gpu_restore(xmd_gpu_ctx *ctx, int32_t rep, const void *buf, int64_t bytes);

/* ---- hot path ------------------------------------------------------------ */
/* Forces and per-term energies at the current state of one replica (the
 * force phase of one step, without integration).  The neighbour list is
 * verified and rebuilt first if needed (verify.cpp:4-23).  F[3n], V[XMD_NUM_TERMS]. */
int xmd_gpu_eval_forces(xmd_gpu_ctx *ctx, int32_t rep, double *F, double *V);
/* Advance every replica by nsteps Langevin predictor-corrector steps. */
int xmd_gpu_step(xmd_gpu_ctx *ctx, int32_t nsteps);
/* Observables of one replica (total_energy.cpp:4-11, gyration.cpp:4-19,
 * report_structure.cpp:85): E = V + K, K, Rg, Q (active native fraction). */
int xmd_gpu_observables(xmd_gpu_ctx *ctx, int32_t rep, double *E, double *K,
                        double *Rg, double *Q);
/* Live quasi-adiabatic contacts of one replica in slot order, as
 * report_structure lists them (src/io/report_structure.cpp): out4[4*k] =
 * (i1, i2, contact type, status 0 = forming/formed, 1 = breaking), ref_time[k]
 * (may be NULL).  Returns the number of live contacts through *count (entries
 * beyond cap are not written). */
int xmd_gpu_qa_contacts(xmd_gpu_ctx *ctx, int32_t rep, int32_t cap, int32_t *out4,
                        double *ref_time, int32_t *count);
/* Valence counters sync[n][4] = back, side_all, side_polar, side_hydrophobic
 * (include/xmd/forces/qa/sync_data.h). */
int xmd_gpu_qa_sync(xmd_gpu_ctx *ctx, int32_t rep, int8_t *out);
/* The replica's current Verlet list as kept for the pair terms: pairs (i, j),
 * i < j, in (i, j) order, out2[2*k]; flags[k] bit 0 = Pauli list
 * (update_pauli_pairs, pauli.cpp:9-24), bit 1 = ES list (update_es_base,
 * es_pair.cpp:6-23), bit 2 = PID bundle (update_pid_bundles,
 * pid/bundle.cpp:6-29).  Pairs no pair term keeps are not stored.  The number of
 * pairs is returned through *count (entries beyond cap are not written). */
int xmd_gpu_verlet_pairs(xmd_gpu_ctx *ctx, int32_t rep, int32_t cap, int32_t *out2,
                         uint8_t *flags, int32_t *count);

/* Device-side error word of the last step/eval (0 = none). */
int xmd_gpu_device_status(xmd_gpu_ctx *ctx, int32_t *status);
int xmd_gpu_synchronize(xmd_gpu_ctx *ctx);

/* ---- packed host-buffer path and instrumentation --------------------------- */
/* All replicas at once, beads in replica order (replica r starts after the
 * beads of replicas 0..r-1).  y: [6][3*N] history with y0 = positions (pinned
 * host memory makes the copy asynchronous).  Uploading restarts the skin test
 * from the new positions (the next step verifies and rebuilds as needed). */
int xmd_gpu_upload_history_all(xmd_gpu_ctx *ctx, const double *y);
int xmd_gpu_download_positions_all(xmd_gpu_ctx *ctx, double *r);
/* The whole [6][3*N] history of all replicas (the layout the upload takes):
 * a host-driven loop can carry the state through host memory and upload it
 * back unchanged without altering the trajectory. */
int xmd_gpu_download_history_all(xmd_gpu_ctx *ctx, double *y);
/* The CUDA stream (cudaStream_t) all work of the context is ordered on. */
int xmd_gpu_get_stream(xmd_gpu_ctx *ctx, void **stream);
/* Counters, see XMD_STAT_*; out[XMD_NUM_STATS]. */
int xmd_gpu_stats(xmd_gpu_ctx *ctx, int64_t *out);
/* When on, CUDA events bracket every force and list-rebuild launch; the sums
 * are returned (ms, launches) by xmd_gpu_kernel_times and reset on enabling. */
int xmd_gpu_set_kernel_timing(xmd_gpu_ctx *ctx, int on);

/* ---- launch shapes and the autotuner ------------------------------------------
 * No counterpart in the reference (its OpenMP loop has no launch shape).
 * shape[4] = {beads per step-kernel block (32, 64, 128), resident tile-build
 * blocks per SM (0 = as many as fit), steps per captured graph (8, 16, 32, 64),
 * threads per bead in the step kernel (1, 2, 4)}.
 * Results never depend on the shape.  xmd_gpu_autotune times every candidate
 * on a clone of the context (same replicas, same starting state; the
 * context's own state is untouched), keeps the fastest and returns it with
 * its time per step.  Static contexts only (replicas added, states set). */
int xmd_gpu_autotune(xmd_gpu_ctx *ctx, int32_t steps, int32_t *shape, double *ms_per_step);
int xmd_gpu_set_tuning(xmd_gpu_ctx *ctx, const int32_t *shape);
int xmd_gpu_get_tuning(xmd_gpu_ctx *ctx, int32_t *shape);
int xmd_gpu_kernel_times(xmd_gpu_ctx *ctx, double *force_ms, int64_t *force_launches,
                         double *rebuild_ms, int64_t *rebuild_launches);

/* ---- dynamic membership ----------------------------------------------------- */
/* No counterpart in the reference (its driver simulates one system).  After
 * xmd_gpu_reserve the context holds fixed device capacities; replicas can then
 * be added (placed at the next eval/step, or by xmd_gpu_server admission) and
 * removed between steps, their slots and device ranges reused.  A replica's
 * results do not depend on which other replicas share the context. */
int xmd_gpu_reserve(xmd_gpu_ctx *ctx, int32_t beads, int32_t replicas, int32_t native_entries);
int xmd_gpu_remove_replica(xmd_gpu_ctx *ctx, int32_t rep);
/* per-replica step budget: the replica stops (state kept) after nsteps more
 * steps; -1 = no bound (the default) */
int xmd_gpu_set_steps(xmd_gpu_ctx *ctx, int32_t rep, int64_t nsteps);
/* out[k] = steps left for replica slot k (-1 unbounded, -2 free slot);
 * out holds the reserved replica capacity (or the replica count) */
int xmd_gpu_steps_left(xmd_gpu_ctx *ctx, int64_t *out);

/* ---- serving: continuous batching ------------------------------------------- */
/* No counterpart in the reference.  A server owns one context and a worker
 * thread.  Requests (one independent system each: any number of chains, its
 * own temperature, seed and step count) are admitted first come first served
 * into replica slots while the capacity reserved from `hbm_budget_bytes`
 * (and at most `max_beads` beads) has room; every admitted request advances
 * in the same batched launches, `chunk_steps` steps at a time, and leaves as
 * soon as its steps are done.  Input arrays are copied at submission. */
typedef struct xmd_gpu_server xmd_gpu_server;
typedef struct {
    int32_t n;                                   /* beads */
    const int32_t *chain_idx, *seq_idx;          /* [n] */
    const uint8_t *atype;                        /* [n] amino-acid codes */
    const double *cell;                          /* [3] box (0 = open), NULL = open */
    double temperature;                          /* eps/kB; <= 0: langevin: temperature */
    uint64_t seed;
    int32_t n_tethers;  const int32_t *teth_i1, *teth_i2;  const double *teth_d;
    int32_t n_angles;   const int32_t *ang_i1, *ang_i2, *ang_i3;  const double *ang_theta;
    int32_t n_dihedrals; const int32_t *dih_i1, *dih_i2, *dih_i3, *dih_i4; const double *dih_phi;
    int32_t n_natives;  const int32_t *nat_i1, *nat_i2;  const double *nat_d;
    const double *r, *v;                         /* [3n] initial positions, velocities (NULL = 0) */
    int64_t nsteps;
} xmd_request;
enum { XMD_REQ_QUEUED = 0, XMD_REQ_RUNNING = 1, XMD_REQ_DONE = 2, XMD_REQ_FAILED = -1 };
enum {
    XMD_SRV_P50_S = 0, XMD_SRV_P99_S, XMD_SRV_BEAD_STEPS_PER_S, XMD_SRV_COMPLETED, XMD_SRV_QUEUED,
    XMD_SRV_RUNNING, XMD_SRV_CHUNKS, XMD_SRV_PEAK_RUNNING, XMD_SRV_CAP_BEADS, XMD_SRV_BEAD_STEPS,
    XMD_SRV_SPAN_S, XMD_SRV_FAILED,
    XMD_SRV_DEVICE_BYTES,     /* device memory the serving context holds           */
    XMD_SRV_BUDGET_BYTES,     /* the HBM budget it was created with                */
    XMD_SRV_BYTES_PER_BEAD,   /* measured device cost of one reserved bead slot    */
    XMD_SRV_ADMIT_S,          /* worker time between step chunks (admit, retire)   */
    XMD_SRV_STEP_S,           /* worker time inside step chunks                    */
    XMD_SRV_NUM
};
int xmd_gpu_server_create(const char *yaml_text, int64_t hbm_budget_bytes, int32_t max_beads,
                          int32_t chunk_steps, xmd_gpu_server **out);
int xmd_gpu_server_submit(xmd_gpu_server *srv, const xmd_request *req, int64_t *id);
/* *state = XMD_REQ_* */
int xmd_gpu_server_poll(xmd_gpu_server *srv, int64_t id, int32_t *state);
/* waits for the request, copies its final state ([3n] each, NULL skips) and
 * latency (submission to completion, s), and forgets it */
int xmd_gpu_server_result(xmd_gpu_server *srv, int64_t id, double *r, double *v, double *t, double *latency_s);
int xmd_gpu_server_wait_all(xmd_gpu_server *srv);
/* out[XMD_SRV_NUM]: latency percentiles of completed requests, throughput
 * (bead-steps of completed requests over first submission to last
 * completion), counters */
int xmd_gpu_server_stats(xmd_gpu_server *srv, double *out);
int xmd_gpu_server_destroy(xmd_gpu_server *srv);

/* ---- allocation-free pair search --------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory where they need a pair list: code running while a CUDA graph is
 * captured on its stream, hosts whose device memory belongs to a fixed pool
 * or a framework allocator, loops that cannot take cudaMalloc's implicit
 * device synchronisation.  Every input and output is a device pointer the
 * caller owns; the function calls no cudaMalloc, cudaFree or allocating
 * library routine.  Its scratch is a file-scope __device__ array of about
 * 1.75 MiB that every GPU which loads the library holds until exit, sized for
 * XMD_NOALLOC_MAX_BEADS beads; larger n is rejected with XMD_ERR_CAPACITY.
 *
 * Computes, on `stream` (a cudaStream_t; NULL = legacy default stream), the
 * pairs i < j of the engine's Verlet search: not in the same chain with
 * |seq_i - seq_j| < 3, minimum-image distance below `cutoff`
 * (legacy_update.cpp:24-29 semantics), written as (i, j) into d_pairs[2*k] in
 * (i, j) order, at most `cap` pairs; *d_count receives the number found.
 * When that number exceeds cap, d_pairs holds the first cap pairs of the
 * full (i, j)-ordered list.  d_r = positions [3n], d_chain / d_seq = [n];
 * cell = host array, 0 = open along that axis.  Each bead's row is kept sorted
 * by insertion in one thread, O(m^2) for m partners: meant for Verlet-list
 * densities, slow when most beads lie within the cutoff of most others.
 *
 * The first call on a device looks up the scratch's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  All calls share the scratch and leave their contents in it; each
 * call clears what must start at zero.  Calls that overlap on the GPU (on
 * different streams, or from different threads without ordering) race on the
 * scratch and must be serialised by the caller. */
#define XMD_NOALLOC_MAX_BEADS 65536
int xmd_gpu_verlet_pairs_noalloc(const double *d_r, const int32_t *d_chain, const int32_t *d_seq,
                                 int32_t n, const double cell[3], double cutoff, int32_t *d_pairs,
                                 int32_t cap, int32_t *d_count, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* XMD_GPU_H */
