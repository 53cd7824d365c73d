/*
 * xmd_oracle.c - CPU restatement of XMD's per-step hot path (TEST ORACLE).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine and the timed CPU
 * baseline.  Nothing in the engine links, loads or calls this file.
 *
 * Every routine restates one reference function and cites it (paths relative
 * to the reference project's xmd/ directory).  Arithmetic follows the
 * reference's operation order so that the FP64 results agree with the
 * reference's own translation units (compiled with real = double by
 * oracle/ref/build_ref.sh) to rounding.
 *
 * Where the reference's list plumbing is broken (it does not compile or never
 * fills its lists) the INTENDED semantics are restated; each such deviation
 * is tagged [Dn] and listed in the project's design notes:
 *   [D1] the Verlet list fills (gentypes push_back never grows, vector.h:331)
 *   [D2] the native-contact merge advances (legacy_update.cpp:33-55 spins)
 *   [D3] non-native pairs go to the non-native list (legacy_update.cpp:57-59)
 *        and "particle_pairs" (pauli.cpp:15, es_pair.cpp:11, free_pair.cpp:12)
 *        means that list
 *   [D4] QA valence counters start at the residue limits (main.cpp:662-672
 *        appends after n zeros)
 *   [D5] QA free pairs use max_formation_min_dist = max req_min_dist
 *        (main.cpp:742-746; never assigned) and skip pairs already in contact
 *   [D6] QA contact potentials are looked up as ljs[type-1]: contact_type got
 *        a NONE=0 entry (contact_type.h:10) but lj_variants::operator[]
 *        (lj_variants.h:16-23) still counts from BB=0
 *   [D7] process_contacts runs every step after process_candidates, in the
 *        order of eval_qa_forces::operator() (qa.cpp:20-31)
 *   [D8] lang_pc_step gets dt and the particle count (main.cpp:209-253 never
 *        sets them)
 */
#include "xmd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(double s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
/* norm_squared, norm, norm_inv, dot, cross, unit: include/xmd/types/vec3.h:133-158,349-360 */
static inline double nsq(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double nrm(v3 a) { return sqrt(nsq(a)); }
static inline double ninv(v3 a) { return 1.0 / nrm(a); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 unit(v3 a) { return scl(ninv(a), a); }
/* clamp: include/xmd/utils/math.h:77-80 (NaN maps to max_value) */
static inline double clampd(double v, double lo, double hi) {
    return v < lo ? lo : (v < hi ? v : hi);
}
/* acos with argument clamped to [-1, 1]: math.h:41-45 */
static inline double acos_c(double x) {
    double x_ = x < -1.0 ? -1.0 : (x > 1.0 ? 1.0 : x);
    return acos(x_);
}
static inline double ipow6(double s) { return s * (s * (s * (s * (s * s)))); }

/* ---- generator: include/xmd/random/rand_gen.h:22-58 ---------------------- */
uint64_t xo_rng_next(uint64_t *state) {
    uint64_t res = *state * 0xd989bcacc137dcd5ull;
    *state ^= *state >> 11;
    *state ^= *state << 31;
    *state ^= *state >> 18;
    return res;
}
static inline double rng_uniform(uint64_t *st) {
    double inv = 1.0 / (double)(1ull << 32);
    uint64_t val = xo_rng_next(st);
    return (double)(val >> 32) * inv;
}
static inline void rng_normal_x2(uint64_t *st, double *a, double *b) {
    double r1 = rng_uniform(st), r2 = rng_uniform(st);
    double r = sqrt(-2.0 * log(r1));
    if (isnan(r)) r = 0.0;
    double t = (2.0 * M_PI) * r2;
    *a = r * cos(t);
    *b = r * sin(t);
}
double xo_rng_normal(uint64_t *st) {
    double r1 = rng_uniform(st), r2 = rng_uniform(st);
    double r = sqrt(-2.0 * log(r1));
    if (isnan(r)) r = 0.0;
    double t = (2.0 * M_PI) * r2;
    return r * cos(t);
}

/* ---- system ---------------------------------------------------------------- */
typedef struct { int32_t i1, i2; double d; } pair_d;
typedef struct { int32_t i1, i2; } pair_i;
typedef struct { int32_t i1, i2, free_idx, type; int8_t d1[4], d2[4]; } qa_cand;
typedef struct {
    int32_t i1, i2, type, status, vacant;
    double ref_time;
    int8_t d1[4], d2[4];
} qa_cont;
typedef struct { int32_t i1, i2, vacant; } qa_free;

enum { FORMING_OR_FORMED = 0, BREAKING = 1 };   /* contact.h:7-9 */

struct xo_sys {
    xmd_params p;
    int32_t n;
    int32_t *chain, *seq, *prev, *next;
    uint8_t *atype;
    double cell[3], cell_inv[3];
    double temperature;
    /* bonded lists */
    int32_t n_teth; int32_t *teth_i; double *teth_d;
    int32_t n_ang; int32_t *ang_i; double *ang_t;
    int32_t n_dih; int32_t *dih_i; double *dih_p;
    int32_t n_nat; pair_d *nat;
    int32_t n_chir; int32_t *chir_i; double *chir_f, *chir_n;   /* chiral_quad (chiral.h) */
    int32_t n_ss_all; pair_i *ss_all;                           /* native ssbonds (nat_ss) */
    pair_i *ss; int32_t n_ss;                                   /* update_nat_ssbonds' list */
    int32_t n_hang; int32_t *hang_i; int8_t *hang_t;            /* heur_ang (angle/heurestic.h) */
    int32_t n_hdih; int32_t *hdih_i; int8_t *hdih_t;            /* heur_dih (dihedral/heurestic.h) */
    int32_t n_vafm; int32_t *vafm_i; double *vafm_o, *vafm_v;   /* vel_afm_tip (velocity_afm.h) */
    int32_t n_fafm; int32_t *fafm_i; double *fafm_F;            /* force_afm_tip (force_afm.h) */
    int32_t n_wall[2]; double wall[2][XMD_MAX_WALLS][6];       /* planes (origin, normal): solid, LJ attractive */
    int8_t *ljw_status; double *ljw_joint, *ljw_ref;           /* lj_attr_pair per (wall, bead) */
    double pid_cut;                                            /* update_pid_bundles::cutoff */
    pair_i *pid; int64_t n_pid, cap_pid;                       /* pid_bundle{i1, i2} (type from atype) */
    /* state */
    double *r, *v, *y[6], *F;
    double t, true_t;
    uint64_t rng;
    /* derived constants */
    double max_cutoff, pad_req, req_r, max_form;
    double const_es_Vf, const_es_sdi, rel_es_Vf, rel_es_sdi;
    double qa_factor, qa_cycle_inv;
    double req_min_dist[4 + XMD_NUM_SS];
    /* neighbour-list state (nl/data.h:8-14) */
    int first_time, invalid;
    double orig_pad, orig_cell[3];
    double *orig_r;
    pair_i *nl; int64_t n_nl, cap_nl;
    int64_t n_rebuilds;
    /* term lists */
    pair_d *go; int32_t n_go;
    pair_i *pauli; int64_t n_pauli, cap_pauli;
    pair_d *es; int64_t n_es, cap_es;
    /* QA state */
    qa_free *fp; int64_t n_fp, cap_fp;
    qa_cand *cand; int64_t n_cand, cap_cand;
    qa_cont *cont; int64_t n_cont, cap_cont;
    int8_t *sync;               /* [n][4]: back, side_all, side_polar, side_hydrophobic */
    double *qn, *qh;            /* [n][3] */
    double V[XMD_NUM_TERMS];
};

static inline v3 ld(const double *a, int i) { return mk(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
static inline void st3(double *a, int i, v3 v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
static inline void acc(double *a, int i, v3 v) { a[3 * i] += v.x; a[3 * i + 1] += v.y; a[3 * i + 2] += v.z; }
static inline void dec(double *a, int i, v3 v) { a[3 * i] -= v.x; a[3 * i + 1] -= v.y; a[3 * i + 2] -= v.z; }

/* box::wrap / box::r_uv: include/xmd/model/box.h:36-49 */
static inline v3 r_uv(const xo_sys *s, v3 u, v3 w) {
    v3 d = sub(w, u);
    d.x -= s->cell[0] * nearbyint(d.x * s->cell_inv[0]);
    d.y -= s->cell[1] * nearbyint(d.y * s->cell_inv[1]);
    d.z -= s->cell[2] * nearbyint(d.z * s->cell_inv[2]);
    return d;
}

#define GROW(ptr, cnt, cap, T)                                                     \
    do {                                                                           \
        if ((cnt) >= (cap)) {                                                      \
            (cap) = (cap) ? 2 * (cap) : 1024;                                      \
            (ptr) = (T *)realloc((ptr), sizeof(T) * (size_t)(cap));                \
        }                                                                          \
    } while (0)

static void derive_cutoffs(xo_sys *s) {
    const xmd_params *p = &s->p;
    /* max_cutoff accumulation: main.cpp:500, 545-551, 628-630, 642-644, 742-746 */
    double mc = 0.0;
    if (p->on[XMD_TERM_PAULI]) mc = fmax(mc, p->pauli_r_excl);
    if (p->on[XMD_TERM_NAT_SS]) mc = fmax(mc, 2.0 * p->nat_ss_dist);   /* harmonic::cutoff, main.cpp:596-597 */
    if (p->on[XMD_TERM_GO]) {
        double c = 0.0;
        for (int k = 0; k < s->n_nat; ++k) c = fmax(c, 2.0 * s->nat[k].d); /* lj::cutoff lj.cpp:8-10 */
        mc = fmax(mc, c);
    }
    if (p->on[XMD_TERM_CONST_ES]) mc = fmax(mc, 2.0 * p->const_es_screen_dist);
    if (p->on[XMD_TERM_REL_ES]) mc = fmax(mc, 2.0 * p->rel_es_screen_dist);
    /* req_min_dist: main.cpp:681-697 */
    memset(s->req_min_dist, 0, sizeof s->req_min_dist);
    s->req_min_dist[1] = p->lj_bb_r_min;
    s->req_min_dist[2] = p->lj_bs_r_min;
    s->req_min_dist[3] = p->lj_bs_r_min;
    for (int a1 = 0; a1 < XMD_NUM_AA; ++a1)
        for (int a2 = 0; a2 < XMD_NUM_AA; ++a2)
            s->req_min_dist[4 + a1 + XMD_NUM_AA * a2] = p->ss_r_max[a1 * XMD_NUM_AA + a2];
    double mf = 0.0;
    for (int t = 0; t < 4 + XMD_NUM_SS; ++t) mf = fmax(mf, s->req_min_dist[t]);
    s->max_form = mf;                                              /* [D5] */
    if (p->on[XMD_TERM_QA]) mc = fmax(mc, mf);
    /* PID: the largest LJ-variant cutoff (lj::cutoff = 2 r_min, sink_lj::cutoff
       = 2 r_max), main.cpp:801-810 */
    {
        double c = fmax(2.0 * p->lj_bb_r_min, 2.0 * p->lj_bs_r_min);
        for (int k = 0; k < XMD_NUM_SS; ++k) c = fmax(c, 2.0 * p->ss_r_max[k]);
        s->pid_cut = c;
        if (p->on[XMD_TERM_PID]) mc = fmax(mc, c);
    }
    if (p->nl_cutoff > 0.0) mc = p->nl_cutoff;
    s->max_cutoff = mc;
    /* legacy_update.cpp:7-8 */
    s->pad_req = p->nl_skin > 0.0 ? p->nl_skin : p->pad_factor * mc;
    s->req_r = mc + s->pad_req;
    /* main.cpp:619-645 */
    s->const_es_Vf = 1.0 / (4.0 * M_PI * p->const_es_permittivity);
    s->const_es_sdi = 1.0 / p->const_es_screen_dist;
    s->rel_es_Vf = 1.0 / (4.0 * M_PI * p->rel_es_factor);
    s->rel_es_sdi = 1.0 / p->rel_es_screen_dist;
    /* main.cpp:719-723: factor = breaking_factor * (real)pow(2.0f, -1.0f/6.0f) */
    s->qa_factor = p->qa_breaking_factor * (double)powf(2.0f, -1.0f / 6.0f);
    s->qa_cycle_inv = 1.0 / p->qa_phase_duration;
}

xo_sys *xo_create(const xmd_params *p, int32_t n, const int32_t *chain_idx,
                  const int32_t *seq_idx, const uint8_t *atype, const double cell[3],
                  double temperature, uint64_t seed) {
    if (!p || n <= 0 || !chain_idx || !seq_idx || !atype) return NULL;
    xo_sys *s = (xo_sys *)calloc(1, sizeof(xo_sys));
    s->p = *p;
    s->n = n;
    s->chain = (int32_t *)malloc(sizeof(int32_t) * n);
    s->seq = (int32_t *)malloc(sizeof(int32_t) * n);
    s->prev = (int32_t *)malloc(sizeof(int32_t) * n);
    s->next = (int32_t *)malloc(sizeof(int32_t) * n);
    s->atype = (uint8_t *)malloc(n);
    memcpy(s->chain, chain_idx, sizeof(int32_t) * n);
    memcpy(s->seq, seq_idx, sizeof(int32_t) * n);
    memcpy(s->atype, atype, n);
    /* prev/next: main.cpp:163-185 (consecutive beads of one chain) */
    for (int i = 0; i < n; ++i) {
        s->prev[i] = (i > 0 && chain_idx[i - 1] == chain_idx[i] && seq_idx[i - 1] == seq_idx[i] - 1) ? i - 1 : -1;
        s->next[i] = (i + 1 < n && chain_idx[i + 1] == chain_idx[i] && seq_idx[i + 1] == seq_idx[i] + 1) ? i + 1 : -1;
    }
    for (int a = 0; a < 3; ++a) {
        s->cell[a] = cell ? cell[a] : 0.0;
        s->cell_inv[a] = s->cell[a] != 0.0 ? 1.0 / s->cell[a] : 0.0;   /* box.h:12-22 */
        s->orig_cell[a] = s->cell[a];
    }
    s->temperature = temperature > 0.0 ? temperature : p->temperature;
    s->rng = seed;
    s->r = (double *)calloc(3 * (size_t)n, sizeof(double));
    s->v = (double *)calloc(3 * (size_t)n, sizeof(double));
    s->F = (double *)calloc(3 * (size_t)n, sizeof(double));
    for (int k = 0; k < 6; ++k) s->y[k] = (double *)calloc(3 * (size_t)n, sizeof(double));
    s->orig_r = (double *)calloc(3 * (size_t)n, sizeof(double));
    s->qn = (double *)calloc(3 * (size_t)n, sizeof(double));
    s->qh = (double *)calloc(3 * (size_t)n, sizeof(double));
    s->sync = (int8_t *)calloc(4 * (size_t)n, 1);
    for (int i = 0; i < n; ++i)                                         /* [D4] */
        for (int k = 0; k < 4; ++k) s->sync[4 * i + k] = (int8_t)p->limits[atype[i]][k];
    s->first_time = 1;
    s->invalid = 1;
    derive_cutoffs(s);
    return s;
}

void xo_destroy(xo_sys *s) {
    if (!s) return;
    free(s->chain); free(s->seq); free(s->prev); free(s->next); free(s->atype);
    free(s->teth_i); free(s->teth_d); free(s->ang_i); free(s->ang_t);
    free(s->dih_i); free(s->dih_p); free(s->nat);
    free(s->chir_i); free(s->chir_f); free(s->chir_n); free(s->ss_all); free(s->ss);
    free(s->hang_i); free(s->hang_t); free(s->hdih_i); free(s->hdih_t);
    free(s->vafm_i); free(s->vafm_o); free(s->vafm_v); free(s->fafm_i); free(s->fafm_F);
    free(s->ljw_status); free(s->ljw_joint); free(s->ljw_ref);
    free(s->pid);
    free(s->r); free(s->v); free(s->F);
    for (int k = 0; k < 6; ++k) free(s->y[k]);
    free(s->orig_r); free(s->nl); free(s->go); free(s->pauli); free(s->es);
    free(s->fp); free(s->cand); free(s->cont); free(s->sync); free(s->qn); free(s->qh);
    free(s);
}

int xo_set_tethers(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                   const double *nat_dist) {
    free(s->teth_i); free(s->teth_d);
    s->n_teth = n;
    s->teth_i = (int32_t *)malloc(sizeof(int32_t) * 2 * (n ? n : 1));
    s->teth_d = (double *)malloc(sizeof(double) * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->teth_i[2 * k] = i1[k]; s->teth_i[2 * k + 1] = i2[k];
        /* tether.length.value_or(def_length): main.cpp:409-413 */
        s->teth_d[k] = (nat_dist && nat_dist[k] > 0.0) ? nat_dist[k] : s->p.tether_def_length;
    }
    return 0;
}
int xo_set_angles(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                  const int32_t *i3, const double *th) {
    free(s->ang_i); free(s->ang_t);
    s->n_ang = n;
    s->ang_i = (int32_t *)malloc(sizeof(int32_t) * 3 * (n ? n : 1));
    s->ang_t = (double *)malloc(sizeof(double) * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->ang_i[3 * k] = i1[k]; s->ang_i[3 * k + 1] = i2[k]; s->ang_i[3 * k + 2] = i3[k];
        s->ang_t[k] = th[k];
    }
    return 0;
}
int xo_set_dihedrals(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                     const int32_t *i3, const int32_t *i4, const double *ph) {
    free(s->dih_i); free(s->dih_p);
    s->n_dih = n;
    s->dih_i = (int32_t *)malloc(sizeof(int32_t) * 4 * (n ? n : 1));
    s->dih_p = (double *)malloc(sizeof(double) * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->dih_i[4 * k] = i1[k]; s->dih_i[4 * k + 1] = i2[k];
        s->dih_i[4 * k + 2] = i3[k]; s->dih_i[4 * k + 3] = i4[k];
        s->dih_p[k] = ph[k];
    }
    return 0;
}
static int cmp_pair_d(const void *a, const void *b) {
    const pair_d *x = (const pair_d *)a, *y = (const pair_d *)b;
    if (x->i1 != y->i1) return x->i1 < y->i1 ? -1 : 1;
    if (x->i2 != y->i2) return x->i2 < y->i2 ? -1 : 1;
    return 0;
}
int xo_set_native_contacts(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2,
                           const double *nat_dist) {
    free(s->nat);
    s->n_nat = n;
    s->nat = (pair_d *)malloc(sizeof(pair_d) * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        int a = i1[k], b = i2[k];
        s->nat[k].i1 = a < b ? a : b;
        s->nat[k].i2 = a < b ? b : a;
        s->nat[k].d = nat_dist[k];
    }
    /* the merge of legacy_update.cpp:33-43 needs the list sorted (nl/pair.h:19-25) */
    qsort(s->nat, n, sizeof(pair_d), cmp_pair_d);
    derive_cutoffs(s);
    s->first_time = 1;
    return 0;
}

/* chiral quads (main.cpp:372-398): parameters from the native structure */
int xo_set_chirals(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                   const int32_t *i4, const double *nat_factor, const double *nat_chir) {
    free(s->chir_i); free(s->chir_f); free(s->chir_n);
    s->n_chir = n;
    s->chir_i = (int32_t *)malloc(sizeof(int32_t) * 4 * (n ? n : 1));
    s->chir_f = (double *)malloc(sizeof(double) * (n ? n : 1));
    s->chir_n = (double *)malloc(sizeof(double) * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->chir_i[4 * k] = i1[k]; s->chir_i[4 * k + 1] = i2[k];
        s->chir_i[4 * k + 2] = i3[k]; s->chir_i[4 * k + 3] = i4[k];
        s->chir_f[k] = nat_factor[k];
        s->chir_n[k] = nat_chir[k];
    }
    return 0;
}
/* heur_ang_type / heur_dih_type: GLY = 0, PRO = 1, others = 2 and
   type = 3 t1 + t2 (angle/heurestic.cpp:9-15, dihedral/heurestic.cpp:8-14) */
static int8_t heur_type(uint8_t a, uint8_t b) {
    int ca = a == 7 ? 0 : (a == 14 ? 1 : 2), cb = b == 7 ? 0 : (b == 14 ? 1 : 2);
    return (int8_t)(3 * ca + cb);
}
/* heuristic angles: type of (i1, i2) */
int xo_set_heuristic_angles(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3) {
    free(s->hang_i); free(s->hang_t);
    s->n_hang = n;
    s->hang_i = (int32_t *)malloc(sizeof(int32_t) * 3 * (n ? n : 1));
    s->hang_t = (int8_t *)malloc(n ? n : 1);
    for (int k = 0; k < n; ++k) {
        s->hang_i[3 * k] = i1[k]; s->hang_i[3 * k + 1] = i2[k]; s->hang_i[3 * k + 2] = i3[k];
        s->hang_t[k] = heur_type(s->atype[i1[k]], s->atype[i2[k]]);
    }
    return 0;
}
/* heuristic dihedrals: type of (i2, i3) */
int xo_set_heuristic_dihedrals(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                               const int32_t *i4) {
    free(s->hdih_i); free(s->hdih_t);
    s->n_hdih = n;
    s->hdih_i = (int32_t *)malloc(sizeof(int32_t) * 4 * (n ? n : 1));
    s->hdih_t = (int8_t *)malloc(n ? n : 1);
    for (int k = 0; k < n; ++k) {
        s->hdih_i[4 * k] = i1[k]; s->hdih_i[4 * k + 1] = i2[k];
        s->hdih_i[4 * k + 2] = i3[k]; s->hdih_i[4 * k + 3] = i4[k];
        s->hdih_t[k] = heur_type(s->atype[i2[k]], s->atype[i3[k]]);
    }
    return 0;
}
/* AFM tips (main.cpp:876-906): origins given explicitly */
int xo_set_velocity_afm(xo_sys *s, int32_t n, const int32_t *bead, const double *orig, const double *vel) {
    free(s->vafm_i); free(s->vafm_o); free(s->vafm_v);
    s->n_vafm = n;
    s->vafm_i = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    s->vafm_o = (double *)malloc(sizeof(double) * 3 * (n ? n : 1));
    s->vafm_v = (double *)malloc(sizeof(double) * 3 * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->vafm_i[k] = bead[k];
        for (int a = 0; a < 3; ++a) { s->vafm_o[3 * k + a] = orig[3 * k + a]; s->vafm_v[3 * k + a] = vel[3 * k + a]; }
    }
    return 0;
}
int xo_set_force_afm(xo_sys *s, int32_t n, const int32_t *bead, const double *F) {
    free(s->fafm_i); free(s->fafm_F);
    s->n_fafm = n;
    s->fafm_i = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    s->fafm_F = (double *)malloc(sizeof(double) * 3 * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->fafm_i[k] = bead[k];
        for (int a = 0; a < 3; ++a) s->fafm_F[3 * k + a] = F[3 * k + a];
    }
    return 0;
}
/* wall planes (main.cpp:815-871); the LJ attractive pairs start free */
int xo_set_walls(xo_sys *s, int32_t kind, int32_t n, const double *origin, const double *normal) {
    if (kind < 0 || kind > 1 || n < 0 || n > XMD_MAX_WALLS) return -1;
    s->n_wall[kind] = n;
    for (int k = 0; k < n; ++k)
        for (int a = 0; a < 3; ++a) { s->wall[kind][k][a] = origin[3 * k + a]; s->wall[kind][k][3 + a] = normal[3 * k + a]; }
    if (kind == 1) {
        free(s->ljw_status); free(s->ljw_joint); free(s->ljw_ref);
        size_t m = (size_t)(n ? n : 1) * (size_t)s->n;
        s->ljw_status = (int8_t *)calloc(m, 1);
        s->ljw_joint = (double *)calloc(3 * m, sizeof(double));
        s->ljw_ref = (double *)calloc(m, sizeof(double));
    }
    return 0;
}
static int cmp_pair_i0(const void *a, const void *b) {
    const pair_i *x = (const pair_i *)a, *y = (const pair_i *)b;
    if (x->i1 != y->i1) return x->i1 < y->i1 ? -1 : 1;
    if (x->i2 != y->i2) return x->i2 < y->i2 ? -1 : 1;
    return 0;
}
/* native disulfides (model contacts of type NAT_SS, main.cpp:554-598) */
int xo_set_ssbonds(xo_sys *s, int32_t n, const int32_t *i1, const int32_t *i2) {
    free(s->ss_all);
    s->n_ss_all = n;
    s->ss_all = (pair_i *)malloc(sizeof(pair_i) * (n ? n : 1));
    for (int k = 0; k < n; ++k) {
        s->ss_all[k].i1 = i1[k] < i2[k] ? i1[k] : i2[k];
        s->ss_all[k].i2 = i1[k] < i2[k] ? i2[k] : i1[k];
    }
    qsort(s->ss_all, n, sizeof(pair_i), cmp_pair_i0);
    s->first_time = 1;
    return 0;
}

int xo_set_state(xo_sys *s, const double *r, const double *v) {
    size_t nb = sizeof(double) * 3 * (size_t)s->n;
    memcpy(s->r, r, nb);
    if (v) memcpy(s->v, v, nb); else memset(s->v, 0, nb);
    /* y0 = r, y1 = v*dt, y2..5 = 0: main.cpp:229-248 (v starts at 0 there) */
    memcpy(s->y[0], r, nb);
    for (size_t k = 0; k < 3 * (size_t)s->n; ++k) s->y[1][k] = s->v[k] * s->p.dt;
    for (int k = 2; k < 6; ++k) memset(s->y[k], 0, nb);
    s->t = s->true_t = 0.0;
    s->first_time = 1;
    return 0;
}
int xo_set_history(xo_sys *s, const double *y, double t, uint64_t rng_state) {
    size_t n3 = 3 * (size_t)s->n;
    for (int k = 0; k < 6; ++k) memcpy(s->y[k], y + k * n3, sizeof(double) * n3);
    memcpy(s->r, s->y[0], sizeof(double) * n3);
    for (size_t k = 0; k < n3; ++k) s->v[k] = s->y[1][k] * (1.0 / s->p.dt);
    s->t = s->true_t = t;
    s->rng = rng_state;
    s->first_time = 1;
    return 0;
}
int xo_get_state(const xo_sys *s, double *r, double *v, double *t) {
    size_t nb = sizeof(double) * 3 * (size_t)s->n;
    if (r) memcpy(r, s->r, nb);
    if (v) memcpy(v, s->v, nb);
    if (t) *t = s->t;
    return 0;
}
int xo_get_history(const xo_sys *s, double *y, double *t, uint64_t *rng_state) {
    size_t n3 = 3 * (size_t)s->n;
    if (y) for (int k = 0; k < 6; ++k) memcpy(y + k * n3, s->y[k], sizeof(double) * n3);
    if (t) *t = s->t;
    if (rng_state) *rng_state = s->rng;
    return 0;
}

/* ---- neighbour list --------------------------------------------------------- */

/* nl::verify::operator(): src/nl/verify.cpp:4-23 */
static void nl_verify(xo_sys *s) {
    if (s->first_time) {
        s->first_time = 0;
        s->invalid = 1;
        return;
    }
    double max_r_disp = 0.0;
    for (int i = 0; i < s->n; ++i) {
        v3 dr = r_uv(s, ld(s->r, i), ld(s->orig_r, i));
        max_r_disp = fmax(max_r_disp, nrm(dr));
    }
    double box_disp = fabs(s->cell[0] - s->orig_cell[0]) + fabs(s->cell[1] - s->orig_cell[1]) +
                      fabs(s->cell[2] - s->orig_cell[2]);
    double total_disp = 2.0 * max_r_disp + box_disp;
    if (total_disp > s->orig_pad) s->invalid = 1;
}

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Candidate partners j > i of bead i within adjacent cells (a pure
 * acceleration of the all-pairs scan of legacy_update.cpp:16-27: every pair
 * closer than req_r lies in adjacent cells; the exact distance test below
 * decides). */
typedef struct {
    int dims[3], per[3];
    double lo[3], cs[3];
    int *head, *cnt, *items;
    int ncell;
} cgrid;

static void grid_build(const xo_sys *s, cgrid *g) {
    double rr = s->req_r;
    long total = 1;
    for (int a = 0; a < 3; ++a) {
        g->per[a] = s->cell[a] != 0.0;
        if (g->per[a]) {
            int d = (int)floor(s->cell[a] / rr);
            g->dims[a] = d < 1 ? 1 : d;
            g->lo[a] = 0.0;
            g->cs[a] = s->cell[a] / g->dims[a];
        } else {
            double mn = 1e300, mx = -1e300;
            for (int i = 0; i < s->n; ++i) {
                double x = s->r[3 * i + a];
                mn = fmin(mn, x); mx = fmax(mx, x);
            }
            double ext = mx - mn;
            int d = (int)floor(ext / rr);
            if (d < 1) d = 1;
            if (d > 256) d = 256;
            g->dims[a] = d;
            g->lo[a] = mn;
            g->cs[a] = fmax(ext / d, rr);
        }
        total *= g->dims[a];
    }
    g->ncell = (int)total;
    g->head = (int *)calloc(total + 1, sizeof(int));
    g->cnt = (int *)calloc(total, sizeof(int));
    g->items = (int *)malloc(sizeof(int) * s->n);
    int *cid = (int *)malloc(sizeof(int) * s->n);
    for (int i = 0; i < s->n; ++i) {
        int c[3];
        for (int a = 0; a < 3; ++a) {
            double x = s->r[3 * i + a];
            int k;
            if (g->per[a]) {
                double f = x / s->cell[a];
                f -= floor(f);
                k = (int)(f * g->dims[a]);
            } else {
                k = (int)floor((x - g->lo[a]) / g->cs[a]);
            }
            if (k < 0) k = 0;
            if (k >= g->dims[a]) k = g->dims[a] - 1;
            c[a] = k;
        }
        cid[i] = (c[2] * g->dims[1] + c[1]) * g->dims[0] + c[0];
        g->cnt[cid[i]]++;
    }
    for (int c = 0; c < g->ncell; ++c) g->head[c + 1] = g->head[c] + g->cnt[c];
    memset(g->cnt, 0, sizeof(int) * g->ncell);
    for (int i = 0; i < s->n; ++i) g->items[g->head[cid[i]] + g->cnt[cid[i]]++] = i;
    free(cid);
}

static int grid_partners(const xo_sys *s, const cgrid *g, int i, int *out) {
    int c[3];
    for (int a = 0; a < 3; ++a) {
        double x = s->r[3 * i + a];
        int k;
        if (g->per[a]) {
            double f = x / s->cell[a];
            f -= floor(f);
            k = (int)(f * g->dims[a]);
        } else {
            k = (int)floor((x - g->lo[a]) / g->cs[a]);
        }
        if (k < 0) k = 0;
        if (k >= g->dims[a]) k = g->dims[a] - 1;
        c[a] = k;
    }
    int offs[3][3], noff[3];
    for (int a = 0; a < 3; ++a) {
        noff[a] = 0;
        for (int d = -1; d <= 1; ++d) {
            int k = c[a] + d;
            if (g->per[a]) k = ((k % g->dims[a]) + g->dims[a]) % g->dims[a];
            else if (k < 0 || k >= g->dims[a]) continue;
            int dup = 0;
            for (int q = 0; q < noff[a]; ++q) dup |= offs[a][q] == k;
            if (!dup) offs[a][noff[a]++] = k;
        }
    }
    int m = 0;
    for (int az = 0; az < noff[2]; ++az)
        for (int ay = 0; ay < noff[1]; ++ay)
            for (int ax = 0; ax < noff[0]; ++ax) {
                int cc = (offs[2][az] * g->dims[1] + offs[1][ay]) * g->dims[0] + offs[0][ax];
                for (int q = g->head[cc]; q < g->head[cc + 1]; ++q) {
                    int j = g->items[q];
                    if (j > i) out[m++] = j;
                }
            }
    qsort(out, m, sizeof(int), cmp_int);
    return m;
}

static int contact_exists(const xo_sys *s, const pair_i *live, int64_t nlive, int i1, int i2) {
    int64_t lo = 0, hi = nlive - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) / 2;
        if (live[mid].i1 == i1 && live[mid].i2 == i2) return 1;
        if (live[mid].i1 < i1 || (live[mid].i1 == i1 && live[mid].i2 < i2)) lo = mid + 1;
        else hi = mid - 1;
    }
    (void)s;
    return 0;
}
static int cmp_pair_i(const void *a, const void *b) {
    const pair_i *x = (const pair_i *)a, *y = (const pair_i *)b;
    if (x->i1 != y->i1) return x->i1 < y->i1 ? -1 : 1;
    if (x->i2 != y->i2) return x->i2 < y->i2 ? -1 : 1;
    return 0;
}

/* nl::legacy_update::operator(): src/nl/legacy_update.cpp:6-70 [D1-D3],
 * followed by the list builders of the enabled terms:
 * update_pauli_pairs pauli.cpp:9-24, update_go_contacts go.cpp:8-23,
 * update_es_base es_pair.cpp:6-23, update_free_pairs free_pair.cpp:6-21. */
static void nl_rebuild(xo_sys *s) {
    const xmd_params *p = &s->p;
    double pad = s->pad_req;
    double req_r = s->req_r;
    s->n_nl = 0;
    cgrid g;
    grid_build(s, &g);
    int *part = (int *)malloc(sizeof(int) * s->n);
    int64_t nat_idx = 0, ss_idx = 0;
    for (int i1 = 0; i1 < s->n; ++i1) {
        v3 r1 = ld(s->r, i1);
        int chain1 = s->chain[i1], seq1 = s->seq[i1];
        int m = grid_partners(s, &g, i1, part);
        for (int q = 0; q < m; ++q) {
            int i2 = part[q];
            int chain2 = s->chain[i2], seq2 = s->seq[i2];
            int diff = seq1 > seq2 ? seq1 - seq2 : seq2 - seq1;
            if (chain1 == chain2 && diff < 3) continue;
            double orig_dist = nrm(r_uv(s, r1, ld(s->r, i2)));
            if (orig_dist < req_r) {
                int non_native = 1;
                /* sorted merge against the native list [D2] */
                /* the native list takes part only with native contacts
                   enabled (main.cpp:504-530 wires all_nat_cont there) */
                while (p->on[XMD_TERM_GO] && nat_idx < s->n_nat &&
                       (s->nat[nat_idx].i1 < i1 || (s->nat[nat_idx].i1 == i1 && s->nat[nat_idx].i2 < i2)))
                    ++nat_idx;
                if (p->on[XMD_TERM_GO] && nat_idx < s->n_nat && s->nat[nat_idx].i1 == i1 && s->nat[nat_idx].i2 == i2)
                    non_native = 0;
                /* the same merge against the native disulfides, which take
                   part with that term enabled (main.cpp:579-580) */
                while (p->on[XMD_TERM_NAT_SS] && ss_idx < s->n_ss_all &&
                       (s->ss_all[ss_idx].i1 < i1 || (s->ss_all[ss_idx].i1 == i1 && s->ss_all[ss_idx].i2 < i2)))
                    ++ss_idx;
                if (p->on[XMD_TERM_NAT_SS] && ss_idx < s->n_ss_all && s->ss_all[ss_idx].i1 == i1 &&
                    s->ss_all[ss_idx].i2 == i2)
                    non_native = 0;
                if (non_native) {                                       /* [D3] */
                    GROW(s->nl, s->n_nl, s->cap_nl, pair_i);
                    s->nl[s->n_nl].i1 = i1;
                    s->nl[s->n_nl].i2 = i2;
                    s->n_nl++;
                }
            }
        }
    }
    free(part);
    free(g.head); free(g.cnt); free(g.items);
    s->orig_pad = pad;
    memcpy(s->orig_r, s->r, sizeof(double) * 3 * (size_t)s->n);
    memcpy(s->orig_cell, s->cell, sizeof s->cell);
    s->invalid = 0;
    s->n_rebuilds++;

    /* update_pauli_pairs: pauli.cpp:9-24 */
    s->n_pauli = 0;
    if (p->on[XMD_TERM_PAULI]) {
        double min_norm_inv = 1.0 / (p->pauli_r_excl + s->orig_pad);
        for (int64_t k = 0; k < s->n_nl; ++k) {
            int i1 = s->nl[k].i1, i2 = s->nl[k].i2;
            if (ninv(r_uv(s, ld(s->r, i1), ld(s->r, i2))) > min_norm_inv) {
                GROW(s->pauli, s->n_pauli, s->cap_pauli, pair_i);
                s->pauli[s->n_pauli].i1 = i1;
                s->pauli[s->n_pauli].i2 = i2;
                s->n_pauli++;
            }
        }
    }
    /* update_pid_bundles: pid/bundle.cpp:6-27 (beads with both chain
       neighbours, r < cutoff + pad at the rebuild) */
    s->n_pid = 0;
    if (p->on[XMD_TERM_PID]) {
        double min_norm_inv = 1.0 / (s->pid_cut + s->orig_pad);
        for (int64_t k = 0; k < s->n_nl; ++k) {
            int i1 = s->nl[k].i1, i2 = s->nl[k].i2;
            if (ninv(r_uv(s, ld(s->r, i1), ld(s->r, i2))) > min_norm_inv) {
                if (s->prev[i1] < 0 || s->next[i1] < 0 || s->prev[i2] < 0 || s->next[i2] < 0) continue;
                GROW(s->pid, s->n_pid, s->cap_pid, pair_i);
                s->pid[s->n_pid].i1 = i1;
                s->pid[s->n_pid].i2 = i2;
                s->n_pid++;
            }
        }
    }
    /* update_nat_ssbonds: native_ss.cpp:8-19, cutoff = harmonic::cutoff(nat_r)
       = 2 nat_r [D14] */
    free(s->ss);
    s->ss = (pair_i *)malloc(sizeof(pair_i) * (s->n_ss_all ? s->n_ss_all : 1));
    s->n_ss = 0;
    if (p->on[XMD_TERM_NAT_SS]) {
        for (int k = 0; k < s->n_ss_all; ++k)
            if (nrm(r_uv(s, ld(s->r, s->ss_all[k].i1), ld(s->r, s->ss_all[k].i2))) < 2.0 * p->nat_ss_dist + s->orig_pad)
                s->ss[s->n_ss++] = s->ss_all[k];
    }
    /* update_go_contacts: go.cpp:8-23 */
    free(s->go);
    s->go = (pair_d *)malloc(sizeof(pair_d) * (s->n_nat ? s->n_nat : 1));
    s->n_go = 0;
    if (p->on[XMD_TERM_GO]) {
        for (int k = 0; k < s->n_nat; ++k) {
            double cutoff = 2.0 * s->nat[k].d;
            if (nrm(r_uv(s, ld(s->r, s->nat[k].i1), ld(s->r, s->nat[k].i2))) < cutoff + s->orig_pad)
                s->go[s->n_go++] = s->nat[k];
        }
    }
    /* update_es_base: es_pair.cpp:6-23 (the const-ES builder when both are on, main.cpp:611-613) */
    s->n_es = 0;
    if (p->on[XMD_TERM_CONST_ES] || p->on[XMD_TERM_REL_ES]) {
        double cutoff = p->on[XMD_TERM_CONST_ES] ? 2.0 * p->const_es_screen_dist
                                                 : 2.0 * p->rel_es_screen_dist;
        double min_norm_inv = 1.0 / (cutoff + s->orig_pad);
        for (int64_t k = 0; k < s->n_nl; ++k) {
            int i1 = s->nl[k].i1, i2 = s->nl[k].i2;
            if (ninv(r_uv(s, ld(s->r, i1), ld(s->r, i2))) > min_norm_inv) {
                double q1_x_q2 = p->charge[s->atype[i1]] * p->charge[s->atype[i2]];
                if (q1_x_q2 != 0.0) {
                    GROW(s->es, s->n_es, s->cap_es, pair_d);
                    s->es[s->n_es].i1 = i1;
                    s->es[s->n_es].i2 = i2;
                    s->es[s->n_es].d = q1_x_q2;
                    s->n_es++;
                }
            }
        }
    }
    /* update_free_pairs: free_pair.cpp:6-21 [D5] */
    s->n_fp = 0;
    if (p->on[XMD_TERM_QA]) {
        int64_t nlive = 0;
        pair_i *live = (pair_i *)malloc(sizeof(pair_i) * (s->n_cont ? s->n_cont : 1));
        for (int64_t k = 0; k < s->n_cont; ++k)
            if (!s->cont[k].vacant) {
                live[nlive].i1 = s->cont[k].i1;
                live[nlive].i2 = s->cont[k].i2;
                nlive++;
            }
        qsort(live, nlive, sizeof(pair_i), cmp_pair_i);
        double min_norm_inv = 1.0 / (s->max_form + s->orig_pad);
        for (int64_t k = 0; k < s->n_nl; ++k) {
            int i1 = s->nl[k].i1, i2 = s->nl[k].i2;
            if (ninv(r_uv(s, ld(s->r, i1), ld(s->r, i2))) > min_norm_inv) {
                if (contact_exists(s, live, nlive, i1, i2)) continue;
                GROW(s->fp, s->n_fp, s->cap_fp, qa_free);
                s->fp[s->n_fp].i1 = i1;
                s->fp[s->n_fp].i2 = i2;
                s->fp[s->n_fp].vacant = 0;
                s->n_fp++;
            }
        }
        free(live);
    }
}

static void ensure_nl(xo_sys *s) {
    nl_verify(s);
    if (s->invalid) nl_rebuild(s);
}

/* ---- force terms ------------------------------------------------------------ */

/* eval_tether_forces::iter: src/forces/tether.cpp:21-36; harmonic.h:18-25 */
static void tether_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->teth_i[2 * idx], i2 = s->teth_i[2 * idx + 1];
    double nat_dist = s->teth_d[idx];
    v3 r12 = sub(ld(s->r, i2), ld(s->r, i1));
    double r12_n = nrm(r12);
    double dr = r12_n - nat_dist, dr2 = dr * dr;
    double V_ = 0.5 * dr2 * (s->p.tether_H1 + s->p.tether_H2 * dr2);
    double dV_dr = dr * (s->p.tether_H1 + 2.0 * s->p.tether_H2 * dr2);
    V_ = clampd(V_, -1.0e3, 1.0e3);
    dV_dr = clampd(dV_dr, -1.0e3, 1.0e3);
    v3 r12_u = mk(r12.x / r12_n, r12.y / r12_n, r12.z / r12_n);
    *V += V_;
    acc(F, i1, scl(dV_dr, r12_u));
    dec(F, i2, scl(dV_dr, r12_u));
}

/* eval_native_angle_forces::iter: src/forces/angle/native.cpp:13-39 */
static void angle_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->ang_i[3 * idx], i2 = s->ang_i[3 * idx + 1], i3 = s->ang_i[3 * idx + 2];
    double nat_theta = s->ang_t[idx];
    v3 r1 = ld(s->r, i1), r2 = ld(s->r, i2), r3 = ld(s->r, i3);
    v3 r12 = sub(r2, r1), r23 = sub(r3, r2);
    v3 x12_23 = cross(r12, r23);
    double r12_rn = ninv(r12), r23_rn = ninv(r23);
    v3 d1 = scl(r12_rn, unit(cross(r12, x12_23)));
    v3 d3 = scl(r23_rn, unit(cross(r23, x12_23)));
    v3 d2 = sub(neg(d1), d3);
    double cos_theta = -dot(r12, r23) * r12_rn * r23_rn;
    double theta = acos_c(cos_theta);
    double dtheta = theta - nat_theta;
    *V += 0.5 * s->p.nat_ang_k * dtheta * dtheta;
    double dV = s->p.nat_ang_k * dtheta;
    dec(F, i1, scl(dV, d1));
    dec(F, i2, scl(dV, d2));
    dec(F, i3, scl(dV, d3));
}

/* shared dihedral geometry of complex_native.cpp:19-43 / simple_native.cpp:17-37 */
static double dih_geom(const xo_sys *s, int idx, double nat_phi, v3 *d1, v3 *d2, v3 *d3, v3 *d4) {
    int i1 = s->dih_i[4 * idx], i2 = s->dih_i[4 * idx + 1], i3 = s->dih_i[4 * idx + 2],
        i4 = s->dih_i[4 * idx + 3];
    v3 r1 = ld(s->r, i1), r2 = ld(s->r, i2), r3 = ld(s->r, i3), r4 = ld(s->r, i4);
    v3 r12 = sub(r2, r1), r23 = sub(r3, r2), r34 = sub(r4, r3);
    v3 x12_23 = cross(r12, r23), x23_34 = cross(r23, r34);
    double x12_23_rn = ninv(x12_23), x23_34_rn = ninv(x23_34);
    v3 x12_23_u = scl(x12_23_rn, x12_23), x23_34_u = scl(x23_34_rn, x23_34);
    double cos_phi = dot(x12_23_u, x23_34_u);
    double phi = acos_c(cos_phi);
    if (dot(x12_23, r34) < 0.0) phi = -phi;
    double r23_n = nrm(r23);
    *d1 = scl(x12_23_rn, scl(r23_n, neg(x12_23_u)));
    *d4 = scl(x23_34_rn, scl(r23_n, x23_34_u));
    double k1 = dot(r12, r23), k4 = dot(r23, r34), den = r23_n * r23_n;
    v3 df = mk((-d1->x * k1 + d4->x * k4) / den, (-d1->y * k1 + d4->y * k4) / den,
               (-d1->z * k1 + d4->z * k4) / den);
    *d2 = add(neg(*d1), df);
    *d3 = sub(neg(*d4), df);
    return phi - nat_phi;
}

/* eval_cnd_forces::iter: src/forces/dihedral/complex_native.cpp:13-49 */
static void cnd_iter(const xo_sys *s, int idx, double *F, double *V) {
    v3 d1, d2, d3, d4;
    double diff = dih_geom(s, idx, s->dih_p[idx], &d1, &d2, &d3, &d4);
    double sin_diff = sin(diff), cos_diff = cos(diff);
    double sin_3diff = sin(3.0 * diff), cos_3diff = cos(3.0 * diff);
    *V += s->p.cnd_CDA * (1.0 - cos_diff) + s->p.cnd_CDB * (1.0 - cos_3diff);
    double dV = s->p.cnd_CDA * sin_diff + s->p.cnd_CDB * 3.0 * sin_3diff;
    int *ii = s->dih_i + 4 * idx;
    dec(F, ii[0], scl(dV, d1));
    dec(F, ii[1], scl(dV, d2));
    dec(F, ii[2], scl(dV, d3));
    dec(F, ii[3], scl(dV, d4));
}

/* eval_snd_forces::iter: src/forces/dihedral/simple_native.cpp:13-45 */
static void snd_iter(const xo_sys *s, int idx, double *F, double *V) {
    v3 d1, d2, d3, d4;
    double diff = dih_geom(s, idx, s->dih_p[idx], &d1, &d2, &d3, &d4);
    *V += 0.5 * s->p.snd_CDH * diff * diff;
    double dV = s->p.snd_CDH * diff;
    int *ii = s->dih_i + 4 * idx;
    dec(F, ii[0], scl(dV, d1));
    dec(F, ii[1], scl(dV, d2));
    dec(F, ii[2], scl(dV, d3));
    dec(F, ii[3], scl(dV, d4));
}

/* lj::operator(): include/xmd/forces/primitives/lj.h:22-30 */
static inline void lj_eval(double depth, double r_min, double r_inv, double *V, double *dV) {
    double sv = r_inv * r_min, s6 = ipow6(sv), s12 = s6 * s6;
    double V_ = depth * (s12 - 2.0 * s6);
    double dV_dr = 12.0 * depth * r_inv * (s6 - s12);
    *V = clampd(V_, -1.0e3, 1.0e3);
    *dV = clampd(dV_dr, -1.0e3, 1.0e3);
}

/* eval_go_forces::iter: src/forces/go.cpp:31-46 */
static void go_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->go[idx].i1, i2 = s->go[idx].i2;
    v3 r12 = r_uv(s, ld(s->r, i1), ld(s->r, i2));
    double r12_rn = ninv(r12);
    v3 r12_u = scl(r12_rn, r12);
    double V_, dV;
    lj_eval(s->p.go_depth, s->go[idx].d, r12_rn, &V_, &dV);
    *V += V_;
    acc(F, i1, scl(dV, r12_u));
    dec(F, i2, scl(dV, r12_u));
}

/* eval_pauli_exclusion_forces::iter: src/forces/pauli.cpp:32-48; shifted_lj.h:14-21 */
static void pauli_iter(const xo_sys *s, int64_t idx, double *F, double *V) {
    int i1 = s->pauli[idx].i1, i2 = s->pauli[idx].i2;
    v3 r12 = r_uv(s, ld(s->r, i1), ld(s->r, i2));
    double r12_rn = ninv(r12);
    double r_excl = s->p.pauli_r_excl, depth = s->p.pauli_depth;
    if (1.0 < r12_rn * r_excl) {
        v3 r12_u = scl(r12_rn, r12);
        double sv = r12_rn * r_excl, s6 = ipow6(sv), s12 = s6 * s6;
        double V_ = depth * (s12 - 2.0 * s6 + 1.0);
        double dV_dr = 12.0 * depth * r12_rn * (s6 - s12);
        V_ = clampd(V_, -1.0e3, 1.0e3);
        dV_dr = clampd(dV_dr, -1.0e3, 1.0e3);
        *V += V_;
        acc(F, i1, scl(dV_dr, r12_u));
        dec(F, i2, scl(dV_dr, r12_u));
    }
}

/* eval_const_es_forces::iter src/forces/es/const.cpp:13-32 (rel = 0) and
 * eval_relative_es_forces::iter src/forces/es/relative.cpp:13-32 (rel = 1) */
static void es_iter(const xo_sys *s, int64_t idx, int rel, double *F, double *V) {
    int i1 = s->es[idx].i1, i2 = s->es[idx].i2;
    double q1_x_q2 = s->es[idx].d;
    v3 r12 = r_uv(s, ld(s->r, i1), ld(s->r, i2));
    double r12_n = nrm(r12), r12_rn = 1.0 / r12_n;
    v3 r12_u = scl(r12_rn, r12);
    double Vf = rel ? s->rel_es_Vf : s->const_es_Vf;
    double sdi = rel ? s->rel_es_sdi : s->const_es_sdi;
    double Vij = Vf * q1_x_q2 * exp(-r12_n * sdi) * r12_rn * r12_rn;
    double dVij_dr = rel ? -Vij * (sdi + 2.0 * r12_rn) : -Vij * (sdi + r12_rn);
    *V += Vij;
    v3 f = scl(dVij_dr, r12_u);
    acc(F, i1, f);
    dec(F, i2, f);
}

/* ---- quasi-adiabatic contacts ------------------------------------------------ */

/* qa::precompute_nh::iter: src/forces/qa/precompute_nh.cpp:12-20 */
static void qa_nh_iter(xo_sys *s, int idx) {
    int iprev = s->prev[idx], inext = s->next[idx];
    if (iprev < 0 || inext < 0) return;
    v3 rprev = ld(s->r, iprev), rcur = ld(s->r, idx), rnext = ld(s->r, inext);
    v3 v1 = sub(rcur, rprev), v2 = sub(rnext, rcur);
    st3(s->qn, idx, unit(sub(v2, v1)));
    st3(s->qh, idx, unit(cross(v2, v1)));
}

static inline int sync_valid(const int8_t *a) { return a[0] >= 0 && a[1] >= 0 && a[2] >= 0 && a[3] >= 0; }

/* qa::sift_candidates::iter: src/forces/qa/sift_candidates.cpp:15-77.
 * Returns 1 and fills *c when free pair `idx` is a candidate. */
static int qa_sift_iter(const xo_sys *s, int64_t idx, qa_cand *c) {
    const qa_free *node = &s->fp[idx];
    if (node->vacant) return 0;
    const xmd_params *p = &s->p;
    int i1 = node->i1, i2 = node->i2;
    v3 r12 = r_uv(s, ld(s->r, i1), ld(s->r, i2));
    double r12_rn = ninv(r12);
    v3 r12_u = scl(r12_rn, r12);
    v3 n1 = ld(s->qn, i1), n2 = ld(s->qn, i2), h1 = ld(s->qh, i1), h2 = ld(s->qh, i2);
    int back1 = fabs(dot(h1, r12_u)) > p->qa_min_cos_hr;
    int back2 = fabs(dot(h2, r12_u)) > p->qa_min_cos_hr;
    int bb_extra = fabs(dot(h1, h2)) > p->qa_min_cos_hh;
    int side1 = dot(n1, r12_u) < p->qa_max_cos_nr;
    int side2 = -dot(n2, r12_u) < p->qa_max_cos_nr;
    int a1 = s->atype[i1], a2 = s->atype[i2];
    int type = 0;
    if (back1 && back2 && bb_extra) type = 1;
    else if (back1 && side2) type = 2;
    else if (side1 && back2) type = 3;
    else if (side1 && side2) type = 4 + a1 + XMD_NUM_AA * a2;   /* contact_type.h:26-31 */
    if (type == 0) return 0;
    if (1.0 > r12_rn * s->req_min_dist[type]) return 0;
    int ptype2 = p->polarization[a2];
    int8_t d1[4] = {(int8_t)back1, (int8_t)side1, (int8_t)(side1 && ptype2 == 1),
                    (int8_t)(side1 && ptype2 == 2)};
    int8_t after1[4];
    for (int k = 0; k < 4; ++k) after1[k] = (int8_t)(s->sync[4 * i1 + k] - d1[k]);
    if (!sync_valid(after1)) return 0;
    int ptype1 = p->polarization[a1];
    int8_t d2[4] = {(int8_t)back2, (int8_t)side2, (int8_t)(side2 && ptype1 == 1),
                    (int8_t)(side2 && ptype1 == 2)};
    int8_t after2[4];
    for (int k = 0; k < 4; ++k) after2[k] = (int8_t)(s->sync[4 * i2 + k] - d2[k]);
    if (!sync_valid(after2)) return 0;
    c->i1 = i1; c->i2 = i2; c->free_idx = (int32_t)idx; c->type = type;
    memcpy(c->d1, d1, 4); memcpy(c->d2, d2, 4);
    return 1;
}

/* qa::process_candidates::iter: src/forces/qa/process_candidates.cpp:10-29 */
static void qa_accept(xo_sys *s) {
    for (int64_t idx = 0; idx < s->n_cand; ++idx) {
        qa_cand *c = &s->cand[idx];
        int8_t n1[4], n2[4];
        for (int k = 0; k < 4; ++k) {
            n1[k] = (int8_t)(s->sync[4 * c->i1 + k] - c->d1[k]);
            n2[k] = (int8_t)(s->sync[4 * c->i2 + k] - c->d2[k]);
        }
        if (sync_valid(n1) && sync_valid(n2)) {
            GROW(s->cont, s->n_cont, s->cap_cont, qa_cont);
            qa_cont *q = &s->cont[s->n_cont++];
            q->i1 = c->i1; q->i2 = c->i2; q->type = c->type;
            q->status = FORMING_OR_FORMED; q->ref_time = s->t; q->vacant = 0;
            memcpy(q->d1, c->d1, 4); memcpy(q->d2, c->d2, 4);
            for (int k = 0; k < 4; ++k) {
                s->sync[4 * c->i1 + k] -= c->d1[k];
                s->sync[4 * c->i2 + k] -= c->d2[k];
            }
            s->fp[c->free_idx].vacant = 1;
        }
    }
}

/* Potential of contact type t: ljs[t-1] with lj_variants::operator[]
 * (lj_variants.h:16-23) over the table of lj_variants.cpp:8-63 [D6]. */
static void qa_lj(const xo_sys *s, int type, double *depth, double *r_min, double *r_max) {
    const xmd_params *p = &s->p;
    int k = type - 1;
    if (k == 0) { *depth = p->lj_bb_depth; *r_min = *r_max = p->lj_bb_r_min; }
    else if (k == 1 || k == 2) { *depth = p->lj_bs_depth; *r_min = *r_max = p->lj_bs_r_min; }
    else {
        int ss = k - 3;
        *depth = p->ss_depth[ss];
        *r_max = p->ss_r_max[ss];
        *r_min = p->ss_sinking ? p->lj_bb_r_min : p->ss_r_max[ss];
    }
}

/* sink_lj::operator(): include/xmd/forces/primitives/sink_lj.h:24-33 */
static inline void sink_lj_eval(double depth, double r_min, double r_max, double r,
                                double r_inv, double *V, double *dV) {
    double r_eff = (r < r_min ? r_min : (r < r_max ? r : r_max));
    double sv = r_inv * r_eff, s6 = ipow6(sv), s12 = s6 * s6;
    double V_ = depth * (s12 - 2.0 * s6);
    double dV_dr = 12.0 * depth * r_inv * (s6 - s12);
    dV_dr = (r_min < r && r < r_max) ? 0 : dV_dr;
    *V = clampd(V_, -1.0e3, 1.0e3);
    *dV = clampd(dV_dr, -1.0e3, 1.0e3);
}

/* Force part of qa::process_contacts::iter: process_contacts.cpp:14-40 */
static void qa_contact_force(const xo_sys *s, int64_t idx, double *F, double *V) {
    const qa_cont *c = &s->cont[idx];
    if (c->vacant) return;
    v3 r12 = r_uv(s, ld(s->r, c->i1), ld(s->r, c->i2));
    double r12_rn = ninv(r12);
    v3 r12_u = scl(r12_rn, r12);
    double sat = fmin(s->t - c->ref_time, s->p.qa_phase_duration) * s->qa_cycle_inv;
    if (c->status == BREAKING) sat = 1.0 - sat;
    double depth, r_min, r_max;
    qa_lj(s, c->type, &depth, &r_min, &r_max);
    double r12_n = r12_rn * nsq(r12);
    double Vij, dVij;
    sink_lj_eval(depth, r_min, r_max, r12_n, r12_rn, &Vij, &dVij);
    *V += sat * Vij;
    v3 f = scl(sat * dVij, r12_u);
    acc(F, c->i1, f);
    dec(F, c->i2, f);
}

/* State part of qa::process_contacts::iter: process_contacts.cpp:42-56 */
static void qa_contact_transition(xo_sys *s, int64_t idx) {
    qa_cont *c = &s->cont[idx];
    if (c->vacant) return;
    v3 r12 = r_uv(s, ld(s->r, c->i1), ld(s->r, c->i2));
    double r12_rn = ninv(r12);
    double sat = fmin(s->t - c->ref_time, s->p.qa_phase_duration) * s->qa_cycle_inv;
    if (c->status == BREAKING) sat = 1.0 - sat;
    double depth, r_min, r_max;
    qa_lj(s, c->type, &depth, &r_min, &r_max);
    if (c->status == FORMING_OR_FORMED && sat == 1.0) {
        if (s->qa_factor * r_min * r12_rn < 1.0) {
            c->status = BREAKING;
            c->ref_time = s->t;
        }
    } else if (c->status == BREAKING && sat == 0.0) {
        c->vacant = 1;
        for (int k = 0; k < 4; ++k) {
            s->sync[4 * c->i1 + k] += c->d1[k];
            s->sync[4 * c->i2 + k] += c->d2[k];
        }
        GROW(s->fp, s->n_fp, s->cap_fp, qa_free);
        s->fp[s->n_fp].i1 = c->i1;
        s->fp[s->n_fp].i2 = c->i2;
        s->fp[s->n_fp].vacant = 0;
        s->n_fp++;
    }
}

/* ---- force phase ------------------------------------------------------------- */

/* eval_heurestic_angle_forces::iter: src/forces/angle/heurestic.cpp:29-59,
   with the 7 coefficients a0..a6 of the type's table row */
static void heur_angle_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->hang_i[3 * idx], i2 = s->hang_i[3 * idx + 1], i3 = s->hang_i[3 * idx + 2];
    const double *a = s->p.heur_ang_coeffs[s->hang_t[idx]];
    v3 r1 = ld(s->r, i1), r2 = ld(s->r, i2), r3 = ld(s->r, i3);
    v3 r12 = sub(r2, r1), r23 = sub(r3, r2);
    v3 x12_23 = cross(r12, r23);
    double r12_rn = ninv(r12), r23_rn = ninv(r23);
    v3 d1 = scl(r12_rn, unit(cross(r12, x12_23)));
    v3 d3 = scl(r23_rn, unit(cross(r23, x12_23)));
    v3 d2 = sub(neg(d1), d3);
    double cos_theta = -dot(r12, r23) * r12_rn * r23_rn;
    double theta = acos_c(cos_theta);
    double angle_V = 0.0, dV = 0.0;
    for (int d = 6; d >= 0; --d) {
        if (d > 0) dV = (double)d * a[d] + theta * dV;
        angle_V = a[d] + theta * angle_V;
    }
    *V += angle_V;
    dec(F, i1, scl(dV, d1));
    dec(F, i2, scl(dV, d2));
    dec(F, i3, scl(dV, d3));
}

/* eval_heurestic_dihedral_forces::iter: src/forces/dihedral/heurestic.cpp:29-70,
   with phi = acos(cos_phi) (line 43 takes cos) and dV/dphi the derivative
   of V (lines 52-54 add 2 c4 sin cos where d(cos^2)/dphi = -2 sin cos) */
static void heur_dihedral_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->hdih_i[4 * idx], i2 = s->hdih_i[4 * idx + 1], i3 = s->hdih_i[4 * idx + 2],
        i4 = s->hdih_i[4 * idx + 3];
    const double *c = s->p.heur_dih_coeffs[s->hdih_t[idx]];
    v3 r1 = ld(s->r, i1), r2 = ld(s->r, i2), r3 = ld(s->r, i3), r4 = ld(s->r, i4);
    v3 r12 = sub(r2, r1), r23 = sub(r3, r2), r34 = sub(r4, r3);
    v3 x12_23 = cross(r12, r23), x23_34 = cross(r23, r34);
    double x12_23_rn = ninv(x12_23), x23_34_rn = ninv(x23_34);
    v3 x12_23_u = scl(x12_23_rn, x12_23), x23_34_u = scl(x23_34_rn, x23_34);
    double cos_phi = dot(x12_23_u, x23_34_u);
    double phi = acos_c(cos_phi);
    if (dot(x12_23, r34) < 0.0) phi = -phi;
    double sin_phi = sin(phi);
    double sin2 = sin_phi * sin_phi, cos2 = cos_phi * cos_phi, sc = sin_phi * cos_phi;
    *V += c[0] + c[1] * sin_phi + c[2] * cos_phi + c[3] * sin2 + c[4] * cos2 + c[5] * sc;
    double dV = c[1] * cos_phi - c[2] * sin_phi + 2.0 * (c[3] - c[4]) * sc + c[5] * (cos2 - sin2);
    double r23_n = nrm(r23);
    v3 d1 = scl(x12_23_rn, scl(r23_n, neg(x12_23_u)));
    v3 d4 = scl(x23_34_rn, scl(r23_n, x23_34_u));
    double k1 = dot(r12, r23), k4 = dot(r23, r34), den = r23_n * r23_n;
    v3 df = mk((-d1.x * k1 + d4.x * k4) / den, (-d1.y * k1 + d4.y * k4) / den, (-d1.z * k1 + d4.z * k4) / den);
    v3 d2 = add(neg(d1), df), d3 = sub(neg(d4), df);
    dec(F, i1, scl(dV, d1));
    dec(F, i2, scl(dV, d2));
    dec(F, i3, scl(dV, d3));
    dec(F, i4, scl(dV, d4));
}

/* eval_velocity_afm_forces::iter: src/forces/velocity_afm.cpp; afm_force is
   harmonic(H1, H2, nat_r = 0) (main.cpp sets H1 and H2 only) */
static void vel_afm_iter(const xo_sys *s, int idx, double *F) {
    int i = s->vafm_i[idx];
    v3 r_ = ld(s->r, i);
    v3 cur = add(ld(s->vafm_o, idx), scl(s->t, ld(s->vafm_v, idx)));
    v3 r_afm = sub(cur, r_);
    double r_afm_n = nrm(r_afm), r_afm_rn = 1.0 / r_afm_n;
    if (r_afm_n == 0.0) return;   /* the spring at rest: no force (the shipped code gives 0 * inf) [D21] */
    v3 r_afm_u = scl(r_afm_rn, r_afm);
    double dr = r_afm_n - 0.0, dr2 = dr * dr;
    double dV_dr = dr * (s->p.vel_afm_H1 + 2.0 * s->p.vel_afm_H2 * dr2);
    dV_dr = clampd(dV_dr, -1.0e3, 1.0e3);
    acc(F, i, scl(dV_dr, r_afm_u));
}
/* box::wrap (include/xmd/model/box.h:37-43) */
static v3 wrap(const xo_sys *s, v3 v) {
    v.x -= s->cell[0] * nearbyint(v.x * s->cell_inv[0]);
    v.y -= s->cell[1] * nearbyint(v.y * s->cell_inv[1]);
    v.z -= s->cell[2] * nearbyint(v.z * s->cell_inv[2]);
    return v;
}
static double signed_dist(v3 p, const double *pl) {   /* utils/geometry.h:17-20 */
    return dot(mk(pl[3], pl[4], pl[5]), sub(p, mk(pl[0], pl[1], pl[2])));
}
/* eval_solid_wall_forces::iter (walls/solid.cpp:12-27): V = eps / (9 x^9)
   inside the cutoff, with the force -dV/dx along the normal (the shipped
   dV_dx = V * (-9 x) is added along +normal) [D22] */
static void solid_wall_iter(const xo_sys *s, int idx, double *F, double *V) {
    v3 part_r = wrap(s, ld(s->r, idx));
    for (int w = 0; w < s->n_wall[0]; ++w) {
        const double *pl = s->wall[0][w];
        double x = signed_dist(part_r, pl);
        if (x < s->p.solid_wall_cutoff) {
            double x3 = x * x * x;
            double V_ = s->p.solid_wall_depth / (9.0 * (x3 * x3 * x3));
            double dV_dx = -9.0 * V_ / x;
            *V += V_;
            acc(F, idx, scl(-dV_dx, mk(pl[3], pl[4], pl[5])));
        }
    }
}
/* Force part of eval_lj_attr_wall_forces::loop (walls/lj_attr.cpp:16-31),
   lj_depth = `depth` (never set by main.cpp:836-843) [D22] */
static void lj_wall_force(const xo_sys *s, int w, int idx, double *F, double *V) {
    size_t q = (size_t)w * s->n + idx;
    int st = s->ljw_status[q];
    if (st == 0) return;
    v3 r_ = wrap(s, ld(s->r, idx));
    double sat = fmin(s->t - s->ljw_ref[q], s->p.lj_wall_phase_duration) * (1.0 / s->p.lj_wall_phase_duration);
    if (st == 2) sat = 1.0 - sat;
    v3 r12 = sub(ld(s->ljw_joint, (int)q), r_);
    double r12_rn = ninv(r12);
    double V_, dV_dr;
    lj_eval(s->p.lj_wall_depth, s->p.lj_wall_min_dist, r12_rn, &V_, &dV_dr);
    *V += V_ * sat;
    v3 r12_u = scl(r12_rn, r12);
    acc(F, idx, scl(sat * dV_dr, r12_u));
}
/* State part of the same loop (lj_attr.cpp:8-14, 32-40), after the forces */
static void lj_wall_transition(xo_sys *s, int w, int idx) {
    size_t q = (size_t)w * s->n + idx;
    int st = s->ljw_status[q];
    v3 r_ = wrap(s, ld(s->r, idx));
    const double *pl = s->wall[1][w];
    if (st == 0) {
        double x = signed_dist(r_, pl);
        if (fabs(x) < s->p.lj_wall_min_dist) {
            s->ljw_status[q] = 1;
            v3 j = sub(r_, scl(x, mk(pl[3], pl[4], pl[5])));
            st3(s->ljw_joint, (int)q, j);
            s->ljw_ref[q] = s->t;
        }
        return;
    }
    double sat = fmin(s->t - s->ljw_ref[q], s->p.lj_wall_phase_duration) * (1.0 / s->p.lj_wall_phase_duration);
    if (st == 2) sat = 1.0 - sat;
    double r12_rn = ninv(sub(ld(s->ljw_joint, (int)q), r_));
    double factor = s->p.lj_wall_breaking_factor * pow(2.0, -1.0 / 6.0);
    if (st == 1 && sat == 1.0) {
        if (factor * s->p.lj_wall_min_dist * r12_rn < 1.0) { s->ljw_status[q] = 2; s->ljw_ref[q] = s->t; }
    } else if (st == 2 && sat == 0.0) {
        s->ljw_status[q] = 0;
    }
}
static void lj_wall_phase(xo_sys *s) {
    if (!s->p.on[XMD_TERM_LJ_WALL]) return;
    for (int w = 0; w < s->n_wall[1]; ++w)
        for (int i = 0; i < s->n; ++i) lj_wall_transition(s, w, i);
}

/* pid::lambda_func (pid/lambda.h:29-56): support and (value, derivative) */
static int pid_supp(double alpha, double psi0, double psi) { return fabs(alpha * (psi - psi0)) < M_PI; }
static void pid_lam(int version, double alpha, double psi0, double psi, double *val, double *deriv) {
    double sv = alpha * (psi - psi0);
    if (version == 0) {
        *val = 0.5 * cos(sv) + 0.5;
        *deriv = -0.5 * alpha * sin(sv);
    } else {
        double t = fabs(sv / M_PI);
        double x_inv = 1.0 / (2.0 * t * t - 2.0 * t - 1);
        *val = (t * t - 2.0 * t + 1.0) * x_inv;
        /* d val / d psi = 2 (t - 1)(t - 2) / den^2 * alpha / pi (the shipped
           line 47 has 2 t (t - 1) and no alpha) [D23] */
        *deriv = (2.0 * (t - 1.0) * (t - 2.0)) * x_inv * x_inv * alpha / M_PI;
        *deriv *= (sv < 0.0 ? -1.0 : 1.0);
    }
}
/* One side of eval_pid_forces::iter (eval_forces.cpp:27-62): the
   pseudo-improper dihedral psi of (r1_, r2_, r3_; r4_) and its derivatives
   along the four beads */
static double pid_psi(const xo_sys *s, v3 r1_, v3 r2_, v3 r3_, v3 r4_, v3 *d1, v3 *d2, v3 *d3, v3 *d4) {
    v3 r24 = r_uv(s, r2_, r4_);
    v3 r12 = sub(r2_, r1_), r23 = sub(r3_, r2_), r13 = sub(r3_, r1_);
    v3 r14 = add(r12, r24);
    v3 rij = neg(r23), rkj = neg(r13), rkl = neg(r14);
    v3 rm = cross(r23, r12), rn = cross(r13, r14);
    double rm_rn = ninv(rm), rn_rn = ninv(rn), rkj_n = nrm(rkj);
    /* atoms i = r2_, j = r3_, k = r1_, l = r4_ of rij = ri - rj, rkj, rkl;
       the dihedral's gradient (Bekker): dpsi/dri = |rkj| m / |m|^2,
       dpsi/drl = -|rkj| n / |n|^2, and j, k from them [D23] */
    v3 gi = scl(rkj_n * rm_rn * rm_rn, rm);
    v3 gl = neg(scl(rkj_n * rn_rn * rn_rn, rn));
    double a = dot(rij, rkj) / (rkj_n * rkj_n), b = dot(rkl, rkj) / (rkj_n * rkj_n);
    v3 gj = sub(scl(a - 1.0, gi), scl(b, gl));
    v3 gk = sub(scl(b - 1.0, gl), scl(a, gi));
    *d1 = gk;      /* r1_: previous bead */
    *d2 = gi;      /* r2_: the bead */
    *d3 = gj;      /* r3_: next bead */
    *d4 = gl;      /* r4_: the partner */
    double psi = acos(dot(rm, rn) * rm_rn * rn_rn);
    if (dot(rij, rn) < 0.0) psi = -psi;
    return psi;
}
/* eval_pid_forces::iter (eval_forces.cpp:14-141) with the forces the
   energy's gradient [D23]: the shipped lines 64-98 write the second side's
   derivatives into dpsi1_* (dpsi2_* stay unset), and each side's derivatives
   go to the wrong beads with 1/|m|, 1/|n| for 1/|m|^2, 1/|n|^2; the pair
   part's sign is that of the Go term (F1 = +dV/dr r12_u, go.cpp:42-44),
   where the shipped lines 136-139 subtract it */
static void pid_iter(const xo_sys *s, int64_t idx, double *F, double *V) {
    const xmd_params *p = &s->p;
    int i1 = s->pid[idx].i1, i2 = s->pid[idx].i2;
    int i1p = s->prev[i1], i1n = s->next[i1], i2p = s->prev[i2], i2n = s->next[i2];
    v3 r1p = ld(s->r, i1p), r1 = ld(s->r, i1), r1n = ld(s->r, i1n);
    v3 r2p = ld(s->r, i2p), r2 = ld(s->r, i2), r2n = ld(s->r, i2n);
    v3 a1p, a1, a1n, a2, b2p, b2, b2n, b1;
    double psi1 = pid_psi(s, r1p, r1, r1n, r2, &a1p, &a1, &a1n, &a2);
    double psi2 = pid_psi(s, r2p, r2, r2n, r1, &b2p, &b2, &b2n, &b1);
    v3 r12 = r_uv(s, r1, r2);
    double r12_n = nrm(r12), r12_rn = 1.0 / r12_n;
    double A = 0.0, B = 0.0, C = 0.0, V_ = 0.0;
    const double *bb[2] = {p->pid_bbp, p->pid_bbm};
    for (int k = 0; k < 2; ++k) {
        const double *q = bb[k];
        if (pid_supp(q[0], q[1], psi1) && pid_supp(q[0], q[1], psi2)) {
            double lam1, d1, lam2, d2, lV, ldV;
            pid_lam(p->pid_lambda, q[0], q[1], psi1, &lam1, &d1);
            pid_lam(p->pid_lambda, q[0], q[1], psi2, &lam2, &d2);
            lj_eval(q[3], q[2], r12_rn, &lV, &ldV);
            V_ += lam1 * lam2 * lV;
            A += d1 * lam2 * lV;
            B += d2 * lam1 * lV;
            C += lam1 * lam2 * ldV;
        }
    }
    if (pid_supp(p->pid_ss[0], p->pid_ss[1], psi1) && pid_supp(p->pid_ss[0], p->pid_ss[1], psi2)) {
        /* ss_ljs[type], type = atype1 * NUM_AA + atype2 (bundle.cpp:20-22) */
        int ss = (int)s->atype[i1] * XMD_NUM_AA + (int)s->atype[i2];
        double depth = p->ss_depth[ss], r_max = p->ss_r_max[ss];
        double r_min = p->ss_sinking ? p->lj_bb_r_min : r_max;
        double lam1, d1, lam2, d2, lV, ldV;
        pid_lam(p->pid_lambda, p->pid_ss[0], p->pid_ss[1], psi1, &lam1, &d1);
        pid_lam(p->pid_lambda, p->pid_ss[0], p->pid_ss[1], psi2, &lam2, &d2);
        sink_lj_eval(depth, r_min, r_max, r12_n, r12_rn, &lV, &ldV);
        V_ += lam1 * lam2 * lV;
        A += d1 * lam2 * lV;
        B += d2 * lam1 * lV;
        C += lam1 * lam2 * ldV;
    }
    *V += V_;
    v3 r12_u = scl(r12_rn, r12);
    dec(F, i1p, scl(A, a1p));
    dec(F, i1, sub(add(scl(A, a1), scl(B, b1)), scl(C, r12_u)));
    dec(F, i1n, scl(A, a1n));
    dec(F, i2p, scl(B, b2p));
    dec(F, i2, add(add(scl(A, a2), scl(B, b2)), scl(C, r12_u)));
    dec(F, i2n, scl(B, b2n));
}

/* eval_force_afm_forces::iter: src/forces/force_afm.cpp */
static void force_afm_iter(const xo_sys *s, int idx, double *F) {
    acc(F, s->fafm_i[idx], ld(s->fafm_F, idx));
}

/* eval_chiral_forces::iter: src/forces/chiral.cpp:15-37 */
static void chiral_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->chir_i[4 * idx], i2 = s->chir_i[4 * idx + 1], i3 = s->chir_i[4 * idx + 2], i4 = s->chir_i[4 * idx + 3];
    double nat_chir = s->chir_n[idx], nat_factor = s->chir_f[idx];
    v3 r1 = ld(s->r, i1), r2 = ld(s->r, i2), r3 = ld(s->r, i3), r4 = ld(s->r, i4);
    v3 r12 = sub(r2, r1), r23 = sub(r3, r2), r34 = sub(r4, r3);
    v3 x12_23 = cross(r12, r23), x12_34 = cross(r12, r34), x23_34 = cross(r23, r34);
    double chir = dot(r12, x23_34) * nat_factor;
    double chir_diff = chir - nat_chir;
    *V += 0.5 * s->p.chir_e_chi * chir_diff * chir_diff;
    double f = s->p.chir_e_chi * chir_diff * nat_factor;
    acc(F, i1, scl(f, x12_23));
    dec(F, i2, scl(f, add(x12_34, x23_34)));
    acc(F, i3, scl(f, add(x12_23, x12_34)));
    dec(F, i4, scl(f, x12_23));
}

/* eval_nat_ssbond_forces::iter: src/forces/native_ss.cpp:27-40 */
static void ss_iter(const xo_sys *s, int idx, double *F, double *V) {
    int i1 = s->ss[idx].i1, i2 = s->ss[idx].i2;
    v3 r12 = r_uv(s, ld(s->r, i1), ld(s->r, i2));
    double r12_n = nrm(r12);
    /* harmonic(H1, 0, nat_r): harmonic.h:18-25 */
    double dr = r12_n - s->p.nat_ss_dist, dr2 = dr * dr;
    double V_ = 0.5 * dr2 * (s->p.nat_ss_H1 + 0.0 * dr2);
    double dV_dr = dr * (s->p.nat_ss_H1 + 2.0 * 0.0 * dr2);
    V_ = clampd(V_, -1.0e3, 1.0e3);
    dV_dr = clampd(dV_dr, -1.0e3, 1.0e3);
    v3 r12_u = {r12.x / r12_n, r12.y / r12_n, r12.z / r12_n};   /* r12 / r12_n: per component */
    *V += V_;
    acc(F, i1, scl(dV_dr, r12_u));
    dec(F, i2, scl(dV_dr, r12_u));
}

static void pure_forces(const xo_sys *s, double *F, double *V) {
    const xmd_params *p = &s->p;
    memset(F, 0, sizeof(double) * 3 * (size_t)s->n);
    for (int k = 0; k < XMD_NUM_TERMS; ++k) V[k] = 0.0;
    if (p->on[XMD_TERM_TETHER]) for (int k = 0; k < s->n_teth; ++k) tether_iter(s, k, F, &V[XMD_TERM_TETHER]);
    if (p->on[XMD_TERM_NAT_ANG]) for (int k = 0; k < s->n_ang; ++k) angle_iter(s, k, F, &V[XMD_TERM_NAT_ANG]);
    if (p->on[XMD_TERM_CND]) for (int k = 0; k < s->n_dih; ++k) cnd_iter(s, k, F, &V[XMD_TERM_CND]);
    if (p->on[XMD_TERM_SND]) for (int k = 0; k < s->n_dih; ++k) snd_iter(s, k, F, &V[XMD_TERM_SND]);
    if (p->on[XMD_TERM_PAULI]) for (int64_t k = 0; k < s->n_pauli; ++k) pauli_iter(s, k, F, &V[XMD_TERM_PAULI]);
    if (p->on[XMD_TERM_GO]) for (int k = 0; k < s->n_go; ++k) go_iter(s, k, F, &V[XMD_TERM_GO]);
    if (p->on[XMD_TERM_CONST_ES]) for (int64_t k = 0; k < s->n_es; ++k) es_iter(s, k, 0, F, &V[XMD_TERM_CONST_ES]);
    if (p->on[XMD_TERM_REL_ES]) for (int64_t k = 0; k < s->n_es; ++k) es_iter(s, k, 1, F, &V[XMD_TERM_REL_ES]);
    if (p->on[XMD_TERM_QA]) for (int64_t k = 0; k < s->n_cont; ++k) qa_contact_force(s, k, F, &V[XMD_TERM_QA]);
    if (p->on[XMD_TERM_CHIR]) for (int k = 0; k < s->n_chir; ++k) chiral_iter(s, k, F, &V[XMD_TERM_CHIR]);
    if (p->on[XMD_TERM_NAT_SS]) for (int k = 0; k < s->n_ss; ++k) ss_iter(s, k, F, &V[XMD_TERM_NAT_SS]);
    if (p->on[XMD_TERM_HEUR_ANG]) for (int k = 0; k < s->n_hang; ++k) heur_angle_iter(s, k, F, &V[XMD_TERM_HEUR_ANG]);
    if (p->on[XMD_TERM_HEUR_DIH]) for (int k = 0; k < s->n_hdih; ++k) heur_dihedral_iter(s, k, F, &V[XMD_TERM_HEUR_DIH]);
    if (p->on[XMD_TERM_VEL_AFM]) for (int k = 0; k < s->n_vafm; ++k) vel_afm_iter(s, k, F);
    if (p->on[XMD_TERM_FORCE_AFM]) for (int k = 0; k < s->n_fafm; ++k) force_afm_iter(s, k, F);
    if (p->on[XMD_TERM_PID]) for (int64_t k = 0; k < s->n_pid; ++k) pid_iter(s, k, F, &V[XMD_TERM_PID]);
    if (p->on[XMD_TERM_SOLID_WALL]) for (int k = 0; k < s->n; ++k) solid_wall_iter(s, k, F, &V[XMD_TERM_SOLID_WALL]);
    if (p->on[XMD_TERM_LJ_WALL])
        for (int w = 0; w < s->n_wall[1]; ++w)
            for (int k = 0; k < s->n; ++k) lj_wall_force(s, w, k, F, &V[XMD_TERM_LJ_WALL]);
}

/* Forces at positions r with the current lists (no rebuild); the state is
   left as it was (a checker of derivatives) */
int xo_eval_at(xo_sys *s, const double *r, double *F, double *V) {
    size_t nb = sizeof(double) * 3 * (size_t)s->n;
    double *keep = (double *)malloc(nb);
    memcpy(keep, s->r, nb);
    memcpy(s->r, r, nb);
    double Vl[XMD_NUM_TERMS];
    double *Ft = (double *)malloc(nb);
    pure_forces(s, Ft, Vl);
    if (F) memcpy(F, Ft, nb);
    if (V) memcpy(V, Vl, sizeof Vl);
    memcpy(s->r, keep, nb);
    free(keep);
    free(Ft);
    return 0;
}

int xo_eval_forces(xo_sys *s, double *F, double *V) {
    if (s->first_time) ensure_nl(s);
    double Vl[XMD_NUM_TERMS];
    pure_forces(s, s->F, Vl);
    if (F) memcpy(F, s->F, sizeof(double) * 3 * (size_t)s->n);
    if (V) memcpy(V, Vl, sizeof Vl);
    return 0;
}

/* QA stage order of eval_qa_forces::operator(): qa.cpp:20-31 [D7].
 * The force of each contact is taken in pure_forces() from the contact set
 * as it stood before this step's acceptance; contacts accepted this step have
 * saturation 0 and add nothing, so the order is equivalent. */
static void qa_state_phase(xo_sys *s) {
    for (int i = 0; i < s->n; ++i) qa_nh_iter(s, i);
    s->n_cand = 0;                                                  /* omp_prep */
    for (int64_t k = 0; k < s->n_fp; ++k) {
        qa_cand c;
        if (qa_sift_iter(s, k, &c)) {
            GROW(s->cand, s->n_cand, s->cap_cand, qa_cand);
            s->cand[s->n_cand++] = c;
        }
    }
    qa_accept(s);
    int64_t n_before = s->n_cont;
    for (int64_t k = 0; k < n_before; ++k) qa_contact_transition(s, k);
}

/* lang_pc_step::operator(): src/dynamics/lang_pc.cpp:5-41 [D8] (mass = 1,
 * main.cpp:156) */
static void lang_pc(xo_sys *s) {
    uint64_t local_gen = s->rng;
    double dt = s->p.dt, gamma_factor = s->p.gamma_factor;
    double noise_factor = sqrt(2.0 * 1.0 * s->temperature);
    double dt_inv = 1.0 / dt;
    double gamma_factor_sqrt = sqrt(gamma_factor);
    const double mass = 1.0, mass_inv = 1.0, mass_rsqrt = 1.0;
    for (int idx = 0; idx < s->n; ++idx) {
        double gamma = gamma_factor * mass;
        double noise_sd = noise_factor * gamma_factor_sqrt * mass_rsqrt;
        double nx, ny;
        rng_normal_x2(&local_gen, &nx, &ny);
        double nz = xo_rng_normal(&local_gen);
        double *y0 = s->y[0] + 3 * idx, *y1 = s->y[1] + 3 * idx, *y2 = s->y[2] + 3 * idx,
               *y3 = s->y[3] + 3 * idx, *y4 = s->y[4] + 3 * idx, *y5 = s->y[5] + 3 * idx;
        double noise[3] = {nx, ny, nz};
        for (int a = 0; a < 3; ++a) {
            double a_ = s->F[3 * idx + a] * mass_inv - gamma * s->v[3 * idx + a] + noise_sd * noise[a];
            double error = y2[a] - a_ * (dt * dt / 2.0);
            y0[a] -= 3.0 / 16.0 * error;
            y1[a] -= 251.0 / 360.0 * error;
            y2[a] -= 1.0 * error;
            y3[a] -= 11.0 / 18.0 * error;
            y4[a] -= 1.0 / 6.0 * error;
            y5[a] -= 1.0 / 60.0 * error;
            y0[a] += y1[a] + y2[a] + y3[a] + y4[a] + y5[a];
            y1[a] += 2.0 * y2[a] + 3.0 * y3[a] + 4.0 * y4[a] + 5.0 * y5[a];
            y2[a] += 3.0 * y3[a] + 6.0 * y4[a] + 10.0 * y5[a];
            y3[a] += 4.0 * y4[a] + 10.0 * y5[a];
            y4[a] += 5.0 * y5[a];
            s->r[3 * idx + a] = y0[a];
            s->v[3 * idx + a] = y1[a] * dt_inv;
        }
    }
    s->true_t += dt;
    s->t = s->true_t;
    s->rng = local_gen;
}

/* One iteration of the step loop of main.cpp:1028-1076 (serial). */
int xo_step(xo_sys *s, int32_t nsteps) {
    if (s->first_time) ensure_nl(s);
    for (int32_t k = 0; k < nsteps; ++k) {
        pure_forces(s, s->F, s->V);
        if (s->p.on[XMD_TERM_QA]) qa_state_phase(s);
        lj_wall_phase(s);
        if (s->p.langevin_on) lang_pc(s);
        ensure_nl(s);
    }
    return 0;
}

/* The same step with the reference's OpenMP structure (main.cpp:909-1077):
 * every thread owns thread_F/thread_V (main.cpp:917-925), each term runs as
 * `omp for schedule(static) nowait`, reduce_vf adds them atomically
 * (reduce_vf.cpp:4-11), the master thread integrates and rebuilds. */
int xo_step_omp(xo_sys *s, int32_t nsteps, int32_t nthreads) {
#ifdef _OPENMP
    if (s->first_time) ensure_nl(s);
    const xmd_params *p = &s->p;
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
    size_t n3 = 3 * (size_t)s->n;
    double *tF = (double *)malloc(sizeof(double) * n3 * (size_t)nt);
    qa_cand **tc = (qa_cand **)calloc((size_t)nt, sizeof(qa_cand *));
    int64_t *tcn = (int64_t *)calloc((size_t)nt, sizeof(int64_t));
    int64_t *tcc = (int64_t *)calloc((size_t)nt, sizeof(int64_t));
#pragma omp parallel num_threads(nt)
    {
        int tid = omp_get_thread_num();
        double *F = tF + n3 * (size_t)tid;
        for (int32_t step = 0; step < nsteps; ++step) {
            double V[XMD_NUM_TERMS] = {0};
            memset(F, 0, sizeof(double) * n3);                     /* reset_thread_vf */
#pragma omp single
            {
                memset(s->F, 0, sizeof(double) * n3);              /* reset_vf */
                for (int k = 0; k < XMD_NUM_TERMS; ++k) s->V[k] = 0.0;
            }
            if (p->on[XMD_TERM_TETHER]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_teth; ++k) tether_iter(s, k, F, &V[XMD_TERM_TETHER]);
            }
            if (p->on[XMD_TERM_NAT_ANG]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_ang; ++k) angle_iter(s, k, F, &V[XMD_TERM_NAT_ANG]);
            }
            if (p->on[XMD_TERM_CND]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_dih; ++k) cnd_iter(s, k, F, &V[XMD_TERM_CND]);
            }
            if (p->on[XMD_TERM_SND]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_dih; ++k) snd_iter(s, k, F, &V[XMD_TERM_SND]);
            }
            if (p->on[XMD_TERM_PAULI]) {
#pragma omp for schedule(static) nowait
                for (int64_t k = 0; k < s->n_pauli; ++k) pauli_iter(s, k, F, &V[XMD_TERM_PAULI]);
            }
            if (p->on[XMD_TERM_GO]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_go; ++k) go_iter(s, k, F, &V[XMD_TERM_GO]);
            }
            if (p->on[XMD_TERM_CONST_ES]) {
#pragma omp for schedule(static) nowait
                for (int64_t k = 0; k < s->n_es; ++k) es_iter(s, k, 0, F, &V[XMD_TERM_CONST_ES]);
            }
            if (p->on[XMD_TERM_REL_ES]) {
#pragma omp for schedule(static) nowait
                for (int64_t k = 0; k < s->n_es; ++k) es_iter(s, k, 1, F, &V[XMD_TERM_REL_ES]);
            }
            if (p->on[XMD_TERM_CHIR]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_chir; ++k) chiral_iter(s, k, F, &V[XMD_TERM_CHIR]);
            }
            if (p->on[XMD_TERM_NAT_SS]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_ss; ++k) ss_iter(s, k, F, &V[XMD_TERM_NAT_SS]);
            }
            if (p->on[XMD_TERM_HEUR_ANG]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_hang; ++k) heur_angle_iter(s, k, F, &V[XMD_TERM_HEUR_ANG]);
            }
            if (p->on[XMD_TERM_HEUR_DIH]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_hdih; ++k) heur_dihedral_iter(s, k, F, &V[XMD_TERM_HEUR_DIH]);
            }
            if (p->on[XMD_TERM_VEL_AFM]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_vafm; ++k) vel_afm_iter(s, k, F);
            }
            if (p->on[XMD_TERM_FORCE_AFM]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n_fafm; ++k) force_afm_iter(s, k, F);
            }
            if (p->on[XMD_TERM_PID]) {
#pragma omp for schedule(static) nowait
                for (int64_t k = 0; k < s->n_pid; ++k) pid_iter(s, k, F, &V[XMD_TERM_PID]);
            }
            if (p->on[XMD_TERM_SOLID_WALL]) {
#pragma omp for schedule(static) nowait
                for (int k = 0; k < s->n; ++k) solid_wall_iter(s, k, F, &V[XMD_TERM_SOLID_WALL]);
            }
            if (p->on[XMD_TERM_LJ_WALL]) {
                for (int w = 0; w < s->n_wall[1]; ++w) {
#pragma omp for schedule(static) nowait
                    for (int k = 0; k < s->n; ++k) lj_wall_force(s, w, k, F, &V[XMD_TERM_LJ_WALL]);
                }
            }
            if (p->on[XMD_TERM_QA]) {
#pragma omp for schedule(static) nowait
                for (int64_t k = 0; k < s->n_cont; ++k) qa_contact_force(s, k, F, &V[XMD_TERM_QA]);
#pragma omp for schedule(static)
                for (int i = 0; i < s->n; ++i) qa_nh_iter(s, i);
                tcn[tid] = 0;
                /* static chunks are contiguous and ordered by thread id, so
                   concatenating per-thread candidates in thread order gives the
                   serial free-pair order */
#pragma omp for schedule(static)
                for (int64_t k = 0; k < s->n_fp; ++k) {
                    qa_cand c;
                    if (qa_sift_iter(s, k, &c)) {
                        GROW(tc[tid], tcn[tid], tcc[tid], qa_cand);
                        tc[tid][tcn[tid]++] = c;
                    }
                }
            }
            /* reduce_vf: reduce_vf.cpp:4-11 */
            for (int k = 0; k < XMD_NUM_TERMS; ++k) {
                if (V[k] != 0.0) {
#pragma omp atomic update
                    s->V[k] += V[k];
                }
            }
            for (size_t q = 0; q < n3; ++q) {
#pragma omp atomic update
                s->F[q] += F[q];
            }
#pragma omp barrier
#pragma omp master
            {
                if (p->on[XMD_TERM_QA]) {
                    s->n_cand = 0;
                    for (int t = 0; t < nt; ++t)
                        for (int64_t q = 0; q < tcn[t]; ++q) {
                            GROW(s->cand, s->n_cand, s->cap_cand, qa_cand);
                            s->cand[s->n_cand++] = tc[t][q];
                        }
                    qa_accept(s);
                    int64_t n_before = s->n_cont;
                    for (int64_t k = 0; k < n_before; ++k) qa_contact_transition(s, k);
                }
                lj_wall_phase(s);
                if (p->langevin_on) lang_pc(s);
                ensure_nl(s);
            }
#pragma omp barrier
        }
    }
    for (int t = 0; t < nt; ++t) free(tc[t]);
    free(tc); free(tcn); free(tcc); free(tF);
    return 0;
#else
    (void)nthreads;
    return xo_step(s, nsteps);
#endif
}

/* compute_total_energy (total_energy.cpp:4-11), compute_gyration_radius
 * (gyration.cpp:4-19), active native contacts (report_structure.cpp:85). */
int xo_observables(xo_sys *s, double *E, double *K, double *Rg, double *Q) {
    double V[XMD_NUM_TERMS];
    xo_eval_forces(s, NULL, V);
    double Vt = 0.0;
    for (int k = 0; k < XMD_NUM_TERMS; ++k) Vt += V[k];
    double K_ = 0.0;
    for (int i = 0; i < s->n; ++i) K_ += 0.5 * 1.0 * nsq(ld(s->v, i));
    v3 com = mk(0, 0, 0);
    double tm = 0.0;
    for (int i = 0; i < s->n; ++i) { com = add(com, ld(s->r, i)); tm += 1.0; }
    com = scl(1.0 / tm, com);
    double g = 0.0;
    for (int i = 0; i < s->n; ++i) g += nsq(sub(ld(s->r, i), com));
    double act = 0.0;
    double thr = s->p.go_active_threshold * pow(2.0, -1.0 / 6.0);
    for (int k = 0; k < s->n_nat; ++k) {
        double d = nrm(sub(ld(s->r, s->nat[k].i1), ld(s->r, s->nat[k].i2)));
        if (d < thr * s->nat[k].d) act += 1.0;
    }
    if (E) *E = Vt + K_;
    if (K) *K = K_;
    if (Rg) *Rg = sqrt(g / s->n);
    if (Q) *Q = s->n_nat ? act / s->n_nat : 0.0;
    return 0;
}

int xo_counts(const xo_sys *s, int64_t *c) {
    int64_t live_fp = 0, live_c = 0;
    for (int64_t k = 0; k < s->n_fp; ++k) live_fp += !s->fp[k].vacant;
    for (int64_t k = 0; k < s->n_cont; ++k) live_c += !s->cont[k].vacant;
    c[0] = s->n_go; c[1] = s->n_pauli; c[2] = s->n_es; c[3] = live_fp;
    c[4] = s->n_fp; c[5] = live_c; c[6] = s->n_cont; c[7] = s->n_rebuilds;
    return 0;
}
int xo_qa_contacts(const xo_sys *s, int32_t cap, int32_t *out4, double *ref_time) {
    int32_t m = 0;
    for (int64_t k = 0; k < s->n_cont; ++k) {
        if (s->cont[k].vacant) continue;
        if (m < cap) {
            out4[4 * m] = s->cont[k].i1; out4[4 * m + 1] = s->cont[k].i2;
            out4[4 * m + 2] = s->cont[k].type; out4[4 * m + 3] = s->cont[k].status;
            if (ref_time) ref_time[m] = s->cont[k].ref_time;
        }
        ++m;
    }
    return m;
}
int xo_free_pairs(const xo_sys *s, int32_t cap, int32_t *out2) {
    int32_t m = 0;
    for (int64_t k = 0; k < s->n_fp; ++k) {
        if (s->fp[k].vacant) continue;
        if (m < cap) { out2[2 * m] = s->fp[k].i1; out2[2 * m + 1] = s->fp[k].i2; }
        ++m;
    }
    return m;
}
int xo_nl_pairs(const xo_sys *s, int64_t cap, int32_t *out2) {
    for (int64_t k = 0; k < s->n_nl && k < cap; ++k) {
        out2[2 * k] = s->nl[k].i1;
        out2[2 * k + 1] = s->nl[k].i2;
    }
    return (int)s->n_nl;
}
int xo_sync(const xo_sys *s, int8_t *out) {
    memcpy(out, s->sync, 4 * (size_t)s->n);
    return 0;
}
int xo_cutoffs(const xo_sys *s, double *out3) {
    out3[0] = s->max_cutoff;
    out3[1] = s->pad_req;
    out3[2] = s->req_r;
    return 0;
}
