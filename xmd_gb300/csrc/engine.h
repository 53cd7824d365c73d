// engine.h - host-side state of one engine context.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/xmd_gpu.h"
#include "types.h"

namespace xmdg {

// bead flags (bflags)
enum : uint32_t {
    BF_TETH = 1u,  // bond (i, i+1)
    BF_ANG = 2u,   // angle (i-1, i, i+1)
    BF_DIH = 4u,   // dihedral (i-1, i, i+1, i+2)
    BF_CHIR = 32u, // chiral quad (i-1, i, i+1, i+2)
    BF_PREV = 8u,  // i-1 is the previous bead of the same chain
    BF_NEXT = 16u, // i+1 is the next bead of the same chain
    BF_HANG = 64u, // heuristic angle (i-1, i, i+1); type in bits 8-11
    BF_HDIH = 128u, // heuristic dihedral (i-1, i, i+1, i+2); type in bits 12-15
    BF_AFM = 65536u // the bead is pulled by AFM tips; their slot in bits 17-31
};
constexpr int BF_HANG_SHIFT = 8, BF_HDIH_SHIFT = 12, BF_AFM_SHIFT = 17;
constexpr int AFM_MAX_TIPS = 1 << 15;

// one (bead, LJ attractive wall) pair: lj_attr_pair{status, joint_r, ref_t}
// (walls/lj_attr.h); status 0 = free, 1 = forming or formed, 2 = breaking
struct LjWallState {
    double jx, jy, jz, ref_t;
    int status, pad_;
};

// the AFM tips on one bead: a velocity tip (vel_afm_tip{res_idx, afm_orig,
// afm_vel}, velocity_afm.h) and the sum of its force tips
// (force_afm_tip{res_idx, pull_force}, force_afm.h)
struct AfmTip {
    double ox, oy, oz, vx, vy, vz;
    double fx, fy, fz;
    int has_vel, pad_;
};

// per-replica device record
struct RepDev {
    BoxD box;
    double pad, req_r, noise_sd;
    double es_min_inv, pauli_min_inv, qa_min_inv, pid_min_inv;
    // squared-distance forms of the list tests: s < s_req <=> sqrt(s) < req_r,
    // s < s_pa <=> 1/sqrt(s) > pauli_min_inv, etc. (correctly rounded FP64)
    double s_req, s_pa, s_es, s_qa, s_pid;
    double s_ss;             // disulfide list: s < s_ss <=> r < 2 nat_r + pad (native_ss.cpp:15)
    double t;
    int begin, n;
    int cell_off, cell_budget;
    int per[3];
    int dims[3];             // cells along periodic axes
    double lo[3], cs[3];     // bounding-box minimum and 1/cell edge along open axes
    int hashed;              // cells hashed into the bucket budget
    int tile;                // Verlet build by whole-replica tiles (no cell grid)
    float pre2;              // squared FP32 pre-filter radius of the Verlet build
    double band_m;           // FP32 distance error bound of the cell build
    float band_lo[5], band_hi[5];   // cell build: FP32 bands of the list radius, r_excl + pad, 2D + pad,
                                    // QA radius + pad, PID cutoff + pad
    float band_mf;           // band_m rounded up to FP32
    int first, rebuild;
    int chunk_off, nchunk;   // tile-build chunks of the replica in Dev::chunks
    int active;              // slot holds a placed replica
    int fault;               // a bead's force was non-finite: the replica is frozen
    long long steps_left;    // steps this replica still takes (-1: no bound)
    unsigned long long maxdisp;
    unsigned long long rebuilds;
    // quasi-adiabatic lists: free pairs [fp_off, fp_off + fp_n) of capacity
    // fp_cap, contacts [ct_off, ct_off + ct_n) of capacity ct_cap
    int fp_off, fp_cap, fp_n;
    int qa_bchunk_off, qa_nbchunk;   // chunks of QA_BCHUNK beads in QaDev::bchunk
    int ct_off, ct_cap, ct_n;
    int qa_removed;          // contacts removed at this step (k_qa_trans; k_qa_refree clears it)
    int afm;                 // some bead of the replica is pulled by an AFM tip
};

constexpr int QA_REF_CAP = 16;   // contacts per bead (valence bounds it by 10)
constexpr int QA_TMP_CAP = 256;  // free-pair partners j > i per bead at a rebuild
constexpr int QA_FP_PER_BEAD = 96;   // free-pair slots per bead of a replica (+256)
constexpr int QA_CT_PER_BEAD = 8;    // contact slots per bead of a replica (+256)
constexpr int QA_SIFT = 256;         // free-pair slots per block of the candidate sift
constexpr int QA_BCHUNK = 1024;      // beads per chunk of the free-pair re-listing

// device record of the quasi-adiabatic state
struct QaDev {
    float *nh;                   // [6][N]: n then h (precompute_nh.cpp:12-20) to FP32 accuracy
    int32_t *sync;               // [N] packed int8 x4: back | side_all | side_polar | side_hydrophobic
    int32_t *ref_cnt, *ref;      // [N], [QA_REF_CAP][N] contact slots per bead
    int32_t *tmp_cnt, *tmp;      // [N], [QA_TMP_CAP][N] partners collected at a rebuild
    int32_t *tmp_off;            // [N] offset of a bead's partners within its chunk
    int2 *bchunk;                // (replica, first bead) of each chunk of QA_BCHUNK beads
    int32_t *bcsum, *bcbase;     // per chunk: partners, first free-pair slot
    int nbchunk;
    int32_t *fp_i1, *fp_i2, *fp_rep;   // free-pair slots
    uint8_t *fp_vac;
    int32_t *cand_type, *cand_d1, *cand_d2;   // per free-pair slot, 0 = not a candidate
    int32_t *cand_list, *cand_blk;   // per sift block of QA_SIFT slots: its candidates in slot order, their count
    int32_t *ct_i1, *ct_i2, *ct_type, *ct_d1, *ct_d2;
    uint8_t *ct_status, *ct_vac;
    uint8_t *ct_rm;              // removed at this step (re-freed by k_qa_refree)
    int32_t *ct_rep;             // contact slot -> replica owning it
    double *ct_ref;
    const double *req_min_dist;  // [404] by contact type (main.cpp:681-697)
    const double *ss_depth, *ss_rmin, *ss_rmax;   // [400] ss potentials (lj_variants.cpp)
    const int32_t *ptype;        // [20] polarization
    int fp_total, ct_total;
    double min_cos_hr, min_cos_hh, max_cos_nr;
    // a squared distance above which no contact type passes the formation
    // distance test (the largest req_min_dist, widened by 1e-9)
    double req_out2;
    // FP32 forms of the sift's thresholds (the gate widened by 1e-4)
    float req_out2_f, min_cos_hr_f, min_cos_hh_f, max_cos_nr_f;
};

// everything a kernel needs, passed by value
struct Dev {
    int N, R, nl_cap;
    double4_32a *pos[2];        // x, y, z, charge; double-buffered
    double *yh;             // [15][N]: y1x y1y y1z y2x ... y5z
    double4_32a *orig;          // positions at the last list rebuild
    double *F;              // [3N] force output of eval
    double *Vrep;           // [R][XMD_NUM_TERMS] energies of eval
    int32_t *rep_of;        // bead -> replica
    uint32_t *bflags;
    int32_t *chain, *seq;
    uint8_t *atype;
    double *teth_r0, *ang_t0, *dih_p0;
    double2 *chir;          // (nat_factor, nat_chir) per centre i2 of a chiral quad
    float2 *chir_f32;       // the same in FP32 (mixed path)
    const double *heur_ang;     // [9][7] heuristic angle coefficients a0..a6
    const double *heur_dih;     // [9][6] heuristic dihedral coefficients c0..c5
    const float *heur_dih_f;    // the same in FP32 (mixed path)
    AfmTip *afm;            // AFM tips, one slot per pulled bead
    double *wall;           // [2][XMD_MAX_WALLS][6] planes (origin, normal): solid, then LJ attractive
    LjWallState *ljw;       // [n_ljw][N] LJ attractive wall pairs
    double *fext;           // [3N] external force of the step (k_ext: AFM, walls)
    int32_t *ss_start, *ss_end, *ss_j;   // native disulfide partners per bead (CSR, both directions)
    uint8_t *ss_on;         // in the list of the last rebuild (update_nat_ssbonds, native_ss.cpp:8-19)
    float4 *bond_f;         // (r0, theta0, phi0) in FP32 for the mixed path
    int32_t *nat_start, *nat_end, *nat_j;   // natives of bead i: [nat_start[i], nat_end[i])
    double *nat_d;
    float *nat_df;          // nat_d in FP32 for the mixed path
    double *nat_T;          // Go-list threshold 2 r_nat + pad of each entry (go.cpp:11-22)
    double *nat_S;          // its squared form: s < nat_S <=> sqrt(s) < nat_T
    uint8_t *nat_on;
    int32_t *nl_row, *nl_cnt;
    int32_t *cell_cnt, *cell_start, *cell_fill, *cell_items, *bead_cell;
    float4 *cell_pos;       // bucket-sorted FP32 coordinates (+ bead index bits)
    int32_t *bead_slot;     // bead -> its slot in cell_pos
    int2 *cell_cs;          // (chain, sequence index) of each slot of cell_pos
    int32_t *cell_rep;      // bucket of the pool -> replica owning it (-1: free)
    int ncells;             // buckets in the pool
    uint64_t *rng;          // per-bead generator state
    uint64_t *jump;         // [R][16][16] nibble tables of the GF(2) jump (4 N_r draws)
    RepDev *rep;
    int *any_rebuild;       // [0]: some replica flagged at the last check; [1..3]: gate
    // gate of the graphs that rebuild on the host (halted, steps done,
    // budget): while gate[0] is set every step kernel returns at once
    int *gate;
    int *status;            // device error word
    unsigned long long *ctr;  // [0]: list-rebuild passes launched
    int2 *chunks;           // (replica, first bead) of each tile-build block
    int nchunks;
    int *work;              // chunks of the replicas flagged at the last skin check
    int *nwork;             // number of entries in `work`
    int any_cell;           // some replica uses the cell-grid build
    uint8_t *blk_on;        // force blocks (FB beads) holding at least one placed bead
    int qa_on;
    QaDev qa;
    // pseudo-improper dihedral potential: per bead its bundles' forces on
    // itself, on its previous and on its next bead ([3][3N], k_pid), and the
    // side-chain LJ table by pair type ([400] depth, r_min, r_max)
    double *pid_f;
    const double *pid_sd, *pid_smin, *pid_smax;
};

struct RepHost {
    bool in_use = true;      // slot taken (false after remove)
    bool placed = false;     // static data and state are on the device
    int n = 0;
    std::vector<int32_t> chain, seq;
    std::vector<uint8_t> atype;
    double cell[3] = {0, 0, 0};
    double temperature = 0;
    uint64_t seed = 0;
    std::vector<double> teth_r0, ang_t0, dih_p0;   // per centre, NaN = absent
    std::vector<double> chir_f, chir_n;            // chirality per centre (i2), NaN = absent
    std::vector<int32_t> ss_i1, ss_i2;             // native disulfides
    std::vector<int8_t> hang_t, hdih_t;            // heuristic angle / dihedral type per centre, -1 = absent
    std::vector<int32_t> vafm_i, fafm_i;           // AFM tips: pulled bead
    std::vector<double> vafm_o, vafm_v, fafm_F;    // [3 per tip] origin (NaN: placed position), velocity, force
    int afm_off = 0, afm_len = 0;       // AFM tip slots
    std::vector<int32_t> nat_i1, nat_i2;
    std::vector<double> nat_d;
    std::vector<double> r, v;                      // initial state
    bool have_state = false;
    int begin = 0;
    int nat_off = 0, nat_len = 0;       // native CSR entries
    int ss_off = 0, ss_len = 0;         // disulfide CSR entries
    int cell_off = 0, cell_len = 0;     // cell buckets (cell-grid build)
    int chunk_off = 0, chunk_len = 0;   // tile-build chunks
    int fp_off = 0, fp_len = 0, ct_off = 0, ct_len = 0;   // quasi-adiabatic slots
    long long steps_left = -1;
    bool staged = false;     // device data uploading on the side stream, not yet active
};

// first-fit allocator of index ranges [0, n)
class RangeAlloc {
public:
    void init(int n) {
        free_.clear();
        if (n > 0) free_[0] = n;
    }
    int alloc(int n) {
        if (n <= 0) return 0;
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n) {
                int s = it->first, l = it->second;
                free_.erase(it);
                if (l > n) free_[s + n] = l - n;
                return s;
            }
        return -1;
    }
    void release(int s, int n) {
        if (n <= 0) return;
        auto it = free_.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && s + n == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    int largest() const {
        int m = 0;
        for (auto &kv : free_) m = std::max(m, kv.second);
        return m;
    }

private:
    std::map<int, int> free_;   // start -> length
};

class Engine {
public:
    explicit Engine(const xmd_params &p);
    ~Engine();

    xmd_params params;
    std::vector<RepHost> reps;
    bool finalized = false;
    int nl_cap = 64;

    int add_replica(int n, const int32_t *chain, const int32_t *seq, const uint8_t *atype,
                    const double cell[3], double temperature, uint64_t seed);
    // dynamic membership: fixed capacities, replicas placed and removed
    // between steps (slots and device ranges are reused)
    void reserve(int beads, int replicas, int natives);
    void remove_replica(int rep);
    void set_steps(int rep, long long nsteps);
    void steps_left(long long *out);   // per replica slot, -2 for a free slot
    void place_now(int rep);           // place a replica now (XMD_ERR_CAPACITY: no room yet)
    // Overlapped placement (dynamic contexts): stage() allocates the
    // replica's device ranges and uploads its data on a side stream while
    // earlier work runs; activate_staged() then makes every staged replica
    // live on the step stream, ordered after those uploads.  A staged replica
    // takes no step before it is activated.
    void stage(int rep);               // XMD_ERR_CAPACITY (length_error): no room yet
    void activate_staged();
    // step() in two halves: launch the steps, then wait for them and report
    void step_async(int nsteps);
    void step_wait();
    int capacity_replicas() const { return cap.reps; }
    // device memory this context holds (its allocations, rows at their current capacity)
    size_t device_bytes() const { return alloc_bytes; }
    // a non-finite force freezes its replica (steps_left reports -3) instead
    // of failing the step, so a serving loop can retire it alone
    void set_isolate_faults(bool on) { isolate_faults = on; }
    // launch shapes (the trajectory does not depend on them), chosen by
    // autotune() or set directly
    struct Tune {
        int fb = 64;             // beads per step-kernel block: 32, 64 or 128
        int tile_per_sm = 0;     // resident tile-build blocks per SM (0: as many as fit)
        int graph_steps = 16;    // steps per captured graph: 8, 16 or 32
        int lpb = 4;             // threads per bead in the step kernel: 1, 2 or 4
    };
    Tune tuning() const { return tune; }
    void set_tuning(const Tune &t);
    // times every candidate shape on a clone of this context (same replicas,
    // same starting state) and keeps the fastest; this context's state is
    // not touched.  ms_out (optional) receives the best time per step.
    Tune autotune(int steps, double *ms_out = nullptr);
    Tune tune;
    void set_tethers(int rep, int n, const int32_t *i1, const int32_t *i2, const double *d);
    void set_angles(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                    const double *th);
    void set_dihedrals(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                       const int32_t *i4, const double *ph);
    void set_native(int rep, int n, const int32_t *i1, const int32_t *i2, const double *d);
    void set_chirals(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3, const int32_t *i4,
                     const double *factor, const double *chir);
    void set_ssbonds(int rep, int n, const int32_t *i1, const int32_t *i2);
    void set_heuristic_angles(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3);
    void set_velocity_afm(int rep, int n, const int32_t *bead, const double *orig, const double *vel);
    void set_force_afm(int rep, int n, const int32_t *bead, const double *F);
    void set_walls(int kind, int n, const double *origin, const double *normal);
    std::vector<double> walls[2];           // planes (origin, normal) per kind
    void set_heuristic_dihedrals(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                                 const int32_t *i4);
    void set_state(int rep, const double *r, const double *v);
    void set_history(int rep, const double *y, double t, uint64_t rng);
    void get_state(int rep, double *r, double *v, double *t);
    void get_history(int rep, double *y, double *t, uint64_t *rng);
    // whole mutable state of a replica (positions, history, generators, lists,
    // quasi-adiabatic state) for an exact resume; restore into the same slot
    // of a context built the same way
    size_t snapshot_size(int rep);
    void snapshot(int rep, void *buf, size_t bytes);
    void restore(int rep, const void *buf, size_t bytes);
    uint64_t topo_hash(int rep) const;
    // cap_rows >= 0: size of a snapshot whose Verlet rows have that capacity
    size_t snapshot_io(int rep, unsigned char *buf, size_t bytes, bool save, int cap_rows = -1);
    void resize_rows(int ncap);
    void eval_forces(int rep, double *F, double *V);
    void step(int nsteps);
    void observables(int rep, double *E, double *K, double *Rg, double *Q);
    int device_status();
    void sync();
    void upload_history_all(const double *y);
    void download_positions_all(double *r);
    void download_history_all(double *y);
    cudaStream_t get_stream() const { return stream; }
    void stats(int64_t *out);
    void set_kernel_timing(bool on);
    int qa_contacts(int rep, int cap, int32_t *out4, double *ref_time);
    int verlet_pairs(int rep, int cap, int32_t *out2, uint8_t *flags);
    void qa_sync(int rep, int8_t *out);
    void kernel_times(double *force_ms, int64_t *nf, double *rebuild_ms, int64_t *nr);
    void use_device() const;

private:
    Dev d{};
    int cur = 0;                 // which pos buffer is current
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    size_t alloc_bytes = 0;   // device memory held by this context
    int *h_any = nullptr;        // pinned
    TermP tp{};
    int64_t launches = 0, md_steps = 0;
    double *staging = nullptr;   // packed host-layout buffer [18 N]
    bool timing = false;
    bool isolate_faults = false;
    void launch_force(int mode, int c);
    int tile_sms = 1, tile_max_per_sm = 1;     // for the tile build's resident grid
    // the QA sift's fixed grid: four blocks per SM, each taking at most
    // QA_SIFT groups of free-pair slots
    int sift_grid() const {
        const int ng = (d.qa.fp_total + QA_SIFT - 1) / QA_SIFT;
        return std::max(4 * tile_sms, (ng + QA_SIFT - 1) / QA_SIFT);
    }
    // graphs rebuild with a plain row-build node instead of an IF node
    bool plain_rebuild() const { return any_tile && !any_cell && !d.qa_on; }
    // graphs without rebuild nodes: a flagged check halts the graph's
    // remaining steps and the host rebuilds (static contexts with cell-path
    // replicas or the quasi-adiabatic term, where the rebuild is a chain of
    // kernels and rebuilds are rare)
    bool gated_graphs() const { return !plain_rebuild() && !dynamic; }
    // the QA transitions' fixed grid (groups of 256 contact slots)
    int trans_grid() const {
        const int ng = (d.qa.ct_total + 255) / 256;
        return std::max(4 * tile_sms, (ng + 255) / 256);
    }
    std::vector<cudaEvent_t> ev_force, ev_rebuild;   // start/stop pairs
    size_t n_ev_force = 0, n_ev_rebuild = 0;

    void record(std::vector<cudaEvent_t> &pool, size_t &n);
    void launch_force_step();

    // graph-captured step chunks, per (precision, kind: gated or with IF
    // rebuild nodes, starting buffer, steps)
    struct GraphSet {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
    };
    std::map<int, GraphSet> graphs;
    bool use_graphs = true;
    bool auto_grow = true;       // grow Verlet rows instead of failing
    int cond_graphs_left = 0;    // gated contexts: IF-node graphs to run before the next gated one
    cudaGraphExec_t graph_for(int start_cur, bool gated, int len);
    bool any_cell = false, any_tile = false;   // which Verlet builds the replicas use
    size_t tile_smem = 0;                      // dynamic shared memory of k_nl_tile
    int tile_grid = 1;                         // resident blocks of k_nl_tile over all SMs
    void add_rebuild_nodes(cudaGraph_t body, int cn);
    bool grow_rows(double frac);
    void drop_graphs();

    struct Caps {
        int beads = 0, reps = 0, nat = 0, cells = 0, chunks = 0, fp = 0, ct = 0, qab = 0, ss = 0, afm = 0;
    } cap;
    bool dynamic = false;
    RangeAlloc a_beads, a_nat, a_cells, a_chunks, a_fp, a_ct, a_ss, a_afm;
    int qa_bchunk_next = 0;   // next free chunk of the QA re-listing (static contexts)
    std::vector<int32_t> owner_h;              // bead slot -> replica (or -1)
    void allocate();
    // the staged replicas' activation data: bead -> replica, bucket ->
    // replica and the replica record, written on the step stream
    struct Staged {
        int k = 0;
        std::vector<int32_t> rep_of, cell_rep;
        RepDev rd{};
    };
    std::vector<Staged> staged_reps;
    cudaStream_t ustream = nullptr;            // side stream of staged uploads
    cudaEvent_t ev_staged = nullptr, ev_removed = nullptr;
    void place(int k, Staged *st = nullptr);
    void place_pending();
    void ready();                              // allocated, every replica placed
    void ready_alloc();
    void update_blocks(int b0, int b1, bool wait = true);
    void *dalloc(size_t bytes);
    void finalize();
    void release();
    void derive_rep(int r, RepDev &rd);
    void ensure_nl();
    void launch_rebuild();
    void check_status(const char *where);
    void upload_state(int rep);
    void upload_state_data(int rep, cudaStream_t us);
};

std::string &last_error();
uint64_t rng_jump(uint64_t state, uint64_t n_draws);
int verlet_pairs_noalloc(const double *d_r, const int32_t *d_chain, const int32_t *d_seq, int32_t n,
                         const double cell[3], double cutoff, int32_t *d_pairs, int32_t cap, int32_t *d_count,
                         void *stream);

}  // namespace xmdg
