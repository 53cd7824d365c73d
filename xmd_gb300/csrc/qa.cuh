// qa.cuh - quasi-adiabatic contacts on the device (included by engine.cu).
//
// Per replica the reference keeps three tombstoned sets (free pairs,
// candidates, contacts; gentypes set<T>, _templates/set.h.j2:47-104) whose
// SLOT ORDER decides which candidate wins a shared valence
// (process_candidates.cpp:4-29) and where re-freed pairs land
// (process_contacts.cpp:48-55).  Here each replica owns contiguous regions of
// free-pair and contact slots; slot order is kept by ordered block-wide
// compaction, and the order-dependent greedy acceptance decides the compacted
// candidates of a replica in dependency rounds (k_qa_step).  Geometry that
// feeds a yes/no decision is evaluated with explicitly rounded FP64 operations
// so the decisions match an uncontracted CPU build.
#pragma once

namespace xmdg {

enum : int { QA_FORMING = 0, QA_BREAKING = 1 };

// ---- exactly rounded vector helpers (no FMA contraction) -------------------
struct D3 { double x, y, z; };
__device__ __forceinline__ D3 d3sub(D3 a, D3 b) { return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ double d3dot(D3 a, D3 b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ D3 d3cross(D3 a, D3 b) {
    return {__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
            __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ D3 d3scl(double s, D3 a) { return {__dmul_rn(s, a.x), __dmul_rn(s, a.y), __dmul_rn(s, a.z)}; }
// unit(): norm_inv(e) * e (vec3.h:154, 357)
__device__ __forceinline__ D3 d3unit(D3 a) { return d3scl(__ddiv_rn(1.0, __dsqrt_rn(d3dot(a, a))), a); }
__device__ __forceinline__ D3 d3of(double4_32a p) { return {p.x, p.y, p.z}; }
// box::r_uv with explicit rounding
__device__ __forceinline__ D3 d3ruv(const BoxD &b, double4_32a u, double4_32a w) {
    double d[3] = {__dsub_rn(w.x, u.x), __dsub_rn(w.y, u.y), __dsub_rn(w.z, u.z)};
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = __dsub_rn(d[a], __dmul_rn(b.cell[a], rint(__dmul_rn(d[a], b.cell_inv[a]))));
    return {d[0], d[1], d[2]};
}

// packed valence counters
__device__ __forceinline__ int sbyte(int32_t v, int k) { return (int)(int8_t)((v >> (8 * k)) & 0xff); }
__device__ __forceinline__ bool sync_ok_after(int32_t s, int32_t dpk) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (sbyte(s, k) - sbyte(dpk, k) < 0) return false;
    return true;
}
__device__ __forceinline__ int32_t pack4(int a, int b, int c, int e) {
    return (a & 0xff) | ((b & 0xff) << 8) | ((c & 0xff) << 16) | ((e & 0xff) << 24);
}

// the potential of contact type t: ljs[t-1] through lj_variants::operator[]
// (lj_variants.h:16-23); sink_lj(lj) has r_max = r_min (sink_lj.h:21-22)
__device__ __forceinline__ void qa_lj(const TermP &p, const QaDev &q, int type, double *depth, double *rmin,
                                      double *rmax) {
    int k = type - 1;
    if (k == 0) { *depth = p.lj_bb_depth; *rmin = *rmax = p.lj_bb_r_min; }
    else if (k <= 2) { *depth = p.lj_bs_depth; *rmin = *rmax = p.lj_bs_r_min; }
    else { *depth = q.ss_depth[k - 3]; *rmin = q.ss_rmin[k - 3]; *rmax = q.ss_rmax[k - 3]; }
}

// precompute_nh::iter (precompute_nh.cpp:12-20) from three positions
__device__ __forceinline__ void qa_nh(double4_32a rp, double4_32a rc, double4_32a rn, D3 *n, D3 *h) {
    D3 v1 = d3sub(d3of(rc), d3of(rp)), v2 = d3sub(d3of(rn), d3of(rc));
    *n = d3unit(d3sub(v2, v1));
    *h = d3unit(d3cross(v2, v1));
}
// the same to FP32 accuracy: bond vectors, their difference and their cross
// product in float-float from split positions (within ~2^-44 of the exact
// values however straight the chain), normalised in FP32; each component
// is within ~3e-7 of the FP64 unit vector's
__device__ __forceinline__ V3<float> unit_f(V3<float> a) {
    const float s = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return V3<float>{a.x * s, a.y * s, a.z * s};
}
__device__ __forceinline__ void qa_nh_f(double4_32a rp, double4_32a rc, double4_32a rn, V3<float> *n, V3<float> *h) {
    const P2 sp = split_p(rp), sc = split_p(rc), sn = split_p(rn);
    const V3<FF> v1{ff_diff(sp.x, sc.x), ff_diff(sp.y, sc.y), ff_diff(sp.z, sc.z)};
    const V3<FF> v2{ff_diff(sc.x, sn.x), ff_diff(sc.y, sn.y), ff_diff(sc.z, sn.z)};
    const V3<FF> dv{ff_sub(v2.x, v1.x), ff_sub(v2.y, v1.y), ff_sub(v2.z, v1.z)};
    const V3<FF> x = ff_cross(v2, v1);
    *n = unit_f(V3<float>{dv.x.h, dv.y.h, dv.z.h});
    *h = unit_f(V3<float>{x.x.h, x.y.h, x.z.h});
}

// ---- block-wide helpers (blockDim.x == 1024) ------------------------------------
// Exclusive prefix of an int over the block; returns the total.
__device__ __forceinline__ int block_exscan(int v, int *out, int *s_warp) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = s_warp[lane], sx = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, sx, o);
            if (lane >= o) sx += y;
        }
        s_warp[lane] = sx - s;
        if (lane == 31) s_warp[32] = sx;
    }
    __syncthreads();
    *out = s_warp[w] + x - v;
    int total = s_warp[32];
    __syncthreads();
    return total;
}

// ---- sift_candidates::iter (sift_candidates.cpp:15-77), one thread per slot ----
// Each block also lists its candidates in slot order (cand_list, cand_blk),
// so the acceptance visits candidates instead of every free-pair slot.
//
// The decisions are taken in FP32 where they are certain: the pair vector
// from split positions (float-float differences, error <= 2^-24 of each
// component), its unit vector, and n, h to FP32 accuracy (qa_nh_f, written by
// the step kernel); every dot product of unit vectors is then within 2e-6 of
// its FP64 value and the squared distance within 1e-6 of it (relative).  A pair whose value lies
// within QA_BAND of any threshold it is tested against is decided again from
// scratch in FP64 with explicit rounding (the reference's operations), so the
// candidate set is exactly the FP64 one.
constexpr float QA_BAND = 1.0e-5f;

// the FP64 decision (the reference's arithmetic, no contraction): the type
// and the five geometric tests (back1, back2, bb, side1, side2 in bits 0-4)
__device__ __noinline__ int qa_sift_fp64(const Dev &d, const RepDev &rp, int i1, int i2, int cur, int *tests) {
    const QaDev &q = d.qa;
    const double4_32a *pos = d.pos[cur];
    const D3 r12 = d3ruv(rp.box, pos[i1], pos[i2]);
    *tests = 0;
    if (!(d3dot(r12, r12) <= q.req_out2)) return 0;
    const double r12_rn = __ddiv_rn(1.0, __dsqrt_rn(d3dot(r12, r12)));
    const D3 u = d3scl(r12_rn, r12);
    // n and h of both beads in FP64, as precompute_nh computes them
    D3 n1{0.0, 0.0, 0.0}, h1 = n1, n2 = n1, h2 = n1;
    const uint32_t both = BF_PREV | BF_NEXT;
    if ((d.bflags[i1] & both) == both) qa_nh(pos[i1 - 1], pos[i1], pos[i1 + 1], &n1, &h1);
    if ((d.bflags[i2] & both) == both) qa_nh(pos[i2 - 1], pos[i2], pos[i2 + 1], &n2, &h2);
    const bool back1 = fabs(d3dot(h1, u)) > q.min_cos_hr;
    const bool back2 = fabs(d3dot(h2, u)) > q.min_cos_hr;
    const bool bb_extra = fabs(d3dot(h1, h2)) > q.min_cos_hh;
    const bool side1 = d3dot(n1, u) < q.max_cos_nr;
    const bool side2 = -d3dot(n2, u) < q.max_cos_nr;
    const int a1 = d.atype[i1], a2 = d.atype[i2];
    int type = 0;
    if (back1 && back2 && bb_extra) type = 1;
    else if (back1 && side2) type = 2;
    else if (side1 && back2) type = 3;
    else if (side1 && side2) type = 4 + a1 + XMD_NUM_AA * a2;
    if (type != 0 && 1.0 > __dmul_rn(r12_rn, q.req_min_dist[type])) type = 0;
    *tests = (back1 ? 1 : 0) | (back2 ? 2 : 0) | (bb_extra ? 4 : 0) | (side1 ? 8 : 0) | (side2 ? 16 : 0);
    return type;
}

__device__ __forceinline__ V3<float> nh_f(const QaDev &q, size_t N, int i, int off) {
    return V3<float>{q.nh[(off + 0) * N + i], q.nh[(off + 1) * N + i], q.nh[(off + 2) * N + i]};
}
// x > T (or, with less, x < T) decided in FP32; *unsure when x is within
// the band of T
__device__ __forceinline__ bool cmp_band(float x, float T, bool less, bool *unsure) {
    *unsure |= fabsf(x - T) <= QA_BAND;
    return less ? x < T : x > T;
}

// one group of QA_SIFT free-pair slots: the decisions, then the ordered
// compaction of the group's candidates into its cand_list segment
__device__ __forceinline__ void qa_sift_group(const Dev &d, const TermP &p, int cur, int sg) {
    const int slot = sg * QA_SIFT + threadIdx.x;
    const QaDev &q = d.qa;
    bool live = slot < q.fp_total;
    const int r = live ? q.fp_rep[slot] : 0;
    const RepDev &rp = d.rep[r];
    live = live && slot - rp.fp_off < rp.fp_n;
    int type = 0, tests = 0;
    int32_t d1p = 0, d2p = 0;
    int i1 = 0, i2 = 0;
    if (live && !q.fp_vac[slot]) {
        i1 = q.fp_i1[slot];
        i2 = q.fp_i2[slot];
        const double4_32a *pos = d.pos[cur];
        const bool per = (rp.per[0] | rp.per[1] | rp.per[2]) != 0;
        const PairGeo<float> geo(rp.box, per, pos[i1]);
        const V3<float> r12 = geo.to(pos[i2]);
        const float d2 = r12.x * r12.x + r12.y * r12.y + r12.z * r12.z;
        // beyond every type's formation distance no pair is a candidate (the
        // widened FP32 gate keeps every pair the FP64 gate keeps)
        if (d2 <= q.req_out2_f) {
            const float rn = 1.0f / sqrtf(d2);
            const V3<float> u{r12.x * rn, r12.y * rn, r12.z * rn};
            const size_t N = d.N;
            const V3<float> n1 = nh_f(q, N, i1, 0), n2 = nh_f(q, N, i2, 0);
            const V3<float> h1 = nh_f(q, N, i1, 3), h2 = nh_f(q, N, i2, 3);
            bool unsure = false;
            const bool back1 = cmp_band(fabsf(dot(h1, u)), q.min_cos_hr_f, false, &unsure);
            const bool back2 = cmp_band(fabsf(dot(h2, u)), q.min_cos_hr_f, false, &unsure);
            const bool bb_extra = cmp_band(fabsf(dot(h1, h2)), q.min_cos_hh_f, false, &unsure);
            const bool side1 = cmp_band(dot(n1, u), q.max_cos_nr_f, true, &unsure);
            const bool side2 = cmp_band(-dot(n2, u), q.max_cos_nr_f, true, &unsure);
            const int a1 = d.atype[i1], a2 = d.atype[i2];
            if (back1 && back2 && bb_extra) type = 1;
            else if (back1 && side2) type = 2;
            else if (side1 && back2) type = 3;
            else if (side1 && side2) type = 4 + a1 + XMD_NUM_AA * a2;
            if (type != 0) {
                // r < req_min_dist[type], on squared distances
                const float rq = narrow_f(q.req_min_dist[type]);
                const float rq2 = rq * rq;
                unsure |= fabsf(d2 - rq2) <= QA_BAND * rq2;
                if (!(d2 < rq2)) type = 0;
            }
            tests = (back1 ? 1 : 0) | (back2 ? 2 : 0) | (bb_extra ? 4 : 0) | (side1 ? 8 : 0) | (side2 ? 16 : 0);
            if (unsure) type = qa_sift_fp64(d, rp, i1, i2, cur, &tests);
        }
        if (type != 0) {
            const int a1 = d.atype[i1], a2 = d.atype[i2];
            const int pt2 = q.ptype[a2], pt1 = q.ptype[a1];
            const bool back1 = tests & 1, back2 = tests & 2, side1 = tests & 8, side2 = tests & 16;
            d1p = pack4(back1, side1, side1 && pt2 == 1, side1 && pt2 == 2);
            d2p = pack4(back2, side2, side2 && pt1 == 1, side2 && pt1 == 2);
            if (!sync_ok_after(q.sync[i1], d1p) || !sync_ok_after(q.sync[i2], d2p)) type = 0;
        }
    }
    // only listed candidates are read (k_qa_step)
    if (type != 0) {
        q.cand_type[slot] = type;
        q.cand_d1[slot] = d1p;
        q.cand_d2[slot] = d2p;
    }
    // ordered compaction of the group's candidates
    __shared__ int s_wc[QA_SIFT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, type != 0);
    if (lane == 0) s_wc[w] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
#pragma unroll
    for (int k = 0; k < QA_SIFT / 32; ++k) {
        before += k < w ? s_wc[k] : 0;
        total += s_wc[k];
    }
    if (type != 0) q.cand_list[(size_t)sg * QA_SIFT + before + __popc(bal & ((1u << lane) - 1u))] = slot;
    if (threadIdx.x == 0) q.cand_blk[sg] = total;
    __syncthreads();   // s_wc is reused by the next group
}

// A fixed grid: block b takes groups b, b + G, b + 2G, ... (G blocks), finds
// with one round of parallel loads which of them hold live slots (a
// replica's live slots are a prefix of its region, and the free-pair
// capacity is far above the live count), then sifts only those.  Dealing the
// groups round-robin spreads a replica's live prefix over all blocks, so one
// large replica is sifted by the whole grid.  Groups without a live slot are
// never read (k_qa_step reads the groups of each replica's live range).
__global__ void __launch_bounds__(QA_SIFT, 4) k_qa_sift(Dev d, TermP p, int cur) {
    if (d.gate[0]) return;   // a halted graph step
    const QaDev &q = d.qa;
    const int t = threadIdx.x;
    // the per-bead contact references are listed again at this step's end
    // (k_qa_trans); nothing reads them before that
    for (int k = blockIdx.x * blockDim.x + t; k < d.N; k += gridDim.x * blockDim.x) q.ref_cnt[k] = 0;
    const int ng = (q.fp_total + QA_SIFT - 1) / QA_SIFT, G = gridDim.x;
    const int per = (ng - (int)blockIdx.x + G - 1) / G;   // <= QA_SIFT (the grid is sized for it)
    bool lv = false;
    if (t < per) {
        const int first = (blockIdx.x + t * G) * QA_SIFT, last = min(first + QA_SIFT, q.fp_total) - 1;
        const int r1 = q.fp_rep[first], r2 = q.fp_rep[last];
        const RepDev &a = d.rep[r1];
        lv = first - a.fp_off < a.fp_n;               // the group starts inside r1's live prefix
        if (r2 != r1) lv = lv || d.rep[r2].fp_n > 0;  // r2's region starts inside the group
    }
    __shared__ unsigned s_live[QA_SIFT / 32];
    const unsigned bl = __ballot_sync(0xffffffffu, lv);
    if ((t & 31) == 0) s_live[t >> 5] = bl;
    __syncthreads();
    for (int k = 0; k < per; ++k)
        if ((s_live[k >> 5] >> (k & 31)) & 1u) qa_sift_group(d, p, cur, blockIdx.x + k * G);
}

// ---- acceptance: process_candidates::iter (process_candidates.cpp:10-29) in
// candidate order, one block per replica; the transitions follow in
// k_qa_trans.
//
// The greedy choice is sequential by definition: a candidate is accepted when
// both beads still have the valence it needs after every EARLIER candidate
// was decided.  Only earlier candidates that share a bead with it matter, so
// the block decides in rounds: in each round a pending candidate decides when
// it is the lowest-ordered pending candidate of both its beads (an atomicMin
// per bead into a shared table).  At that moment every earlier candidate on
// its beads has decided and no later one has, so it sees exactly the valences
// the sequential loop would; candidates deciding in one round share no bead.
// The table is hashed (bead mod QA_HASH): two beads in one entry only make
// the later candidate wait a round, and the lowest pending candidate always
// decides, so every round makes progress.  Accepted contacts then take their
// slots in candidate order (an ordered compaction).  A chunk that could
// overflow the replica's contact region runs the plain sequential loop, which
// stops at the first candidate without a slot.
constexpr int QA_HASH = 4096;
__global__ void __launch_bounds__(1024) k_qa_step(Dev d, TermP p, int cur) {
    if (d.gate[0]) return;
    const int r = blockIdx.x, t = threadIdx.x;
    RepDev &rp = d.rep[r];
    const QaDev &q = d.qa;
    __shared__ int s_slots[1024];
    __shared__ int s_warp[33];
    __shared__ int s_first[QA_HASH];
    __shared__ int s_ct_n, s_fp_n, s_err;
    if (t == 0) { s_ct_n = rp.ct_n; s_fp_n = rp.fp_n; s_err = 0; }
    for (int k = t; k < QA_HASH; k += 1024) s_first[k] = INT_MAX;
    __syncthreads();
    const double tnow = rp.t;
    const int fp_off = rp.fp_off, ct_off = rp.ct_off, ct_cap = rp.ct_cap;
    const int fp_n0 = s_fp_n;
    // 1. greedy acceptance in free-pair slot order, over the sift blocks'
    //    ordered candidate lists (slots outside this replica's live range are
    //    skipped: blocks at the edges are shared)
    __shared__ int s_i1[1024], s_i2[1024], s_d1[1024], s_d2[1024], s_ty[1024];
    // each thread takes a contiguous run of the replica's sift blocks, so
    // one block-wide scan orders every candidate
    const int sb0 = fp_off / QA_SIFT, sb1 = (fp_off + fp_n0 + QA_SIFT - 1) / QA_SIFT;
    {
        const int per = (sb1 - sb0 + 1023) / 1024;
        const int b0 = min(sb0 + t * per, sb1), b1 = min(b0 + per, sb1);
        int cnt = 0;
        for (int blk = b0; blk < b1; ++blk) cnt += q.cand_blk[blk];
        int pos;
        const int total = block_exscan(cnt, &pos, s_warp);
        for (int g0 = 0; g0 < total; g0 += 1024) {
            // gather candidates [g0, g0 + 1024) of this round with their data
            if (cnt && pos < g0 + 1024 && pos + cnt > g0) {
                int o = pos;
                for (int blk = b0; blk < b1 && o < g0 + 1024; ++blk) {
                    const int c = q.cand_blk[blk];
                    for (int k = 0; k < c && o < g0 + 1024; ++k, ++o) {
                        if (o < g0) continue;
                        const int s = q.cand_list[(size_t)blk * QA_SIFT + k];
                        const int so = o - g0;
                        const bool mine = s >= fp_off && s < fp_off + fp_n0;
                        s_slots[so] = mine ? s : -1;
                        if (mine) {
                            s_i1[so] = q.fp_i1[s]; s_i2[so] = q.fp_i2[s];
                            s_d1[so] = q.cand_d1[s]; s_d2[so] = q.cand_d2[s]; s_ty[so] = q.cand_type[s];
                        }
                    }
                }
            }
            __syncthreads();
            const int m = min(1024, total - g0);
            if (s_ct_n + m > ct_cap) {
                // the sequential loop (can run out of contact slots)
                if (t == 0) {
                    for (int k = 0; k < m; ++k) {
                        const int s = s_slots[k];
                        if (s < 0) continue;
                        const int i1 = s_i1[k], i2 = s_i2[k];
                        const int32_t d1p = s_d1[k], d2p = s_d2[k];
                        const int32_t y1 = q.sync[i1], y2 = q.sync[i2];
                        if (sync_ok_after(y1, d1p) && sync_ok_after(y2, d2p)) {
                            if (s_ct_n >= ct_cap) { s_err = 1; break; }
                            const int c = ct_off + s_ct_n++;
                            q.ct_i1[c] = i1; q.ct_i2[c] = i2; q.ct_type[c] = s_ty[k];
                            q.ct_status[c] = QA_FORMING; q.ct_ref[c] = tnow; q.ct_vac[c] = 0;
                            q.ct_d1[c] = d1p; q.ct_d2[c] = d2p;
                            q.sync[i1] = y1 - d1p;   // bytes never borrow: each stays >= 0
                            q.sync[i2] = (i2 == i1 ? y1 - d1p : y2) - d2p;
                            q.fp_vac[s] = 1;
                        }
                    }
                }
                __syncthreads();
                continue;
            }
            // rounds: candidate t decides once it is the lowest pending one
            // of both its beads
            bool pend = t < m && s_slots[t] >= 0, acc = false;
            int i1 = 0, i2 = 0;
            int32_t d1p = 0, d2p = 0;
            if (pend) { i1 = s_i1[t]; i2 = s_i2[t]; d1p = s_d1[t]; d2p = s_d2[t]; }
            const int h1 = i1 & (QA_HASH - 1), h2 = i2 & (QA_HASH - 1);
            while (__syncthreads_or(pend)) {
                if (pend) { atomicMin(&s_first[h1], t); atomicMin(&s_first[h2], t); }
                __syncthreads();
                const bool go = pend && s_first[h1] == t && s_first[h2] == t;
                __syncthreads();
                if (pend) { s_first[h1] = INT_MAX; s_first[h2] = INT_MAX; }
                if (go) {
                    const int32_t y1 = q.sync[i1], y2 = q.sync[i2];
                    if (sync_ok_after(y1, d1p) && sync_ok_after(y2, d2p)) {
                        acc = true;
                        q.sync[i1] = y1 - d1p;
                        q.sync[i2] = (i2 == i1 ? y1 - d1p : y2) - d2p;
                    }
                    pend = false;
                }
            }
            // contact slots in candidate order
            int at;
            const int nacc = block_exscan(acc ? 1 : 0, &at, s_warp);
            if (acc) {
                const int s = s_slots[t];
                const int c = ct_off + s_ct_n + at;
                q.ct_i1[c] = i1; q.ct_i2[c] = i2; q.ct_type[c] = s_ty[t];
                q.ct_status[c] = QA_FORMING; q.ct_ref[c] = tnow; q.ct_vac[c] = 0;
                q.ct_d1[c] = d1p; q.ct_d2[c] = d2p;
                q.fp_vac[s] = 1;
            }
            __syncthreads();
            if (t == 0) s_ct_n += nacc;
            __syncthreads();
        }
    }
    __syncthreads();
    if (t == 0) rp.ct_n = s_ct_n;
    if (t == 0 && s_err) atomicOr(d.status, 4);
}

// ---- process_contacts::iter, state part (process_contacts.cpp:42-56) -----------
// One thread per contact slot of the pool: saturation, forming -> breaking,
// and removal (valence returned, slot vacated, flagged for re-freeing).
// Contacts accepted at this step have saturation 0 and stay as they are.
// The contacts that stay are then listed per bead (the references the next
// step's forces and list builds read; cleared by the sift).
__device__ __forceinline__ void qa_trans_slot(const Dev &d, const TermP &p, int cur, int slot) {
    const QaDev &q = d.qa;
    if (slot >= q.ct_total) return;
    q.ct_rm[slot] = 0;
    const int r = q.ct_rep[slot];
    if (r < 0) return;
    const RepDev &rp = d.rep[r];
    if (!rp.active || slot - rp.ct_off >= rp.ct_n || q.ct_vac[slot]) return;
    const double tnow = rp.t;
    const int i1 = q.ct_i1[slot], i2 = q.ct_i2[slot];
    int status = q.ct_status[slot];
    double sat = __dmul_rn(fmin(__dsub_rn(tnow, q.ct_ref[slot]), p.qa_cycle), p.qa_cycle_inv);
    if (status == QA_BREAKING) sat = __dsub_rn(1.0, sat);
    if (status == QA_FORMING && sat == 1.0) {
        // the breaking test needs the distance (only formed contacts)
        double depth, rmin, rmax;
        qa_lj(p, q, q.ct_type[slot], &depth, &rmin, &rmax);
        const D3 r12 = d3ruv(rp.box, d.pos[cur][i1], d.pos[cur][i2]);
        const double r12_rn = __ddiv_rn(1.0, __dsqrt_rn(d3dot(r12, r12)));
        if (__dmul_rn(__dmul_rn(p.qa_factor, rmin), r12_rn) < 1.0) {
            q.ct_status[slot] = QA_BREAKING;
            q.ct_ref[slot] = tnow;
        }
    } else if (status == QA_BREAKING && sat == 0.0) {
        atomicAdd(&d.rep[r].qa_removed, 1);
        q.ct_vac[slot] = 1;
        atomicAdd(&q.sync[i1], q.ct_d1[slot]);   // bytes stay <= 127: no carry
        atomicAdd(&q.sync[i2], q.ct_d2[slot]);
        q.ct_rm[slot] = 1;
        return;
    }
    // per-bead contact references of the contacts that stay
    const int k1 = atomicAdd(&q.ref_cnt[i1], 1), k2 = atomicAdd(&q.ref_cnt[i2], 1);
    if (k1 < QA_REF_CAP) q.ref[(size_t)k1 * d.N + i1] = slot;
    if (k2 < QA_REF_CAP) q.ref[(size_t)k2 * d.N + i2] = slot;
    if (k1 >= QA_REF_CAP || k2 >= QA_REF_CAP) atomicOr(d.status, 4);
}
// A fixed grid, as the sift: block b takes groups b, b + G, ... of 256
// contact slots and processes the groups that hold live slots (a replica's
// live contacts are a prefix of its region; re-freeing reads the removal
// flags of live slots only).
constexpr int QA_TG = 256;
__global__ void __launch_bounds__(QA_TG) k_qa_trans(Dev d, TermP p, int cur) {
    if (d.gate[0]) return;
    const QaDev &q = d.qa;
    const int t = threadIdx.x;
    const int ng = (q.ct_total + QA_TG - 1) / QA_TG, G = gridDim.x;
    const int per = (ng - (int)blockIdx.x + G - 1) / G;   // <= QA_TG (the grid is sized for it)
    bool lv = false;
    if (t < per) {
        const int first = (blockIdx.x + t * G) * QA_TG, last = min(first + QA_TG, q.ct_total) - 1;
        const int r1 = q.ct_rep[first], r2 = q.ct_rep[last];
        if (r1 >= 0) {
            const RepDev &a = d.rep[r1];
            lv = first - a.ct_off < a.ct_n;
        }
        if (r2 >= 0 && r2 != r1) lv = lv || d.rep[r2].ct_n > 0;
    }
    __shared__ unsigned s_live[QA_TG / 32];
    const unsigned bl = __ballot_sync(0xffffffffu, lv);
    if ((t & 31) == 0) s_live[t >> 5] = bl;
    __syncthreads();
    for (int k = 0; k < per; ++k)
        if ((s_live[k >> 5] >> (k & 31)) & 1u) qa_trans_slot(d, p, cur, (blockIdx.x + k * G) * QA_TG + t);
}

// Removed pairs re-freed at the end of the free-pair list in contact-slot
// order (process_contacts.cpp:48-55); replicas without a removal at this step
// return at once.
// (the body of k_qa_refree: one 1024-thread block per replica)
__device__ __forceinline__ void qa_refree_block(const Dev &d) {
    const int r = blockIdx.x, t = threadIdx.x;
    RepDev &rp = d.rep[r];
    if (!rp.active || rp.ct_cap == 0) return;
    // most steps remove no contact: nothing to re-free
    if (rp.qa_removed == 0) return;
    const QaDev &q = d.qa;
    __shared__ int s_warp[33];
    __shared__ int s_err;
    if (t == 0) s_err = 0;
    const int fp_off = rp.fp_off, ct_off = rp.ct_off, ct_n = rp.ct_n, fp_n0 = rp.fp_n, fp_cap = rp.fp_cap;
    // each thread takes a contiguous run of contact slots, so one block-wide
    // scan places every removed pair in slot order
    const int per = (ct_n + 1023) / 1024;
    const int k0 = min(t * per, ct_n), k1 = min(k0 + per, ct_n);
    int cnt = 0;
    for (int k = k0; k < k1; ++k) cnt += q.ct_rm[ct_off + k];
    int pos;
    const int total = block_exscan(cnt, &pos, s_warp);
    for (int k = k0; k < k1 && cnt; ++k) {
        const int slot = ct_off + k;
        if (!q.ct_rm[slot]) continue;
        const int o = fp_n0 + pos++;
        if (o < fp_cap) {
            q.fp_i1[fp_off + o] = q.ct_i1[slot];
            q.fp_i2[fp_off + o] = q.ct_i2[slot];
            q.fp_vac[fp_off + o] = 0;
        } else {
            s_err = 1;
        }
    }
    __syncthreads();
    if (t == 0) {
        rp.qa_removed = 0;
        rp.fp_n = min(fp_n0 + total, fp_cap);
        if (s_err) atomicOr(d.status, 4);
    }
}

// ---- after a Verlet rebuild: the free-pair list re-listed ------------------------
// update_free_pairs (free_pair.cpp:6-21): non-native list pairs within
// max_formation_min_dist + pad, in (i1, i2) order, minus pairs in contact.
// The builds leave each bead's partners in ascending j (tmp rows); the list
// is their concatenation in bead order, placed by a scan over chunks of
// QA_BCHUNK beads of each replica (grid-wide: the writes are spread over
// every SM).
__global__ void __launch_bounds__(QA_BCHUNK) k_qa_fp_scan(Dev d) {
    const QaDev &q = d.qa;
    const int2 ch = q.bchunk[blockIdx.x];
    const RepDev &rp = d.rep[ch.x];
    if (!rp.active || !rp.rebuild) return;
    __shared__ int s_warp[33];
    const int i = ch.y + threadIdx.x, end = rp.begin + rp.n;
    const int cnt = i < end ? min(q.tmp_cnt[i], QA_TMP_CAP) : 0;
    int pos;
    const int total = block_exscan(cnt, &pos, s_warp);
    if (i < end) q.tmp_off[i] = pos;
    if (threadIdx.x == 0) q.bcsum[blockIdx.x] = total;
}
__global__ void __launch_bounds__(1024) k_qa_fp_base(Dev d) {
    const int r = blockIdx.x, t = threadIdx.x;
    RepDev &rp = d.rep[r];
    if (!rp.active || !rp.rebuild) return;
    const QaDev &q = d.qa;
    __shared__ int s_warp[33];
    __shared__ int s_run;
    if (t == 0) s_run = 0;
    __syncthreads();
    const int off = rp.qa_bchunk_off, nb = rp.qa_nbchunk;
    for (int base = 0; base < nb; base += 1024) {
        const int c = base + t;
        const int v = c < nb ? q.bcsum[off + c] : 0;
        int pos;
        const int total = block_exscan(v, &pos, s_warp);
        if (c < nb) q.bcbase[off + c] = s_run + pos;
        __syncthreads();
        if (t == 0) s_run += total;
        __syncthreads();
    }
    if (t == 0) {
        if (s_run > rp.fp_cap) atomicOr(d.status, 4);
        rp.fp_n = min(s_run, rp.fp_cap);
    }
}
__global__ void __launch_bounds__(QA_BCHUNK) k_qa_fp_fill(Dev d) {
    const QaDev &q = d.qa;
    const int2 ch = q.bchunk[blockIdx.x];
    const RepDev &rp = d.rep[ch.x];
    if (!rp.active || !rp.rebuild) return;
    const int i = ch.y + threadIdx.x;
    if (i >= rp.begin + rp.n) return;
    const int cnt = min(q.tmp_cnt[i], QA_TMP_CAP);
    const int o0 = q.bcbase[blockIdx.x] + q.tmp_off[i];
    for (int k = 0; k < cnt; ++k) {
        const int o = o0 + k;
        if (o < rp.fp_cap) {
            q.fp_i1[rp.fp_off + o] = i;
            q.fp_i2[rp.fp_off + o] = q.tmp[(size_t)k * d.N + i];
            q.fp_vac[rp.fp_off + o] = 0;
        }
    }
}

// Contact slots compacted in order when the replica's region is three
// quarters used (tombstones of removed contacts accumulate between; the order
// of the live contacts, which decides transitions and re-freeing, is kept),
// with the per-bead references rebuilt for the moved slots.
__global__ void __launch_bounds__(1024) k_qa_compact(Dev d) {
    const int r = blockIdx.x, t = threadIdx.x;
    RepDev &rp = d.rep[r];
    if (!rp.active || !rp.rebuild || 4 * rp.ct_n <= 3 * rp.ct_cap) return;
    const QaDev &q = d.qa;
    __shared__ int s_warp[33];
    __shared__ int s_out;
    const int b = rp.begin, n = rp.n;
    const int ct_off = rp.ct_off, ct_n = rp.ct_n;
    if (t == 0) s_out = 0;
    __syncthreads();
    for (int base = 0; base < ct_n; base += 1024) {
        int slot = ct_off + base + t;
        int live = (base + t < ct_n) && !q.ct_vac[slot];
        int a1 = 0, a2 = 0, ty = 0, d1 = 0, d2 = 0;
        uint8_t st = 0;
        double rf = 0;
        if (live) {
            a1 = q.ct_i1[slot]; a2 = q.ct_i2[slot]; ty = q.ct_type[slot]; d1 = q.ct_d1[slot];
            d2 = q.ct_d2[slot]; st = q.ct_status[slot]; rf = q.ct_ref[slot];
        }
        int pos;
        int total = block_exscan(live, &pos, s_warp);
        if (live) {
            int o = ct_off + s_out + pos;
            q.ct_i1[o] = a1; q.ct_i2[o] = a2; q.ct_type[o] = ty; q.ct_d1[o] = d1; q.ct_d2[o] = d2;
            q.ct_status[o] = st; q.ct_ref[o] = rf; q.ct_vac[o] = 0;
        }
        __syncthreads();
        if (t == 0) s_out += total;
        __syncthreads();
    }
    const int nct = s_out;
    for (int i = b + t; i < b + n; i += 1024) q.ref_cnt[i] = 0;
    __syncthreads();
    for (int k = t; k < nct; k += 1024) {
        int slot = ct_off + k;
        int i1 = q.ct_i1[slot], i2 = q.ct_i2[slot];
        int k1 = atomicAdd(&q.ref_cnt[i1], 1), k2 = atomicAdd(&q.ref_cnt[i2], 1);
        if (k1 < QA_REF_CAP) q.ref[(size_t)k1 * d.N + i1] = slot;
        if (k2 < QA_REF_CAP) q.ref[(size_t)k2 * d.N + i2] = slot;
    }
    __syncthreads();
    if (t == 0) rp.ct_n = nct;
}

}  // namespace xmdg
