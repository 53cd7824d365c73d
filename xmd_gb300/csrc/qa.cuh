// qa.cuh - quasi-adiabatic contacts on the device (included by engine.cu).
//
// Per replica the reference keeps three tombstoned sets (free pairs,
// candidates, contacts; gentypes set<T>, _templates/set.h.j2:47-104) whose
// SLOT ORDER decides which candidate wins a shared valence
// (process_candidates.cpp:4-29) and where re-freed pairs land
// (process_contacts.cpp:48-55).  Here each replica owns contiguous regions of
// free-pair and contact slots; slot order is kept by ordered block-wide
// compaction, and the order-dependent greedy acceptance runs sequentially on
// one thread per replica over the (few) compacted candidates.  Geometry that
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
__global__ void __launch_bounds__(256) k_qa_sift(Dev d, TermP p, int cur) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    const QaDev &q = d.qa;
    if (slot >= q.fp_total) return;
    const int r = q.fp_rep[slot];
    const RepDev &rp = d.rep[r];
    if (slot - rp.fp_off >= rp.fp_n) return;
    int type = 0;
    int32_t d1p = 0, d2p = 0;
    if (!q.fp_vac[slot]) {
        const int i1 = q.fp_i1[slot], i2 = q.fp_i2[slot];
        const double4_32a *pos = d.pos[cur];
        D3 r12 = d3ruv(rp.box, pos[i1], pos[i2]);
        double r12_rn = __ddiv_rn(1.0, __dsqrt_rn(d3dot(r12, r12)));
        D3 u = d3scl(r12_rn, r12);
        const size_t N = d.N;
        D3 n1{q.nh[i1], q.nh[N + i1], q.nh[2 * N + i1]}, n2{q.nh[i2], q.nh[N + i2], q.nh[2 * N + i2]};
        D3 h1{q.nh[3 * N + i1], q.nh[4 * N + i1], q.nh[5 * N + i1]};
        D3 h2{q.nh[3 * N + i2], q.nh[4 * N + i2], q.nh[5 * N + i2]};
        bool back1 = fabs(d3dot(h1, u)) > q.min_cos_hr;
        bool back2 = fabs(d3dot(h2, u)) > q.min_cos_hr;
        bool bb_extra = fabs(d3dot(h1, h2)) > q.min_cos_hh;
        bool side1 = d3dot(n1, u) < q.max_cos_nr;
        bool side2 = -d3dot(n2, u) < q.max_cos_nr;
        int a1 = d.atype[i1], a2 = d.atype[i2];
        if (back1 && back2 && bb_extra) type = 1;
        else if (back1 && side2) type = 2;
        else if (side1 && back2) type = 3;
        else if (side1 && side2) type = 4 + a1 + XMD_NUM_AA * a2;
        if (type != 0 && 1.0 > __dmul_rn(r12_rn, q.req_min_dist[type])) type = 0;
        if (type != 0) {
            int pt2 = q.ptype[a2], pt1 = q.ptype[a1];
            d1p = pack4(back1, side1, side1 && pt2 == 1, side1 && pt2 == 2);
            d2p = pack4(back2, side2, side2 && pt1 == 1, side2 && pt1 == 2);
            if (!sync_ok_after(q.sync[i1], d1p) || !sync_ok_after(q.sync[i2], d2p)) type = 0;
        }
    }
    q.cand_type[slot] = type;
    q.cand_d1[slot] = d1p;
    q.cand_d2[slot] = d2p;
}

// ---- acceptance, contact transitions and per-bead references: block/replica ----
// process_candidates::iter (process_candidates.cpp:10-29) in candidate order,
// then process_contacts::iter's state part (process_contacts.cpp:42-56) in
// contact-slot order.
__global__ void __launch_bounds__(1024) k_qa_step(Dev d, TermP p, int cur) {
    const int r = blockIdx.x, t = threadIdx.x;
    RepDev &rp = d.rep[r];
    const QaDev &q = d.qa;
    __shared__ int s_slots[1024];
    __shared__ int s_warp[33];
    __shared__ int s_ct_n, s_fp_n, s_err;
    if (t == 0) { s_ct_n = rp.ct_n; s_fp_n = rp.fp_n; s_err = 0; }
    __syncthreads();
    const double tnow = rp.t;
    const int fp_off = rp.fp_off, ct_off = rp.ct_off;
    const int fp_n0 = s_fp_n;
    // 1. greedy acceptance in free-pair slot order
    for (int base = 0; base < fp_n0; base += 1024) {
        int slot = fp_off + base + t;
        int flag = (base + t < fp_n0) && q.cand_type[slot] != 0;
        int pos;
        int total = block_exscan(flag, &pos, s_warp);
        if (flag) s_slots[pos] = slot;
        __syncthreads();
        if (t == 0) {
            for (int k = 0; k < total; ++k) {
                int s = s_slots[k];
                int i1 = q.fp_i1[s], i2 = q.fp_i2[s];
                int32_t d1p = q.cand_d1[s], d2p = q.cand_d2[s];
                int32_t y1 = q.sync[i1], y2 = q.sync[i2];
                if (sync_ok_after(y1, d1p) && sync_ok_after(y2, d2p)) {
                    if (s_ct_n >= rp.ct_cap) { s_err = 1; break; }
                    int c = ct_off + s_ct_n++;
                    q.ct_i1[c] = i1; q.ct_i2[c] = i2; q.ct_type[c] = q.cand_type[s];
                    q.ct_status[c] = QA_FORMING; q.ct_ref[c] = tnow; q.ct_vac[c] = 0;
                    q.ct_d1[c] = d1p; q.ct_d2[c] = d2p;
                    q.sync[i1] = y1 - d1p;   // bytes never borrow: each stays >= 0
                    q.sync[i2] = (i2 == i1 ? y1 - d1p : y2) - d2p;
                    q.fp_vac[s] = 1;
                }
            }
        }
        __syncthreads();
    }
    // 2. transitions in contact-slot order; removals re-free the pair at the
    //    end of the free-pair list, in slot order
    const int ct_n = s_ct_n;
    for (int base = 0; base < ct_n; base += 1024) {
        int slot = ct_off + base + t;
        int removed = 0;
        if (base + t < ct_n && !q.ct_vac[slot]) {
            int i1 = q.ct_i1[slot], i2 = q.ct_i2[slot];
            D3 r12 = d3ruv(rp.box, d.pos[cur][i1], d.pos[cur][i2]);
            double r12_rn = __ddiv_rn(1.0, __dsqrt_rn(d3dot(r12, r12)));
            int status = q.ct_status[slot];
            double sat = __dmul_rn(fmin(__dsub_rn(tnow, q.ct_ref[slot]), p.qa_cycle), p.qa_cycle_inv);
            if (status == QA_BREAKING) sat = __dsub_rn(1.0, sat);
            double depth, rmin, rmax;
            qa_lj(p, q, q.ct_type[slot], &depth, &rmin, &rmax);
            if (status == QA_FORMING && sat == 1.0) {
                if (__dmul_rn(__dmul_rn(p.qa_factor, rmin), r12_rn) < 1.0) {
                    q.ct_status[slot] = QA_BREAKING;
                    q.ct_ref[slot] = tnow;
                }
            } else if (status == QA_BREAKING && sat == 0.0) {
                q.ct_vac[slot] = 1;
                atomicAdd(&q.sync[i1], q.ct_d1[slot]);   // bytes stay <= 127: no carry
                atomicAdd(&q.sync[i2], q.ct_d2[slot]);
                removed = 1;
            }
        }
        int pos;
        int total = block_exscan(removed, &pos, s_warp);
        if (removed) {
            int fs = fp_off + s_fp_n + pos;
            if (s_fp_n + pos < rp.fp_cap) {
                q.fp_i1[fs] = q.ct_i1[slot];
                q.fp_i2[fs] = q.ct_i2[slot];
                q.fp_vac[fs] = 0;
            } else {
                s_err = 1;
            }
        }
        __syncthreads();
        if (t == 0) s_fp_n = min(s_fp_n + total, rp.fp_cap);
        __syncthreads();
    }
    // 3. per-bead contact references
    for (int i = rp.begin + t; i < rp.begin + rp.n; i += 1024) q.ref_cnt[i] = 0;
    __syncthreads();
    for (int base = 0; base < ct_n; base += 1024) {
        int slot = ct_off + base + t;
        if (base + t < ct_n && !q.ct_vac[slot]) {
            int i1 = q.ct_i1[slot], i2 = q.ct_i2[slot];
            int k1 = atomicAdd(&q.ref_cnt[i1], 1), k2 = atomicAdd(&q.ref_cnt[i2], 1);
            if (k1 < QA_REF_CAP) q.ref[(size_t)k1 * d.N + i1] = slot; else s_err = 1;
            if (k2 < QA_REF_CAP) q.ref[(size_t)k2 * d.N + i2] = slot; else s_err = 1;
        }
    }
    __syncthreads();
    if (t == 0) {
        rp.ct_n = s_ct_n;
        rp.fp_n = s_fp_n;
        if (s_err) atomicOr(d.status, 4);
    }
}

// ---- after a Verlet rebuild: free pairs re-listed, contacts compacted -----------
// update_free_pairs (free_pair.cpp:6-21): non-native list pairs within
// max_formation_min_dist + pad, in (i1, i2) order, minus pairs in contact.
__global__ void __launch_bounds__(1024) k_qa_rebuild(Dev d) {
    const int r = blockIdx.x, t = threadIdx.x;
    RepDev &rp = d.rep[r];
    if (!rp.rebuild) return;
    const QaDev &q = d.qa;
    __shared__ int s_warp[33];
    __shared__ int s_base, s_err;
    if (t == 0) { s_base = 0; s_err = 0; }
    __syncthreads();
    const int b = rp.begin, n = rp.n, fp_off = rp.fp_off;
    for (int c0 = 0; c0 < n; c0 += 1024) {
        int i = b + c0 + t;
        int cnt = (c0 + t < n) ? min(q.tmp_cnt[i], QA_TMP_CAP) : 0;
        int pos;
        int total = block_exscan(cnt, &pos, s_warp);
        if (cnt) {
            int loc[QA_TMP_CAP];
            for (int k = 0; k < cnt; ++k) loc[k] = q.tmp[(size_t)k * d.N + i];
            for (int x = 1; x < cnt; ++x) {   // ascending j
                int v = loc[x], y = x - 1;
                while (y >= 0 && loc[y] > v) { loc[y + 1] = loc[y]; --y; }
                loc[y + 1] = v;
            }
            for (int k = 0; k < cnt; ++k) {
                int o = s_base + pos + k;
                if (o < rp.fp_cap) {
                    q.fp_i1[fp_off + o] = i;
                    q.fp_i2[fp_off + o] = loc[k];
                    q.fp_vac[fp_off + o] = 0;
                } else {
                    s_err = 1;
                }
            }
        }
        __syncthreads();
        if (t == 0) s_base += total;
        __syncthreads();
    }
    if (t == 0) rp.fp_n = min(s_base, rp.fp_cap);
    // in-place ordered compaction of the contact slots
    const int ct_off = rp.ct_off, ct_n = rp.ct_n;
    __shared__ int s_out;
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
    if (t == 0) {
        rp.ct_n = nct;
        if (s_err) atomicOr(d.status, 4);
    }
}

}  // namespace xmdg
