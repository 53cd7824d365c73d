// engine.cu - sm_103a kernels of the hot path and the context that runs them.
//
// Data layout in HBM (N beads of all replicas packed, replica r owning the
// contiguous range [begin_r, begin_r + n_r)):
//   pos[2]   double4_32a (x, y, z, charge), double-buffered: one step reads
//            pos[cur] and writes pos[cur^1]; y0 of the predictor-corrector IS
//            the position.
//   yh       y1..y5 as 15 SoA double arrays (coalesced per component).
//   orig     double4_32a positions of the last Verlet rebuild (skin test).
//   bonded   per-centre parameters (bond i->i+1, angle at i, dihedral with
//            second bead i) and a flag word per bead; chains are contiguous,
//            so bonded partners are i-3..i+3 and come from a shared-memory
//            tile of the block.
//   natives  CSR per bead (both directions) with an "in Go list" byte.
//   Verlet   ELL rows nl_row[k*N + i] = j | flags<<30 holding only pairs that
//            some enabled pair term keeps (Pauli r < r_excl+pad, ES r < 2D+pad
//            with q_i q_j != 0); pairs no term keeps are dropped at build time.
//   cells    per-replica grids (cell budget fixed per replica), counting sort
//            with a deterministic in-cell order.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "device.cuh"
#include "engine.h"
#include "qa.cuh"

namespace xmdg {

std::string &last_error() {
    static thread_local std::string e;
    return e;
}

#define CK(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess)                                                       \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + \
                                     " at " #call);                                  \
    } while (0)

constexpr int BLK_ON = 32;           // beads per granule of the force blocks' occupancy map
constexpr int NL_MASK = 0x1FFFFFFF;
constexpr int NL_PID = 1 << 29;
constexpr int NL_PAULI = 1 << 30;
constexpr int NL_ES = (int)(1u << 31);

enum : int { ST_CAPACITY = 1, ST_NONFINITE = 2 };

// ---- generator jump-ahead (host) ---------------------------------------------
using GF2 = std::array<uint64_t, 64>;
static uint64_t xs_step(uint64_t s) {
    s ^= s >> 11;
    s ^= s << 31;
    s ^= s >> 18;
    return s;
}
static uint64_t gf2_apply_h(const GF2 &m, uint64_t x) {
    uint64_t y = 0;
    for (int k = 0; k < 64; ++k)
        if ((x >> k) & 1) y ^= m[k];
    return y;
}
static GF2 gf2_mul(const GF2 &a, const GF2 &b) {
    GF2 c;
    for (int k = 0; k < 64; ++k) c[k] = gf2_apply_h(a, b[k]);
    return c;
}
// matrix of `draws` generator steps
static GF2 gf2_jump(uint64_t draws) {
    GF2 m, r;
    for (int k = 0; k < 64; ++k) {
        m[k] = xs_step(1ull << k);
        r[k] = 1ull << k;
    }
    while (draws) {
        if (draws & 1) r = gf2_mul(m, r);
        m = gf2_mul(m, m);
        draws >>= 1;
    }
    return r;
}

uint64_t rng_jump(uint64_t state, uint64_t n_draws) { return gf2_apply_h(gf2_jump(n_draws), state); }

// ---- exact squared-distance thresholds (host) ---------------------------------
// The list tests of the reference take a square root (and a reciprocal) of
// the squared distance and compare.  Both are correctly rounded and monotone
// in IEEE FP64, so each test equals s < S for one threshold S on the squared
// distance, found here by stepping through adjacent doubles; the builds then
// compare squared distances (no FP64 square root or division per pair).
// smallest s with RN(sqrt(s)) >= T: sqrt(s) < T <=> s < sq_below(T)
static double sq_below(double T) {
    if (!(T > 0.0)) return 0.0;
    double s = T * T;
    while (s > 0.0 && std::sqrt(s) >= T) s = std::nextafter(s, 0.0);
    while (std::sqrt(s) < T) s = std::nextafter(s, INFINITY);
    return s;
}
// smallest x with RN(1/x) <= v: 1/x > v <=> x < inv_above(v)
static double inv_above(double v) {
    if (!(v > 0.0)) return INFINITY;
    double x = 1.0 / v;
    while (x > 0.0 && 1.0 / x <= v) x = std::nextafter(x, 0.0);
    while (1.0 / x > v) x = std::nextafter(x, INFINITY);
    return x;
}

// ---- device helpers -----------------------------------------------------------
// maximum over the warp of non-negative doubles, compared as their bit
// patterns (the same order) on the integer pipe
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long v) {
    for (int o = 16; o; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    return v;
}

template <class FT>
__device__ __forceinline__ void add3(double &fx, double &fy, double &fz, V3<FT> f) {
    fx += (double)f.x;
    fy += (double)f.y;
    fz += (double)f.z;
}

// finiteness from the exponent bits (integer pipe)
__device__ __forceinline__ bool finite_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// native distance of Go-list entry k in the path's type
template <class FT> __device__ __forceinline__ FT nat_dist(const Dev &d, int k);
template <> __device__ __forceinline__ double nat_dist<double>(const Dev &d, int k) { return d.nat_d[k]; }
template <> __device__ __forceinline__ float nat_dist<float>(const Dev &d, int k) { return d.nat_df[k]; }

// ---- force (+ integrate) kernel --------------------------------------------------
// MODE 0: forces and per-term energies at pos[cur] (eval).
// MODE 1: forces, then one Langevin predictor-corrector step (lang_pc.cpp:5-41)
//         writing pos[cur^1], y1..y5, the generator state and the skin-test
//         displacement (verify.cpp:10-15).
// Wall forces on one bead at its wrapped position rw.  ljw points at the bead's state for the first LJ attractive
// wall (stride N); step = true advances the pair states.
struct WallOut { double fx, fy, fz, vs, vl; };
__device__ __forceinline__ WallOut wall_forces(const double *wall, LjWallState *ljw, size_t N, V3<double> rw,
                                            double tt, bool step, int n_solid, int n_ljw, double solid_eps,
                                            double solid_cutoff, double min_dist, double factor, double cycle,
                                            double cycle_inv, double depth) {
    WallOut o{0.0, 0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < n_solid; ++w) {
        // eval_solid_wall_forces::iter (walls/solid.cpp:12-27): V = eps /
        // (9 x^9) inside the cutoff, its force -dV/dx along the normal [the
        // shipped dV_dx = V (-9 x), added along +normal]
        const double *pl = wall + 6 * w;
        const double x = pl[3] * (rw.x - pl[0]) + pl[4] * (rw.y - pl[1]) + pl[5] * (rw.z - pl[2]);
        if (x < solid_cutoff) {
            const double x3 = x * x * x, V_ = solid_eps / (9.0 * (x3 * x3 * x3));
            const double mdV = 9.0 * V_ / x;   // -dV/dx
            o.vs += V_;
            o.fx += mdV * pl[3]; o.fy += mdV * pl[4]; o.fz += mdV * pl[5];
        }
    }
    for (int w = 0; w < n_ljw; ++w) {
        // eval_lj_attr_wall_forces::loop (walls/lj_attr.cpp:5-43)
        const double *pl = wall + 6 * (XMD_MAX_WALLS + w);
        LjWallState st = ljw[(size_t)w * N];
        if (st.status == 0) {
            const double x = pl[3] * (rw.x - pl[0]) + pl[4] * (rw.y - pl[1]) + pl[5] * (rw.z - pl[2]);
            if (step && fabs(x) < min_dist) {
                st.status = 1;
                st.jx = rw.x - pl[3] * x; st.jy = rw.y - pl[4] * x; st.jz = rw.z - pl[5] * x;
                st.ref_t = tt;
                ljw[(size_t)w * N] = st;
            }
        } else {
            double sat = fmin(tt - st.ref_t, cycle) * cycle_inv;
            if (st.status == 2) sat = 1.0 - sat;
            const V3<double> r12{st.jx - rw.x, st.jy - rw.y, st.jz - rw.z};
            const double r12_rn = 1.0 / norm(r12);
            double V_, dV;
            lj_eval<double>(depth, min_dist, r12_rn, &V_, &dV);
            o.vl += V_ * sat;
            const double f = sat * dV;
            o.fx += f * (r12_rn * r12.x); o.fy += f * (r12_rn * r12.y); o.fz += f * (r12_rn * r12.z);
            if (step) {
                if (st.status == 1 && sat == 1.0) {
                    if (factor * min_dist * r12_rn < 1.0) { st.status = 2; st.ref_t = tt; }
                } else if (st.status == 2 && sat == 0.0) {
                    st.status = 0;
                }
                ljw[(size_t)w * N] = st;
            }
        }
    }
    return o;
}

// External forces of the step, one thread per bead, before the step kernel
// (contexts with AFM tips or walls only): the AFM pulls and the wall forces
// at the step's positions, into fext; MODE 0 adds their energies, MODE 1
// advances the LJ attractive wall pairs.  Kept out of the step kernel, whose
// registers they would raise for every context.
template <int MODE>
__global__ void __launch_bounds__(256) k_ext(Dev d, TermP p, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N || (MODE == 1 && d.gate[0])) return;
    double *fo = d.fext + 3 * (size_t)i;
    fo[0] = fo[1] = fo[2] = 0.0;
    const int r = d.rep_of[i];
    if (r < 0) return;
    if (MODE == 1 && d.rep[r].steps_left == 0) return;
    const double4_32a pi = d.pos[cur][i];
    const double tt = d.rep[r].t;
    V3<double> f{0.0, 0.0, 0.0};
    if (d.rep[r].afm) {
        const uint32_t fl_i = d.bflags[i];
        if (fl_i & BF_AFM) {
            const AfmTip tp = d.afm[fl_i >> BF_AFM_SHIFT];
            if (tp.has_vel && p.on[XMD_TERM_VEL_AFM]) {
                // eval_velocity_afm_forces::iter (velocity_afm.cpp): a
                // harmonic(H1, H2, 0) spring to the tip at orig + t vel
                const V3<double> ra{tp.ox + tt * tp.vx - pi.x, tp.oy + tt * tp.vy - pi.y, tp.oz + tt * tp.vz - pi.z};
                const double rn = norm(ra), rrn = 1.0 / rn;
                const double dr2 = rn * rn;
                double dV = rn * (p.vel_afm_H1 + 2.0 * p.vel_afm_H2 * dr2);
                dV = clampv<double>(dV, -1.0e3, 1.0e3);
                // the spring at rest pulls nothing (0 * inf in the shipped code)
                if (rn > 0.0) f = f + dV * (rrn * ra);
            }
            if (p.on[XMD_TERM_FORCE_AFM]) f = f + V3<double>{tp.fx, tp.fy, tp.fz};
        }
    }
    if (p.n_solid | p.n_ljw) {
        // walls act on the position wrapped into the box (box::wrap)
        const BoxD bx = d.rep[r].box;
        V3<double> rw{pi.x, pi.y, pi.z};
        rw.x -= bx.cell[0] * rint(rw.x * bx.cell_inv[0]);
        rw.y -= bx.cell[1] * rint(rw.y * bx.cell_inv[1]);
        rw.z -= bx.cell[2] * rint(rw.z * bx.cell_inv[2]);
        const WallOut wo = wall_forces(d.wall, d.ljw + i, (size_t)d.N, rw, tt, MODE == 1, p.n_solid, p.n_ljw,
                                       p.solid_eps, p.solid_cutoff, p.ljw_min_dist, p.ljw_factor, p.ljw_cycle,
                                       p.ljw_cycle_inv, p.ljw_depth);
        f = f + V3<double>{wo.fx, wo.fy, wo.fz};
        if (MODE == 0) {
            if (p.n_solid) atomicAdd(&d.Vrep[r * XMD_NUM_TERMS + XMD_TERM_SOLID_WALL], wo.vs);
            if (p.n_ljw) atomicAdd(&d.Vrep[r * XMD_NUM_TERMS + XMD_TERM_LJ_WALL], wo.vl);
        }
    }
    fo[0] = f.x; fo[1] = f.y; fo[2] = f.z;
}

// ---- pseudo-improper dihedral potential: eval_pid_forces::iter
// (pid/eval_forces.cpp:14-141), bundles from update_pid_bundles
// (pid/bundle.cpp:6-29) ------------------------------------------------------------
// Evaluated in FP64 on both paths with every operation rounded on its own
// (DN), in the operation order of the oracle's restatement; the forces are
// the energy's gradient (the shipped kernel leaves one side's derivatives
// unset and scales the others by 1/|m|, 1/|n| for 1/|m|^2, 1/|n|^2).
using D3N = V3<DN>;
constexpr double PID_PI = 3.14159265358979323846;

// lambda_func (pid/lambda.h:29-56): inside the support, value and derivative
__device__ __forceinline__ bool pid_supp(DN alpha, DN psi0, DN psi) { return dn_fabs(alpha * (psi - psi0)) < DN(PID_PI); }
__device__ __forceinline__ void pid_lam(int version, DN alpha, DN psi0, DN psi, DN *val, DN *deriv) {
    const DN sv = alpha * (psi - psi0);
    if (version == 0) {
        *val = DN(0.5) * dn_cos(sv) + DN(0.5);
        *deriv = (DN(-0.5) * alpha) * sin(sv);
    } else {
        const DN t = dn_fabs(sv / DN(PID_PI));
        const DN x_inv = DN(1.0) / (DN(2.0) * t * t - DN(2.0) * t - DN(1.0));
        *val = (t * t - DN(2.0) * t + DN(1.0)) * x_inv;
        DN dv = (DN(2.0) * (t - DN(1.0)) * (t - DN(2.0))) * x_inv * x_inv * alpha / DN(PID_PI);
        if (sv < DN(0.0)) dv = -dv;
        *deriv = dv;
    }
}
__device__ __forceinline__ D3N d3n(double4_32a p) { return D3N{DN(p.x), DN(p.y), DN(p.z)}; }
__device__ __forceinline__ D3N pid_ruv(const BoxD &b, D3N u, D3N w) {
    D3N d = w - u;
    d.x = d.x - DN(b.cell[0]) * dn_rint(d.x * DN(b.cell_inv[0]));
    d.y = d.y - DN(b.cell[1]) * dn_rint(d.y * DN(b.cell_inv[1]));
    d.z = d.z - DN(b.cell[2]) * dn_rint(d.z * DN(b.cell_inv[2]));
    return d;
}
// one side: psi of (previous, bead, next; partner) and its derivatives along
// the four beads (d1 previous, d2 bead, d3 next, d4 partner)
__device__ __forceinline__ DN pid_psi(const BoxD &b, D3N r1_, D3N r2_, D3N r3_, D3N r4_, D3N *d1, D3N *d2, D3N *d3,
                                      D3N *d4) {
    const D3N r24 = pid_ruv(b, r2_, r4_);
    const D3N r12 = r2_ - r1_, r23 = r3_ - r2_, r13 = r3_ - r1_;
    const D3N r14 = r12 + r24;
    const D3N rij = -r23, rkj = -r13, rkl = -r14;
    const D3N rm = cross(r23, r12), rn = cross(r13, r14);
    const DN rm_rn = ninv(rm), rn_rn = ninv(rn), rkj_n = norm(rkj);
    const D3N gi = (rkj_n * rm_rn * rm_rn) * rm;
    const D3N gl = -((rkj_n * rn_rn * rn_rn) * rn);
    const DN a = dot(rij, rkj) / (rkj_n * rkj_n), bb = dot(rkl, rkj) / (rkj_n * rkj_n);
    *d1 = (bb - DN(1.0)) * gl - a * gi;
    *d2 = gi;
    *d3 = (a - DN(1.0)) * gi - bb * gl;
    *d4 = gl;
    DN psi = DN(acos((dot(rm, rn) * rm_rn * rn_rn).v));
    if (dot(rij, rn) < DN(0.0)) psi = -psi;
    return psi;
}

// One thread per bead: the bundles (i, j) of its Verlet row (both beads with
// their chain neighbours, r < PID cutoff + pad at the rebuild), each taken in
// its canonical order (i1, i2) = (min, max).  The bead keeps the forces of
// its side: on itself, its previous and its next bead, into pid_f; the step
// kernel adds to a bead its own part and its neighbours' parts for it.
// MODE 0 adds the energy of the bundles with i < j.
template <int MODE>
__global__ void __launch_bounds__(128) k_pid(Dev d, TermP p, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N || (MODE == 1 && d.gate[0])) return;
    const size_t N = d.N;
    double *Fs = d.pid_f, *Fp = d.pid_f + 3 * N, *Fn = d.pid_f + 6 * N;
    D3N fs{DN(0.0), DN(0.0), DN(0.0)}, fp = fs, fn = fs;
    double Vsum = 0.0;
    const int r = d.rep_of[i];
    const bool both = (d.bflags[i] & (BF_PREV | BF_NEXT)) == (BF_PREV | BF_NEXT);
    if (r >= 0 && both && !(MODE == 1 && d.rep[r].steps_left == 0)) {
        const double4_32a *pos = d.pos[cur];
        const BoxD bx = d.rep[r].box;
        const int cnt = d.nl_cnt[i];
        const DN bbq[2][4] = {{DN(p.pid_bbp[0]), DN(p.pid_bbp[1]), DN(p.pid_bbp[2]), DN(p.pid_bbp[3])},
                              {DN(p.pid_bbm[0]), DN(p.pid_bbm[1]), DN(p.pid_bbm[2]), DN(p.pid_bbm[3])}};
        const DN ssa = DN(p.pid_ss[0]), ssp = DN(p.pid_ss[1]);
        for (int k = 0; k < cnt; ++k) {
            const int e = d.nl_row[(size_t)k * N + i];
            if (!(e & NL_PID)) continue;
            const int j = e & NL_MASK;
            const int i1 = min(i, j), i2 = max(i, j);
            const D3N r1p = d3n(pos[i1 - 1]), r1 = d3n(pos[i1]), r1n = d3n(pos[i1 + 1]);
            const D3N r2p = d3n(pos[i2 - 1]), r2 = d3n(pos[i2]), r2n = d3n(pos[i2 + 1]);
            D3N a1p, a1, a1n, a2, b2p, b2, b2n, b1;
            const DN psi1 = pid_psi(bx, r1p, r1, r1n, r2, &a1p, &a1, &a1n, &a2);
            const DN psi2 = pid_psi(bx, r2p, r2, r2n, r1, &b2p, &b2, &b2n, &b1);
            const D3N r12 = pid_ruv(bx, r1, r2);
            const DN r12_n = norm(r12), r12_rn = DN(1.0) / r12_n;
            DN A(0.0), B(0.0), C(0.0), V(0.0);
            for (int q = 0; q < 2; ++q) {
                if (pid_supp(bbq[q][0], bbq[q][1], psi1) && pid_supp(bbq[q][0], bbq[q][1], psi2)) {
                    DN lam1, g1, lam2, g2, lV, ldV;
                    pid_lam(p.pid_lambda, bbq[q][0], bbq[q][1], psi1, &lam1, &g1);
                    pid_lam(p.pid_lambda, bbq[q][0], bbq[q][1], psi2, &lam2, &g2);
                    lj_eval<DN>(bbq[q][3], bbq[q][2], r12_rn, &lV, &ldV);
                    V = V + lam1 * lam2 * lV;
                    A = A + g1 * lam2 * lV;
                    B = B + g2 * lam1 * lV;
                    C = C + lam1 * lam2 * ldV;
                }
            }
            if (pid_supp(ssa, ssp, psi1) && pid_supp(ssa, ssp, psi2)) {
                // ss_ljs[type], type = atype1 * NUM_AA + atype2 (bundle.cpp:20-22)
                const int ty = (int)d.atype[i1] * XMD_NUM_AA + (int)d.atype[i2];
                DN lam1, g1, lam2, g2, lV, ldV;
                pid_lam(p.pid_lambda, ssa, ssp, psi1, &lam1, &g1);
                pid_lam(p.pid_lambda, ssa, ssp, psi2, &lam2, &g2);
                sink_lj_eval<DN>(DN(d.pid_sd[ty]), DN(d.pid_smin[ty]), DN(d.pid_smax[ty]), r12_n, r12_rn, &lV, &ldV);
                V = V + lam1 * lam2 * lV;
                A = A + g1 * lam2 * lV;
                B = B + g2 * lam1 * lV;
                C = C + lam1 * lam2 * ldV;
            }
            const D3N u = r12_rn * r12;
            if (i == i1) {
                fp = fp - A * a1p;
                fs = fs - ((A * a1 + B * b1) - C * u);
                fn = fn - A * a1n;
                if (MODE == 0) Vsum += V.v;
            } else {
                fp = fp - B * b2p;
                fs = fs - ((A * a2 + B * b2) + C * u);
                fn = fn - B * b2n;
            }
        }
    }
    Fs[3 * i] = fs.x.v; Fs[3 * i + 1] = fs.y.v; Fs[3 * i + 2] = fs.z.v;
    Fp[3 * i] = fp.x.v; Fp[3 * i + 1] = fp.y.v; Fp[3 * i + 2] = fp.z.v;
    Fn[3 * i] = fn.x.v; Fn[3 * i + 1] = fn.y.v; Fn[3 * i + 2] = fn.z.v;
    if (MODE == 0 && Vsum != 0.0) atomicAdd(&d.Vrep[r * XMD_NUM_TERMS + XMD_TERM_PID], Vsum);
}

// Lanes of a bead in the step kernel.  A bead's pair entries (native
// contacts, disulfides, Verlet row, quasi-adiabatic contacts) are dealt to
// VL = 4 virtual lanes, entry k of a list to virtual lane k mod 4, each with
// its own partial force; the partials are combined as ((v0 + v1) + (v2 + v3)).
// The virtual lanes run on LPB = 1, 2 or 4 adjacent threads of one warp
// (thread ln of a bead holds virtual lanes ln, ln + LPB, ...), a launch shape
// chosen by the autotuner: the sums, and so the trajectory, are the same bits
// for every LPB.  A bead's bonded centres are split in two tasks; its
// integrator runs axis a on thread a mod LPB, with the generator, the new
// position and the skin test on the last thread of the bead.
constexpr int VL = 4;

template <int LPB> __device__ __forceinline__ unsigned bead_mask(int t) {
    return ((1u << LPB) - 1u) << ((t & 31) & ~(LPB - 1));
}
__device__ __forceinline__ double vadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ FF vadd(FF a, FF b) { return ff_add(a, b); }
__device__ __forceinline__ double xlane(unsigned m, double v, int o, int w) { return __shfl_xor_sync(m, v, o, w); }
__device__ __forceinline__ FF xlane(unsigned m, FF v, int o, int w) {
    return FF{__shfl_xor_sync(m, v.h, o, w), __shfl_xor_sync(m, v.l, o, w)};
}
// ((v0 + v1) + (v2 + v3)) of a bead's virtual lanes, the same bits on every
// thread of the bead and for every LPB (each addition is commutative bit for
// bit, for FP64 and for the float-float sum, so a thread may add its
// partner's value to its own)
template <int LPB, class T> __device__ __forceinline__ T vl_sum(unsigned m, const T (&a)[VL / LPB]) {
    if constexpr (LPB == 4) {
        const T s = vadd(a[0], xlane(m, a[0], 1, 4));
        return vadd(s, xlane(m, s, 2, 4));
    } else if constexpr (LPB == 2) {
        // thread 0 holds v0 and v2, thread 1 v1 and v3
        return vadd(vadd(a[0], xlane(m, a[0], 1, 2)), vadd(a[1], xlane(m, a[1], 1, 2)));
    } else {
        return vadd(vadd(a[0], a[1]), vadd(a[2], a[3]));
    }
}
template <int LPB, class FT> __device__ __forceinline__ Acc3<FT> vl_sum3(unsigned m, const Acc3<FT> (&a)[VL / LPB]) {
    constexpr int U = VL / LPB;
    decltype(a[0].x) cx[U], cy[U], cz[U];
#pragma unroll
    for (int u = 0; u < U; ++u) { cx[u] = a[u].x; cy[u] = a[u].y; cz[u] = a[u].z; }
    Acc3<FT> r;
    r.x = vl_sum<LPB>(m, cx);
    r.y = vl_sum<LPB>(m, cy);
    r.z = vl_sum<LPB>(m, cz);
    return r;
}
// sum over the threads of a bead (energies of the evaluation pass)
template <int LPB> __device__ __forceinline__ double lane_sum(unsigned m, double v) {
#pragma unroll
    for (int o = 1; o < LPB; o <<= 1) v += __shfl_xor_sync(m, v, o, LPB);
    return v;
}
// add f to the accumulator of the thread's m-th entry: virtual lane slot
// m mod (VL / LPB)
template <int LPB, class FT> __device__ __forceinline__ void acc_slot(Acc3<FT> (&acc)[VL / LPB], int m, V3<FT> f) {
    if constexpr (LPB == 4) {
        acc[0].add(f);
    } else if constexpr (LPB == 2) {
        if (m & 1) acc[1].add(f);
        else acc[0].add(f);
    } else {
        switch (m & 3) {
        case 0: acc[0].add(f); break;
        case 1: acc[1].add(f); break;
        case 2: acc[2].add(f); break;
        default: acc[3].add(f); break;
        }
    }
}
__device__ __forceinline__ double comp3(double4_32a v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// beads of a step-kernel block of FB bead slots (a block of FB - 3 beads,
// whose bonded tasks would fill its threads exactly once, measured slower on
// config 4: at one thread per bead its grid no longer fits one wave)
template <int FB, int LPB> constexpr int force_beads() { return FB; }

template <class FT, int MODE, int FB, int LPB>
__device__ __forceinline__ void force_block(const Dev &d, const TermP &p, int cur) {
    constexpr int NT = FB * LPB;
    constexpr int FBT = force_beads<FB, LPB>();
    constexpr int U = VL / LPB;                 // virtual lanes per thread
    constexpr int AX = (3 + LPB - 1) / LPB;     // integrator axes per thread
    const double4_32a *__restrict__ pin = d.pos[cur];
    const int N = d.N, t = threadIdx.x, i0 = blockIdx.x * FBT;
    const int bs = t / LPB, ln = t % LPB;   // bead slot in the block, thread of the bead
    const int i = i0 + bs;
    const unsigned qm = bead_mask<LPB>(t);  // the bead's threads in the warp
    __shared__ double4_32a P[FBT + 6];
    __shared__ V3<FT> Ct[FBT + 3], Ca[3][FBT + 3], Cd[4][FBT + 3];
    // mixed path: every position of the tile split into float-float parts
    // (integer operations); bond vectors e_k = P[k+1] - P[k] and cross
    // products x_k = e_{k-1} x e_k formed once per tile slot in float-float
    // arithmetic (~2^-44 relative, FP64-class where the FP32 forms lose
    // everything: nearly straight triples) and shared by the tether, angle and
    // dihedral centres that use them
    constexpr int NE = sizeof(FT) == 4 ? FBT + 5 : 1;
    __shared__ P2 S[sizeof(FT) == 4 ? FBT + 6 : 1];
    __shared__ V3<FF> Eff[NE], Xff[NE];
    __shared__ V3<float> Ef[NE], Xf[NE];
    // quasi-adiabatic contact slots of each bead, in ascending order
    __shared__ int Qs[FBT][QA_REF_CAP];

    // mixed path: the integrator's per-bead state does not depend on the
    // forces, so its loads are issued first and their latency passes under
    // the force work (each thread the history of its axes, the last thread
    // the generator and the list origin); the FP64 path is bound by its FP64
    // pipe instead and loads them where they are used
    constexpr bool EARLY = MODE == 1 && sizeof(FT) == 4;
    const bool live = bs < FBT && i < N;
    double yv[5 * AX];
    uint64_t st0 = 0;
    double4_32a o_i = make_double4_32a(0, 0, 0, 0);
    int pf_n0 = 0, pf_n1 = 0, pf_cnt = 0;   // the pair loops' bounds, loaded first too
    if (live) {
        pf_n0 = d.nat_start[i];
        pf_n1 = d.nat_end[i];
        pf_cnt = d.nl_cnt[i];
    }
    const size_t Ns = (size_t)N;
    if (EARLY && live) {
#pragma unroll
        for (int u = 0; u < AX; ++u) {
            const int a = ln + LPB * u;
            if (a < 3) {
#pragma unroll
                for (int q = 0; q < 5; ++q) yv[q * AX + u] = d.yh[(size_t)(q * 3 + a) * Ns + i];
            }
        }
        if (ln == LPB - 1) {
            st0 = d.rng[i];
            o_i = d.orig[i];
        }
    }

    for (int k = t; k < FBT + 6; k += NT) {
        int idx = i0 - 3 + k;
        P[k] = (idx >= 0 && idx < N) ? pin[idx] : make_double4_32a(0, 0, 0, 0);
        if constexpr (sizeof(FT) == 4) S[k] = split_p(P[k]);
    }
    __syncthreads();
    if constexpr (sizeof(FT) == 4) {
        for (int k = t; k < NE; k += NT) {
            const V3<FF> e{ff_diff(S[k].x, S[k + 1].x), ff_diff(S[k].y, S[k + 1].y), ff_diff(S[k].z, S[k + 1].z)};
            Eff[k] = e;
            Ef[k] = V3<float>{e.x.h, e.y.h, e.z.h};
        }
        __syncthreads();
        for (int k = t + 1; k < NE; k += NT) {
            const V3<FF> x = ff_cross(Eff[k - 1], Eff[k]);
            Xff[k] = x;
            Xf[k] = V3<float>{x.x.h, x.y.h, x.z.h};
        }
        __syncthreads();
    }

    // bonded contributions of centres c in [i0-2, i0+FBT].  A centre is two
    // tasks, (tether, angle) and (dihedral, chirality).  With one thread per
    // bead a thread takes both tasks of its centres; with more, the tasks are
    // dealt so that the 32 threads of a warp take one task of 32 consecutive
    // centres (no divergence between the two).
    constexpr int NC = FBT + 3, NC32 = (NC + 31) / 32 * 32;
    constexpr int NW = LPB == 1 ? NC : 2 * NC32;
    auto bonded = [&](const int sc, const int task) {
        const int c = i0 - 2 + sc;
        const uint32_t fl = (c >= 0 && c < N) ? d.bflags[c] : 0u;
        const V3<FT> z{FT(0), FT(0), FT(0)};
        const int sp = c - (i0 - 3);
        const bool own = (c >= i0 && c < i0 + FBT && c < N);
        const int rc = own ? d.rep_of[c] : 0;
        // a centre's angle and dihedral are native or heuristic (seq-file
        // models: those without a native value); both kinds share one call
        if (task == 0) {
            V3<FT> ft = z, a1 = z, a2 = z, a3 = z;
            if ((fl & BF_TETH) && p.on[XMD_TERM_TETHER]) {
                FT V_;
                if constexpr (sizeof(FT) == 4) ft = tether_vec(p, Ef[sp], d.bond_f[c].x, &V_);
                else {
                    DN Vn;
                    ft = v3d(tether_term<DN>(p, P[sp], P[sp + 1], DN(d.teth_r0[c]), &Vn));
                    V_ = (double)Vn;
                }
                if (MODE == 0 && own) atomicAdd(&d.Vrep[rc * XMD_NUM_TERMS + XMD_TERM_TETHER], (double)V_);
            }
            const bool h_ang = (fl & BF_HANG) && p.on[XMD_TERM_HEUR_ANG];
            const bool do_ang = ((fl & BF_ANG) && p.on[XMD_TERM_NAT_ANG]) || h_ang;
            const double *hac = h_ang ? d.heur_ang + 7 * ((fl >> BF_HANG_SHIFT) & 15u) : nullptr;
            const int ang_slot = h_ang ? XMD_TERM_HEUR_ANG : XMD_TERM_NAT_ANG;
            if (do_ang) {
                double V_;
                if constexpr (sizeof(FT) == 8) {
                    // every operation rounded on its own (DN), as the
                    // reference's uncontracted build: near-straight triples
                    // make the bonded terms ill-conditioned
                    V3<DN> b1, b2, b3;
                    DN Vn;
                    angle_term<DN>(p, P[sp - 1], P[sp], P[sp + 1], DN(d.ang_t0[c]), hac, &b1, &b2, &b3, &Vn);
                    a1 = v3d(b1); a2 = v3d(b2); a3 = v3d(b3);
                    V_ = (double)Vn;
                } else {
                    // mixed path: float-float bond vectors and cross products
                    // (shared slots), FP32 forces
                    float Vf;
                    angle_mixed(p, Ef[sp - 1], Ef[sp], Xf[sp], d.bond_f[c].y, hac, &a1, &a2, &a3, &Vf);
                    V_ = (double)Vf;
                }
                if (MODE == 0 && own) atomicAdd(&d.Vrep[rc * XMD_NUM_TERMS + ang_slot], V_);
            }
            Ct[sc] = ft;
            Ca[0][sc] = a1; Ca[1][sc] = a2; Ca[2][sc] = a3;
        } else {
            V3<FT> q[4] = {z, z, z, z};
            const bool h_dih = (fl & BF_HDIH) && p.on[XMD_TERM_HEUR_DIH];
            const bool do_dih = ((fl & BF_DIH) && (p.on[XMD_TERM_CND] || p.on[XMD_TERM_SND])) || h_dih;
            const int hdt = (int)((fl >> BF_HDIH_SHIFT) & 15u);
            if (do_dih) {
                double Vc, Vs;
                if constexpr (sizeof(FT) == 8) {
                    V3<DN> qn[4];
                    DN Vcn, Vsn;
                    dihedral_term<DN>(p, P[sp - 1], P[sp], P[sp + 1], P[sp + 2], DN(d.dih_p0[c]),
                                      p.on[XMD_TERM_CND] != 0, p.on[XMD_TERM_SND] != 0,
                                      h_dih ? reinterpret_cast<const DN *>(d.heur_dih) + 6 * hdt : nullptr, qn,
                                      &Vcn, &Vsn);
#pragma unroll
                    for (int k = 0; k < 4; ++k) q[k] = v3d(qn[k]);
                    Vc = (double)Vcn;
                    Vs = (double)Vsn;
                } else {
                    float Vcf, Vsf;
                    const float X = dot(Xf[sp], Xf[sp + 1]), T = ff_dot(Xff[sp], Eff[sp + 1]).h;
                    dihedral_mixed(p, Ef[sp - 1], Ef[sp], Ef[sp + 1], Xf[sp], Xf[sp + 1], X, T, d.bond_f[c].z,
                                   p.on[XMD_TERM_CND] != 0, p.on[XMD_TERM_SND] != 0,
                                   h_dih ? d.heur_dih_f + 6 * hdt : nullptr, q, &Vcf, &Vsf);
                    Vc = (double)Vcf;
                    Vs = (double)Vsf;
                }
                if (MODE == 0 && own) {
                    if (h_dih) atomicAdd(&d.Vrep[rc * XMD_NUM_TERMS + XMD_TERM_HEUR_DIH], Vc);
                    else {
                        if (p.on[XMD_TERM_CND]) atomicAdd(&d.Vrep[rc * XMD_NUM_TERMS + XMD_TERM_CND], Vc);
                        if (p.on[XMD_TERM_SND]) atomicAdd(&d.Vrep[rc * XMD_NUM_TERMS + XMD_TERM_SND], Vs);
                    }
                }
            }
            // chirality of the quad (c-1, c, c+1, c+2): eval_chiral_forces::iter,
            // chiral.cpp:15-37; its forces join the dihedral slots of the centre
            if ((fl & BF_CHIR) && p.on[XMD_TERM_CHIR]) {
                V3<FT> g[4];
                double Vch;
                if constexpr (sizeof(FT) == 8) {
                    const double2 cp = d.chir[c];
                    V3<DN> gn[4];
                    DN Vn;
                    chiral_term<DN>(p, P[sp - 1], P[sp], P[sp + 1], P[sp + 2], DN(cp.x), DN(cp.y), gn, &Vn);
#pragma unroll
                    for (int k = 0; k < 4; ++k) g[k] = v3d(gn[k]);
                    Vch = (double)Vn;
                } else {
                    const float2 cp = d.chir_f32[c];
                    // the triple product in float-float: planar quads are well conditioned
                    const float tp = ff_dot(Eff[sp - 1], Xff[sp + 1]).h;
                    float Vf;
                    chiral_mixed(p, Ef[sp - 1], Ef[sp], Ef[sp + 1], Xf[sp], Xf[sp + 1], tp, cp.x, cp.y, g, &Vf);
                    Vch = (double)Vf;
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) q[k] = q[k] + g[k];
                if (MODE == 0 && own) atomicAdd(&d.Vrep[rc * XMD_NUM_TERMS + XMD_TERM_CHIR], Vch);
            }
            Cd[0][sc] = q[0]; Cd[1][sc] = q[1]; Cd[2][sc] = q[2]; Cd[3][sc] = q[3];
        }
    };
    for (int w = t; w < NW; w += NT) {
        if constexpr (LPB == 1) {
            bonded(w, 0);
            bonded(w, 1);
        } else {
            const int sc = ((w >> 6) << 5) | (w & 31);
            if (sc < NC) bonded(sc, (w >> 5) & 1);
        }
    }
    __syncthreads();

    // from here on, the threads of a bead take the same branches
    if (!live) return;
    const int r = d.rep_of[i];
    if (r < 0) return;     // free bead slot
    if (MODE == 1 && d.rep[r].steps_left == 0) {
        // the replica has taken its steps: it keeps its state (both buffers)
        if (ln == LPB - 1) d.pos[cur ^ 1][i] = P[bs + 3];
        return;
    }
    const int s = bs + 2;   // centre slot of bead i
    // the partial forces of this thread's virtual lanes; virtual lane 0
    // (thread 0, slot 0) starts from the bonded sum
    Acc3<FT> acc[U];
    if (ln == 0) {
        Acc3<FT> &a0 = acc[0];
        if constexpr (sizeof(FT) == 4) {
            // the bonded contributions, computed in FP32, are summed in FP32
            // and enter the float-float accumulator once
            V3<float> bsum = Ct[s] - Ct[s - 1] + Ca[2][s - 1] + Ca[1][s] + Ca[0][s + 1] + Cd[0][s + 1] +
                             Cd[1][s] + Cd[2][s - 1] + Cd[3][s - 2];
            a0.add(bsum);
        } else {
            a0.add(Ct[s]);
            a0.sub(Ct[s - 1]);
            a0.add(Ca[2][s - 1]);
            a0.add(Ca[1][s]);
            a0.add(Ca[0][s + 1]);
            a0.add(Cd[0][s + 1]);
            a0.add(Cd[1][s]);
            a0.add(Cd[2][s - 1]);
            a0.add(Cd[3][s - 2]);
        }
    }

    const double4_32a pi = P[bs + 3];
    const BoxD bx = d.rep[r].box;
    const bool per = (d.rep[r].per[0] | d.rep[r].per[1] | d.rep[r].per[2]) != 0;
    const PairGeo<FT> geo(bx, per, pi);
    double vgo = 0, vpa = 0, ves = 0;

    // Thread ln takes entries k0 + ln, k0 + ln + LPB, ... of each list; its
    // m-th entry goes to its virtual lane slot m mod U (the same slot on every
    // active thread of the warp, so the slot switch does not diverge).  Each
    // loop body appears once in the code; the loops are software-pipelined
    // (the next entry's index data is loaded while this entry's partner is
    // fetched).
    if (p.on[XMD_TERM_GO]) {
        const int k1 = pf_n1;
        int k = pf_n0 + ln, m = 0;
        int j = 0;
        bool on = false;
        FT nd = FT(0);
        if (k < k1) {
            j = d.nat_j[k];
            on = d.nat_on[k] != 0;
            nd = nat_dist<FT>(d, k);
        }
        for (; k < k1; k += LPB, ++m) {
            int jn = 0;
            bool onn = false;
            FT ndn = FT(0);
            if (k + LPB < k1) {
                jn = d.nat_j[k + LPB];
                onn = d.nat_on[k + LPB] != 0;
                ndn = nat_dist<FT>(d, k + LPB);
            }
            if (on) {
                FT V_;
                const V3<FT> f = go_pair<FT>(p, geo.to(pin[j]), nd, &V_);
                acc_slot<LPB>(acc, m, f);
                if (MODE == 0 && i < j) vgo += (double)V_;
            }
            j = jn;
            on = onn;
            nd = ndn;
        }
    }
    double vss = 0;
    if (p.on[XMD_TERM_NAT_SS]) {
        const int s1 = d.ss_end[i];
        int m = 0;
        for (int k = d.ss_start[i] + ln; k < s1; k += LPB, ++m) {
            if (!d.ss_on[k]) continue;
            const int j = d.ss_j[k];
            FT V_;
            const V3<FT> f = ss_pair<FT>(p, geo.to(pin[j]), &V_);
            acc_slot<LPB>(acc, m, f);
            if (MODE == 0 && i < j) vss += (double)V_;
        }
    }
    {
        const int cnt = pf_cnt;
        int e_next = ln < cnt ? d.nl_row[(size_t)ln * N + i] : 0;
        int m = 0;
        for (int k = ln; k < cnt; k += LPB, ++m) {
            const int e = e_next;
            if (k + LPB < cnt) e_next = d.nl_row[(size_t)(k + LPB) * N + i];
            const int j = e & NL_MASK;
            const double4_32a pj = pin[j];
            const V3<FT> r12 = geo.to(pj);
            V3<FT> f{FT(0), FT(0), FT(0)};
            bool any = false;
            if (e & NL_PAULI) {
                FT V_;
                f = pauli_pair<FT>(p, r12, &V_);
                any = true;
                if (MODE == 0 && i < j) vpa += (double)V_;
            }
            if (e & NL_ES) {
                FT V_;
                const V3<FT> g = es_pair<FT>(p, r12, charge_prod<FT>(pi.w, pj.w), &V_);
                // a pair on both lists adds its two forces one after the other
                if (any) acc_slot<LPB>(acc, m, f);
                f = g;
                any = true;
                if (MODE == 0 && i < j) ves += (double)V_;
            }
            if (any) acc_slot<LPB>(acc, m, f);
        }
    }

    // quasi-adiabatic contacts: the force part of process_contacts::iter
    // (process_contacts.cpp:25-40).  The bead's contact slots (at most
    // QA_REF_CAP, held QA_REF_CAP / LPB per thread) are put in ascending order
    // by rank and dealt to the virtual lanes like a list.
    double vqa = 0;
    if (d.qa_on && p.on[XMD_TERM_QA]) {
        const QaDev &q = d.qa;
        const int nref = min(q.ref_cnt[i], QA_REF_CAP);
        constexpr int HOLD = QA_REF_CAP / LPB;
        int v[HOLD], rk[HOLD];
#pragma unroll
        for (int u = 0; u < HOLD; ++u) {
            const int k = u * LPB + ln;
            v[u] = k < nref ? q.ref[(size_t)k * N + i] : INT_MAX;
            rk[u] = 0;
        }
        for (int m = 0; m < nref; ++m) {
            int x = 0;
#pragma unroll
            for (int u = 0; u < HOLD; ++u) {
                const int y = __shfl_sync(qm, v[u], m % LPB, LPB);
                if (m / LPB == u) x = y;
            }
#pragma unroll
            for (int u = 0; u < HOLD; ++u) rk[u] += x < v[u];
        }
#pragma unroll
        for (int u = 0; u < HOLD; ++u)
            if (u * LPB + ln < nref) Qs[bs][rk[u]] = v[u];
        __syncwarp(qm);
        const double tnow = d.rep[r].t;
        int m = 0;
        for (int k = ln; k < nref; k += LPB, ++m) {
            const int slot = Qs[bs][k];
            int i1 = q.ct_i1[slot], i2 = q.ct_i2[slot];
            V3<FT> r12 = geo.between(pin[i1], pin[i2]);
            FT r12_rn = ninv(r12);
            V3<FT> u = r12_rn * r12;
            double sat = fmin(tnow - q.ct_ref[slot], p.qa_cycle) * p.qa_cycle_inv;
            if (q.ct_status[slot] == QA_BREAKING) sat = 1.0 - sat;
            double depth, rmin, rmax;
            qa_lj(p, q, q.ct_type[slot], &depth, &rmin, &rmax);
            FT V_, dV_;
            sink_lj_eval<FT>((FT)depth, (FT)rmin, (FT)rmax, r12_rn * nsq(r12), r12_rn, &V_, &dV_);
            V3<FT> f = ((FT)sat * dV_) * u;
            acc_slot<LPB>(acc, m, i == i1 ? f : -f);
            if (MODE == 0 && i == i1) vqa += sat * (double)V_;
        }
        if (MODE == 1 && ln == LPB - 1) {
            // n and h at this step's positions (precompute_nh.cpp:12-20) to
            // FP32 accuracy, for the sift's FP32 decisions (which recompute
            // them in FP64 near a threshold)
            V3<float> n{0.0f, 0.0f, 0.0f}, h{0.0f, 0.0f, 0.0f};
            const uint32_t fl = d.bflags[i];
            if ((fl & BF_PREV) && (fl & BF_NEXT)) qa_nh_f(P[bs + 2], P[bs + 3], P[bs + 4], &n, &h);
            q.nh[i] = n.x; q.nh[Ns + i] = n.y; q.nh[2 * Ns + i] = n.z;
            q.nh[3 * Ns + i] = h.x; q.nh[4 * Ns + i] = h.y; q.nh[5 * Ns + i] = h.z;
        }
    }

    // the bead's force: its virtual lanes' partial sums combined (every
    // thread of the bead holds it)
    V3<double> ftot = vl_sum3<LPB>(qm, acc).total();
    if (p.ext_on) {
        // AFM pulls and walls, from k_ext (launched just before)
        ftot = ftot + V3<double>{d.fext[3 * (size_t)i], d.fext[3 * (size_t)i + 1], d.fext[3 * (size_t)i + 2]};
    }
    if (p.on[XMD_TERM_PID]) {
        // pseudo-improper dihedral bundles, from k_pid: the bead's own side,
        // then the parts its chain neighbours' bundles put on it
        const double *pf = d.pid_f;
        const uint32_t fl = d.bflags[i];
        V3<double> g{pf[3 * (size_t)i], pf[3 * (size_t)i + 1], pf[3 * (size_t)i + 2]};
        if (fl & BF_PREV) {
            const double *q = pf + 6 * Ns + 3 * (size_t)(i - 1);   // next-bead part of i - 1
            g = g + V3<double>{q[0], q[1], q[2]};
        }
        if (fl & BF_NEXT) {
            const double *q = pf + 3 * Ns + 3 * (size_t)(i + 1);   // previous-bead part of i + 1
            g = g + V3<double>{q[0], q[1], q[2]};
        }
        ftot = ftot + g;
    }
    const double fx = ftot.x, fy = ftot.y, fz = ftot.z;
    if (!(finite_bits(fx) && finite_bits(fy) && finite_bits(fz))) {
        // the replica is frozen from the next step on (its skin check sets
        // steps_left = 0); this bead keeps its state, so no non-finite
        // position ever reaches a list build
        if (ln == 0) atomicOr(d.status, ST_NONFINITE);
        if (MODE == 1) {
            if (ln == LPB - 1) {
                d.rep[r].fault = 1;
                d.pos[cur ^ 1][i] = pi;
            }
            return;
        }
    }

    if (MODE == 0) {
#pragma unroll
        for (int u = 0; u < AX; ++u) {
            const int a = ln + LPB * u;
            if (a < 3) d.F[3 * (size_t)i + a] = a == 0 ? fx : (a == 1 ? fy : fz);
        }
        vgo = lane_sum<LPB>(qm, vgo);
        vpa = lane_sum<LPB>(qm, vpa);
        ves = lane_sum<LPB>(qm, ves);
        vqa = lane_sum<LPB>(qm, vqa);
        vss = lane_sum<LPB>(qm, vss);
        if (ln == 0) {
            double *Vr = d.Vrep + r * XMD_NUM_TERMS;
            if (vgo != 0.0) atomicAdd(&Vr[XMD_TERM_GO], vgo);
            if (vpa != 0.0) atomicAdd(&Vr[XMD_TERM_PAULI], vpa);
            if (ves != 0.0) atomicAdd(&Vr[p.es_rel ? XMD_TERM_REL_ES : XMD_TERM_CONST_ES], ves);
            if (vqa != 0.0) atomicAdd(&Vr[XMD_TERM_QA], vqa);
            if (vss != 0.0) atomicAdd(&Vr[XMD_TERM_NAT_SS], vss);
        }
        return;
    }

    // ---- lang_pc_step::operator(), lang_pc.cpp:11-37, mass = 1 (main.cpp:156) ----
    // the last thread of the bead: its four generator draws, three normals
    double nz0 = 0.0, nz1 = 0.0, nz2 = 0.0;
    if (ln == LPB - 1) {
        if (!EARLY) {
            st0 = d.rng[i];
            o_i = d.orig[i];
        }
        uint64_t st = st0;
        if constexpr (sizeof(FT) == 8) {
            noise3(st, &nz0, &nz1, &nz2);
        } else {
            float a, b, c;
            noise3m(st, &a, &b, &c);
            nz0 = widen_f(a);
            nz1 = widen_f(b);
            nz2 = widen_f(c);
        }
        d.rng[i] = gf2_apply_nib(d.jump + JUMP_WORDS * r, st);
    }
    if constexpr (LPB > 1) {
        nz0 = __shfl_sync(qm, nz0, LPB - 1, LPB);
        nz1 = __shfl_sync(qm, nz1, LPB - 1, LPB);
        nz2 = __shfl_sync(qm, nz2, LPB - 1, LPB);
    }
    // the Gear-5 corrector and predictor of the thread's axes
    double y0a[AX];
#pragma unroll
    for (int u = 0; u < AX; ++u) {
        const int a = ln + LPB * u;
        y0a[u] = 0.0;
        if (a >= 3) continue;
        const double dt_inv = p.dt_inv, h = p.dt2_half;
        const double gamma = p.gamma_factor * 1.0;
        const double nsd = d.rep[r].noise_sd;
        const double Fa = a == 0 ? fx : (a == 1 ? fy : fz);
        const double nza = a == 0 ? nz0 : (a == 1 ? nz1 : nz2);
        double *yh = d.yh;
        double y0 = comp3(pi, a);
        double y1, y2, y3, y4, y5;
        if constexpr (EARLY) {
            y1 = yv[0 * AX + u]; y2 = yv[1 * AX + u]; y3 = yv[2 * AX + u]; y4 = yv[3 * AX + u];
            y5 = yv[4 * AX + u];
        } else {
            y1 = yh[(size_t)(0 * 3 + a) * Ns + i]; y2 = yh[(size_t)(1 * 3 + a) * Ns + i];
            y3 = yh[(size_t)(2 * 3 + a) * Ns + i]; y4 = yh[(size_t)(3 * 3 + a) * Ns + i];
            y5 = yh[(size_t)(4 * 3 + a) * Ns + i];
        }
        double v = y1 * dt_inv;
        double a_ = Fa * 1.0 - gamma * v + nsd * nza;
        double error = y2 - a_ * h;
        y0 -= 3.0 / 16.0 * error;
        y1 -= 251.0 / 360.0 * error;
        y2 -= 1.0 * error;
        y3 -= 11.0 / 18.0 * error;
        y4 -= 1.0 / 6.0 * error;
        y5 -= 1.0 / 60.0 * error;
        y0 += y1 + y2 + y3 + y4 + y5;
        y1 += 2.0 * y2 + 3.0 * y3 + 4.0 * y4 + 5.0 * y5;
        y2 += 3.0 * y3 + 6.0 * y4 + 10.0 * y5;
        y3 += 4.0 * y4 + 10.0 * y5;
        y4 += 5.0 * y5;
        yh[(size_t)(0 * 3 + a) * Ns + i] = y1;
        yh[(size_t)(1 * 3 + a) * Ns + i] = y2;
        yh[(size_t)(2 * 3 + a) * Ns + i] = y3;
        yh[(size_t)(3 * 3 + a) * Ns + i] = y4;
        yh[(size_t)(4 * 3 + a) * Ns + i] = y5;
        y0a[u] = y0;
    }
    // the last thread: the new position (axis a from thread a mod LPB) and
    // the skin-test displacement
    const double px = __shfl_sync(qm, y0a[0 / LPB], 0 % LPB, LPB);
    const double py = __shfl_sync(qm, y0a[1 / LPB], 1 % LPB, LPB);
    const double pz = __shfl_sync(qm, y0a[2 / LPB], 2 % LPB, LPB);
    double disp = 0.0;
    if (ln == LPB - 1) {
        const double4_32a pn = make_double4_32a(px, py, pz, pi.w);
        d.pos[cur ^ 1][i] = pn;
        // skin test displacement: norm(box->r_uv(r_, orig_r_)), verify.cpp:12-14
        // squared; the check takes one square root of the maximum (sqrt is
        // monotone and correctly rounded, so that equals the max of the norms)
        if constexpr (sizeof(FT) == 4) {
            // mixed path: the displacement from split positions (the FP64
            // difference to FP32 accuracy), squared in FP32
            const V3<float> e = geo.between(o_i, pn);
            disp = widen_f(e.x * e.x + e.y * e.y + e.z * e.z);
        } else {
            // on open axes the wrap subtracts exactly zero: skipping it changes no bit
            disp = per ? dist2_exact(bx, pn, o_i) : dist2_open(pn, o_i);
        }
    }
    const unsigned lane = t & 31;
    int r0 = __shfl_sync(0xffffffffu & __activemask(), r, 0);
    unsigned mask = __activemask();
    if (__all_sync(mask, r == r0) && mask == 0xffffffffu) {
        const unsigned long long m = warp_max_bits((unsigned long long)__double_as_longlong(disp));
        if (lane == 0) atomicMax(&d.rep[r].maxdisp, m);
    } else if (ln == LPB - 1) {
        atomicMax(&d.rep[r].maxdisp, (unsigned long long)__double_as_longlong(disp));
    }
}

// ---- skin decision (nl::verify, verify.cpp:4-23) --------------------------------
// setc 1: also set the conditional handle of the graph's rebuild IF node;
// setc 2: count the step in the gate and halt the graph when a replica is
// flagged or the budget of steps is spent
enum : int { CHECK_PLAIN = 0, CHECK_COND = 1, CHECK_GATE = 2 };
template <int SETC>
__device__ __forceinline__ void nl_check_block(const Dev &d, int advance, double dt, cudaGraphConditionalHandle h) {
    __shared__ int any_s, nwork_s;
    if (threadIdx.x == 0) any_s = nwork_s = 0;
    __syncthreads();
    int any = 0;
    for (int r = threadIdx.x; r < d.R; r += blockDim.x) {
        RepDev &rp = d.rep[r];
        // every field the decision reads, loaded at once (one round trip)
        const int active = rp.active, fault = rp.fault, first = rp.first, tile = rp.tile;
        const int nchunk = rp.nchunk, chunk_off = rp.chunk_off;
        long long left = rp.steps_left;
        const unsigned long long mdb = rp.maxdisp;
        const double pad = rp.pad, tr = rp.t;
        if (!active) continue;
        if (fault) {   // frozen: no further step, no list
            rp.steps_left = 0;
            rp.rebuild = 0;
            continue;
        }
        if (advance && left == 0) {           // took no step (k_force kept it)
            rp.rebuild = 0;
            continue;
        }
        if (advance) {
            rp.t = tr + dt;                   // *t = (*true_t += dt)
            if (left > 0) rp.steps_left = --left;
        }
        const double md = __dsqrt_rn(__longlong_as_double((long long)mdb));
        rp.maxdisp = 0ull;
        int rb = first || (2.0 * md + 0.0 > pad);
        if (advance && left == 0 && !first) rb = 0;   // no further step uses a list
        rp.rebuild = rb;
        any |= rb;
        // the tile build's work list: every chunk of the flagged replicas
        // (order is free: each chunk writes its own rows)
        if (rb && tile) {
            const int at = atomicAdd(&nwork_s, nchunk);
            for (int c = 0; c < nchunk; ++c) d.work[at + c] = chunk_off + c;
        }
    }
    if (any) atomicOr(&any_s, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        *d.any_rebuild = any_s;
        *d.nwork = nwork_s;
        if constexpr (SETC == CHECK_COND) cudaGraphSetConditional(h, any_s ? 1u : 0u);
        if constexpr (SETC == CHECK_GATE) {
            const int done = d.gate[1] + 1;
            d.gate[1] = done;
            if (any_s || done >= d.gate[2]) d.gate[0] = 1;
        }
    }
}
__global__ void k_nl_check(Dev d, int advance, double dt, cudaGraphConditionalHandle h, int setc) {
    if (setc == CHECK_GATE && d.gate[0]) return;
    if (setc == CHECK_COND) nl_check_block<CHECK_COND>(d, advance, dt, h);
    else if (setc == CHECK_GATE) nl_check_block<CHECK_GATE>(d, advance, dt, h);
    else nl_check_block<CHECK_PLAIN>(d, advance, dt, h);
}

// The quasi-adiabatic re-freeing (one block per replica).  With `check` (the
// gated graph steps) the last block to finish also takes the step's skin
// decision, which otherwise is a launch of its own.
__global__ void __launch_bounds__(1024) k_qa_refree(Dev d, double dt, int check) {
    if (d.gate[0]) return;
    qa_refree_block(d);
    if (!check) return;
    __shared__ int last_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last_s = atomicAdd(&d.ctr[2], 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (last_s) {
        __threadfence();
        nl_check_block<CHECK_GATE>(d, 1, dt, (cudaGraphConditionalHandle)0);
        if (threadIdx.x == 0) d.ctr[2] = 0ull;
    }
}

// The step kernel.  `fuse` (graph steps): FUSE_CHECK, the last block to
// finish also takes the skin decision of every replica (the next node, the
// row build, runs on the work list it leaves, empty or not); FUSE_CHECK_GATE,
// the same, and the decision keeps the gate: the kernel returns at once
// while the gate is closed; FUSE_GATE, no decision (a later kernel of the step
// takes it), and the kernel returns at once while the gate is closed.  The
// kernel holds no device-side graph call, so profilers see it in graphs.
// resident blocks the register allocation leaves room for: 16 warps per SM
// (at most 128 registers) with one or two threads per bead, 28 (at most 73)
// with four
template <int FB, int LPB> constexpr int force_min_blocks() {
    return LPB == 4 ? (896 / (FB * 4) > 0 ? 896 / (FB * 4) : 1) : 512 / (FB * LPB);
}
enum : int { FUSE_NONE = 0, FUSE_CHECK = 1, FUSE_CHECK_GATE = 2, FUSE_GATE = 3 };
template <class FT, int MODE, int FB, int LPB>
__global__ void __launch_bounds__(FB * LPB, (force_min_blocks<FB, LPB>())) k_force(Dev d, TermP p, int cur,
                                                                                  int fuse) {
    __shared__ int last_s;
    static_assert(LPB == 1 || LPB == 2 || LPB == 4, "one, two or four threads per bead");
    // uniform: the gate changes between launches
    if (MODE == 1 && (fuse == FUSE_CHECK_GATE || fuse == FUSE_GATE) && d.gate[0]) return;
    constexpr int FBT = force_beads<FB, LPB>();
    // the block runs when an occupancy granule of its beads is on (uniform)
    const int i0 = blockIdx.x * FBT, i1 = min(i0 + FBT, d.N) - 1;
    bool on = false;
    for (int g = i0 / BLK_ON; g <= i1 / BLK_ON; ++g) on |= d.blk_on[g] != 0;
    if (on) force_block<FT, MODE, FB, LPB>(d, p, cur);
    if (MODE == 1 && (fuse == FUSE_CHECK || fuse == FUSE_CHECK_GATE)) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            last_s = atomicAdd(&d.ctr[2], 1ull) == (unsigned long long)(gridDim.x - 1);
        }
        __syncthreads();
        if (last_s) {
            __threadfence();
            if (fuse == FUSE_CHECK_GATE) nl_check_block<CHECK_GATE>(d, 1, p.dt, (cudaGraphConditionalHandle)0);
            else nl_check_block<CHECK_PLAIN>(d, 1, p.dt, (cudaGraphConditionalHandle)0);
            if (threadIdx.x == 0) d.ctr[2] = 0ull;
        }
    }
}

// the replicas whose rebuild overflowed the rows rebuild again at the next
// check (after the rows were reallocated); the others keep their lists
__global__ void k_mark_all(Dev d) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < d.R && d.rep[r].active && d.rep[r].rebuild) d.rep[r].first = 1;
}

// Minimum image of a difference of coordinates wrapped into [0, L) (so
// |d| < L) by compare and select: rintf runs on the slow conversion pipe.
// L = 0 (open axis) leaves d unchanged.
__device__ __forceinline__ float min_image_f(float d, float L) {
    const float h = 0.5f * L;
    d = d > h ? d - L : d;
    return d < -h ? d + L : d;
}

// FP32 error bound of a distance d <= ext between FP32 coordinates of
// magnitude <= ext (relative coordinates, or wrapped into [0, L) with L <=
// ext).  Each coordinate is the FP64 value rounded once (<= 2^-24 ext); a
// difference adds one rounding and the minimum-image shift by the rounded
// box length two more (<= 4 * 2^-24 ext per axis); the three squares and
// their sum add <= 3 * 2^-24 relative to d^2.  In distance terms that is
// <= sqrt(3) * 4 * 2^-24 ext + 1.5 * 2^-24 d < 5e-7 ext; the bound used is
// twice that plus an absolute 1e-5.
__host__ __device__ __forceinline__ double band_margin(double ext) { return 1e-5 + 1e-6 * ext; }

// FP32 decision band around a distance threshold T (error bound m)
struct Band {
    float lo, hi;   // squared FP32 distance: below lo -> inside, above hi -> outside
};
__device__ __forceinline__ Band make_band(double T, double m) {
    double a = T - m, b = T + m;
    return Band{a > 0.0 ? __double2float_rd(a * a) : -1.0f, __double2float_ru(b * b)};
}
__device__ __forceinline__ bool in_band(const Band &B, float d2) { return d2 >= B.lo && d2 <= B.hi; }

// ---- cell lists: one block per flagged replica -----------------------------------
// Cells have an edge of at least the Verlet radius.  Periodic axes are cut
// into dims = floor(L / r) cells (wrapped); open axes count cells from the
// bounding-box minimum without bound.  When every axis is periodic and the
// grid fits the replica's bucket budget, a cell IS a bucket; otherwise cells
// are hashed into the budget (chains in open space occupy few of their
// bounding box's cells).  Buckets are visited once each, so collisions only
// add candidates; the exact distance test decides.
__device__ __forceinline__ int cell_coord(const RepDev &rp, int a, double x) {
    if (rp.per[a]) {
        double f = x * rp.box.cell_inv[a];
        f -= floor(f);
        int k = (int)(f * rp.dims[a]);
        return k < 0 ? 0 : (k >= rp.dims[a] ? rp.dims[a] - 1 : k);
    }
    int k = (int)floor((x - rp.lo[a]) * rp.cs[a]);   // cs holds 1 / cell edge on open axes
    return k < 0 ? 0 : k;
}
__device__ __forceinline__ int cell_key(const RepDev &rp, int cx, int cy, int cz) {
    if (!rp.hashed) return (cz * rp.dims[1] + cy) * rp.dims[0] + cx;
    uint32_t h = (uint32_t)cx * 73856093u ^ (uint32_t)cy * 19349663u ^ (uint32_t)cz * 83492791u;
    return (int)(h % (uint32_t)rp.cell_budget);
}
// FP32 coordinate for the pre-filter: wrapped into [0, L) or taken from the
// bounding-box minimum
__device__ __forceinline__ float rel_coord(const RepDev &rp, int a, double x) {
    if (rp.per[a]) return (float)(x - rp.box.cell[a] * floor(x * rp.box.cell_inv[a]));
    return (float)(x - rp.lo[a]);
}
__device__ __forceinline__ double comp(double4_32a v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

constexpr int CB = 1024;
__global__ void __launch_bounds__(CB) k_cells(Dev d, int cur) {
    const int r = blockIdx.x;
    if (r == 0 && threadIdx.x == 0) atomicAdd(d.ctr, 1ull);
    RepDev &rp = d.rep[r];
    if (!rp.active || !rp.rebuild || rp.tile) return;
    const double4_32a *pos = d.pos[cur];
    const int b = rp.begin, n = rp.n, off = rp.cell_off, bud = rp.cell_budget;
    __shared__ double red_lo[3][32], red_hi[3][32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;

    // bounding box along open axes (none in a fully periodic box); four
    // loads in flight per thread
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    const bool any_open = !(rp.per[0] && rp.per[1] && rp.per[2]);
    for (int i0 = b + t; any_open && i0 < b + n; i0 += 4 * CB) {
        double4_32a q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = pos[min(i0 + u * CB, b + n - 1)];   // repeats are harmless
#pragma unroll
        for (int u = 0; u < 4; ++u)
            for (int a = 0; a < 3; ++a) {
                lo[a] = fmin(lo[a], comp(q[u], a));
                hi[a] = fmax(hi[a], comp(q[u], a));
            }
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o; o >>= 1) {
            lo[a] = fmin(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmax(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
        if (lane == 0) { red_lo[a][w] = lo[a]; red_hi[a][w] = hi[a]; }
    }
    __syncthreads();
    if (t == 0) {
        const double rr = rp.req_r * (1.0 + 1e-9);
        long total = 1;
        bool all_per = true;
        double ext = 0.0;
        for (int a = 0; a < 3; ++a) {
            double l = 1e300, hh = -1e300;
            for (int q = 0; q < CB / 32; ++q) { l = fmin(l, red_lo[a][q]); hh = fmax(hh, red_hi[a][q]); }
            if (rp.per[a]) {
                int dm = (int)floor(rp.box.cell[a] / rr);
                dm = dm < 1 ? 1 : (dm > 4096 ? 4096 : dm);
                rp.dims[a] = dm;
                rp.lo[a] = 0.0;
                rp.cs[a] = 0.0;
                total *= dm;
                ext = fmax(ext, rp.box.cell[a]);
            } else {
                all_per = false;
                rp.dims[a] = 0;
                rp.lo[a] = l;
                rp.cs[a] = 1.0 / rr;
                ext = fmax(ext, hh - l);
            }
        }
        rp.hashed = !(all_per && total <= bud);
        // FP32 error bound of a distance (see band_margin); the pre-filter
        // radius req_r + m never rejects a pair inside req_r
        rp.band_m = band_margin(fmax(ext, rp.req_r));
        double m = rp.req_r + rp.band_m;
        rp.pre2 = __double2float_ru(m * m);
        const double T[5] = {rp.req_r, 1.0 / rp.pauli_min_inv, 1.0 / rp.es_min_inv, 1.0 / rp.qa_min_inv,
                             1.0 / rp.pid_min_inv};
        for (int k = 0; k < 5; ++k) {
            const Band B = make_band(T[k], rp.band_m);
            rp.band_lo[k] = B.lo;
            rp.band_hi[k] = B.hi;
        }
        rp.band_mf = __double2float_ru(rp.band_m);
        rp.first = 0;
        rp.rebuilds += 1;
    }
    __syncthreads();
    const int ncell = rp.hashed ? bud : rp.dims[0] * rp.dims[1] * rp.dims[2];
    for (int c = t; c < ncell; c += CB) {
        d.cell_cnt[off + c] = 0;
        d.cell_fill[off + c] = 0;
    }
}

// The bucket sort of the flagged replicas, over the whole grid: count, scan
// (one block per replica, over its buckets), scatter, then per bucket a
// deterministic order (ascending bead index) and the FP32 coordinates.
__device__ __forceinline__ bool cell_flagged(const Dev &d, int r) {
    if (r < 0) return false;
    const RepDev &rp = d.rep[r];
    return rp.active && rp.rebuild && !rp.tile;
}
__global__ void k_cell_count(Dev d, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const int r = d.rep_of[i];
    if (!cell_flagged(d, r)) return;
    const RepDev &rp = d.rep[r];
    const double4_32a q = d.pos[cur][i];
    const int c = rp.cell_off + cell_key(rp, cell_coord(rp, 0, q.x), cell_coord(rp, 1, q.y), cell_coord(rp, 2, q.z));
    d.bead_cell[i] = c;
    atomicAdd(&d.cell_cnt[c], 1);
}
__global__ void __launch_bounds__(CB) k_cell_scan(Dev d) {
    const int r = blockIdx.x;
    if (!cell_flagged(d, r)) return;
    const RepDev &rp = d.rep[r];
    __shared__ int scan_s[CB];
    const int t = threadIdx.x, off = rp.cell_off;
    const int ncell = rp.hashed ? rp.cell_budget : rp.dims[0] * rp.dims[1] * rp.dims[2];
    // exclusive scan of the counts, contiguous chunk per thread
    const int chunk = (ncell + CB - 1) / CB;
    const int c0 = t * chunk, c1 = min(ncell, c0 + chunk);
    int sum = 0;
    for (int c = c0; c < c1; ++c) sum += d.cell_cnt[off + c];
    scan_s[t] = sum;
    __syncthreads();
    for (int o = 1; o < CB; o <<= 1) {
        int v = t >= o ? scan_s[t - o] : 0;
        __syncthreads();
        scan_s[t] += v;
        __syncthreads();
    }
    int run = rp.begin + scan_s[t] - sum;
    for (int c = c0; c < c1; ++c) {
        d.cell_start[off + c] = run;
        run += d.cell_cnt[off + c];
    }
}
__global__ void k_cell_scatter(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    if (!cell_flagged(d, d.rep_of[i])) return;
    const int c = d.bead_cell[i];
    const int slot = atomicAdd(&d.cell_fill[c], 1);
    d.cell_items[d.cell_start[c] + slot] = i;
}
// one warp per bucket of the pool: the bucket's beads put in ascending index
// order (each item's rank among the bucket's items; buckets of more than
// 8 x 32 beads are sorted by one lane), then their FP32 coordinates
constexpr int CF_WARPS = 8, CF_HOLD = 8;
__global__ void __launch_bounds__(CF_WARPS * 32) k_cell_finish(Dev d, int cur) {
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * CF_WARPS + (threadIdx.x >> 5);
    if (c >= d.ncells) return;   // warp-uniform exits
    const int r = d.cell_rep[c];
    if (!cell_flagged(d, r)) return;
    const RepDev &rp = d.rep[r];
    const int ncell = rp.hashed ? rp.cell_budget : rp.dims[0] * rp.dims[1] * rp.dims[2];
    if (c - rp.cell_off >= ncell) return;
    const int s0 = d.cell_start[c], m = d.cell_cnt[c];
    int *it = d.cell_items + s0;
    const unsigned FULL = 0xffffffffu;
    if (m <= 32 * CF_HOLD) {
        int v[CF_HOLD], rk[CF_HOLD];
#pragma unroll
        for (int u = 0; u < CF_HOLD; ++u) {
            v[u] = u * 32 + lane < m ? it[u * 32 + lane] : 0x7fffffff;
            rk[u] = 0;
        }
        for (int k = 0; k < m; ++k) {
            int x = 0;
#pragma unroll
            for (int u = 0; u < CF_HOLD; ++u)
                if ((k >> 5) == u) x = __shfl_sync(FULL, v[u], k & 31);
#pragma unroll
            for (int u = 0; u < CF_HOLD; ++u) rk[u] += x < v[u];
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < CF_HOLD; ++u)
            if (u * 32 + lane < m) it[rk[u]] = v[u];
    } else if (lane == 0) {
        for (int x = 1; x < m; ++x) {
            int vv = it[x], y = x - 1;
            while (y >= 0 && it[y] > vv) { it[y + 1] = it[y]; --y; }
            it[y + 1] = vv;
        }
    }
    __syncwarp();
    const double4_32a *pos = d.pos[cur];
    for (int k = s0 + lane; k < s0 + m; k += 32) {
        const int i = d.cell_items[k];
        const double4_32a q = pos[i];
        d.cell_pos[k] = make_float4(rel_coord(rp, 0, q.x), rel_coord(rp, 1, q.y), rel_coord(rp, 2, q.z),
                                    __int_as_float(i));
        d.cell_cs[k] = make_int2(d.chain[i], d.seq[i]);
        d.bead_slot[i] = k;
    }
}

// ---- Verlet rows (legacy_update.cpp:16-62 + the update_* filters) ---------------

// ---- Verlet rows of the cell build (legacy_update.cpp:16-62 + the update_*
// filters), one warp per bead i --------------------------------------------------
// A pair is decided in FP32 when its FP32 distance is outside the bands of
// the replica (k_cells: the list radius, r_excl + pad, 2D + pad, the QA
// formation radius + pad, each widened by the FP32 error bound), and by the
// exact FP64 test inside them.  The candidates of each neighbouring bucket
// are taken 32 at a time by the lanes: loads of a bucket are contiguous, the
// row is compacted by ballot, and the bead's latency chain is one bucket deep
// instead of one candidate deep.  Buckets are visited z, then y, then x
// offset (first occurrence of each key).  Quasi-adiabatic partners are ranked
// by j within the warp at the end, so the free-pair source list is ordered as
// update_free_pairs (free_pair.cpp:9-19) walks it.
constexpr int NC_WARPS = 8;
__global__ void __launch_bounds__(NC_WARPS * 32, 4) k_nl_cells(Dev d, TermP p, int cur) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * NC_WARPS + (threadIdx.x >> 5);
    if (i >= d.N) return;   // warp-uniform exits
    const int r = d.rep_of[i];
    if (r < 0) return;
    const RepDev &rp = d.rep[r];
    if (!rp.rebuild || rp.tile) return;
    const double4_32a *pos = d.pos[cur];
    const double4_32a pi = pos[i];
    const BoxD bx = rp.box;
    const int ci = d.chain[i], si = d.seq[i];
    const int n0 = d.nat_start[i], n1 = d.nat_end[i];
    const unsigned FULL = 0xffffffffu, lt = (1u << lane) - 1u;
    const PairGeo<float> geo(bx, (rp.per[0] | rp.per[1] | rp.per[2]) != 0, pi);
    const float mf = rp.band_mf;

    // Go list: update_go_contacts, go.cpp:11-22 (lanes over the natives)
    for (int k = n0 + lane; k < n1; k += 32) {
        const double4_32a pj = pos[d.nat_j[k]];
        const V3<float> e = geo.to(pj);
        const float d2 = e.x * e.x + e.y * e.y + e.z * e.z;
        // band around T = 2 r_nat + pad, as in the tile build (split
        // differences carry <= 1 ulp, inside the margin)
        const double T = d.nat_T[k];
        const float Tf = narrow_f(T);
        const float mm = __fmaf_ru(Tf, 1.2e-7f, mf);
        const float blo = __fsub_rd(Tf, mm), bhi = __fadd_ru(Tf, mm);
        const Band B{blo > 0.0f ? __fmul_rd(blo, blo) : -1.0f, __fmul_ru(bhi, bhi)};
        d.nat_on[k] = in_band(B, d2) ? dist2_exact(bx, pi, pj) < d.nat_S[k] : d2 < B.lo;
    }

    // neighbouring buckets: lane l < 27 takes offsets (l/9, l/3 % 3, l % 3) - 1
    int key = -1;
    if (lane < 27) {
        const int off[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
        int cc[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
            int k = cell_coord(rp, a, a == 0 ? pi.x : (a == 1 ? pi.y : pi.z)) + off[a];
            if (rp.per[a]) k = ((k % rp.dims[a]) + rp.dims[a]) % rp.dims[a];
            else if (k < 0) ok = false;
            cc[a] = k;
        }
        if (ok) key = cell_key(rp, cc[0], cc[1], cc[2]);
    }
    // first occurrence of each key in lane order
    const unsigned same = __match_any_sync(FULL, key);
    const bool lead = key >= 0 && (same & lt) == 0u;
    // each lead lane fetches its bucket's range up front
    int kq0 = 0, kq1 = 0;
    if (lead) {
        const int c = rp.cell_off + key;
        kq0 = d.cell_start[c];
        kq1 = kq0 + d.cell_cnt[c];
    }

    const float4 me = d.cell_pos[d.bead_slot[i]];
    const float mx = me.x, my = me.y, mz = me.z;
    const float Lx = narrow_f(bx.cell[0]), Ly = narrow_f(bx.cell[1]), Lz = narrow_f(bx.cell[2]);
    const bool periodic = (rp.per[0] | rp.per[1] | rp.per[2]) != 0;
    const float pre2 = rp.pre2;
    const Band Breq{rp.band_lo[0], rp.band_hi[0]}, Bpa{rp.band_lo[1], rp.band_hi[1]};
    const Band Bes{rp.band_lo[2], rp.band_hi[2]}, Bqa{rp.band_lo[3], rp.band_hi[3]};
    const Band Bpid{rp.band_lo[4], rp.band_hi[4]};
    const bool pauli_on = p.on[XMD_TERM_PAULI] != 0;
    // PID bundles join beads that both have their chain neighbours
    const bool pid_on = p.on[XMD_TERM_PID] != 0 && (d.bflags[i] & (BF_PREV | BF_NEXT)) == (BF_PREV | BF_NEXT);
    const bool go_on = p.on[XMD_TERM_GO] != 0;
    const bool es_on = (p.on[XMD_TERM_CONST_ES] || p.on[XMD_TERM_REL_ES]);
    const bool qa_on = d.qa_on && p.on[XMD_TERM_QA];
    const int nref = qa_on ? min(d.qa.ref_cnt[i], QA_REF_CAP) : 0;
    const int nnat = n1 - n0;
    const int my_nat = lane < nnat ? d.nat_j[n0 + lane] : -1;
    // disulfide list (update_nat_ssbonds, native_ss.cpp:8-19) and partners
    const bool ss_on = p.on[XMD_TERM_NAT_SS] != 0;
    const int ss0 = d.ss_start[i], ss1 = d.ss_end[i];
    if (ss_on)
        for (int k = ss0 + lane; k < ss1; k += 32)
            d.ss_on[k] = dist2_exact(bx, pi, pos[d.ss_j[k]]) < rp.s_ss;
    const int nss = ss_on ? ss1 - ss0 : 0;
    const int my_ss = lane < nss ? d.ss_j[ss0 + lane] : -1;
    int my_qa = -1;
    if (lane < nref) {
        const int s = d.qa.ref[(size_t)lane * d.N + i];
        my_qa = d.qa.ct_i1[s] == i ? d.qa.ct_i2[s] : d.qa.ct_i1[s];
    }
    const float qi_w = narrow_f(pi.w);
    const int cap = d.nl_cap;
    int cnt = 0, tcnt = 0;
    // the buckets' candidates as one sequence (lead lanes in lane order, each
    // bucket in its ascending bead order), taken 32 at a time: lane l takes
    // entry g = base + l, which lies in the bucket of the last lane whose
    // exclusive prefix of bucket sizes is <= g
    const int csz = kq1 - kq0;
    int pre = csz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, pre, o);
        if (lane >= o) pre += y;
    }
    const int total = __shfl_sync(FULL, pre, 31);
    pre -= csz;   // exclusive
    for (int base = 0; base < total; base += 32) {
        {
            const int g = base + lane;
            int lo = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const int pm = __shfl_sync(FULL, pre, lo + step);
                if (pm <= g) lo += step;
            }
            const int q = __shfl_sync(FULL, kq0, lo) + (g - __shfl_sync(FULL, pre, lo));
            int flags = 0;
            bool qa_free = false;
            int j = -1;
            if (g < total) {
                const float4 f = d.cell_pos[q];
                j = __float_as_int(f.w);
                float ddx = f.x - mx, ddy = f.y - my, ddz = f.z - mz;
                if (periodic) {
                    ddx = min_image_f(ddx, Lx);
                    ddy = min_image_f(ddy, Ly);
                    ddz = min_image_f(ddz, Lz);
                }
                const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                if (j != i && d2 <= pre2) {
                    const int2 cs = d.cell_cs[q];
                    const int cj = cs.x, sj = cs.y;
                    const int df = si > sj ? si - sj : sj - si;
                    if (!(ci == cj && df < 3)) {
                        bool in_req, pa, es, qa, pd;
                        if (in_band(Breq, d2) || (pauli_on && in_band(Bpa, d2)) || (es_on && in_band(Bes, d2)) ||
                            (qa_on && in_band(Bqa, d2)) || (pid_on && in_band(Bpid, d2))) {
                            const double s2 = periodic ? dist2_exact(bx, pi, pos[j]) : dist2_open(pi, pos[j]);
                            in_req = s2 < rp.s_req;
                            pa = s2 < rp.s_pa;
                            es = s2 < rp.s_es;
                            qa = s2 < rp.s_qa;
                            pd = s2 < rp.s_pid;
                        } else {
                            in_req = d2 < Breq.lo;
                            pa = d2 < Bpa.lo;
                            es = d2 < Bes.lo;
                            qa = d2 < Bqa.lo;
                            pd = d2 < Bpid.lo;
                        }
                        if (in_req) {
                            if (pauli_on && pa) flags |= NL_PAULI;
                            if (es_on && es && qi_w * narrow_f(pos[j].w) != 0.0f) flags |= NL_ES;
                            if (pid_on && pd && (d.bflags[j] & (BF_PREV | BF_NEXT)) == (BF_PREV | BF_NEXT))
                                flags |= NL_PID;
                            qa_free = qa_on && j > i && qa;
                        }
                    }
                }
            }
            // a native contact leaves every list (natives leave only with
            // native contacts enabled, main.cpp:504-530); a pair in contact
            // is no free pair.  The bead's natives and contact partners are
            // held one per lane and broadcast.
            if (go_on && __any_sync(FULL, flags != 0 || qa_free)) {
                if (nnat <= 32) {
                    for (int k = 0; k < nnat; ++k)
                        if (__shfl_sync(FULL, my_nat, k) == j) { flags = 0; qa_free = false; }
                } else {
                    for (int k = n0; k < n1; ++k)
                        if (d.nat_j[k] == j) { flags = 0; qa_free = false; }
                }
            }
            if (qa_on && __any_sync(FULL, qa_free))
                for (int k = 0; k < nref; ++k)
                    if (__shfl_sync(FULL, my_qa, k) == j) qa_free = false;
            // a native disulfide is in no non-native list (main.cpp:579-580)
            if (nss && __any_sync(FULL, flags != 0 || qa_free)) {
                if (nss <= 32) {
                    for (int k = 0; k < nss; ++k)
                        if (__shfl_sync(FULL, my_ss, k) == j) { flags = 0; qa_free = false; }
                } else {
                    for (int k = ss0; k < ss1; ++k)
                        if (d.ss_j[k] == j) { flags = 0; qa_free = false; }
                }
            }
            const unsigned km = __ballot_sync(FULL, flags != 0);
            if (flags) {
                const int at = cnt + __popc(km & lt);
                if (at < cap) d.nl_row[(size_t)at * d.N + i] = j | flags;
            }
            cnt += __popc(km);
            if (qa_on) {
                const unsigned qm = __ballot_sync(FULL, qa_free);
                if (qa_free) {
                    const int at = tcnt + __popc(qm & lt);
                    if (at < QA_TMP_CAP) d.qa.tmp[(size_t)at * d.N + i] = j;
                }
                tcnt += __popc(qm);
            }
        }
    }
    if (qa_on && tcnt > 1) {
        // order the partners by j: each entry's rank is the number of smaller
        // ones (partners are distinct beads)
        const int m = min(tcnt, QA_TMP_CAP);
        __syncwarp();
        int vals[QA_TMP_CAP / 32];
#pragma unroll
        for (int u = 0; u < QA_TMP_CAP / 32; ++u) {
            const int k = u * 32 + lane;
            vals[u] = k < m ? d.qa.tmp[(size_t)k * d.N + i] : 0x7fffffff;
        }
        int rank[QA_TMP_CAP / 32];
#pragma unroll
        for (int u = 0; u < QA_TMP_CAP / 32; ++u) rank[u] = 0;
        for (int k = 0; k < m; ++k) {
            int v = 0;
#pragma unroll
            for (int u = 0; u < QA_TMP_CAP / 32; ++u)
                if (k / 32 == u) v = __shfl_sync(FULL, vals[u], k & 31);
#pragma unroll
            for (int u = 0; u < QA_TMP_CAP / 32; ++u) rank[u] += v < vals[u];
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < QA_TMP_CAP / 32; ++u) {
            const int k = u * 32 + lane;
            if (k < m) d.qa.tmp[(size_t)rank[u] * d.N + i] = vals[u];
        }
    }
    if (lane == 0) {
        atomicMax(&d.ctr[1], (unsigned long long)cnt);   // longest row needed
        if (cnt > cap) {
            atomicOr(d.status, ST_CAPACITY);
            cnt = cap;
        }
        d.nl_cnt[i] = cnt;
        d.orig[i] = pi;
        if (qa_on) {
            if (tcnt > QA_TMP_CAP) atomicOr(d.status, ST_CAPACITY);
            d.qa.tmp_cnt[i] = min(tcnt, QA_TMP_CAP);
        }
    }
}

// ---- Verlet build for replicas of at most TILE_MAX beads ---------------------------
// A block takes chunks of TL_CH beads i from the work list of the last skin
// check (the chunks of every flagged replica); for each it holds the whole replica in
// shared memory (FP32 coordinates relative to the replica, chain and sequence
// index) and each warp scans every bead j of the replica for one bead i at a
// time, lane k taking j = j0 + k.  A pair is decided in FP32 when its FP32
// distance is farther than the error margin m from every threshold (the list
// radius, r_excl + pad, 2D + pad, the QA formation radius + pad); otherwise the
// exact FP64 test decides it.  The margin (band_margin) bounds the FP32 error
// of a distance between coordinates of magnitude <= ext, so both paths keep
// exactly the same pairs.
// Rows come out ordered by j (ballot compaction in lane order).
constexpr int TL_CH = 8;       // rows per chunk: one per warp (a pass of a few replicas spreads over more blocks)
constexpr int TL_THREADS = 256;
constexpr int TL_WARPS = TL_THREADS / 32;
constexpr int TILE_MAX = 4096;

// dynamic shared memory of a tile block for a replica of n beads: the box of
// each group of 32 consecutive beads (lo, hi), then the FP32 coordinates, then
// chain and sequence indices
__host__ __device__ constexpr size_t tile_bytes(int n) {
    return 2 * sizeof(float4) * (size_t)((n + 31) / 32) + (sizeof(float4) + sizeof(int2)) * (size_t)n;
}

// FP32 coordinate of the pre-filter: wrapped into [0, L) on periodic axes,
// else relative to the replica's first bead (from split positions: the FP64
// difference to within 2^-46, then rounded to FP32, with no FP64 instruction)
__device__ __forceinline__ float tl_rel(const RepDev &rp, int a, double x, F2 ref) {
    if (rp.per[a]) return (float)(x - rp.box.cell[a] * floor(x * rp.box.cell_inv[a]));
    return ff_diff(ref, split_d(x)).h;
}



__device__ __forceinline__ void tl_chunk(const Dev &d, const TermP &p, int cur, const int2 chk) {
    const int r = chk.x;
    if (r < 0) return;   // free chunk slot
    RepDev &rp = d.rep[r];
    if (!rp.active || !rp.rebuild || !rp.tile) return;
    extern __shared__ float4 tl_smem[];
    const int b = rp.begin, n = rp.n;
    const int ng = (n + 31) / 32;
    float4 *gbox = tl_smem;
    float4 *sq = gbox + 2 * ng;
    int2 *scs = (int2 *)(sq + n);
    __shared__ float ext_s[TL_WARPS];
    const double4_32a *pos = d.pos[cur];
    const BoxD bx = rp.box;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const P2 p0 = split_p(pos[b]);

    float ext = 0.0f;
    // two loops on a block-uniform flag, so the open-box loop carries no
    // FP64 work (a select between the two forms would execute both)
    if ((rp.per[0] | rp.per[1] | rp.per[2]) == 0) {
        for (int k = t; k < n; k += TL_THREADS) {
            const double4_32a q = pos[b + k];
            const float x = ff_diff(p0.x, split_d(q.x)).h, y = ff_diff(p0.y, split_d(q.y)).h,
                        z = ff_diff(p0.z, split_d(q.z)).h;
            sq[k] = make_float4(x, y, z, narrow_f(q.w));
            scs[k] = make_int2(d.chain[b + k], d.seq[b + k]);
            ext = fmaxf(ext, fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z))));
        }
    } else {
        for (int k = t; k < n; k += TL_THREADS) {
            const double4_32a q = pos[b + k];
            const float x = tl_rel(rp, 0, q.x, p0.x), y = tl_rel(rp, 1, q.y, p0.y), z = tl_rel(rp, 2, q.z, p0.z);
            sq[k] = make_float4(x, y, z, narrow_f(q.w));
            scs[k] = make_int2(d.chain[b + k], d.seq[b + k]);
            ext = fmaxf(ext, fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z))));
        }
    }
    for (int o = 16; o; o >>= 1) ext = fmaxf(ext, __shfl_xor_sync(0xffffffffu, ext, o));
    if (lane == 0) ext_s[w] = ext;
    __syncthreads();
    ext = 0.0f;
    for (int q = 0; q < TL_WARPS; ++q) ext = fmaxf(ext, ext_s[q]);
    // decision bands of the chunk, formed once (FP64 work off the scan)
    // (one thread per band: the reciprocals are FP64 divisions)
    __shared__ Band bands_s[5];
    __shared__ float mf_s;
    if (t < 5) {
        double exd = fmax((double)ext, rp.req_r);
        for (int a = 0; a < 3; ++a) exd = fmax(exd, bx.cell[a]);
        const double m = band_margin(exd);
        const double inv = t == 1 ? rp.pauli_min_inv : t == 2 ? rp.es_min_inv : t == 3 ? rp.qa_min_inv
                                                                                       : rp.pid_min_inv;
        bands_s[t] = make_band(t == 0 ? rp.req_r : 1.0 / inv, m);
        if (t == 0) mf_s = __double2float_ru(m);
    }
    // bounding box of each group of 32 beads j (one warp per group)
    for (int g = w; g < ng; g += TL_WARPS) {
        const float4 q = sq[min(g * 32 + lane, n - 1)];
        float lx = q.x, ly = q.y, lz = q.z, hx = q.x, hy = q.y, hz = q.z;
        for (int o = 16; o; o >>= 1) {
            lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
            ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
            lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
            hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
            hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
            hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
        }
        if (lane == 0) {
            gbox[2 * g] = make_float4(lx, ly, lz, 0.0f);
            gbox[2 * g + 1] = make_float4(hx, hy, hz, 0.0f);
        }
    }
    __syncthreads();
    const float mf = mf_s;

    const bool pauli_on = p.on[XMD_TERM_PAULI] != 0;
    const bool go_on = p.on[XMD_TERM_GO] != 0;
    const bool es_on = (p.on[XMD_TERM_CONST_ES] || p.on[XMD_TERM_REL_ES]);
    const bool qa_on = d.qa_on && p.on[XMD_TERM_QA];
    const bool ss_on = p.on[XMD_TERM_NAT_SS] != 0;
    const Band Breq = bands_s[0], Bpa = bands_s[1], Bes = bands_s[2], Bqa = bands_s[3], Bpid = bands_s[4];
    const bool pid_term = p.on[XMD_TERM_PID] != 0;
    const float Lx = narrow_f(bx.cell[0]), Ly = narrow_f(bx.cell[1]), Lz = narrow_f(bx.cell[2]);
    const bool periodic = (rp.per[0] | rp.per[1] | rp.per[2]) != 0;
    const int cap = d.nl_cap;
    const unsigned lt = (1u << lane) - 1u;
    const float skip2 = Breq.hi * 1.0001f;

    if (t == 0 && chk.y == b) {
        rp.first = 0;
        rp.rebuilds += 1;
    }
    const int i_end = min(chk.y + TL_CH, b + n);
    for (int i = chk.y + w; i < i_end; i += TL_WARPS) {
        const int li = i - b;
        const float4 qi = sq[li];
        const int2 ci = scs[li];
        const double4_32a pi = pos[i];
        const int n0 = d.nat_start[i], n1 = d.nat_end[i];
        // PID bundles join beads that both have their chain neighbours
        const bool pid_on = pid_term && (d.bflags[i] & (BF_PREV | BF_NEXT)) == (BF_PREV | BF_NEXT);

        // Go list: update_go_contacts, go.cpp:11-22
        for (int k = n0 + lane; k < n1; k += 32) {
            const int j = d.nat_j[k];
            const float4 qj = sq[j - b];
            float dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
            if (periodic) {
                dx = min_image_f(dx, Lx);
                dy = min_image_f(dy, Ly);
                dz = min_image_f(dz, Lz);
            }
            const float d2 = dx * dx + dy * dy + dz * dz;
            // band around T = 2 r_nat + pad in FP32 with directed rounding,
            // widened by the narrowing error of T: at least as wide as the
            // FP64-formed band, so the exact test decides the same pairs
            const double T = d.nat_T[k];
            const float Tf = narrow_f(T);
            const float mm = __fmaf_ru(Tf, 1.2e-7f, mf);
            const float blo = __fsub_rd(Tf, mm), bhi = __fadd_ru(Tf, mm);
            const Band B{blo > 0.0f ? __fmul_rd(blo, blo) : -1.0f, __fmul_ru(bhi, bhi)};
            bool on;
            if (in_band(B, d2)) on = dist2_exact(bx, pi, pos[j]) < d.nat_S[k];
            else on = d2 < B.lo;
            d.nat_on[k] = on;
        }

        // disulfide list: update_nat_ssbonds, native_ss.cpp:8-19 (exact test;
        // a bead has at most a few disulfides)
        const int ss0 = d.ss_start[i], ss1 = d.ss_end[i];
        if (ss_on)
            for (int k = ss0 + lane; k < ss1; k += 32) {
                const double4_32a pj = pos[d.ss_j[k]];
                d.ss_on[k] = (periodic ? dist2_exact(bx, pi, pj) : dist2_open(pi, pj)) < rp.s_ss;
            }
        const int nss = ss_on ? ss1 - ss0 : 0;
        const int my_ss = lane < nss ? d.ss_j[ss0 + lane] : -1;

        int nref = 0;
        if (qa_on) nref = min(d.qa.ref_cnt[i], QA_REF_CAP);
        // the row's natives and contact partners, one per lane (broadcast by
        // shuffle in the exclusion checks)
        const int nnat = n1 - n0;
        const int my_nat = lane < nnat ? d.nat_j[n0 + lane] : -1;
        int my_qa = -1;
        if (lane < nref) {
            const int s = d.qa.ref[(size_t)lane * d.N + i];
            my_qa = d.qa.ct_i1[s] == i ? d.qa.ct_i2[s] : d.qa.ct_i1[s];
        }
        int cnt = 0, tcnt = 0;
        for (int j0 = 0; j0 < n; j0 += 32) {
            if (!periodic) {
                // a group whose box is beyond the list radius holds no pair
                // (FP32 rounding is monotone, so the box distance never exceeds
                // a member's distance; the factor covers contraction order)
                const float4 lo = gbox[2 * (j0 >> 5)], hi = gbox[2 * (j0 >> 5) + 1];
                const float gx = fmaxf(fmaxf(lo.x - qi.x, qi.x - hi.x), 0.0f);
                const float gy = fmaxf(fmaxf(lo.y - qi.y, qi.y - hi.y), 0.0f);
                const float gz = fmaxf(fmaxf(lo.z - qi.z, qi.z - hi.z), 0.0f);
                if (gx * gx + gy * gy + gz * gz > skip2) continue;
            }
            const int lj = j0 + lane;
            int flags = 0;
            bool qa_free = false;
            if (lj < n && lj != li) {
                const float4 qj = sq[lj];
                float dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
                if (periodic) {
                    dx = min_image_f(dx, Lx);
                    dy = min_image_f(dy, Ly);
                    dz = min_image_f(dz, Lz);
                }
                const float d2 = dx * dx + dy * dy + dz * dz;
                const int2 cj = scs[lj];
                const int df = ci.y > cj.y ? ci.y - cj.y : cj.y - ci.y;
                if (d2 <= Breq.hi && !(ci.x == cj.x && df < 3)) {
                    bool in_req, pa, es, qa, pd;
                    if (in_band(Breq, d2) || (pauli_on && in_band(Bpa, d2)) || (es_on && in_band(Bes, d2)) ||
                        (qa_on && in_band(Bqa, d2)) || (pid_on && in_band(Bpid, d2))) {
                        const double s2 = periodic ? dist2_exact(bx, pi, pos[b + lj]) : dist2_open(pi, pos[b + lj]);
                        in_req = s2 < rp.s_req;
                        pa = s2 < rp.s_pa;
                        es = s2 < rp.s_es;
                        qa = s2 < rp.s_qa;
                        pd = s2 < rp.s_pid;
                    } else {
                        in_req = d2 < Breq.lo;
                        pa = d2 < Bpa.lo;
                        es = d2 < Bes.lo;
                        qa = d2 < Bqa.lo;
                        pd = d2 < Bpid.lo;
                    }
                    if (in_req) {
                        if (pauli_on && pa) flags |= NL_PAULI;
                        if (es_on && es && qi.w * qj.w != 0.0f) flags |= NL_ES;
                        if (pid_on && pd && (d.bflags[b + lj] & (BF_PREV | BF_NEXT)) == (BF_PREV | BF_NEXT))
                            flags |= NL_PID;
                        qa_free = qa_on && lj > li && qa;
                    }
                }
            }
            // natives leave the list only with native contacts enabled
            // (main.cpp:504-530); the loop is warp-uniform
            if (go_on && __any_sync(0xffffffffu, flags != 0 || qa_free)) {
                if (nnat <= 32) {
                    for (int k = 0; k < nnat; ++k)
                        if (__shfl_sync(0xffffffffu, my_nat, k) == b + lj) { flags = 0; qa_free = false; }
                } else {
                    for (int k = n0; k < n1; ++k)
                        if (d.nat_j[k] == b + lj) { flags = 0; qa_free = false; }
                }
            }
            if (qa_on && __any_sync(0xffffffffu, qa_free))
                for (int k = 0; k < nref; ++k)
                    if (__shfl_sync(0xffffffffu, my_qa, k) == b + lj) qa_free = false;
            // a native disulfide is in no non-native list (legacy_update's
            // merge against all_nat_ss, main.cpp:579-580)
            if (nss && __any_sync(0xffffffffu, flags != 0 || qa_free)) {
                if (nss <= 32) {
                    for (int k = 0; k < nss; ++k)
                        if (__shfl_sync(0xffffffffu, my_ss, k) == b + lj) { flags = 0; qa_free = false; }
                } else {
                    for (int k = ss0; k < ss1; ++k)
                        if (d.ss_j[k] == b + lj) { flags = 0; qa_free = false; }
                }
            }
            const unsigned km = __ballot_sync(0xffffffffu, flags != 0);
            if (flags) {
                const int at = cnt + __popc(km & lt);
                if (at < cap) d.nl_row[(size_t)at * d.N + i] = (b + lj) | flags;
            }
            cnt += __popc(km);
            if (qa_on) {
                const unsigned qm = __ballot_sync(0xffffffffu, qa_free);
                if (qa_free) {
                    const int at = tcnt + __popc(qm & lt);
                    if (at < QA_TMP_CAP) d.qa.tmp[(size_t)at * d.N + i] = b + lj;
                }
                tcnt += __popc(qm);
            }
        }
        if (lane == 0) {
            atomicMax(&d.ctr[1], (unsigned long long)cnt);
            if (cnt > cap) {
                atomicOr(d.status, ST_CAPACITY);
                cnt = cap;
            }
            d.nl_cnt[i] = cnt;
            d.orig[i] = pi;
            if (qa_on) {
                if (tcnt > QA_TMP_CAP) atomicOr(d.status, ST_CAPACITY);
                d.qa.tmp_cnt[i] = min(tcnt, QA_TMP_CAP);
            }
        }
    }
}

// `count`: a pass with work adds to the pass counter (launches that run
// every step, with or without work, are counted where they are issued)
__global__ void __launch_bounds__(TL_THREADS, 4) k_nl_tile(Dev d, TermP p, int cur, int count) {
    const int nw = *d.nwork;
    if (count && blockIdx.x == 0 && threadIdx.x == 0 && !d.any_cell && nw > 0) atomicAdd(d.ctr, 1ull);
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        tl_chunk(d, p, cur, d.chunks[d.work[w]]);
        __syncthreads();   // the next chunk overwrites the shared tile
    }
}

// =================================================================== host ==

// the step kernel of a precision, mode and launch shape (beads per block and
// threads per bead, the shapes the autotuner chooses from); the evaluation
// pass has one shape
constexpr int EVAL_FB = 64, EVAL_LPB = 4;
static int force_block_beads(int fb, int) { return fb; }
static void *force_kernel(bool mixed, int mode, int fb, int lpb) {
#define XMD_FK(M, B, L) (mixed ? (void *)k_force<float, M, B, L> : (void *)k_force<double, M, B, L>)
    if (mode == 0) return XMD_FK(0, EVAL_FB, EVAL_LPB);
    switch (fb * 8 + lpb) {
    case 32 * 8 + 1: return XMD_FK(1, 32, 1);
    case 32 * 8 + 2: return XMD_FK(1, 32, 2);
    case 32 * 8 + 4: return XMD_FK(1, 32, 4);
    case 64 * 8 + 1: return XMD_FK(1, 64, 1);
    case 64 * 8 + 2: return XMD_FK(1, 64, 2);
    case 64 * 8 + 4: return XMD_FK(1, 64, 4);
    case 128 * 8 + 1: return XMD_FK(1, 128, 1);
    case 128 * 8 + 2: return XMD_FK(1, 128, 2);
    default: return XMD_FK(1, 128, 4);
    }
#undef XMD_FK
}

void Engine::launch_force(int mode, int c) {
    if (tp.ext_on) {
        if (mode == 0) k_ext<0><<<(d.N + 255) / 256, 256, 0, stream>>>(d, tp, c);
        else k_ext<1><<<(d.N + 255) / 256, 256, 0, stream>>>(d, tp, c);
    }
    if (tp.on[XMD_TERM_PID]) {
        if (mode == 0) k_pid<0><<<(d.N + 127) / 128, 128, 0, stream>>>(d, tp, c);
        else k_pid<1><<<(d.N + 127) / 128, 128, 0, stream>>>(d, tp, c);
    }
    const int fb = mode == 0 ? EVAL_FB : tune.fb, lpb = mode == 0 ? EVAL_LPB : tune.lpb;
    const int nb = (d.N + force_block_beads(fb, lpb) - 1) / force_block_beads(fb, lpb);
    int fuse = FUSE_NONE;
    void *args[] = {&d, &tp, &c, &fuse};
    CK(cudaLaunchKernel(force_kernel(params.precision == XMD_PREC_MIXED, mode, fb, lpb), dim3(nb), dim3(fb * lpb),
                        args, 0, stream));
}

Engine::Engine(const xmd_params &p) : params(p) {
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (ndev < 1) throw std::runtime_error("no CUDA device");
    device = p.device;
    if (device < 0 || device >= ndev) throw std::invalid_argument("engine: device out of range");
    use_device();
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ustream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev_staged, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_removed, cudaEventDisableTiming));
    CK(cudaMallocHost(&h_any, sizeof(int) * 4));
}

Engine::~Engine() {
    cudaSetDevice(device);
    for (auto &kv : graphs) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    }
    for (auto e : ev_force) cudaEventDestroy(e);
    for (auto e : ev_rebuild) cudaEventDestroy(e);
    release();
    if (h_any) cudaFreeHost(h_any);
    if (ev_staged) cudaEventDestroy(ev_staged);
    if (ev_removed) cudaEventDestroy(ev_removed);
    if (ustream) cudaStreamDestroy(ustream);
    if (stream) cudaStreamDestroy(stream);
}

void *Engine::dalloc(size_t bytes) {
    void *p = nullptr;
    CK(cudaMalloc(&p, bytes < 16 ? 16 : bytes));
    CK(cudaMemsetAsync(p, 0, bytes < 16 ? 16 : bytes, stream));
    allocs.push_back(p);
    alloc_bytes += bytes < 16 ? 16 : bytes;
    return p;
}

void Engine::release() {
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
    alloc_bytes = 0;
    d = Dev{};
    finalized = false;
}

int Engine::add_replica(int n, const int32_t *chain, const int32_t *seq, const uint8_t *atype,
                        const double cell[3], double temperature, uint64_t seed) {
    if (finalized && !dynamic)
        throw std::invalid_argument("replicas must be added before the first eval/step (or reserve capacity)");
    if (n <= 0 || n > NL_MASK) throw std::invalid_argument("bead count out of range");
    if (!chain || !seq || !atype) throw std::invalid_argument("null topology array");
    RepHost r;
    r.n = n;
    r.chain.assign(chain, chain + n);
    r.seq.assign(seq, seq + n);
    r.atype.assign(atype, atype + n);
    for (int i = 0; i < n; ++i)
        if (atype[i] >= XMD_NUM_AA) throw std::invalid_argument("atype out of range (0..19)");
    for (int a = 0; a < 3; ++a) {
        r.cell[a] = cell ? cell[a] : 0.0;
        if (r.cell[a] < 0 || !std::isfinite(r.cell[a])) throw std::invalid_argument("bad cell");
    }
    r.temperature = temperature > 0 ? temperature : params.temperature;
    r.seed = seed;
    const double nan = std::nan("");
    r.teth_r0.assign(n, nan);
    r.ang_t0.assign(n, nan);
    r.dih_p0.assign(n, nan);
    r.chir_f.assign(n, nan);
    r.chir_n.assign(n, nan);
    r.hang_t.assign(n, -1);
    r.hdih_t.assign(n, -1);
    if (dynamic) {
        // reuse a free slot; the replica is placed at the next eval/step
        for (int k = 0; k < (int)reps.size(); ++k)
            if (!reps[k].in_use) {
                reps[k] = std::move(r);
                return k;
            }
        if ((int)reps.size() >= cap.reps) throw std::length_error("engine: every reserved replica slot is taken");
    }
    reps.push_back(std::move(r));
    return (int)reps.size() - 1;
}

static void check_rep(const std::vector<RepHost> &reps, int rep) {
    if (rep < 0 || rep >= (int)reps.size() || !reps[rep].in_use)
        throw std::invalid_argument("replica id out of range");
}

void Engine::reserve(int beads, int replicas, int natives) {
    if (finalized) throw std::logic_error("reserve must precede the first eval/step");
    if (params.on[XMD_TERM_QA]) throw std::invalid_argument("reserve: the quasi-adiabatic term needs a static context");
    if (beads < 1 || replicas < 1 || natives < 0) throw std::invalid_argument("reserve: bad capacity");
    int nb = 0;
    for (auto &r : reps) nb += r.n;
    if (nb > beads || (int)reps.size() > replicas) throw std::invalid_argument("reserve: replicas already exceed it");
    dynamic = true;
    cap = Caps{};
    cap.beads = beads;
    cap.reps = replicas;
    cap.nat = natives;
    cap.ss = natives;   // disulfide entries share the native budget
    // bucket pool for replicas above the tile limit; chunk slots for the rest
    cap.cells = params.nl_build == XMD_NL_BUILD_TILE ? 0 : std::max(64, 2 * beads);
    cap.chunks = params.nl_build == XMD_NL_BUILD_CELL ? 0 : beads / TL_CH + replicas;
    finalize();
}

void Engine::remove_replica(int rep) {
    check_rep(reps, rep);
    if (!dynamic) throw std::logic_error("remove_replica needs a context with reserved capacity");
    RepHost &r = reps[rep];
    if (r.placed) {
        use_device();
        const int b = r.begin, n = r.n;
        CK(cudaStreamSynchronize(stream));
        CK(cudaMemsetAsync(d.rep_of + b, 0xff, sizeof(int32_t) * n, stream));
        CK(cudaMemsetAsync(d.bflags + b, 0, sizeof(uint32_t) * n, stream));
        CK(cudaMemsetAsync(d.nl_cnt + b, 0, sizeof(int32_t) * n, stream));
        if (r.nat_len) CK(cudaMemsetAsync(d.nat_on + r.nat_off, 0, r.nat_len, stream));
        if (r.chunk_len) CK(cudaMemsetAsync(d.chunks + r.chunk_off, 0xff, sizeof(int2) * r.chunk_len, stream));
        if (r.cell_len) CK(cudaMemsetAsync(d.cell_rep + r.cell_off, 0xff, sizeof(int32_t) * r.cell_len, stream));
        CK(cudaMemsetAsync(d.rep + rep, 0, sizeof(RepDev), stream));
        CK(cudaStreamSynchronize(stream));
        for (int i = 0; i < n; ++i) owner_h[b + i] = -1;
        update_blocks(b, b + n);
        a_beads.release(b, n);
        a_nat.release(r.nat_off, r.nat_len);
        a_ss.release(r.ss_off, r.ss_len);
        CK(cudaMemsetAsync(d.ss_start + b, 0, sizeof(int32_t) * n, stream));
        CK(cudaMemsetAsync(d.ss_end + b, 0, sizeof(int32_t) * n, stream));
        a_cells.release(r.cell_off, r.cell_len);
        a_chunks.release(r.chunk_off, r.chunk_len);
        a_afm.release(r.afm_off, r.afm_len);
        // staged uploads into these ranges wait for the clears above
        CK(cudaEventRecord(ev_removed, stream));
    } else if (r.staged) {
        // staged, never activated: its uploads are ordered before any later
        // staging on the side stream, so its ranges can be reused at once
        for (size_t q = 0; q < staged_reps.size(); ++q)
            if (staged_reps[q].k == rep) {
                staged_reps.erase(staged_reps.begin() + (long)q);
                break;
            }
        a_beads.release(r.begin, r.n);
        a_nat.release(r.nat_off, r.nat_len);
        a_ss.release(r.ss_off, r.ss_len);
        a_cells.release(r.cell_off, r.cell_len);
        a_chunks.release(r.chunk_off, r.chunk_len);
        a_afm.release(r.afm_off, r.afm_len);
    }
    r = RepHost{};
    r.in_use = false;
}

void Engine::stage(int rep) {
    check_rep(reps, rep);
    if (!dynamic) throw std::logic_error("stage needs a context with reserved capacity");
    ready_alloc();
    RepHost &r = reps[rep];
    if (r.placed || r.staged) return;
    if (!r.have_state) throw std::logic_error("set_state must precede placement");
    use_device();
    Staged st;
    place(rep, &st);
    staged_reps.push_back(std::move(st));
}

void Engine::activate_staged() {
    if (staged_reps.empty()) return;
    use_device();
    CK(cudaEventRecord(ev_staged, ustream));
    CK(cudaStreamWaitEvent(stream, ev_staged, 0));
    for (Staged &st : staged_reps) {
        RepHost &r = reps[st.k];
        CK(cudaMemcpyAsync(d.rep_of + r.begin, st.rep_of.data(), sizeof(int32_t) * r.n, cudaMemcpyHostToDevice,
                           stream));
        if (!st.cell_rep.empty())
            CK(cudaMemcpyAsync(d.cell_rep + r.cell_off, st.cell_rep.data(), sizeof(int32_t) * st.cell_rep.size(),
                               cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(d.rep + st.k, &st.rd, sizeof(RepDev), cudaMemcpyHostToDevice, stream));
        for (int i = 0; i < r.n; ++i) owner_h[r.begin + i] = st.k;
        update_blocks(r.begin, r.begin + r.n, false);
        r.staged = false;
        r.placed = true;
    }
    staged_reps.clear();
}

void Engine::step_async(int nsteps) {
    use_device();
    ready();
    if (!params.langevin_on) throw std::invalid_argument("langevin: enabled is false; nothing integrates");
    ensure_nl();
    int s = 0;
    if (!timing && use_graphs) {
        const int gsteps = tune.graph_steps;
        // launches per step of each graph form: the step kernel, plus the
        // quasi-adiabatic kernels with that term, the external-force and PID
        // kernels, and the plain form's row-build node or the IF form's
        // separate check (gated QA graphs take the decision in the
        // re-freeing kernel); rebuild kernels of IF nodes and of the host's
        // rebuilds are counted per pass in stats()
        const int64_t extra = (tp.ext_on ? 1 : 0) + (tp.on[XMD_TERM_PID] ? 1 : 0);
        const int64_t per_plain = 2 + extra, per_gated = (d.qa_on ? 5 : 1) + extra,
                      per_cond = (d.qa_on ? 6 : 2) + extra;
        // graphs of graph_steps steps, and the rest in graphs of the largest
        // powers of two that fit
        auto chunk = [&](int left) {
            if (left >= gsteps) return gsteps;
            int l = 1;
            while (2 * l <= left) l *= 2;
            return l;
        };
        if (gated_graphs()) {
            // each graph runs until a check flags a replica (or its steps are
            // done); the host then rebuilds and goes on from the steps taken.
            // While rebuilds come every few steps (a relaxing start) the
            // halted steps would be launches for nothing: graphs with IF
            // rebuild nodes run instead for a while.  The gate is open
            // outside the gated graphs (per-launch steps read it).
            struct Open {
                Engine *e;
                ~Open() { cudaMemsetAsync(e->d.gate, 0, sizeof(int) * 3, e->stream); }
            } open_gate{this};
            while (s < nsteps) {
                const int len = chunk(nsteps - s);
                if (cond_graphs_left > 0) {
                    CK(cudaGraphLaunch(graph_for(cur, false, len), stream));
                    launches += per_cond * len;
                    md_steps += len;
                    s += len;
                    cur ^= len & 1;
                    --cond_graphs_left;
                    continue;
                }
                h_any[0] = 0; h_any[1] = 0; h_any[2] = 0; h_any[3] = len;
                CK(cudaMemcpyAsync(d.any_rebuild, h_any, sizeof(int) * 4, cudaMemcpyHostToDevice, stream));
                CK(cudaGraphLaunch(graph_for(cur, true, len), stream));
                CK(cudaMemcpyAsync(h_any, d.any_rebuild, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
                CK(cudaStreamSynchronize(stream));
                const int done = h_any[2];
                if (done < 1 || done > len) throw std::logic_error("engine: graph step count out of range");
                CK(cudaMemsetAsync(d.gate, 0, sizeof(int) * 3, stream));   // open for what follows
                launches += per_gated * len;
                md_steps += done;
                s += done;
                cur ^= done & 1;
                if (h_any[0]) {
                    launch_rebuild();
                    if (done < len / 4) cond_graphs_left = 8;
                }
            }
        } else {
            const int64_t per = plain_rebuild() ? per_plain : per_cond;
            while (s < nsteps) {
                const int len = chunk(nsteps - s);
                CK(cudaGraphLaunch(graph_for(cur, false, len), stream));
                launches += per * len;
                md_steps += len;
                s += len;
                cur ^= len & 1;
            }
        }
    }
    for (; s < nsteps; ++s) {
        launch_force_step();
        cur ^= 1;
        k_nl_check<<<1, 1024, 0, stream>>>(d, 1, params.dt, (cudaGraphConditionalHandle)0, 0);
        ++launches;
        ++md_steps;
        CK(cudaMemcpyAsync(h_any, d.any_rebuild, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (*h_any) launch_rebuild();
    }
}

void Engine::step_wait() {
    use_device();
    check_status("step");
    if (auto_grow) grow_rows(0.6);
}

void Engine::set_steps(int rep, long long nsteps) {
    check_rep(reps, rep);
    if (params.on[XMD_TERM_QA]) throw std::invalid_argument("per-replica step budgets exclude the quasi-adiabatic term");
    reps[rep].steps_left = nsteps < 0 ? -1 : nsteps;
    if (reps[rep].placed) {
        use_device();
        long long v = reps[rep].steps_left;
        CK(cudaMemcpyAsync((char *)(d.rep + rep) + offsetof(RepDev, steps_left), &v, sizeof v,
                           cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
    }
}

void Engine::place_now(int rep) {
    check_rep(reps, rep);
    ready_alloc();
    if (!reps[rep].placed) {
        if (!reps[rep].have_state) throw std::logic_error("set_state must precede placement");
        use_device();
        place(rep);
    }
}

void Engine::steps_left(long long *out) {
    use_device();
    std::vector<RepDev> rd(std::max(1, d.R));
    if (finalized) {
        CK(cudaMemcpyAsync(rd.data(), d.rep, sizeof(RepDev) * d.R, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
    }
    for (int k = 0; k < (int)reps.size(); ++k)
        out[k] = !reps[k].in_use ? -2
                 : (reps[k].placed ? (rd[k].fault ? -3 : rd[k].steps_left) : reps[k].steps_left);
}
static bool consecutive(const RepHost &r, int a, int b) {
    return a >= 0 && b < r.n && b == a + 1 && r.chain[a] == r.chain[b] && r.seq[b] == r.seq[a] + 1;
}

void Engine::set_tethers(int rep, int n, const int32_t *i1, const int32_t *i2, const double *dd) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::fill(r.teth_r0.begin(), r.teth_r0.end(), std::nan(""));
    for (int k = 0; k < n; ++k) {
        int a = std::min(i1[k], i2[k]), b = std::max(i1[k], i2[k]);
        if (!consecutive(r, a, b)) throw std::invalid_argument("tether is not a bond between consecutive beads of a chain");
        if (!std::isnan(r.teth_r0[a])) throw std::invalid_argument("duplicate tether");
        // tether.length.value_or(def_length), main.cpp:409-413
        r.teth_r0[a] = (dd && dd[k] > 0) ? dd[k] : params.tether_def_length;
    }
}
void Engine::set_angles(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                        const double *th) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::fill(r.ang_t0.begin(), r.ang_t0.end(), std::nan(""));
    for (int k = 0; k < n; ++k) {
        if (!consecutive(r, i1[k], i2[k]) || !consecutive(r, i2[k], i3[k]))
            throw std::invalid_argument("angle must be (i-1, i, i+1) of one chain");
        if (!std::isnan(r.ang_t0[i2[k]])) throw std::invalid_argument("duplicate angle");
        if (r.hang_t[i2[k]] >= 0) throw std::invalid_argument("angle is already heuristic");
        if (!std::isfinite(th[k])) throw std::invalid_argument("non-finite native angle");
        r.ang_t0[i2[k]] = th[k];
    }
}
void Engine::set_dihedrals(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                           const int32_t *i4, const double *ph) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::fill(r.dih_p0.begin(), r.dih_p0.end(), std::nan(""));
    for (int k = 0; k < n; ++k) {
        if (!consecutive(r, i1[k], i2[k]) || !consecutive(r, i2[k], i3[k]) || !consecutive(r, i3[k], i4[k]))
            throw std::invalid_argument("dihedral must be (i-1, i, i+1, i+2) of one chain");
        if (!std::isnan(r.dih_p0[i2[k]])) throw std::invalid_argument("duplicate dihedral");
        if (r.hdih_t[i2[k]] >= 0) throw std::invalid_argument("dihedral is already heuristic");
        if (!std::isfinite(ph[k])) throw std::invalid_argument("non-finite native dihedral");
        r.dih_p0[i2[k]] = ph[k];
    }
}
void Engine::set_native(int rep, int n, const int32_t *i1, const int32_t *i2, const double *dd) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::vector<std::tuple<int, int, double>> v;
    for (int k = 0; k < n; ++k) {
        int a = std::min(i1[k], i2[k]), b = std::max(i1[k], i2[k]);
        if (a < 0 || b >= r.n || a == b) throw std::invalid_argument("native contact index out of range");
        if (!(dd[k] > 0)) throw std::invalid_argument("native distance must be positive");
        v.emplace_back(a, b, dd[k]);
    }
    std::sort(v.begin(), v.end());
    for (size_t k = 1; k < v.size(); ++k)
        if (std::get<0>(v[k]) == std::get<0>(v[k - 1]) && std::get<1>(v[k]) == std::get<1>(v[k - 1]))
            throw std::invalid_argument("duplicate native contact");
    r.nat_i1.clear(); r.nat_i2.clear(); r.nat_d.clear();
    for (auto &[a, b, x] : v) { r.nat_i1.push_back(a); r.nat_i2.push_back(b); r.nat_d.push_back(x); }
}

void Engine::set_chirals(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                         const int32_t *i4, const double *f, const double *c) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::fill(r.chir_f.begin(), r.chir_f.end(), std::nan(""));
    std::fill(r.chir_n.begin(), r.chir_n.end(), std::nan(""));
    for (int k = 0; k < n; ++k) {
        if (!consecutive(r, i1[k], i2[k]) || !consecutive(r, i2[k], i3[k]) || !consecutive(r, i3[k], i4[k]))
            throw std::invalid_argument("chiral quad must be (i-1, i, i+1, i+2) of one chain");
        if (!std::isnan(r.chir_f[i2[k]])) throw std::invalid_argument("duplicate chiral quad");
        if (!std::isfinite(f[k]) || !std::isfinite(c[k])) throw std::invalid_argument("non-finite chiral parameter");
        r.chir_f[i2[k]] = f[k];
        r.chir_n[i2[k]] = c[k];
    }
}
// heur_ang_type / heur_dih_type: G = 0, P = 1, any other residue = 2,
// type = 3 t1 + t2 (angle/heurestic.cpp:9-15, dihedral/heurestic.cpp:8-14)
static int8_t heur_type(uint8_t a, uint8_t b) {
    auto cls = [](uint8_t x) { return x == 7 ? 0 : (x == 14 ? 1 : 2); };   // GLY, PRO of amino_acid.h:10-13
    return (int8_t)(3 * cls(a) + cls(b));
}
void Engine::set_heuristic_angles(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::fill(r.hang_t.begin(), r.hang_t.end(), (int8_t)-1);
    for (int k = 0; k < n; ++k) {
        if (!consecutive(r, i1[k], i2[k]) || !consecutive(r, i2[k], i3[k]))
            throw std::invalid_argument("heuristic angle must be (i-1, i, i+1) of one chain");
        if (r.hang_t[i2[k]] >= 0) throw std::invalid_argument("duplicate heuristic angle");
        if (!std::isnan(r.ang_t0[i2[k]])) throw std::invalid_argument("angle is already native");
        r.hang_t[i2[k]] = heur_type(r.atype[i1[k]], r.atype[i2[k]]);
    }
}
void Engine::set_heuristic_dihedrals(int rep, int n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                                     const int32_t *i4) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::fill(r.hdih_t.begin(), r.hdih_t.end(), (int8_t)-1);
    for (int k = 0; k < n; ++k) {
        if (!consecutive(r, i1[k], i2[k]) || !consecutive(r, i2[k], i3[k]) || !consecutive(r, i3[k], i4[k]))
            throw std::invalid_argument("heuristic dihedral must be (i-1, i, i+1, i+2) of one chain");
        if (r.hdih_t[i2[k]] >= 0) throw std::invalid_argument("duplicate heuristic dihedral");
        if (!std::isnan(r.dih_p0[i2[k]])) throw std::invalid_argument("dihedral is already native");
        r.hdih_t[i2[k]] = heur_type(r.atype[i2[k]], r.atype[i3[k]]);
    }
}
void Engine::set_velocity_afm(int rep, int n, const int32_t *bead, const double *orig, const double *vel) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    if (dynamic) throw std::invalid_argument("AFM tips need a static context");
    RepHost &r = reps[rep];
    std::vector<int32_t> seen;
    for (int k = 0; k < n; ++k) {
        if (bead[k] < 0 || bead[k] >= r.n) throw std::invalid_argument("AFM tip bead out of range");
        if (std::find(seen.begin(), seen.end(), bead[k]) != seen.end())
            throw std::invalid_argument("one velocity AFM tip per bead");
        seen.push_back(bead[k]);
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(vel[3 * k + a]) || std::isinf(orig[3 * k + a]))
                throw std::invalid_argument("non-finite AFM tip");
    }
    r.vafm_i.assign(bead, bead + n);
    r.vafm_o.assign(orig, orig + 3 * n);
    r.vafm_v.assign(vel, vel + 3 * n);
}
void Engine::set_force_afm(int rep, int n, const int32_t *bead, const double *F) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    if (dynamic) throw std::invalid_argument("AFM tips need a static context");
    RepHost &r = reps[rep];
    for (int k = 0; k < n; ++k) {
        if (bead[k] < 0 || bead[k] >= r.n) throw std::invalid_argument("AFM tip bead out of range");
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(F[3 * k + a])) throw std::invalid_argument("non-finite AFM force");
    }
    r.fafm_i.assign(bead, bead + n);
    r.fafm_F.assign(F, F + 3 * n);
}
void Engine::set_walls(int kind, int n, const double *origin, const double *normal) {
    if (kind != 0 && kind != 1) throw std::invalid_argument("wall kind must be 0 (solid) or 1 (LJ attractive)");
    if (n < 0 || n > XMD_MAX_WALLS) throw std::invalid_argument("at most XMD_MAX_WALLS planes per wall kind");
    if (finalized) throw std::invalid_argument("walls are set before the first replica is placed");
    std::vector<double> w;
    for (int k = 0; k < n; ++k) {
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(origin[3 * k + a]) || !std::isfinite(normal[3 * k + a]))
                throw std::invalid_argument("non-finite wall plane");
        for (int a = 0; a < 3; ++a) w.push_back(origin[3 * k + a]);
        for (int a = 0; a < 3; ++a) w.push_back(normal[3 * k + a]);
    }
    walls[kind] = w;
}
// beads of replica r pulled by some AFM tip, in order
static std::vector<int> afm_beads(const RepHost &r) {
    std::vector<int> v(r.vafm_i.begin(), r.vafm_i.end());
    v.insert(v.end(), r.fafm_i.begin(), r.fafm_i.end());
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
}
void Engine::set_ssbonds(int rep, int n, const int32_t *i1, const int32_t *i2) {
    check_rep(reps, rep);
    if (reps[rep].placed) throw std::invalid_argument("topology is fixed once the replica is on the device");
    RepHost &r = reps[rep];
    std::vector<std::pair<int, int>> v;
    for (int k = 0; k < n; ++k) {
        int a = std::min(i1[k], i2[k]), b = std::max(i1[k], i2[k]);
        if (a < 0 || b >= r.n || a == b) throw std::invalid_argument("disulfide index out of range");
        v.emplace_back(a, b);
    }
    std::sort(v.begin(), v.end());
    if (std::adjacent_find(v.begin(), v.end()) != v.end()) throw std::invalid_argument("duplicate disulfide");
    r.ss_i1.clear(); r.ss_i2.clear();
    for (auto &[a, b] : v) { r.ss_i1.push_back(a); r.ss_i2.push_back(b); }
}

void Engine::derive_rep(int ri, RepDev &rd) {
    const RepHost &r = reps[ri];
    const xmd_params &p = params;
    std::memset(&rd, 0, sizeof rd);
    for (int a = 0; a < 3; ++a) {
        rd.box.cell[a] = r.cell[a];
        rd.box.cell_inv[a] = r.cell[a] != 0.0 ? 1.0 / r.cell[a] : 0.0;   // box.h:12-22
        rd.per[a] = r.cell[a] != 0.0;
    }
    // max_cutoff: main.cpp:500, 545-551, 628-630, 642-644, 742-746
    double mc = 0.0;
    if (p.on[XMD_TERM_PAULI]) mc = std::max(mc, p.pauli_r_excl);
    if (p.on[XMD_TERM_NAT_SS]) mc = std::max(mc, 2.0 * p.nat_ss_dist);   // harmonic::cutoff, main.cpp:596-597
    if (p.on[XMD_TERM_GO]) for (double x : r.nat_d) mc = std::max(mc, 2.0 * x);
    if (p.on[XMD_TERM_CONST_ES]) mc = std::max(mc, 2.0 * p.const_es_screen_dist);
    if (p.on[XMD_TERM_REL_ES]) mc = std::max(mc, 2.0 * p.rel_es_screen_dist);
    // max req_min_dist over contact types (main.cpp:742-746), also the
    // intended max_formation_min_dist of update_free_pairs
    double max_form = std::max(p.lj_bb_r_min, p.lj_bs_r_min);
    for (int k = 0; k < XMD_NUM_SS; ++k) max_form = std::max(max_form, p.ss_r_max[k]);
    if (p.on[XMD_TERM_QA]) mc = std::max(mc, max_form);
    // PID bundles: the largest LJ-variant cutoff (lj::cutoff = 2 r_min,
    // sink_lj::cutoff = 2 r_max), main.cpp:801-810
    double pid_cut = std::max(2.0 * p.lj_bb_r_min, 2.0 * p.lj_bs_r_min);
    for (int k = 0; k < XMD_NUM_SS; ++k) pid_cut = std::max(pid_cut, 2.0 * p.ss_r_max[k]);
    if (p.on[XMD_TERM_PID]) mc = std::max(mc, pid_cut);
    if (p.nl_cutoff > 0.0) mc = p.nl_cutoff;
    rd.pad = p.nl_skin > 0.0 ? p.nl_skin : p.pad_factor * mc;   // legacy_update.cpp:7-8
    rd.req_r = mc + rd.pad;
    double es_cut = p.on[XMD_TERM_CONST_ES] ? 2.0 * p.const_es_screen_dist : 2.0 * p.rel_es_screen_dist;
    rd.es_min_inv = 1.0 / (es_cut + rd.pad);                      // es_pair.cpp:9
    rd.pauli_min_inv = 1.0 / (p.pauli_r_excl + rd.pad);           // pauli.cpp:12-13
    rd.qa_min_inv = 1.0 / (max_form + rd.pad);                     // free_pair.cpp:9-10
    rd.pid_min_inv = 1.0 / (pid_cut + rd.pad);                     // pid/bundle.cpp:9-12
    rd.s_req = sq_below(rd.req_r);
    rd.s_pa = sq_below(inv_above(rd.pauli_min_inv));
    rd.s_es = sq_below(inv_above(rd.es_min_inv));
    rd.s_qa = sq_below(inv_above(rd.qa_min_inv));
    rd.s_pid = sq_below(inv_above(rd.pid_min_inv));
    rd.s_ss = sq_below(2.0 * p.nat_ss_dist + rd.pad);   // update_nat_ssbonds, native_ss.cpp:15
    rd.noise_sd = std::sqrt(2.0 * 1.0 * r.temperature) * std::sqrt(p.gamma_factor) * 1.0;
    rd.begin = r.begin;
    rd.n = r.n;
    rd.first = 1;
}

// Capacities: exact totals of the replicas added so far (static contexts), or
// the reservation (dynamic contexts, where replicas come and go between steps).
void Engine::finalize() {
    if (finalized) return;
    if (!dynamic) {
        if (reps.empty()) throw std::logic_error("no replica added");
        for (auto &r : reps)
            if (!r.have_state) throw std::logic_error("set_state must be called for every replica");
        cap = Caps{};
        cap.reps = (int)reps.size();
        for (auto &r : reps) {
            cap.beads += r.n;
            cap.nat += 2 * (int)r.nat_i1.size();
            cap.ss += 2 * (int)r.ss_i1.size();
            cap.afm += (int)afm_beads(r).size();
            const bool tile = params.nl_build == XMD_NL_BUILD_TILE ||
                              (params.nl_build == XMD_NL_BUILD_AUTO && r.n <= TILE_MAX);
            if (tile) cap.chunks += (r.n + TL_CH - 1) / TL_CH;
            else cap.cells += std::max(64, 2 * r.n);
            if (params.on[XMD_TERM_QA]) {
                cap.fp += r.n * QA_FP_PER_BEAD + 256;
                cap.qab += (r.n + QA_BCHUNK - 1) / QA_BCHUNK;
                cap.ct += r.n * QA_CT_PER_BEAD + 256;
            }
        }
    }
    allocate();
    finalized = true;
    place_pending();
}

// every device array at capacity; slots start empty (rep_of = -1)
void Engine::allocate() {
    const xmd_params &p = params;
    const int N = cap.beads, R = cap.reps;
    if (N > NL_MASK) throw std::invalid_argument("the context holds more beads than a Verlet entry can index");
    nl_cap = p.nl_capacity > 0 ? p.nl_capacity : 64;
    auto_grow = p.nl_grow != 0;
    d.N = N;
    d.R = R;
    d.nl_cap = nl_cap;
    const size_t cells = (size_t)std::max(1, cap.cells);
    const size_t NN = (size_t)std::max(1, cap.nat);
    d.pos[0] = (double4_32a *)dalloc(sizeof(double4_32a) * N);
    d.pos[1] = (double4_32a *)dalloc(sizeof(double4_32a) * N);
    d.yh = (double *)dalloc(sizeof(double) * 15 * (size_t)N);
    d.orig = (double4_32a *)dalloc(sizeof(double4_32a) * N);
    d.F = (double *)dalloc(sizeof(double) * 3 * (size_t)N);
    d.Vrep = (double *)dalloc(sizeof(double) * XMD_NUM_TERMS * R);
    d.rep_of = (int32_t *)dalloc(sizeof(int32_t) * N);
    CK(cudaMemsetAsync(d.rep_of, 0xff, sizeof(int32_t) * N, stream));
    d.bflags = (uint32_t *)dalloc(sizeof(uint32_t) * N);
    d.chain = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.seq = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.atype = (uint8_t *)dalloc(N);
    d.teth_r0 = (double *)dalloc(sizeof(double) * N);
    d.ang_t0 = (double *)dalloc(sizeof(double) * N);
    d.dih_p0 = (double *)dalloc(sizeof(double) * N);
    d.bond_f = (float4 *)dalloc(sizeof(float4) * N);
    d.nat_start = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.nat_end = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.nat_j = (int32_t *)dalloc(sizeof(int32_t) * NN);
    d.nat_d = (double *)dalloc(sizeof(double) * NN);
    d.nat_df = (float *)dalloc(sizeof(float) * NN);
    d.nat_T = (double *)dalloc(sizeof(double) * NN);
    d.nat_S = (double *)dalloc(sizeof(double) * NN);
    d.nat_on = (uint8_t *)dalloc(NN);
    {
        const size_t SS = (size_t)std::max(1, cap.ss);
        d.ss_start = (int32_t *)dalloc(sizeof(int32_t) * N);
        d.ss_end = (int32_t *)dalloc(sizeof(int32_t) * N);
        CK(cudaMemsetAsync(d.ss_start, 0, sizeof(int32_t) * N, stream));
        CK(cudaMemsetAsync(d.ss_end, 0, sizeof(int32_t) * N, stream));
        d.ss_j = (int32_t *)dalloc(sizeof(int32_t) * SS);
        d.ss_on = (uint8_t *)dalloc(SS);
        CK(cudaMemsetAsync(d.ss_on, 0, SS, stream));
        d.chir = (double2 *)dalloc(sizeof(double2) * N);
        d.chir_f32 = (float2 *)dalloc(sizeof(float2) * N);
        d.afm = (AfmTip *)dalloc(sizeof(AfmTip) * (size_t)std::max(1, cap.afm));
        // wall planes, and the state of every (bead, LJ attractive wall) pair
        double wt[2 * XMD_MAX_WALLS * 6] = {0};
        for (int kind = 0; kind < 2; ++kind)
            for (size_t q = 0; q < walls[kind].size(); ++q) wt[kind * XMD_MAX_WALLS * 6 + q] = walls[kind][q];
        d.wall = (double *)dalloc(sizeof(wt));
        CK(cudaMemcpyAsync(d.wall, wt, sizeof(wt), cudaMemcpyHostToDevice, stream));
        const size_t nlj = walls[1].size() / 6;
        d.fext = (double *)dalloc(sizeof(double) * 3 * N);
        d.ljw = (LjWallState *)dalloc(sizeof(LjWallState) * std::max<size_t>(1, nlj * N));
        CK(cudaMemsetAsync(d.ljw, 0, sizeof(LjWallState) * std::max<size_t>(1, nlj * N), stream));
        CK(cudaStreamSynchronize(stream));
    }
    {
        // heuristic coefficient tables: constants of the context
        double *ha = (double *)dalloc(sizeof(double) * 9 * 7);
        double *hd = (double *)dalloc(sizeof(double) * 9 * 6);
        float *hdf = (float *)dalloc(sizeof(float) * 9 * 6);
        float tf[9 * 6];
        for (int k = 0; k < 9 * 6; ++k) tf[k] = (float)(&params.heur_dih_coeffs[0][0])[k];
        CK(cudaMemcpyAsync(ha, &params.heur_ang_coeffs[0][0], sizeof(double) * 9 * 7, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(hd, &params.heur_dih_coeffs[0][0], sizeof(double) * 9 * 6, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(hdf, tf, sizeof(float) * 9 * 6, cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        d.heur_ang = ha; d.heur_dih = hd; d.heur_dih_f = hdf;
    }
    d.nl_row = (int32_t *)dalloc(sizeof(int32_t) * (size_t)nl_cap * N);
    d.nl_cnt = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.cell_cnt = (int32_t *)dalloc(sizeof(int32_t) * cells);
    d.cell_start = (int32_t *)dalloc(sizeof(int32_t) * cells);
    d.cell_fill = (int32_t *)dalloc(sizeof(int32_t) * cells);
    d.cell_items = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.bead_cell = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.cell_pos = (float4 *)dalloc(sizeof(float4) * N);
    d.bead_slot = (int32_t *)dalloc(sizeof(int32_t) * N);
    d.cell_cs = (int2 *)dalloc(sizeof(int2) * N);
    d.ncells = (int)cells;
    d.cell_rep = (int32_t *)dalloc(sizeof(int32_t) * cells);
    CK(cudaMemsetAsync(d.cell_rep, 0xff, sizeof(int32_t) * cells, stream));
    d.rng = (uint64_t *)dalloc(sizeof(uint64_t) * N);
    d.jump = (uint64_t *)dalloc(sizeof(uint64_t) * JUMP_WORDS * R);
    d.rep = (RepDev *)dalloc(sizeof(RepDev) * R);
    d.any_rebuild = (int *)dalloc(sizeof(int) * 4);
    d.gate = d.any_rebuild + 1;
    d.status = (int *)dalloc(sizeof(int) * 4);
    d.ctr = (unsigned long long *)dalloc(sizeof(unsigned long long) * 4);
    d.nchunks = std::max(1, cap.chunks);
    d.chunks = (int2 *)dalloc(sizeof(int2) * d.nchunks);
    d.work = (int *)dalloc(sizeof(int) * d.nchunks);
    d.nwork = (int *)dalloc(sizeof(int));
    CK(cudaMemsetAsync(d.nwork, 0, sizeof(int), stream));
    CK(cudaMemsetAsync(d.chunks, 0xff, sizeof(int2) * d.nchunks, stream));
    d.blk_on = (uint8_t *)dalloc((N + BLK_ON - 1) / BLK_ON + 8);
    CK(cudaMemsetAsync(d.blk_on, 0, (N + BLK_ON - 1) / BLK_ON + 8, stream));
    owner_h.assign(N, -1);
    a_beads.init(N);
    a_nat.init(cap.nat);
    a_ss.init(cap.ss);
    if (cap.afm > AFM_MAX_TIPS) throw std::length_error("engine: more AFM-pulled beads than the tip table holds");
    a_afm.init(cap.afm);
    a_cells.init(cap.cells);
    a_chunks.init(cap.chunks);
    a_fp.init(cap.fp);
    a_ct.init(cap.ct);
    any_cell = cap.cells > 0;
    any_tile = cap.chunks > 0;
    d.any_cell = any_cell;
    tile_smem = 0;
    for (auto &r : reps)
        if (r.in_use && r.n <= TILE_MAX) tile_smem = std::max(tile_smem, tile_bytes(r.n));
    if (dynamic) tile_smem = tile_bytes(std::min(TILE_MAX, cap.beads));
    if (tile_smem > 48 * 1024)
        CK(cudaFuncSetAttribute(k_nl_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem));
    {
        // the tile build runs as many blocks as are resident at once (or the
        // tuned number per SM); they take the work list's chunks in turn
        int sms = 0, per_sm = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_nl_tile, TL_THREADS, tile_smem));
        tile_sms = std::max(1, sms);
        tile_max_per_sm = std::max(1, per_sm);
        const int k = tune.tile_per_sm > 0 ? std::min(tune.tile_per_sm, tile_max_per_sm) : tile_max_per_sm;
        tile_grid = std::max(1, std::min(d.nchunks, tile_sms * k));
    }

    // term parameters
    std::memset(&tp, 0, sizeof tp);
    for (int k = 0; k < XMD_NUM_TERMS; ++k) tp.on[k] = p.on[k];
    tp.dt = p.dt;
    tp.dt_inv = 1.0 / p.dt;
    tp.dt2_half = p.dt * p.dt / 2.0;
    tp.gamma_factor = p.gamma_factor;
    tp.tether_H1 = p.tether_H1; tp.tether_H2 = p.tether_H2;
    tp.nat_ang_k = p.nat_ang_k; tp.cnd_CDA = p.cnd_CDA; tp.cnd_CDB = p.cnd_CDB; tp.snd_CDH = p.snd_CDH;
    tp.go_depth = p.go_depth;
    tp.pauli_r_excl = p.pauli_r_excl; tp.pauli_depth = p.pauli_depth;
    if (p.on[XMD_TERM_CONST_ES]) {      // main.cpp:619-631
        tp.es_Vf = 1.0 / (4.0 * M_PI * p.const_es_permittivity);
        tp.es_sdi = 1.0 / p.const_es_screen_dist;
        tp.es_rel = 0;
    } else {                            // main.cpp:633-645
        tp.es_Vf = 1.0 / (4.0 * M_PI * p.rel_es_factor);
        tp.es_sdi = 1.0 / p.rel_es_screen_dist;
        tp.es_rel = 1;
    }
    if (p.on[XMD_TERM_CONST_ES] && p.on[XMD_TERM_REL_ES])
        throw std::invalid_argument("const ES and relative ES cannot both be enabled in this engine");
    tp.qa_cycle = p.qa_phase_duration;
    tp.qa_cycle_inv = 1.0 / p.qa_phase_duration;
    tp.qa_factor = p.qa_breaking_factor * (double)powf(2.0f, -1.0f / 6.0f);   // main.cpp:719-723
    tp.lj_bb_r_min = p.lj_bb_r_min; tp.lj_bb_depth = p.lj_bb_depth;
    tp.lj_bs_r_min = p.lj_bs_r_min; tp.lj_bs_depth = p.lj_bs_depth;
    tp.ss_sinking = p.ss_sinking;
    tp.chir_e_chi = p.chir_e_chi;
    tp.nat_ss_H1 = p.nat_ss_H1;
    tp.nat_ss_dist = p.nat_ss_dist;
    tp.vel_afm_H1 = p.vel_afm_H1;
    tp.vel_afm_H2 = p.vel_afm_H2;
    tp.ext_on = (cap.afm > 0 && (p.on[XMD_TERM_VEL_AFM] || p.on[XMD_TERM_FORCE_AFM])) ||
                (p.on[XMD_TERM_SOLID_WALL] && !walls[0].empty()) || (p.on[XMD_TERM_LJ_WALL] && !walls[1].empty());
    tp.n_solid = p.on[XMD_TERM_SOLID_WALL] ? (int)walls[0].size() / 6 : 0;
    tp.n_ljw = p.on[XMD_TERM_LJ_WALL] ? (int)walls[1].size() / 6 : 0;
    tp.solid_eps = p.solid_wall_depth;
    tp.solid_cutoff = p.solid_wall_cutoff;
    tp.ljw_min_dist = p.lj_wall_min_dist;
    tp.ljw_factor = p.lj_wall_breaking_factor * std::pow(2.0, -1.0 / 6.0);   // main.cpp:842
    tp.ljw_cycle = p.lj_wall_phase_duration;
    tp.ljw_cycle_inv = 1.0 / p.lj_wall_phase_duration;
    tp.ljw_depth = p.lj_wall_depth;
    tp.pid_lambda = p.pid_lambda;
    for (int k = 0; k < 4; ++k) {
        tp.pid_bbp[k] = p.pid_bbp[k];
        tp.pid_bbm[k] = p.pid_bbm[k];
    }
    tp.pid_ss[0] = p.pid_ss[0];
    tp.pid_ss[1] = p.pid_ss[1];
    if (p.on[XMD_TERM_PID]) {
        // bundle forces per bead, and the side-chain LJ table by pair type
        // (lj_variants.cpp:59-62: sink_lj(depth, r_min = bb r_min when
        // sinking else r_max, r_max))
        d.pid_f = (double *)dalloc(sizeof(double) * 9 * (size_t)N);
        std::vector<double> sd(XMD_NUM_SS), smin(XMD_NUM_SS), smax(XMD_NUM_SS);
        for (int k = 0; k < XMD_NUM_SS; ++k) {
            sd[k] = p.ss_depth[k];
            smax[k] = p.ss_r_max[k];
            smin[k] = p.ss_sinking ? p.lj_bb_r_min : p.ss_r_max[k];
        }
        double *t_sd = (double *)dalloc(sizeof(double) * XMD_NUM_SS);
        double *t_smin = (double *)dalloc(sizeof(double) * XMD_NUM_SS);
        double *t_smax = (double *)dalloc(sizeof(double) * XMD_NUM_SS);
        CK(cudaMemcpyAsync(t_sd, sd.data(), sizeof(double) * XMD_NUM_SS, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(t_smin, smin.data(), sizeof(double) * XMD_NUM_SS, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(t_smax, smax.data(), sizeof(double) * XMD_NUM_SS, cudaMemcpyHostToDevice, stream));
        d.pid_sd = t_sd;
        d.pid_smin = t_smin;
        d.pid_smax = t_smax;
        CK(cudaStreamSynchronize(stream));
    }
    tp.f = TermP::F32{(float)tp.tether_H1, (float)tp.tether_H2, (float)tp.nat_ang_k, (float)tp.cnd_CDA,
                      (float)tp.cnd_CDB, (float)tp.snd_CDH, (float)tp.go_depth, (float)tp.pauli_r_excl,
                      (float)tp.pauli_depth, (float)tp.es_Vf, (float)tp.es_sdi, (float)tp.chir_e_chi,
                      (float)tp.nat_ss_H1, (float)tp.nat_ss_dist};
    if (p.on[XMD_TERM_QA]) {
        // quasi-adiabatic state (tables of main.cpp:681-700, lj_variants.cpp:59-62)
        d.qa_on = 1;
        QaDev &q = d.qa;
        q.nh = (float *)dalloc(sizeof(float) * 6 * (size_t)N);
        q.sync = (int32_t *)dalloc(sizeof(int32_t) * N);
        q.ref_cnt = (int32_t *)dalloc(sizeof(int32_t) * N);
        q.ref = (int32_t *)dalloc(sizeof(int32_t) * QA_REF_CAP * (size_t)N);
        q.tmp_cnt = (int32_t *)dalloc(sizeof(int32_t) * N);
        q.tmp = (int32_t *)dalloc(sizeof(int32_t) * QA_TMP_CAP * (size_t)N);
        q.tmp_off = (int32_t *)dalloc(sizeof(int32_t) * N);
        q.nbchunk = std::max(1, cap.qab);
        q.bchunk = (int2 *)dalloc(sizeof(int2) * q.nbchunk);
        CK(cudaMemsetAsync(q.bchunk, 0, sizeof(int2) * q.nbchunk, stream));
        q.bcsum = (int32_t *)dalloc(sizeof(int32_t) * q.nbchunk);
        q.bcbase = (int32_t *)dalloc(sizeof(int32_t) * q.nbchunk);
        qa_bchunk_next = 0;
        const int fp_total = std::max(1, cap.fp), ct_total = std::max(1, cap.ct);
        q.fp_total = fp_total;
        q.ct_total = ct_total;
        q.fp_i1 = (int32_t *)dalloc(sizeof(int32_t) * fp_total);
        q.fp_i2 = (int32_t *)dalloc(sizeof(int32_t) * fp_total);
        q.fp_rep = (int32_t *)dalloc(sizeof(int32_t) * fp_total);
        q.fp_vac = (uint8_t *)dalloc(fp_total);
        q.cand_type = (int32_t *)dalloc(sizeof(int32_t) * fp_total);
        q.cand_d1 = (int32_t *)dalloc(sizeof(int32_t) * fp_total);
        q.cand_d2 = (int32_t *)dalloc(sizeof(int32_t) * fp_total);
        const int nsift = (fp_total + QA_SIFT - 1) / QA_SIFT;
        q.cand_list = (int32_t *)dalloc(sizeof(int32_t) * (size_t)nsift * QA_SIFT);
        q.cand_blk = (int32_t *)dalloc(sizeof(int32_t) * nsift);
        CK(cudaMemsetAsync(q.cand_blk, 0, sizeof(int32_t) * nsift, stream));
        q.ct_i1 = (int32_t *)dalloc(sizeof(int32_t) * ct_total);
        q.ct_i2 = (int32_t *)dalloc(sizeof(int32_t) * ct_total);
        q.ct_type = (int32_t *)dalloc(sizeof(int32_t) * ct_total);
        q.ct_d1 = (int32_t *)dalloc(sizeof(int32_t) * ct_total);
        q.ct_d2 = (int32_t *)dalloc(sizeof(int32_t) * ct_total);
        q.ct_status = (uint8_t *)dalloc(ct_total);
        q.ct_vac = (uint8_t *)dalloc(ct_total);
        q.ct_rm = (uint8_t *)dalloc(ct_total);
        CK(cudaMemsetAsync(q.ct_rm, 0, ct_total, stream));
        q.ct_rep = (int32_t *)dalloc(sizeof(int32_t) * ct_total);
        CK(cudaMemsetAsync(q.ct_rep, 0xff, sizeof(int32_t) * ct_total, stream));
        q.ct_ref = (double *)dalloc(sizeof(double) * ct_total);
        std::vector<double> req(4 + XMD_NUM_SS, 0.0), sd(XMD_NUM_SS), smin(XMD_NUM_SS), smax(XMD_NUM_SS);
        req[1] = p.lj_bb_r_min;
        req[2] = req[3] = p.lj_bs_r_min;
        for (int a1 = 0; a1 < XMD_NUM_AA; ++a1)
            for (int a2 = 0; a2 < XMD_NUM_AA; ++a2)
                req[4 + a1 + XMD_NUM_AA * a2] = p.ss_r_max[a1 * XMD_NUM_AA + a2];
        for (int k = 0; k < XMD_NUM_SS; ++k) {
            sd[k] = p.ss_depth[k];
            smax[k] = p.ss_r_max[k];
            smin[k] = p.ss_sinking ? p.lj_bb_r_min : p.ss_r_max[k];
        }
        double *t_req = (double *)dalloc(sizeof(double) * req.size());
        double *t_sd = (double *)dalloc(sizeof(double) * XMD_NUM_SS);
        double *t_smin = (double *)dalloc(sizeof(double) * XMD_NUM_SS);
        double *t_smax = (double *)dalloc(sizeof(double) * XMD_NUM_SS);
        int32_t *t_pt = (int32_t *)dalloc(sizeof(int32_t) * XMD_NUM_AA);
        CK(cudaMemcpyAsync(t_req, req.data(), sizeof(double) * req.size(), cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(t_sd, sd.data(), sizeof(double) * XMD_NUM_SS, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(t_smin, smin.data(), sizeof(double) * XMD_NUM_SS, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(t_smax, smax.data(), sizeof(double) * XMD_NUM_SS, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(t_pt, p.polarization, sizeof(int32_t) * XMD_NUM_AA, cudaMemcpyHostToDevice, stream));
        q.req_min_dist = t_req;
        q.ss_depth = t_sd;
        q.ss_rmin = t_smin;
        q.ss_rmax = t_smax;
        q.ptype = t_pt;
        q.min_cos_hr = p.qa_min_cos_hr;
        q.min_cos_hh = p.qa_min_cos_hh;
        q.max_cos_nr = p.qa_max_cos_nr;
        double rmax = 0.0;
        for (double v : req) rmax = std::max(rmax, v);
        const double w = rmax * (1.0 + 1e-9);
        q.req_out2 = w * w;
        q.req_out2_f = (float)(q.req_out2 * (1.0 + 1e-4));
        q.min_cos_hr_f = (float)q.min_cos_hr;
        q.min_cos_hh_f = (float)q.min_cos_hh;
        q.max_cos_nr_f = (float)q.max_cos_nr;
    }
    CK(cudaStreamSynchronize(stream));
}

void Engine::ready() {
    finalize();
    place_pending();
}
void Engine::ready_alloc() {
    if (!finalized) finalize();
}

void Engine::place_pending() {
    for (int k = 0; k < (int)reps.size(); ++k)
        if (reps[k].in_use && !reps[k].placed && !reps[k].staged) {
            if (!reps[k].have_state) throw std::logic_error("set_state must be called for every replica");
            place(k);
        }
}

// occupancy granules [b0/BLK_ON, (b1-1)/BLK_ON] on when any bead slot in them
// is placed (a force block runs when any of its granules is on)
void Engine::update_blocks(int b0, int b1, bool wait) {
    if (b1 <= b0) return;
    const int k0 = b0 / BLK_ON, k1 = (b1 - 1) / BLK_ON;
    std::vector<uint8_t> on(k1 - k0 + 1, 0);
    for (int k = k0; k <= k1; ++k)
        for (int i = k * BLK_ON; i < std::min(cap.beads, (k + 1) * BLK_ON); ++i)
            if (owner_h[i] >= 0) { on[k - k0] = 1; break; }
    CK(cudaMemcpyAsync(d.blk_on + k0, on.data(), on.size(), cudaMemcpyHostToDevice, stream));
    if (wait) CK(cudaStreamSynchronize(stream));
}

// static data, lists and state of replica slot k onto the device.  With st
// (staged placement) every upload goes on the side stream, after the last
// removal's clears, and the activation data (bead and bucket owners, the
// replica record) is kept in st for activate_staged().
void Engine::place(int k, Staged *st) {
    const xmd_params &p = params;
    cudaStream_t us = st ? ustream : stream;
    if (st) CK(cudaStreamWaitEvent(ustream, ev_removed, 0));
    RepHost &r = reps[k];
    const int n = r.n;
    const bool tile = p.nl_build == XMD_NL_BUILD_TILE || (p.nl_build == XMD_NL_BUILD_AUTO && n <= TILE_MAX);
    if (tile && n > TILE_MAX)
        throw std::invalid_argument("engine: nl build 'tile' takes replicas of at most " +
                                    std::to_string(TILE_MAX) + " beads");
    const int nnat = 2 * (int)r.nat_i1.size();
    const int nss = 2 * (int)r.ss_i1.size();
    const int nchunk = tile ? (n + TL_CH - 1) / TL_CH : 0;
    const int ncell = tile ? 0 : std::max(64, 2 * n);
    const bool qa = p.on[XMD_TERM_QA] != 0;
    const int nfp = qa ? n * QA_FP_PER_BEAD + 256 : 0, nct = qa ? n * QA_CT_PER_BEAD + 256 : 0;
    // device ranges (all or nothing)
    int b = a_beads.alloc(n), no = a_nat.alloc(nnat), co = a_cells.alloc(ncell), ho = a_chunks.alloc(nchunk);
    const std::vector<int> afm_b = afm_beads(r);
    const int nafm = (int)afm_b.size();
    int fo = a_fp.alloc(nfp), to = a_ct.alloc(nct), so = a_ss.alloc(nss), ao = a_afm.alloc(nafm);
    if (b < 0 || no < 0 || co < 0 || ho < 0 || fo < 0 || to < 0 || so < 0 || ao < 0) {
        if (ao >= 0) a_afm.release(ao, nafm);
        if (so >= 0) a_ss.release(so, nss);
        if (b >= 0) a_beads.release(b, n);
        if (no >= 0) a_nat.release(no, nnat);
        if (co >= 0) a_cells.release(co, ncell);
        if (ho >= 0) a_chunks.release(ho, nchunk);
        if (fo >= 0) a_fp.release(fo, nfp);
        if (to >= 0) a_ct.release(to, nct);
        throw std::length_error("engine: the reserved capacity has no room for this replica");
    }
    r.begin = b;
    r.nat_off = no; r.nat_len = nnat;
    r.ss_off = so; r.ss_len = nss;
    r.cell_off = co; r.cell_len = ncell;
    r.chunk_off = ho; r.chunk_len = nchunk;
    r.fp_off = fo; r.fp_len = nfp;
    r.ct_off = to; r.ct_len = nct;
    r.afm_off = ao; r.afm_len = nafm;

    // per-bead static data; chain ids are local (pairs never cross replicas)
    std::vector<int32_t> rep_of(n, k), seq(r.seq), chain(r.chain), ns(n), ne(n);
    std::vector<uint32_t> bfl(n, 0);
    std::vector<double> tr(n, 0.0), ar(n, 0.0), dr(n, 0.0);
    for (int i = 0; i < n; ++i) {
        uint32_t f = 0;
        if (!std::isnan(r.teth_r0[i])) { f |= BF_TETH; tr[i] = r.teth_r0[i]; }
        if (!std::isnan(r.ang_t0[i])) { f |= BF_ANG; ar[i] = r.ang_t0[i]; }
        if (!std::isnan(r.dih_p0[i])) { f |= BF_DIH; dr[i] = r.dih_p0[i]; }
        if (!std::isnan(r.chir_f[i])) f |= BF_CHIR;
        if (r.hang_t[i] >= 0) f |= BF_HANG | ((uint32_t)r.hang_t[i] << BF_HANG_SHIFT);
        if (r.hdih_t[i] >= 0) f |= BF_HDIH | ((uint32_t)r.hdih_t[i] << BF_HDIH_SHIFT);
        {
            auto it = std::lower_bound(afm_b.begin(), afm_b.end(), i);
            if (it != afm_b.end() && *it == i)
                f |= BF_AFM | ((uint32_t)(ao + (int)(it - afm_b.begin())) << BF_AFM_SHIFT);
        }
        if (i > 0 && consecutive(r, i - 1, i)) f |= BF_PREV;
        if (i + 1 < r.n && consecutive(r, i, i + 1)) f |= BF_NEXT;
        bfl[i] = f;
    }
    // natives of each bead (both directions), ordered by partner: a CSR
    // segment of the replica
    std::vector<std::vector<std::pair<int, double>>> nat(n);
    for (size_t q = 0; q < r.nat_i1.size(); ++q) {
        nat[r.nat_i1[q]].push_back({b + r.nat_i2[q], r.nat_d[q]});
        nat[r.nat_i2[q]].push_back({b + r.nat_i1[q], r.nat_d[q]});
    }
    std::vector<int32_t> nj;
    std::vector<double> nd;
    for (int i = 0; i < n; ++i) {
        std::sort(nat[i].begin(), nat[i].end());
        ns[i] = no + (int)nj.size();
        for (auto &e : nat[i]) { nj.push_back(e.first); nd.push_back(e.second); }
        ne[i] = no + (int)nj.size();
    }
    // (pageable sources: each copy returns once the driver has taken the
    // data, so the host vectors may go out of scope)
    auto up = [&](void *dst, const void *src, size_t bytes_) {
        if (bytes_) CK(cudaMemcpyAsync(dst, src, bytes_, cudaMemcpyHostToDevice, us));
    };
    if (st) st->rep_of = rep_of;
    else up(d.rep_of + b, rep_of.data(), sizeof(int32_t) * n);
    up(d.chain + b, chain.data(), sizeof(int32_t) * n);
    up(d.seq + b, seq.data(), sizeof(int32_t) * n);
    up(d.atype + b, r.atype.data(), n);
    up(d.bflags + b, bfl.data(), sizeof(uint32_t) * n);
    up(d.teth_r0 + b, tr.data(), sizeof(double) * n);
    up(d.ang_t0 + b, ar.data(), sizeof(double) * n);
    up(d.dih_p0 + b, dr.data(), sizeof(double) * n);
    {
        std::vector<double2> ch(n);
        std::vector<float2> chf(n);
        for (int i = 0; i < n; ++i) {
            const bool on = !std::isnan(r.chir_f[i]);
            ch[i] = make_double2(on ? r.chir_f[i] : 0.0, on ? r.chir_n[i] : 0.0);
            chf[i] = make_float2((float)ch[i].x, (float)ch[i].y);
        }
        up(d.chir + b, ch.data(), sizeof(double2) * n);
        up(d.chir_f32 + b, chf.data(), sizeof(float2) * n);
        // disulfide partners per bead, both directions, ordered by partner
        std::vector<std::vector<int>> sp(n);
        for (size_t q = 0; q < r.ss_i1.size(); ++q) {
            sp[r.ss_i1[q]].push_back(b + r.ss_i2[q]);
            sp[r.ss_i2[q]].push_back(b + r.ss_i1[q]);
        }
        std::vector<int32_t> sst(n), sse(n), sj;
        for (int i = 0; i < n; ++i) {
            std::sort(sp[i].begin(), sp[i].end());
            sst[i] = so + (int)sj.size();
            for (int x : sp[i]) sj.push_back(x);
            sse[i] = so + (int)sj.size();
        }
        up(d.ss_start + b, sst.data(), sizeof(int32_t) * n);
        up(d.ss_end + b, sse.data(), sizeof(int32_t) * n);
        up(d.ss_j + so, sj.data(), sizeof(int32_t) * sj.size());
        if (nss) CK(cudaMemsetAsync(d.ss_on + so, 0, nss, us));
    }
    std::vector<float4> bf(n);
    for (int i = 0; i < n; ++i) bf[i] = make_float4((float)tr[i], (float)ar[i], (float)dr[i], 0.0f);
    up(d.bond_f + b, bf.data(), sizeof(float4) * n);
    up(d.nat_start + b, ns.data(), sizeof(int32_t) * n);
    up(d.nat_end + b, ne.data(), sizeof(int32_t) * n);
    up(d.nat_j + no, nj.data(), sizeof(int32_t) * nj.size());
    up(d.nat_d + no, nd.data(), sizeof(double) * nd.size());
    std::vector<float> ndf(nd.begin(), nd.end());
    up(d.nat_df + no, ndf.data(), sizeof(float) * ndf.size());
    CK(cudaMemsetAsync(d.nat_on + no, 0, nnat, us));
    CK(cudaMemsetAsync(d.nl_cnt + b, 0, sizeof(int32_t) * n, us));
    if (ncell) {
        std::vector<int32_t> cr(ncell, k);
        if (st) st->cell_rep = cr;
        else up(d.cell_rep + co, cr.data(), sizeof(int32_t) * ncell);
    }
    std::vector<int2> ch(nchunk);
    for (int c = 0; c < nchunk; ++c) ch[c] = make_int2(k, b + c * TL_CH);
    up(d.chunks + ho, ch.data(), sizeof(int2) * nchunk);

    RepDev rd;
    derive_rep(k, rd);
    {
        std::vector<double> nT(nd.size());
        for (size_t q = 0; q < nd.size(); ++q) nT[q] = 2.0 * nd[q] + rd.pad;   // 2 r_nat is exact
        up(d.nat_T + no, nT.data(), sizeof(double) * nT.size());
        std::vector<double> nS(nT.size());
        for (size_t q = 0; q < nT.size(); ++q) nS[q] = sq_below(nT[q]);
        up(d.nat_S + no, nS.data(), sizeof(double) * nS.size());
    }
    rd.cell_off = co;
    rd.cell_budget = ncell;
    rd.tile = tile;
    rd.fault = 0;
    rd.chunk_off = tile ? ho : 0;
    rd.nchunk = nchunk;
    rd.active = 1;
    rd.steps_left = r.steps_left;
    rd.afm = nafm > 0;
    if (nafm) {
        // the tips of each pulled bead; a velocity tip's origin defaults to
        // the bead's position when placed (main.cpp:884)
        std::vector<AfmTip> tips(nafm);
        for (auto &tp : tips) tp = AfmTip{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        auto slot = [&](int i) { return (int)(std::lower_bound(afm_b.begin(), afm_b.end(), i) - afm_b.begin()); };
        for (size_t q = 0; q < r.vafm_i.size(); ++q) {
            const int i = r.vafm_i[q];
            AfmTip &tp = tips[slot(i)];
            const double *o = &r.vafm_o[3 * q], *v = &r.vafm_v[3 * q];
            tp.ox = std::isnan(o[0]) ? r.r[3 * i] : o[0];
            tp.oy = std::isnan(o[1]) ? r.r[3 * i + 1] : o[1];
            tp.oz = std::isnan(o[2]) ? r.r[3 * i + 2] : o[2];
            tp.vx = v[0]; tp.vy = v[1]; tp.vz = v[2];
            tp.has_vel = 1;
        }
        for (size_t q = 0; q < r.fafm_i.size(); ++q) {
            AfmTip &tp = tips[slot(r.fafm_i[q])];
            tp.fx += r.fafm_F[3 * q]; tp.fy += r.fafm_F[3 * q + 1]; tp.fz += r.fafm_F[3 * q + 2];
        }
        up(d.afm + ao, tips.data(), sizeof(AfmTip) * nafm);
    }
    if (qa) {
        rd.fp_off = fo;
        rd.fp_cap = nfp;
        rd.ct_off = to;
        rd.ct_cap = nct;
        std::vector<int32_t> fprep(nfp, k), sy(n);
        up(d.qa.fp_rep + fo, fprep.data(), sizeof(int32_t) * nfp);
        std::vector<int32_t> ctrep(nct, k);
        up(d.qa.ct_rep + to, ctrep.data(), sizeof(int32_t) * nct);
        const int nbc = (n + QA_BCHUNK - 1) / QA_BCHUNK;
        if (qa_bchunk_next + nbc > d.qa.nbchunk) throw std::logic_error("engine: QA chunk table full");
        std::vector<int2> bch(nbc);
        for (int c = 0; c < nbc; ++c) bch[c] = make_int2(k, b + c * QA_BCHUNK);
        up(d.qa.bchunk + qa_bchunk_next, bch.data(), sizeof(int2) * nbc);
        rd.qa_bchunk_off = qa_bchunk_next;
        rd.qa_nbchunk = nbc;
        qa_bchunk_next += nbc;
        // valences start at the residue limits (intended main.cpp:662-672)
        for (int i = 0; i < n; ++i) {
            const int32_t *lim = p.limits[r.atype[i]];
            sy[i] = (lim[0] & 0xff) | ((lim[1] & 0xff) << 8) | ((lim[2] & 0xff) << 16) | ((lim[3] & 0xff) << 24);
        }
        up(d.qa.sync + b, sy.data(), sizeof(int32_t) * n);
        CK(cudaMemsetAsync(d.qa.ref_cnt + b, 0, sizeof(int32_t) * n, us));
    }
    if (!st) up(d.rep + k, &rd, sizeof(RepDev));
    GF2 j = gf2_jump(4ull * (uint64_t)n);
    std::vector<uint64_t> jt(JUMP_WORDS);
    // nibble tables: entry [q][v] = XOR of the columns 4q+b for the bits b of v
    for (int q = 0; q < 16; ++q)
        for (int v = 0; v < 16; ++v) {
            uint64_t e = 0;
            for (int bb = 0; bb < 4; ++bb)
                if ((v >> bb) & 1) e ^= j[4 * q + bb];
            jt[16 * q + v] = e;
        }
    up(d.jump + (size_t)JUMP_WORDS * k, jt.data(), sizeof(uint64_t) * JUMP_WORDS);
    if (st) {
        // the state (upload_state's data) on the side stream too; the record
        // starts as upload_state leaves it: t = 0, first list build pending
        upload_state_data(k, us);
        rd.t = 0.0;
        rd.first = 1;
        rd.maxdisp = 0;
        rd.fault = 0;
        st->k = k;
        st->rd = rd;
        r.staged = true;
        return;
    }
    CK(cudaStreamSynchronize(stream));
    for (int i = 0; i < n; ++i) owner_h[b + i] = k;
    update_blocks(b, b + n);
    r.placed = true;
    upload_state(k);
}

// positions, history (y1 = v dt, y2..y5 = 0) and generator states of a
// replica, uploaded on stream us
void Engine::upload_state_data(int k, cudaStream_t us) {
    RepHost &r = reps[k];
    int n = r.n, b = r.begin;
    std::vector<double4_32a> pos(n);
    for (int i = 0; i < n; ++i) {
        double q = params.charge[r.atype[i]];
        pos[i] = make_double4_32a(r.r[3 * i], r.r[3 * i + 1], r.r[3 * i + 2], q);
    }
    CK(cudaMemcpyAsync(d.pos[cur] + b, pos.data(), sizeof(double4_32a) * n, cudaMemcpyHostToDevice, us));
    std::vector<double> col(n);
    for (int k2 = 0; k2 < 15; ++k2) {
        for (int i = 0; i < n; ++i) col[i] = k2 < 3 ? r.v[3 * i + k2] * params.dt : 0.0;
        CK(cudaMemcpyAsync(d.yh + (size_t)k2 * d.N + b, col.data(), sizeof(double) * n,
                           cudaMemcpyHostToDevice, us));
    }
    std::vector<uint64_t> st(n);
    uint64_t s = r.seed;
    for (int i = 0; i < n; ++i) {
        st[i] = s;
        for (int q = 0; q < 4; ++q) s = xs_step(s);
    }
    CK(cudaMemcpyAsync(d.rng + b, st.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice, us));
}

void Engine::upload_state(int k) {
    upload_state_data(k, stream);
    RepDev rd;
    CK(cudaMemcpyAsync(&rd, d.rep + k, sizeof(RepDev), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    rd.t = 0.0;
    rd.first = 1;
    rd.maxdisp = 0;
    if (rd.fault) {   // a new state thaws a frozen replica
        rd.fault = 0;
        rd.steps_left = reps[k].steps_left;
    }
    CK(cudaMemcpyAsync(d.rep + k, &rd, sizeof(RepDev), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
}

void Engine::set_state(int rep, const double *r, const double *v) {
    check_rep(reps, rep);
    if (!r) throw std::invalid_argument("null positions");
    RepHost &h = reps[rep];
    h.r.assign(r, r + 3 * (size_t)h.n);
    if (v) h.v.assign(v, v + 3 * (size_t)h.n);
    else h.v.assign(3 * (size_t)h.n, 0.0);
    for (double x : h.r) if (!std::isfinite(x)) throw std::invalid_argument("non-finite position");
    h.have_state = true;
    if (h.placed) upload_state(rep);
}

void Engine::set_history(int rep, const double *y, double t, uint64_t rngs) {
    check_rep(reps, rep);
    ready();
    RepHost &h = reps[rep];
    int n = h.n, b = h.begin;
    size_t n3 = 3 * (size_t)n;
    std::vector<double4_32a> pos(n);
    for (int i = 0; i < n; ++i)
        pos[i] = make_double4_32a(y[3 * i], y[3 * i + 1], y[3 * i + 2], params.charge[h.atype[i]]);
    CK(cudaMemcpyAsync(d.pos[cur] + b, pos.data(), sizeof(double4_32a) * n, cudaMemcpyHostToDevice, stream));
    std::vector<double> col(n);
    for (int ord = 1; ord < 6; ++ord)
        for (int a = 0; a < 3; ++a) {
            for (int i = 0; i < n; ++i) col[i] = y[ord * n3 + 3 * i + a];
            CK(cudaMemcpyAsync(d.yh + (size_t)((ord - 1) * 3 + a) * d.N + b, col.data(), sizeof(double) * n,
                               cudaMemcpyHostToDevice, stream));
        }
    std::vector<uint64_t> st(n);
    uint64_t s = rngs;
    for (int i = 0; i < n; ++i) {
        st[i] = s;
        for (int q = 0; q < 4; ++q) s = xs_step(s);
    }
    CK(cudaMemcpyAsync(d.rng + b, st.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice, stream));
    RepDev rd;
    CK(cudaMemcpyAsync(&rd, d.rep + rep, sizeof(RepDev), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    rd.t = t;
    rd.first = 1;
    rd.maxdisp = 0;
    if (rd.fault) {   // a new state thaws a frozen replica
        rd.fault = 0;
        rd.steps_left = reps[rep].steps_left;
    }
    CK(cudaMemcpyAsync(d.rep + rep, &rd, sizeof(RepDev), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
}

void Engine::get_state(int rep, double *r, double *v, double *t) {
    check_rep(reps, rep);
    ready();
    const RepHost &h = reps[rep];
    int n = h.n, b = h.begin;
    std::vector<double4_32a> pos(n);
    CK(cudaMemcpyAsync(pos.data(), d.pos[cur] + b, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, stream));
    std::vector<double> y1(3 * (size_t)n);
    for (int a = 0; a < 3; ++a)
        CK(cudaMemcpyAsync(y1.data() + (size_t)a * n, d.yh + (size_t)a * d.N + b, sizeof(double) * n,
                           cudaMemcpyDeviceToHost, stream));
    RepDev rd;
    CK(cudaMemcpyAsync(&rd, d.rep + rep, sizeof(RepDev), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    const double dt_inv = 1.0 / params.dt;
    for (int i = 0; i < n; ++i) {
        if (r) { r[3 * i] = pos[i].x; r[3 * i + 1] = pos[i].y; r[3 * i + 2] = pos[i].z; }
        if (v) for (int a = 0; a < 3; ++a) v[3 * i + a] = y1[(size_t)a * n + i] * dt_inv;
    }
    if (t) *t = rd.t;
}

// ---- snapshots: the replica's whole mutable device state -----------------------
// The reference's store (include/xmd/store/store.h; main.cpp's make_saved
// items) keeps positions, the Gear history, time, the pair lists and the QA
// sets, but not the generator (a make_temp), so a resumed run draws new
// noise.  A snapshot here holds everything a step reads and writes:
// positions, Gear history, time, per-bead generators, skin origins, the
// Verlet rows, native and disulfide activity, and the quasi-adiabatic state
// (sync, contacts with their slots, free pairs).  Restoring it continues
// the run bit for bit.  It is taken and restored in place: the replica must
// sit at the same slots of a context built the same way (same parameters,
// the same systems added in the same order); the header checks this.

namespace {
struct SnapHeader {
    char magic[8];
    uint32_t version, precision;
    int32_t rep, n, begin, nl_cap;
    int32_t nat_off, nat_len, ss_off, ss_len;
    int32_t qa_on, fp_off, fp_len, ct_off, ct_len;
    int32_t pad_;
    uint64_t topo;
};
constexpr uint32_t SNAP_VERSION = 1;
constexpr char SNAP_MAGIC[8] = {'X', 'M', 'D', 'S', 'N', 'A', 'P', '1'};
struct SnapRep {   // the mutable scalars of RepDev
    double t;
    int32_t first, rebuild, fault, fp_n, ct_n, pad_;
    long long steps_left;
    unsigned long long maxdisp, rebuilds;
};

uint64_t fnv(uint64_t h, const void *p, size_t bytes) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t k = 0; k < bytes; ++k) h = (h ^ c[k]) * 1099511628211ull;
    return h;
}
}  // namespace

uint64_t Engine::topo_hash(int rep) const {
    const RepHost &r = reps[rep];
    uint64_t h = 1469598103934665603ull;
    h = fnv(h, r.chain.data(), r.chain.size() * sizeof(int32_t));
    h = fnv(h, r.seq.data(), r.seq.size() * sizeof(int32_t));
    h = fnv(h, r.atype.data(), r.atype.size());
    h = fnv(h, r.nat_i1.data(), r.nat_i1.size() * sizeof(int32_t));
    h = fnv(h, r.nat_i2.data(), r.nat_i2.size() * sizeof(int32_t));
    h = fnv(h, r.ss_i1.data(), r.ss_i1.size() * sizeof(int32_t));
    h = fnv(h, r.ss_i2.data(), r.ss_i2.size() * sizeof(int32_t));
    return h;
}

size_t Engine::snapshot_io(int rep, unsigned char *buf, size_t bytes, bool save, int cap_rows) {
    check_rep(reps, rep);
    ready();
    RepHost &h = reps[rep];
    const int n = h.n, b = h.begin;
    const size_t N = (size_t)d.N;
    SnapHeader hd{};
    std::memcpy(hd.magic, SNAP_MAGIC, 8);
    hd.version = SNAP_VERSION;
    hd.precision = (uint32_t)params.precision;
    hd.rep = rep; hd.n = n; hd.begin = b; hd.nl_cap = 0;   // the row capacity may differ (below)
    hd.nat_off = h.nat_off; hd.nat_len = h.nat_len; hd.ss_off = h.ss_off; hd.ss_len = h.ss_len;
    hd.qa_on = d.qa_on; hd.fp_off = h.fp_off; hd.fp_len = h.fp_len; hd.ct_off = h.ct_off; hd.ct_len = h.ct_len;
    // the topology, and the wall planes the saved LJ attractive wall states
    // refer to
    hd.topo = fnv(fnv(topo_hash(rep), walls[0].data(), walls[0].size() * sizeof(double)), walls[1].data(),
                  walls[1].size() * sizeof(double));
    hd.pad_ = (int32_t)(walls[1].size() / 6);   // LJ attractive walls (their pair states are saved)
    size_t off = 0;
    auto host = [&](void *p, size_t nb) {
        if (buf && off + nb <= bytes) {
            if (save) std::memcpy(buf + off, p, nb);
            else std::memcpy(p, buf + off, nb);
        }
        off += nb;
    };
    auto dev = [&](void *p, size_t nb) {
        if (buf && nb && off + nb <= bytes)
            CK(cudaMemcpyAsync(save ? (void *)(buf + off) : p, save ? p : (const void *)(buf + off), nb,
                               save ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice, stream));
        off += nb;
    };
    // rows [k][N] of a per-bead array: the replica's n entries of each row
    auto rows = [&](void *base, size_t elem, int nrows) {
        for (int k = 0; k < nrows; ++k) dev((char *)base + ((size_t)k * N + b) * elem, elem * n);
    };
    if (!save) {
        if (!buf || bytes < sizeof(SnapHeader)) throw std::invalid_argument("snapshot too short");
        SnapHeader got;
        std::memcpy(&got, buf, sizeof got);
        if (std::memcmp(got.magic, SNAP_MAGIC, 8) != 0 || got.version != SNAP_VERSION)
            throw std::invalid_argument("not a snapshot of this format");
        if (std::memcmp(&got, &hd, sizeof hd) != 0)
            throw std::invalid_argument("snapshot of another replica layout (precision, replica sizes or order, "
                                        "topology or wall planes differ)");
        // the whole snapshot must be there before anything of the replica
        // is overwritten: a short buffer leaves the replica as it was
        int32_t scap;
        if (bytes < sizeof(SnapHeader) + sizeof scap) throw std::invalid_argument("snapshot truncated");
        std::memcpy(&scap, buf + sizeof(SnapHeader), sizeof scap);
        if (scap <= 0 || scap > (1 << 20)) throw std::invalid_argument("snapshot: bad row capacity");
        if (bytes < snapshot_io(rep, nullptr, 0, true, scap)) throw std::invalid_argument("snapshot truncated");
    }
    host(&hd, sizeof hd);
    // Verlet row capacity of the snapshot; a restore grows this context's rows
    // to it (capacity does not change the trajectory)
    int32_t cap = cap_rows >= 0 ? cap_rows : nl_cap;
    host(&cap, sizeof cap);
    if (buf && !save) {
        if (cap <= 0 || cap > (1 << 20)) throw std::invalid_argument("snapshot: bad row capacity");
        if (cap > nl_cap) resize_rows(cap);
    }
    CK(cudaStreamSynchronize(stream));
    RepDev rd;
    CK(cudaMemcpy(&rd, d.rep + rep, sizeof(RepDev), cudaMemcpyDeviceToHost));
    SnapRep sr{rd.t, rd.first, rd.rebuild, rd.fault, rd.fp_n, rd.ct_n, 0, rd.steps_left, rd.maxdisp, rd.rebuilds};
    host(&sr, sizeof sr);
    dev(d.pos[cur] + b, sizeof(double4_32a) * n);
    rows(d.yh, sizeof(double), 15);
    dev(d.orig + b, sizeof(double4_32a) * n);
    dev(d.rng + b, sizeof(uint64_t) * n);
    dev(d.nl_cnt + b, sizeof(int32_t) * n);
    rows(d.nl_row, sizeof(int32_t), cap);
    dev(d.nat_on + h.nat_off, h.nat_len);
    dev(d.ss_on + h.ss_off, h.ss_len);
    for (int w = 0; w < hd.pad_; ++w) dev(d.ljw + (size_t)w * N + b, sizeof(LjWallState) * n);
    if (d.qa_on) {
        rows(d.qa.sync, sizeof(int32_t), 1);
        rows(d.qa.ref_cnt, sizeof(int32_t), 1);
        rows(d.qa.ref, sizeof(int32_t), QA_REF_CAP);
        const int fo = h.fp_off, fl = h.fp_len, co = h.ct_off, cl = h.ct_len;
        dev(d.qa.fp_i1 + fo, sizeof(int32_t) * fl);
        dev(d.qa.fp_i2 + fo, sizeof(int32_t) * fl);
        dev(d.qa.fp_rep + fo, sizeof(int32_t) * fl);
        dev(d.qa.fp_vac + fo, fl);
        dev(d.qa.ct_i1 + co, sizeof(int32_t) * cl);
        dev(d.qa.ct_i2 + co, sizeof(int32_t) * cl);
        dev(d.qa.ct_type + co, sizeof(int32_t) * cl);
        dev(d.qa.ct_d1 + co, sizeof(int32_t) * cl);
        dev(d.qa.ct_d2 + co, sizeof(int32_t) * cl);
        dev(d.qa.ct_status + co, cl);
        dev(d.qa.ct_vac + co, cl);
        dev(d.qa.ct_rm + co, cl);
        dev(d.qa.ct_rep + co, sizeof(int32_t) * cl);
        dev(d.qa.ct_ref + co, sizeof(double) * cl);
    }
    CK(cudaStreamSynchronize(stream));
    if (buf && !save) {
        if (off > bytes) throw std::invalid_argument("snapshot truncated");
        rd.t = sr.t; rd.first = sr.first; rd.rebuild = sr.rebuild; rd.fault = sr.fault;
        rd.fp_n = sr.fp_n; rd.ct_n = sr.ct_n; rd.steps_left = sr.steps_left;
        rd.maxdisp = sr.maxdisp; rd.rebuilds = sr.rebuilds;
        CK(cudaMemcpy(d.rep + rep, &rd, sizeof(RepDev), cudaMemcpyHostToDevice));
        h.steps_left = sr.steps_left;
    }
    return off;
}
size_t Engine::snapshot_size(int rep) { return snapshot_io(rep, nullptr, 0, true); }
void Engine::snapshot(int rep, void *buf, size_t bytes) {
    if (bytes < snapshot_size(rep)) throw std::invalid_argument("snapshot buffer too small");
    snapshot_io(rep, (unsigned char *)buf, bytes, true);
}
void Engine::restore(int rep, const void *buf, size_t bytes) {
    snapshot_io(rep, (unsigned char *)const_cast<void *>(buf), bytes, false);
}

void Engine::get_history(int rep, double *y, double *t, uint64_t *rngs) {
    check_rep(reps, rep);
    ready();
    const RepHost &h = reps[rep];
    int n = h.n, b = h.begin;
    size_t n3 = 3 * (size_t)n;
    std::vector<double4_32a> pos(n);
    CK(cudaMemcpyAsync(pos.data(), d.pos[cur] + b, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, stream));
    std::vector<double> col(15 * (size_t)n);
    for (int k = 0; k < 15; ++k)
        CK(cudaMemcpyAsync(col.data() + (size_t)k * n, d.yh + (size_t)k * d.N + b, sizeof(double) * n,
                           cudaMemcpyDeviceToHost, stream));
    uint64_t s0 = 0;
    CK(cudaMemcpyAsync(&s0, d.rng + b, sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
    RepDev rd;
    CK(cudaMemcpyAsync(&rd, d.rep + rep, sizeof(RepDev), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (y) {
        for (int i = 0; i < n; ++i) { y[3 * i] = pos[i].x; y[3 * i + 1] = pos[i].y; y[3 * i + 2] = pos[i].z; }
        for (int ord = 1; ord < 6; ++ord)
            for (int a = 0; a < 3; ++a)
                for (int i = 0; i < n; ++i)
                    y[ord * n3 + 3 * i + a] = col[(size_t)((ord - 1) * 3 + a) * n + i];
    }
    if (t) *t = rd.t;
    if (rngs) *rngs = s0;
}

void Engine::use_device() const { CK(cudaSetDevice(device)); }

void Engine::record(std::vector<cudaEvent_t> &pool, size_t &n) {
    if (n >= pool.size()) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        pool.push_back(e);
    }
    CK(cudaEventRecord(pool[n++], stream));
}

void Engine::launch_rebuild() {
    if (timing) record(ev_rebuild, n_ev_rebuild);
    if (any_cell) {
        const int gb = (d.N + 255) / 256;
        k_cells<<<d.R, CB, 0, stream>>>(d, cur);
        k_cell_count<<<gb, 256, 0, stream>>>(d, cur);
        k_cell_scan<<<d.R, CB, 0, stream>>>(d);
        k_cell_scatter<<<gb, 256, 0, stream>>>(d);
        k_cell_finish<<<(d.ncells + CF_WARPS - 1) / CF_WARPS, CF_WARPS * 32, 0, stream>>>(d, cur);
        k_nl_cells<<<(d.N + NC_WARPS - 1) / NC_WARPS, NC_WARPS * 32, 0, stream>>>(d, tp, cur);
    }
    if (any_tile) k_nl_tile<<<tile_grid, TL_THREADS, tile_smem, stream>>>(d, tp, cur, 1);
    if (d.qa_on) {
        k_qa_fp_scan<<<d.qa.nbchunk, QA_BCHUNK, 0, stream>>>(d);
        k_qa_fp_base<<<d.R, 1024, 0, stream>>>(d);
        k_qa_fp_fill<<<d.qa.nbchunk, QA_BCHUNK, 0, stream>>>(d);
        k_qa_compact<<<d.R, 1024, 0, stream>>>(d);
    }
    if (timing) record(ev_rebuild, n_ev_rebuild);
}

// Grow the Verlet rows when the longest row needed (recorded by the builds)
// reaches `frac` of the capacity.  Returns true when the rows were
// reallocated (lists must then be rebuilt; captured graphs are dropped).
bool Engine::grow_rows(double frac) {
    unsigned long long need = 0;
    CK(cudaMemcpyAsync(&need, d.ctr + 1, sizeof(need), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if ((double)need < frac * nl_cap) return false;
    resize_rows((int)(2 * need + 16));
    return true;
}

// Reallocate the Verlet rows with ncap slots per bead, keeping the rows held.
void Engine::resize_rows(int ncap) {
    int32_t *rows = nullptr;
    CK(cudaMalloc(&rows, sizeof(int32_t) * (size_t)ncap * d.N));
    // rows are slot-major ([k][N]), so the current lists keep their place:
    // growing for headroom leaves them valid without a rebuild
    CK(cudaMemcpyAsync(rows, d.nl_row, sizeof(int32_t) * (size_t)std::min(nl_cap, ncap) * d.N,
                       cudaMemcpyDeviceToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    for (auto &a : allocs)
        if (a == (void *)d.nl_row) {
            CK(cudaFree(a));
            a = rows;
        }
    alloc_bytes += sizeof(int32_t) * (size_t)d.N * ncap;
    alloc_bytes -= std::max<size_t>(16, sizeof(int32_t) * (size_t)nl_cap * d.N);
    d.nl_row = rows;
    d.nl_cap = nl_cap = ncap;
    drop_graphs();
}

void Engine::set_tuning(const Tune &t) {
    if (t.fb != 32 && t.fb != 64 && t.fb != 128)
        throw std::invalid_argument("tuning: step-kernel block size must be 32, 64 or 128 beads");
    if (t.lpb != 1 && t.lpb != 2 && t.lpb != 4)
        throw std::invalid_argument("tuning: threads per bead must be 1, 2 or 4");
    if (t.graph_steps != 8 && t.graph_steps != 16 && t.graph_steps != 32 && t.graph_steps != 64)
        throw std::invalid_argument("tuning: steps per graph must be 8, 16, 32 or 64");
    if (t.tile_per_sm < 0) throw std::invalid_argument("tuning: tile blocks per SM must be >= 0");
    tune = t;
    if (finalized) {
        const int k = tune.tile_per_sm > 0 ? std::min(tune.tile_per_sm, tile_max_per_sm) : tile_max_per_sm;
        tile_grid = std::max(1, std::min(d.nchunks, tile_sms * k));
        drop_graphs();
    }
}

// The autotuner.  Every candidate launch shape (step-kernel block size,
// resident tile-build blocks per SM, steps per graph) runs on a fresh clone of
// this context: the same replicas from the same starting state, so each is
// timed on the same trajectory (the trajectory does not depend on the shape).
// A candidate's time is CUDA-event time per step over `steps` graph steps
// after one warm-up graph (which builds the first lists and captures the
// graph).  This context's device state is not touched.
Engine::Tune Engine::autotune(int steps, double *ms_out) {
    if (dynamic) throw std::logic_error("autotune needs a static context (replicas added before the first step)");
    int live = 0;
    for (auto &r : reps) live += r.in_use ? 1 : 0;
    if (!live) throw std::logic_error("autotune: the context has no replica");
    for (auto &r : reps)
        if (r.in_use && !r.have_state) throw std::logic_error("autotune: set_state must be called for every replica");
    steps = std::max(32, (steps + 31) / 32 * 32);
    // two stages: the step kernel's shape (beads per block x threads per
    // bead) at 16 steps per graph, then graph length and tile residency with
    // the best step-kernel shape
    Tune best = tune;
    double best_ms = 1e300;
    auto trial = [&](const Tune &cand) {
        Engine c(params);
        for (auto &r : reps)
            if (r.in_use) {
                RepHost h = r;
                h.placed = false;
                c.reps.push_back(std::move(h));
            }
        c.tune = cand;
        c.use_device();
        c.ready();
        c.set_tuning(cand);
        c.step(cand.graph_steps);   // first lists, graph capture
        c.sync();
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, c.stream));
        c.step(steps);
        CK(cudaEventRecord(e1, c.stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double per = (double)ms / steps;
        if (per < best_ms) {
            best_ms = per;
            best = cand;
        }
    };
    for (int fb : {32, 64, 128})
        for (int lpb : {1, 2, 4}) trial(Tune{fb, 0, 16, lpb});
    const Tune kshape = best;
    for (int gs : {8, 16, 32, 64})
        for (int tps : {0, 2})
            if (gs != 16 || tps != 0) trial(Tune{kshape.fb, tps, gs, kshape.lpb});
    use_device();
    set_tuning(best);
    if (ms_out) *ms_out = best_ms;
    return best;
}

void Engine::drop_graphs() {
    for (auto &kv : graphs) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    }
    graphs.clear();
}

void Engine::ensure_nl() {
    for (int attempt = 0; attempt < 3; ++attempt) {
        k_nl_check<<<1, 1024, 0, stream>>>(d, 0, 0.0, (cudaGraphConditionalHandle)0, 0);
        ++launches;
        CK(cudaMemcpyAsync(h_any, d.any_rebuild, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (*h_any) launch_rebuild();
        int st = 0;
        CK(cudaMemcpyAsync(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (!(st & ST_CAPACITY) || !auto_grow) {
            if (auto_grow) grow_rows(0.6);   // keep headroom for the run ahead
            return;
        }
        // rows overflowed at this rebuild: grow, clear the flag, rebuild all
        if (!grow_rows(0.0)) return;
        CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
        k_mark_all<<<(d.R + 255) / 256, 256, 0, stream>>>(d);
    }
}

void Engine::launch_force_step() {
    if (timing) record(ev_force, n_ev_force);
    launch_force(1, cur);
    if (timing) record(ev_force, n_ev_force);
    launches += 1 + (tp.ext_on ? 1 : 0) + (tp.on[XMD_TERM_PID] ? 1 : 0);
    if (d.qa_on) {
        // sift + acceptance + transitions at this step's positions (qa.cpp:20-31)
        k_qa_sift<<<sift_grid(), QA_SIFT, 0, stream>>>(d, tp, cur);
        k_qa_step<<<d.R, 1024, 0, stream>>>(d, tp, cur);
        k_qa_trans<<<trans_grid(), QA_TG, 0, stream>>>(d, tp, cur);
        k_qa_refree<<<d.R, 1024, 0, stream>>>(d, 0.0, 0);
        launches += 4;
    }
}

// One graph runs `len` steps (tune.graph_steps, or a power of two for the
// rest of a call).  IF form: per step a force+integrate node, a skin check
// that sets a conditional handle on the device, and an IF node whose body
// rebuilds the lists of the flagged replicas (cells, then rows).  Plain form
// (the rebuild is the row build alone: no cell-path replica, no
// quasi-adiabatic term): the step kernel takes the decision and a row-build
// node follows, which returns at once when the work list is empty (an IF
// node costs more per step than that empty launch).  Gated form (`gated`):
// no rebuild node; the check halts the graph's remaining steps and the host
// rebuilds.  A graph of odd length leaves the position double buffer
// swapped.
cudaGraphExec_t Engine::graph_for(int start_cur, bool gated, int len) {
    const int key = ((len * 2 + (params.precision == XMD_PREC_MIXED ? 1 : 0)) * 2 + (gated ? 1 : 0)) * 2 + start_cur;
    GraphSet &gs = graphs[key];
    if (gs.exec) return gs.exec;
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphNode_t prev = nullptr;
    const int nb = (d.N + force_block_beads(tune.fb, tune.lpb) - 1) / force_block_beads(tune.fb, tune.lpb);
    void *fk = force_kernel(params.precision == XMD_PREC_MIXED, 1, tune.fb, tune.lpb);
    double dt = params.dt;
    // without the quasi-adiabatic term the step kernel takes the skin
    // decision itself (its last block) where no IF node needs it; with it,
    // the re-freeing kernel does in gated graphs
    const bool plain = plain_rebuild();
    const int fuse = d.qa_on ? (gated ? FUSE_GATE : FUSE_NONE) : plain ? FUSE_CHECK
                     : gated ? FUSE_CHECK_GATE : FUSE_NONE;
    int zero = 0;
    for (int s = 0; s < len; ++s) {
        int c = start_cur ^ (s & 1), cn = c ^ 1;
        int adv = 1, setc = gated ? CHECK_GATE : CHECK_COND;
        cudaGraphConditionalHandle h = 0;
        if (!plain && !gated) CK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
        cudaKernelNodeParams kf{};
        int ff = fuse;
        void *fargs[] = {&d, &tp, &c, &ff};
        kf.func = fk;
        kf.gridDim = dim3(nb);
        kf.blockDim = dim3(tune.fb * tune.lpb);
        kf.kernelParams = fargs;
        cudaGraphNode_t nf, nc, ncond;
        void *eargs[] = {&d, &tp, &c};
        if (tp.ext_on) {
            // the step's external forces first (AFM, walls)
            cudaKernelNodeParams ke{};
            ke.func = (void *)k_ext<1>;
            ke.gridDim = dim3((d.N + 255) / 256);
            ke.blockDim = dim3(256);
            ke.kernelParams = eargs;
            cudaGraphNode_t ne;
            CK(cudaGraphAddKernelNode(&ne, g, prev ? &prev : nullptr, prev ? 1 : 0, &ke));
            prev = ne;
        }
        if (tp.on[XMD_TERM_PID]) {
            // the step's pseudo-improper dihedral bundles
            cudaKernelNodeParams kp{};
            kp.func = (void *)k_pid<1>;
            kp.gridDim = dim3((d.N + 127) / 128);
            kp.blockDim = dim3(128);
            kp.kernelParams = eargs;
            cudaGraphNode_t np;
            CK(cudaGraphAddKernelNode(&np, g, prev ? &prev : nullptr, prev ? 1 : 0, &kp));
            prev = np;
        }
        CK(cudaGraphAddKernelNode(&nf, g, prev ? &prev : nullptr, prev ? 1 : 0, &kf));
        if (d.qa_on) {
            cudaKernelNodeParams ks{}, kq{};
            void *sargs[] = {&d, &tp, &c};
            ks.func = (void *)k_qa_sift;
            ks.gridDim = dim3(sift_grid());
            ks.blockDim = dim3(QA_SIFT);
            ks.kernelParams = sargs;
            kq.func = (void *)k_qa_step;
            kq.gridDim = dim3(d.R);
            kq.blockDim = dim3(1024);
            kq.kernelParams = sargs;
            cudaKernelNodeParams kt{}, kr{};
            int rcheck = gated ? 1 : 0;   // the re-freeing's last block takes the skin decision
            void *dargs[] = {&d, &dt, &rcheck};
            kt.func = (void *)k_qa_trans;
            kt.gridDim = dim3(trans_grid());
            kt.blockDim = dim3(QA_TG);
            kt.kernelParams = sargs;
            kr.func = (void *)k_qa_refree;
            kr.gridDim = dim3(d.R);
            kr.blockDim = dim3(1024);
            kr.kernelParams = dargs;
            cudaGraphNode_t n1, n2, n3, n4;
            CK(cudaGraphAddKernelNode(&n1, g, &nf, 1, &ks));
            CK(cudaGraphAddKernelNode(&n2, g, &n1, 1, &kq));
            CK(cudaGraphAddKernelNode(&n3, g, &n2, 1, &kt));
            CK(cudaGraphAddKernelNode(&n4, g, &n3, 1, &kr));
            nf = n4;
        }
        if (fuse == FUSE_CHECK || fuse == FUSE_CHECK_GATE || (d.qa_on && gated)) {
            nc = nf;
        } else {
            cudaKernelNodeParams kc{};
            void *cargs[] = {&d, &adv, &dt, &h, &setc};
            kc.func = (void *)k_nl_check;
            kc.gridDim = dim3(1);
            kc.blockDim = dim3(1024);
            kc.kernelParams = cargs;
            CK(cudaGraphAddKernelNode(&nc, g, &nf, 1, &kc));
        }
        if (gated) {   // the host rebuilds after a halt
            prev = nc;
            continue;
        }
        if (plain) {
            cudaKernelNodeParams kt{};
            void *targs[] = {&d, &tp, &cn, &zero};
            kt.func = (void *)k_nl_tile;
            kt.gridDim = dim3(tile_grid);
            kt.blockDim = dim3(TL_THREADS);
            kt.sharedMemBytes = (unsigned)tile_smem;
            kt.kernelParams = targs;
            CK(cudaGraphAddKernelNode(&ncond, g, &nc, 1, &kt));
            prev = ncond;
            continue;
        }
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        CK(cudaGraphAddNode(&ncond, g, &nc, nullptr, 1, &cp));
        add_rebuild_nodes(cp.conditional.phGraph_out[0], cn);
        prev = ncond;
    }
    CK(cudaGraphInstantiate(&gs.exec, g, 0));
    gs.graph = g;
    return gs.exec;
}

// the list rebuild as a chain of kernel nodes (body of the rebuild IF node)
void Engine::add_rebuild_nodes(cudaGraph_t body, int cn) {
    cudaGraphNode_t last = nullptr;
    auto add = [&](cudaKernelNodeParams &kp) {
        cudaGraphNode_t nn;
        CK(cudaGraphAddKernelNode(&nn, body, last ? &last : nullptr, last ? 1 : 0, &kp));
        last = nn;
    };
    void *a1[] = {&d, &cn};
    void *a2[] = {&d, &tp, &cn};
    void *a3[] = {&d};
    int one = 1;
    void *a4[] = {&d, &tp, &cn, &one};
    if (any_cell) {
        cudaKernelNodeParams k1{}, k2{}, kc{}, ks{}, kx{}, kf{};
        k1.func = (void *)k_cells;
        k1.gridDim = dim3(d.R);
        k1.blockDim = dim3(CB);
        k1.kernelParams = a1;
        add(k1);
        const unsigned gb = (unsigned)((d.N + 255) / 256);
        kc.func = (void *)k_cell_count;
        kc.gridDim = dim3(gb);
        kc.blockDim = dim3(256);
        kc.kernelParams = a1;
        add(kc);
        ks.func = (void *)k_cell_scan;
        ks.gridDim = dim3(d.R);
        ks.blockDim = dim3(CB);
        ks.kernelParams = a3;
        add(ks);
        kx.func = (void *)k_cell_scatter;
        kx.gridDim = dim3(gb);
        kx.blockDim = dim3(256);
        kx.kernelParams = a3;
        add(kx);
        kf.func = (void *)k_cell_finish;
        kf.gridDim = dim3((unsigned)((d.ncells + CF_WARPS - 1) / CF_WARPS));
        kf.blockDim = dim3(CF_WARPS * 32);
        kf.kernelParams = a1;
        add(kf);
        k2.func = (void *)k_nl_cells;
        k2.gridDim = dim3((d.N + NC_WARPS - 1) / NC_WARPS);
        k2.blockDim = dim3(NC_WARPS * 32);
        k2.kernelParams = a2;
        add(k2);
    }
    if (any_tile) {
        cudaKernelNodeParams kt{};
        kt.func = (void *)k_nl_tile;
        kt.gridDim = dim3(tile_grid);
        kt.blockDim = dim3(TL_THREADS);
        kt.sharedMemBytes = (unsigned)tile_smem;
        kt.kernelParams = a4;
        add(kt);
    }
    if (d.qa_on) {
        cudaKernelNodeParams k3{}, k4{}, k5{}, k6{};
        k3.func = (void *)k_qa_fp_scan;
        k3.gridDim = dim3(d.qa.nbchunk);
        k3.blockDim = dim3(QA_BCHUNK);
        k3.kernelParams = a3;
        add(k3);
        k4.func = (void *)k_qa_fp_base;
        k4.gridDim = dim3(d.R);
        k4.blockDim = dim3(1024);
        k4.kernelParams = a3;
        add(k4);
        k5.func = (void *)k_qa_fp_fill;
        k5.gridDim = dim3(d.qa.nbchunk);
        k5.blockDim = dim3(QA_BCHUNK);
        k5.kernelParams = a3;
        add(k5);
        k6.func = (void *)k_qa_compact;
        k6.gridDim = dim3(d.R);
        k6.blockDim = dim3(1024);
        k6.kernelParams = a3;
        add(k6);
    }
}

void Engine::check_status(const char *where) {
    int st = 0;
    CK(cudaMemcpyAsync(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    if (st & ST_CAPACITY)
        throw std::length_error(std::string(where) + ": Verlet row capacity exceeded (raise `engine: nl capacity`)");
    if (st & ST_NONFINITE) {
        // reported once: the faulted replicas are frozen (a new state thaws
        // them); the other replicas of the context go on
        const int keep = st & ~ST_NONFINITE;
        CK(cudaMemcpyAsync(d.status, &keep, sizeof(int), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        if (!isolate_faults) throw std::domain_error(std::string(where) + ": non-finite force");
    }
}

void Engine::eval_forces(int rep, double *F, double *V) {
    check_rep(reps, rep);
    ready();
    ensure_nl();
    CK(cudaMemsetAsync(d.Vrep, 0, sizeof(double) * XMD_NUM_TERMS * d.R, stream));
    launch_force(0, cur);
    const RepHost &h = reps[rep];
    std::vector<double> Ft;
    double *Fh = F;
    if (!Fh) {
        Ft.resize(3 * (size_t)h.n);
        Fh = Ft.data();
    }
    CK(cudaMemcpyAsync(Fh, d.F + 3 * (size_t)h.begin, sizeof(double) * 3 * h.n, cudaMemcpyDeviceToHost, stream));
    if (V) CK(cudaMemcpyAsync(V, d.Vrep + (size_t)rep * XMD_NUM_TERMS, sizeof(double) * XMD_NUM_TERMS,
                              cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    // only this replica's forces decide: a replica frozen by a non-finite
    // force does not fail the evaluation of the others
    const bool iso = isolate_faults;
    isolate_faults = true;
    try {
        check_status("eval_forces");
    } catch (...) {
        isolate_faults = iso;
        throw;
    }
    isolate_faults = iso;
    for (size_t k = 0; k < 3 * (size_t)h.n; ++k)
        if (!std::isfinite(Fh[k])) throw std::domain_error("eval_forces: non-finite force");
}

void Engine::step(int nsteps) {
    step_async(nsteps);
    // rows keep their contents when they grow: no list needs rebuilding, so
    // no replica's trajectory depends on another's row lengths
    step_wait();
}

// ---- packed host-buffer path ----------------------------------------------------
__global__ void k_unpack_history(Dev d, const double *__restrict__ y, int cur) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const size_t n3 = 3 * (size_t)d.N;
    double4_32a p = d.pos[cur][i];
    p.x = y[3 * (size_t)i];
    p.y = y[3 * (size_t)i + 1];
    p.z = y[3 * (size_t)i + 2];
    d.pos[cur][i] = p;
    for (int ord = 1; ord < 6; ++ord)
        for (int a = 0; a < 3; ++a)
            d.yh[(size_t)((ord - 1) * 3 + a) * d.N + i] = y[ord * n3 + 3 * (size_t)i + a];
    // the skin test sees the new positions like any other displacement
    int r = d.rep_of[i];
    if (r < 0) return;
    double disp = dist2_exact(d.rep[r].box, p, d.orig[i]);   // squared, as k_force records it
    atomicMax(&d.rep[r].maxdisp, (unsigned long long)__double_as_longlong(disp));
}
__global__ void k_pack_positions(Dev d, double *__restrict__ r, int cur) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    double4_32a p = d.pos[cur][i];
    r[3 * (size_t)i] = p.x;
    r[3 * (size_t)i + 1] = p.y;
    r[3 * (size_t)i + 2] = p.z;
}

__global__ void k_pack_history(Dev d, double *__restrict__ y, int cur) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const size_t n3 = 3 * (size_t)d.N;
    double4_32a p = d.pos[cur][i];
    y[3 * (size_t)i] = p.x;
    y[3 * (size_t)i + 1] = p.y;
    y[3 * (size_t)i + 2] = p.z;
    for (int ord = 1; ord < 6; ++ord)
        for (int a = 0; a < 3; ++a)
            y[ord * n3 + 3 * (size_t)i + a] = d.yh[(size_t)((ord - 1) * 3 + a) * d.N + i];
}

void Engine::upload_history_all(const double *y) {
    use_device();
    ready();
    if (!staging) staging = (double *)dalloc(sizeof(double) * 18 * (size_t)d.N);
    CK(cudaMemcpyAsync(staging, y, sizeof(double) * 18 * (size_t)d.N, cudaMemcpyHostToDevice, stream));
    k_unpack_history<<<(d.N + 255) / 256, 256, 0, stream>>>(d, staging, cur);
    ++launches;
}

void Engine::download_history_all(double *y) {
    use_device();
    ready();
    if (!staging) staging = (double *)dalloc(sizeof(double) * 18 * (size_t)d.N);
    k_pack_history<<<(d.N + 255) / 256, 256, 0, stream>>>(d, staging, cur);
    ++launches;
    CK(cudaMemcpyAsync(y, staging, sizeof(double) * 18 * (size_t)d.N, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
}

void Engine::download_positions_all(double *r) {
    use_device();
    ready();
    if (!staging) staging = (double *)dalloc(sizeof(double) * 18 * (size_t)d.N);
    k_pack_positions<<<(d.N + 255) / 256, 256, 0, stream>>>(d, staging, cur);
    ++launches;
    CK(cudaMemcpyAsync(r, staging, sizeof(double) * 3 * (size_t)d.N, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
}

void Engine::stats(int64_t *out) {
    use_device();
    for (int k = 0; k < XMD_NUM_STATS; ++k) out[k] = 0;
    int64_t nb = 0;
    int64_t nr = 0;
    for (auto &r : reps)
        if (r.in_use) { nb += r.n; ++nr; }
    out[XMD_STAT_BEADS] = nb;
    out[XMD_STAT_REPLICAS] = nr;
    out[XMD_STAT_LAUNCHES] = launches;
    out[XMD_STAT_MD_STEPS] = md_steps;
    if (!finalized) return;
    std::vector<int32_t> cnt(d.N);
    CK(cudaMemcpyAsync(cnt.data(), d.nl_cnt, sizeof(int32_t) * d.N, cudaMemcpyDeviceToHost, stream));
    const int32_t nn = cap.nat;   // entries of free native ranges are kept at 0
    std::vector<uint8_t> on(nn > 0 ? nn : 1);
    if (nn) CK(cudaMemcpyAsync(on.data(), d.nat_on, nn, cudaMemcpyDeviceToHost, stream));
    std::vector<RepDev> rd(d.R);
    CK(cudaMemcpyAsync(rd.data(), d.rep, sizeof(RepDev) * d.R, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    unsigned long long passes = 0;
    CK(cudaMemcpyAsync(&passes, d.ctr, sizeof(passes), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    out[XMD_STAT_LAUNCHES] = launches + (int64_t)((any_cell ? 6 : 0) + (any_tile ? 1 : 0) + (d.qa_on ? 4 : 0)) * (int64_t)passes;
    for (int i = 0; i < d.N; ++i)
        if (owner_h[i] >= 0) out[XMD_STAT_NL_ENTRIES] += cnt[i];
    for (int k = 0; k < nn; ++k) out[XMD_STAT_GO_ACTIVE] += on[k];
    for (auto &r : rd)
        if (r.active) out[XMD_STAT_REBUILDS] += (int64_t)r.rebuilds;
}

int Engine::qa_contacts(int rep, int cap, int32_t *out4, double *ref_time) {
    check_rep(reps, rep);
    ready();
    if (!d.qa_on) return 0;
    RepDev rd;
    CK(cudaMemcpyAsync(&rd, d.rep + rep, sizeof(RepDev), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    int n = rd.ct_n, o = rd.ct_off;
    std::vector<int32_t> i1(n), i2(n), ty(n);
    std::vector<uint8_t> st(n), vac(n);
    std::vector<double> rf(n);
    if (n) {
        CK(cudaMemcpyAsync(i1.data(), d.qa.ct_i1 + o, 4 * n, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(i2.data(), d.qa.ct_i2 + o, 4 * n, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(ty.data(), d.qa.ct_type + o, 4 * n, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(st.data(), d.qa.ct_status + o, n, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(vac.data(), d.qa.ct_vac + o, n, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(rf.data(), d.qa.ct_ref + o, 8 * n, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
    }
    int m = 0;
    const int b = reps[rep].begin;
    for (int k = 0; k < n; ++k) {
        if (vac[k]) continue;
        if (m < cap) {
            if (out4) {
                out4[4 * m] = i1[k] - b; out4[4 * m + 1] = i2[k] - b;
                out4[4 * m + 2] = ty[k]; out4[4 * m + 3] = st[k];
            }
            if (ref_time) ref_time[m] = rf[k];
        }
        ++m;
    }
    return m;
}

int Engine::verlet_pairs(int rep, int cap, int32_t *out2, uint8_t *flags) {
    check_rep(reps, rep);
    ready();
    ensure_nl();
    const RepHost &h = reps[rep];
    std::vector<int32_t> cnt(h.n), rows((size_t)nl_cap * h.n);
    CK(cudaMemcpyAsync(cnt.data(), d.nl_cnt + h.begin, sizeof(int32_t) * h.n, cudaMemcpyDeviceToHost, stream));
    for (int k = 0; k < nl_cap; ++k)
        CK(cudaMemcpyAsync(rows.data() + (size_t)k * h.n, d.nl_row + (size_t)k * d.N + h.begin,
                           sizeof(int32_t) * h.n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    std::vector<std::tuple<int, int, int>> v;
    for (int i = 0; i < h.n; ++i)
        for (int k = 0; k < cnt[i]; ++k) {
            int e = rows[(size_t)k * h.n + i];
            int j = (e & NL_MASK) - h.begin;
            if (j > i) v.emplace_back(i, j, ((e & NL_PAULI) ? 1 : 0) | ((e & NL_ES) ? 2 : 0) | ((e & NL_PID) ? 4 : 0));
        }
    std::sort(v.begin(), v.end());
    for (size_t k = 0; k < v.size() && (int)k < cap; ++k) {
        out2[2 * k] = std::get<0>(v[k]);
        out2[2 * k + 1] = std::get<1>(v[k]);
        if (flags) flags[k] = (uint8_t)std::get<2>(v[k]);
    }
    return (int)v.size();
}

void Engine::qa_sync(int rep, int8_t *out) {
    check_rep(reps, rep);
    ready();
    const RepHost &h = reps[rep];
    if (!d.qa_on) {
        for (int i = 0; i < h.n; ++i)
            for (int k = 0; k < 4; ++k) out[4 * i + k] = (int8_t)params.limits[h.atype[i]][k];
        return;
    }
    std::vector<int32_t> s(h.n);
    CK(cudaMemcpyAsync(s.data(), d.qa.sync + h.begin, 4 * (size_t)h.n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    for (int i = 0; i < h.n; ++i)
        for (int k = 0; k < 4; ++k) out[4 * i + k] = (int8_t)((s[i] >> (8 * k)) & 0xff);
}

void Engine::set_kernel_timing(bool on) {
    timing = on;
    n_ev_force = n_ev_rebuild = 0;
}

void Engine::kernel_times(double *force_ms, int64_t *nf, double *rebuild_ms, int64_t *nr) {
    use_device();
    CK(cudaStreamSynchronize(stream));
    double f = 0, r = 0;
    for (size_t k = 0; k + 1 < n_ev_force; k += 2) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ev_force[k], ev_force[k + 1]));
        f += ms;
    }
    for (size_t k = 0; k + 1 < n_ev_rebuild; k += 2) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ev_rebuild[k], ev_rebuild[k + 1]));
        r += ms;
    }
    if (force_ms) *force_ms = f;
    if (nf) *nf = (int64_t)(n_ev_force / 2);
    if (rebuild_ms) *rebuild_ms = r;
    if (nr) *nr = (int64_t)(n_ev_rebuild / 2);
}

void Engine::observables(int rep, double *E, double *K, double *Rg, double *Q) {
    check_rep(reps, rep);
    double V[XMD_NUM_TERMS];
    eval_forces(rep, nullptr, V);
    const RepHost &h = reps[rep];
    std::vector<double> r(3 * (size_t)h.n), v(3 * (size_t)h.n);
    get_state(rep, r.data(), v.data(), nullptr);
    double Vt = 0;
    for (double x : V) Vt += x;
    double K_ = 0;   // total_energy.cpp:4-11
    for (int i = 0; i < h.n; ++i)
        K_ += 0.5 * 1.0 * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
    double cm[3] = {0, 0, 0};   // gyration.cpp:4-19
    for (int i = 0; i < h.n; ++i) for (int a = 0; a < 3; ++a) cm[a] += r[3 * i + a];
    for (int a = 0; a < 3; ++a) cm[a] /= h.n;
    double g = 0;
    for (int i = 0; i < h.n; ++i)
        for (int a = 0; a < 3; ++a) g += (r[3 * i + a] - cm[a]) * (r[3 * i + a] - cm[a]);
    double act = 0;   // report_structure.cpp:85
    double thr = params.go_active_threshold * std::pow(2.0, -1.0 / 6.0);
    for (size_t k = 0; k < h.nat_i1.size(); ++k) {
        int a = h.nat_i1[k], b = h.nat_i2[k];
        double dx = r[3 * a] - r[3 * b], dy = r[3 * a + 1] - r[3 * b + 1], dz = r[3 * a + 2] - r[3 * b + 2];
        if (std::sqrt(dx * dx + dy * dy + dz * dz) < thr * h.nat_d[k]) act += 1;
    }
    if (E) *E = Vt + K_;
    if (K) *K = K_;
    if (Rg) *Rg = std::sqrt(g / h.n);
    if (Q) *Q = h.nat_i1.empty() ? 0.0 : act / h.nat_i1.size();
}

int Engine::device_status() {
    if (!finalized) return 0;
    int st = 0;
    CK(cudaMemcpyAsync(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return st;
}

void Engine::sync() { CK(cudaStreamSynchronize(stream)); }

}  // namespace xmdg
