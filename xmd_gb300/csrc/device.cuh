// device.cuh - per-interaction physics of the hot path, precision-templated.
//
// FT is the type the interaction arithmetic runs in: double for the plain
// FP64 path, float for the mixed path (pair and bonded forces in FP32,
// accumulated per bead in FP64 by the caller).  Coordinate differences are
// always taken in FP64 and then narrowed, so FP32 never sees absolute
// coordinates.  Operation order follows the cited reference functions.
#pragma once
#include <cstdint>

#include "../../include/xmd_gpu.h"
#include "types.h"

namespace xmdg {

template <class T> struct V3 { T x, y, z; };

template <class T> __device__ __forceinline__ V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> __device__ __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
// vec3.h:133-158, 349-360
template <class T> __device__ __forceinline__ T nsq(V3<T> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
template <class T> __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double acos_(double x) { return acos(x); }
__device__ __forceinline__ float acos_(float x) { return acosf(x); }
__device__ __forceinline__ double exp_(double x) { return exp(x); }
__device__ __forceinline__ float exp_(float x) { return expf(x); }
__device__ __forceinline__ void sincos_(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void sincos_(float x, float *s, float *c) { sincosf(x, s, c); }

template <class T> __device__ __forceinline__ T norm(V3<T> a) { return sqrt_(nsq(a)); }
template <class T> __device__ __forceinline__ T ninv(V3<T> a) { return T(1) / norm(a); }
template <class T> __device__ __forceinline__ V3<T> unit(V3<T> a) { return ninv(a) * a; }

// clamp: math.h:77-80 (a NaN maps to the upper bound)
template <class T> __device__ __forceinline__ T clampv(T v, T lo, T hi) {
    return v < lo ? lo : (v < hi ? v : hi);
}
// clamped acos: math.h:41-45
template <class T> __device__ __forceinline__ T acos_c(T x) {
    T x_ = x < T(-1) ? T(-1) : (x > T(1) ? T(1) : x);
    return acos_(x_);
}
template <class T> __device__ __forceinline__ T ipow6(T s) { return s * (s * (s * (s * (s * s)))); }

// ---- FP64 without contraction ---------------------------------------------------
// The plain FP64 path evaluates its bonded terms with every product, sum,
// quotient and square root rounded on its own (no fused multiply-add), as the
// uncontracted CPU build of the reference does.  On the extended starts some
// triples are straight to ~1e-6 rad: a dihedral's derivatives there scale as
// 1 / |r12 x r23|^2 and its force reaches ~1e6, so one contracted rounding
// moves that force by ~1e-10 of itself and the first step carries the change
// into the positions at ~1e-8 A.  DN is a double whose operators round each
// operation separately; the bonded templates instantiated on it reproduce
// the reference's arithmetic operation for operation.
struct DN {
    double v;
    DN() = default;
    __host__ __device__ __forceinline__ constexpr DN(double x) : v(x) {}
    __host__ __device__ __forceinline__ explicit operator double() const { return v; }
};
__device__ __forceinline__ DN operator+(DN a, DN b) { return DN(__dadd_rn(a.v, b.v)); }
__device__ __forceinline__ DN operator-(DN a, DN b) { return DN(__dsub_rn(a.v, b.v)); }
__device__ __forceinline__ DN operator*(DN a, DN b) { return DN(__dmul_rn(a.v, b.v)); }
__device__ __forceinline__ DN operator/(DN a, DN b) { return DN(__ddiv_rn(a.v, b.v)); }
__device__ __forceinline__ DN operator-(DN a) { return DN(-a.v); }
__device__ __forceinline__ DN &operator+=(DN &a, DN b) { return a = a + b; }
__device__ __forceinline__ bool operator<(DN a, DN b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(DN a, DN b) { return a.v > b.v; }
__device__ __forceinline__ DN sqrt_(DN x) { return DN(__dsqrt_rn(x.v)); }
__device__ __forceinline__ DN acos_(DN x) { return DN(acos(x.v)); }
__device__ __forceinline__ DN exp_(DN x) { return DN(exp(x.v)); }
__device__ __forceinline__ DN sin(DN x) { return DN(::sin(x.v)); }
__device__ __forceinline__ DN dn_cos(DN x) { return DN(::cos(x.v)); }
__device__ __forceinline__ DN dn_fabs(DN x) { return DN(::fabs(x.v)); }
__device__ __forceinline__ DN dn_rint(DN x) { return DN(::rint(x.v)); }
__device__ __forceinline__ void sincos_(DN x, DN *s, DN *c) { sincos(x.v, &s->v, &c->v); }
template <> __host__ __device__ __forceinline__ DN tpar<DN>(double d, float) { return DN(d); }
__device__ __forceinline__ float ldg_(const float *p) { return __ldg(p); }
__device__ __forceinline__ double ldg_(const double *p) { return __ldg(p); }
__device__ __forceinline__ DN ldg_(const DN *p) { return DN(__ldg(&p->v)); }
template <class T> __device__ __forceinline__ V3<double> v3d(V3<T> a) {
    return V3<double>{(double)a.x, (double)a.y, (double)a.z};
}

// ---- FP32 <-> FP64 on the integer pipe --------------------------------------------
// On GB300 FP64 arithmetic AND the FP32<->FP64 conversion instructions run at
// 2 lanes per clock per SM (FP32: 128).  The mixed path therefore keeps FP64
// instructions out of its per-pair and per-bond work: it moves between the
// formats with integer operations on the bit patterns, and carries extended
// precision as pairs of FP32 values (float-float).
//   narrow_f: round-to-nearest-even, equal to the hardware conversion for
//             results in the normal FP32 range; smaller magnitudes give a
//             signed zero (the hardware would give a denormal); overflow gives
//             infinity and NaN stays NaN.
//   widen_f:  exact for normal values, zeros and infinities; FP32 denormals
//             give a signed zero; NaN stays NaN.
__device__ __forceinline__ float narrow_f(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;   // FP32 biased exponent
    const unsigned sign = hi & 0x80000000u;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    unsigned f = sign | ((unsigned)e << 23) | m;
    f += (unsigned)(rem > 0x10000000u) | ((unsigned)(rem == 0x10000000u) & (m & 1u));
    const bool nan = e == 1151 && (m | rem) != 0u;
    f = e >= 255 ? (sign | 0x7f800000u | (nan ? 0x400000u : 0u)) : f;
    f = e <= 0 ? sign : f;
    return __uint_as_float(f);
}
__device__ __forceinline__ double widen_f(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned sign = u & 0x80000000u;
    const unsigned dex = ex == 0xffu ? 0x7ffu : ex + 896u;
    unsigned hi = sign | (dex << 20) | ((u & 0x7fffffu) >> 3), lo = u << 29;
    hi = ex == 0u ? sign : hi;
    lo = ex == 0u ? 0u : lo;
    return __hiloint2double((int)hi, (int)lo);
}

// A double as an unevaluated sum h + l of two floats: h holds the leading 24
// significant bits (truncated), l the next 24 of the remaining 29 (truncated),
// so |x - (h + l)| <= 2^-47 |x|.  Integer operations only.  Magnitudes below
// the FP32 normal range give 0 + 0 (positions there are zero for every purpose
// of a pair distance); non-finite input gives a non-finite h.
struct F2 { float h, l; };
__device__ __forceinline__ F2 split_d(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int E = (int)((hi >> 20) & 0x7ffu);
    const int e = E - 896;
    const unsigned sign = hi & 0x80000000u;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    unsigned h = sign | ((unsigned)e << 23) | m;
    // remainder rem * 2^(E - 1075): leading one at bit p = 31 - clz
    const int lz = __clz(rem);
    const int el = (31 - lz) + E - 948;                 // FP32 biased exponent of l
    const unsigned ml = lz >= 8 ? rem << (lz - 8) : rem >> (8 - lz);
    unsigned l = sign | ((unsigned)el << 23) | (ml & 0x7fffffu);
    l = (rem == 0u || el <= 0) ? sign : l;
    const bool big = e >= 255;
    h = big ? (sign | 0x7f800000u | ((E == 0x7ff && (m | rem)) ? 0x400000u : 0u)) : h;
    l = big ? 0u : l;
    h = e <= 0 ? sign : h;
    l = e <= 0 ? sign : l;
    return F2{__uint_as_float(h), __uint_as_float(l)};
}

// ---- float-float arithmetic (error-free transformations) ---------------------
// two_sum (Knuth): s + e == a + b exactly.  two_prod: p + e == a * b exactly
// (one FMA).  FF values are unevaluated sums h + l with |l| <= ulp(h).
struct FF { float h, l; };
__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return FF{s, e};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return FF{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.h, -a.l}; }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    FF p = two_prod(a.h, b.h);
    return fast_two_sum(p.h, __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, p.l)));
}
// w - u of two split doubles, as float-float (error <= 2^-46 of the larger
// magnitude of w, u)
__device__ __forceinline__ FF ff_diff(F2 u, F2 w) {
    FF s = two_sum(w.h, -u.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fsub_rn(w.l, u.l)));
}
// accumulation of FP32 terms into a float-float sum (error per addition
// <= 2^-47 of the running magnitude)
__device__ __forceinline__ void ff_acc(FF &acc, float v) {
    FF s = two_sum(acc.h, v);
    acc = fast_two_sum(s.h, __fadd_rn(s.l, acc.l));
}
__device__ __forceinline__ double ff_to_d(FF a) { return widen_f(a.h) + widen_f(a.l); }

__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }
// float-float cross and dot products of float-float vectors
__device__ __forceinline__ V3<FF> ff_cross(const V3<FF> &a, const V3<FF> &b) {
    return V3<FF>{ff_sub(ff_mul(a.y, b.z), ff_mul(a.z, b.y)), ff_sub(ff_mul(a.z, b.x), ff_mul(a.x, b.z)),
                  ff_sub(ff_mul(a.x, b.y), ff_mul(a.y, b.x))};
}
__device__ __forceinline__ FF ff_dot(const V3<FF> &a, const V3<FF> &b) {
    return ff_add(ff_add(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}

// position of a bead split per axis (mixed path)
struct P2 { F2 x, y, z; };
__device__ __forceinline__ P2 split_p(double4_32a p) { return P2{split_d(p.x), split_d(p.y), split_d(p.z)}; }

// FP64 difference, narrowed to FT
template <class T>
__device__ __forceinline__ V3<T> diff(double4_32a u, double4_32a w) {
    return V3<T>{T(w.x - u.x), T(w.y - u.y), T(w.z - u.z)};
}



// box::r_uv: box.h:36-49.  The wrap is done in FP64 before narrowing.
template <class T>
__device__ __forceinline__ V3<T> r_uv(const BoxD &b, double4_32a u, double4_32a w) {
    double dx = w.x - u.x, dy = w.y - u.y, dz = w.z - u.z;
    dx -= b.cell[0] * rint(dx * b.cell_inv[0]);
    dy -= b.cell[1] * rint(dy * b.cell_inv[1]);
    dz -= b.cell[2] * rint(dz * b.cell_inv[2]);
    return V3<T>{T(dx), T(dy), T(dz)};
}

// box::r_uv for a replica that may be open on every axis: there the wrap
// subtracts exactly 0 * rint(0), so skipping it changes no bit.
template <class T>
__device__ __forceinline__ V3<T> r_uv_p(const BoxD &b, bool periodic, double4_32a u, double4_32a w) {
    if (periodic) return r_uv<T>(b, u, w);
    return V3<T>{T(w.x - u.x), T(w.y - u.y), T(w.z - u.z)};
}

// Same minimum image with every product and sum rounded separately, so the
// neighbour-list membership decisions reproduce an uncontracted CPU build
// bit for bit.  dist2_exact is the squared distance (no square root).
__device__ __forceinline__ double dist2_exact(const BoxD &b, double4_32a u, double4_32a w) {
    double d[3] = {__dsub_rn(w.x, u.x), __dsub_rn(w.y, u.y), __dsub_rn(w.z, u.z)};
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = __dsub_rn(d[a], __dmul_rn(b.cell[a], rint(__dmul_rn(d[a], b.cell_inv[a]))));
    return __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
}
__device__ __forceinline__ double dist2_open(double4_32a u, double4_32a w) {
    const double x = __dsub_rn(w.x, u.x), y = __dsub_rn(w.y, u.y), z = __dsub_rn(w.z, u.z);
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}
__device__ __forceinline__ double dist_exact(const BoxD &b, double4_32a u, double4_32a w) {
    return __dsqrt_rn(dist2_exact(b, u, w));
}



// ---- bonded terms: contributions per centre bead ----------------------------

// harmonic bond (c, c+1): eval_tether_forces::iter tether.cpp:21-36,
// harmonic::operator() harmonic.h:18-25.  Returns the force on c (the force on
// c+1 is its negative).
template <class T>
__device__ __forceinline__ V3<T> tether_term(const TermP &p, double4_32a r1, double4_32a r2, T nat_dist, T *V) {
    V3<T> r12 = diff<T>(r1, r2);
    T r12_n = norm(r12);
    T dr = r12_n - nat_dist, dr2 = dr * dr;
    T H1 = tpar<T>(p.tether_H1, p.f.tether_H1), H2 = tpar<T>(p.tether_H2, p.f.tether_H2);
    T V_ = T(0.5) * dr2 * (H1 + H2 * dr2);
    T dV_dr = dr * (H1 + T(2) * H2 * dr2);
    V_ = clampv<T>(V_, T(-1.0e3), T(1.0e3));
    dV_dr = clampv<T>(dV_dr, T(-1.0e3), T(1.0e3));
    *V = V_;
    V3<T> u{r12.x / r12_n, r12.y / r12_n, r12.z / r12_n};
    return dV_dr * u;
}

// ---- heuristic angles and dihedrals -----------------------------------------

// Horner sums of V(theta) = sum_{d=0..6} a_d theta^d and its derivative, in
// the order of eval_heurestic_angle_forces::iter (angle/heurestic.cpp:45-50)
__device__ __forceinline__ void heur_poly(const double *a, double theta, double *V, double *dV) {
    double v = 0.0, dv = 0.0;
#pragma unroll
    for (int d = 6; d >= 0; --d) {
        const double c = __ldg(a + d);
        if (d > 0) dv = (double)d * c + theta * dv;
        v = c + theta * v;
    }
    *V = v;
    *dV = dv;
}

// V(phi) = c0 + c1 sin + c2 cos + c3 sin^2 + c4 cos^2 + c5 sin cos
// (dihedral/heurestic.cpp:48-50) and dV/dphi, its derivative [the shipped
// line 52-54 has +2 c4 sin cos where d(cos^2)/dphi = -2 sin cos]
template <class T>
__device__ __forceinline__ void heur_dih_V(const T *c, T s, T co, T *V, T *dV) {
    const T s2 = s * s, c2 = co * co, sc = s * co;
    *V = c[0] + c[1] * s + c[2] * co + c[3] * s2 + c[4] * c2 + c[5] * sc;
    *dV = c[1] * co - c[2] * s + T(2) * (c[3] - c[4]) * sc + c[5] * (c2 - s2);
}

// Out-of-line forms of the two heuristic sums: called, they leave a real
// branch around them, where inlined the compiler predicates their FP64
// arithmetic into every angle and dihedral centre (2% of the mixed step)
__device__ __noinline__ double2 heur_poly_nl(const double *a, double theta) {
    double v, dv;
    heur_poly(a, theta, &v, &dv);
    return make_double2(v, dv);
}
template <class T>
__device__ __noinline__ void heur_dih_nl(const T *hc, T s, T co, T *V, T *dV) {
    T c[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) c[k] = ldg_(hc + k);
    heur_dih_V<T>(c, s, co, V, dV);
}

// native angle (c-1, c, c+1): eval_native_angle_forces::iter
// angle/native.cpp:13-39; or, with hc (the type's 7 coefficients), the
// heuristic angle of eval_heurestic_angle_forces::iter
// angle/heurestic.cpp:29-59, whose geometry is the same.  Writes the forces
// on the three beads.
template <class T>
__device__ __forceinline__ void angle_term(const TermP &p, double4_32a q1, double4_32a q2, double4_32a q3, T nat_theta,
                                           const double *hc, V3<T> *f1, V3<T> *f2, V3<T> *f3, T *V) {
    V3<T> r12 = diff<T>(q1, q2), r23 = diff<T>(q2, q3);
    V3<T> x12_23 = cross(r12, r23);
    T r12_rn = ninv(r12), r23_rn = ninv(r23);
    V3<T> d1 = r12_rn * unit(cross(r12, x12_23));
    V3<T> d3 = r23_rn * unit(cross(r23, x12_23));
    V3<T> d2 = (-d1) - d3;
    T cos_theta = -dot(r12, r23) * r12_rn * r23_rn;
    T theta = acos_c(cos_theta);
    T dV;
    if (hc) {
        const double2 vd = heur_poly_nl(hc, (double)theta);
        *V = (T)vd.x;
        dV = (T)vd.y;
    } else {
        T dtheta = theta - nat_theta;
        T k = T(p.nat_ang_k);
        *V = T(0.5) * k * dtheta * dtheta;
        dV = k * dtheta;
    }
    *f1 = -(dV * d1);
    *f2 = -(dV * d2);
    *f3 = -(dV * d3);
}

// native dihedral (c-1, c, c+1, c+2): eval_cnd_forces::iter
// dihedral/complex_native.cpp:13-49 and eval_snd_forces::iter
// dihedral/simple_native.cpp:13-45; or, with hc (the type's 6
// coefficients), the heuristic dihedral of
// eval_heurestic_dihedral_forces::iter dihedral/heurestic.cpp:29-70 with
// phi = acos(cos_phi) [line 43 takes cos(cos_phi)], its energy in *Vc
template <class T>
__device__ __forceinline__ void dihedral_term(const TermP &p, double4_32a q1, double4_32a q2, double4_32a q3, double4_32a q4,
                                              T nat_phi, bool cnd, bool snd, const T *hc, V3<T> *f, T *Vc, T *Vs) {
    V3<T> r12 = diff<T>(q1, q2), r23 = diff<T>(q2, q3), r34 = diff<T>(q3, q4);
    V3<T> x12_23 = cross(r12, r23), x23_34 = cross(r23, r34);
    T x12_23_rn = ninv(x12_23), x23_34_rn = ninv(x23_34);
    V3<T> x12_23_u = x12_23_rn * x12_23, x23_34_u = x23_34_rn * x23_34;
    T cos_phi = dot(x12_23_u, x23_34_u);
    T phi = acos_c(cos_phi);
    if (dot(x12_23, r34) < T(0)) phi = -phi;
    T diff_ = phi - nat_phi;
    T dV = T(0);
    *Vc = T(0);
    *Vs = T(0);
    if (hc) {
        heur_dih_nl<T>(hc, sin(phi), cos_phi, Vc, &dV);
    } else if (cnd) {
        T sin_diff, cos_diff, sin_3diff, cos_3diff;
        sincos_(diff_, &sin_diff, &cos_diff);
        sincos_(T(3) * diff_, &sin_3diff, &cos_3diff);
        T CDA = T(p.cnd_CDA), CDB = T(p.cnd_CDB);
        *Vc = CDA * (T(1) - cos_diff) + CDB * (T(1) - cos_3diff);
        dV += CDA * sin_diff + CDB * T(3) * sin_3diff;
    }
    if (snd && !hc) {
        T CDH = T(p.snd_CDH);
        *Vs = T(0.5) * CDH * diff_ * diff_;
        dV += CDH * diff_;
    }
    T r23_n = norm(r23);
    V3<T> d1 = x12_23_rn * (r23_n * (-x12_23_u));
    V3<T> d4 = x23_34_rn * (r23_n * x23_34_u);
    T k1 = dot(r12, r23), k4 = dot(r23, r34), den = r23_n * r23_n;
    V3<T> df{(-d1.x * k1 + d4.x * k4) / den, (-d1.y * k1 + d4.y * k4) / den, (-d1.z * k1 + d4.z * k4) / den};
    V3<T> d2 = (-d1) + df;
    V3<T> d3 = (-d4) - df;
    f[0] = -(dV * d1);
    f[1] = -(dV * d2);
    f[2] = -(dV * d3);
    f[3] = -(dV * d4);
}

// chiral quad (c-1, c, c+1, c+2): eval_chiral_forces::iter chiral.cpp:15-37.
// Writes the forces on the four beads.
template <class T>
__device__ __forceinline__ void chiral_term(const TermP &p, double4_32a q1, double4_32a q2, double4_32a q3,
                                            double4_32a q4, T nat_factor, T nat_chir, V3<T> *f, T *V) {
    V3<T> r12 = diff<T>(q1, q2), r23 = diff<T>(q2, q3), r34 = diff<T>(q3, q4);
    V3<T> x12_23 = cross(r12, r23), x12_34 = cross(r12, r34), x23_34 = cross(r23, r34);
    T chir = dot(r12, x23_34) * nat_factor;
    T chir_diff = chir - nat_chir;
    T e_chi = T(p.chir_e_chi);
    *V = T(0.5) * e_chi * chir_diff * chir_diff;
    T g = e_chi * chir_diff * nat_factor;
    f[0] = g * x12_23;
    f[1] = -(g * (x12_34 + x23_34));
    f[2] = g * (x12_23 + x12_34);
    f[3] = -(g * x12_23);
}

// the same on the mixed path: r12, r23, r34 the narrowed bond vectors,
// x12_23, x23_34 their narrowed float-float crosses, triple = r12 . x23_34
// taken in float-float
__device__ __forceinline__ void chiral_mixed(const TermP &p, V3<float> r12, V3<float> r23, V3<float> r34,
                                             V3<float> x12_23, V3<float> x23_34, float triple, float nat_factor,
                                             float nat_chir, V3<float> *f, float *V) {
    (void)r23;
    const V3<float> x12_34 = cross(r12, r34);
    const float chir_diff = triple * nat_factor - nat_chir;
    const float e_chi = p.f.chir_e_chi;
    *V = 0.5f * e_chi * chir_diff * chir_diff;
    const float g = e_chi * chir_diff * nat_factor;
    f[0] = g * x12_23;
    f[1] = -(g * (x12_34 + x23_34));
    f[2] = g * (x12_23 + x12_34);
    f[3] = -(g * x12_23);
}

// ---- bonded terms of the mixed path -------------------------------------------
// The reference formulation (acos of a clamped cosine; cross products of bond
// vectors) loses all accuracy in FP32 near straight triples, where the stiff
// starting chains live: the reference's own FP32 build misses by ~1e-3.  Here
// the bond vectors, their cross products and the dihedral's triple product are
// formed in FP64 and the angles are taken with atan2 in FP32:
//   theta = atan2(|r12 x r23|, -r12.r23)                    (= acos of the cosine)
//   phi   = atan2(|r23| (x12_23 . r34), x12_23 . x23_34)    (= +-acos, sign of
//            x12_23 . r34 as in complex_native.cpp:27-28)
// after which every FP32 operation is well conditioned.  Force expressions are
// those of angle/native.cpp:25-38 and dihedral/complex_native.cpp:37-48.
__device__ __forceinline__ V3<double> dsub(double4_32a u, double4_32a w) {
    return V3<double>{w.x - u.x, w.y - u.y, w.z - u.z};
}
__device__ __forceinline__ V3<float> f3(V3<double> a) { return V3<float>{(float)a.x, (float)a.y, (float)a.z}; }

// tether of the mixed path from the narrowed bond vector r12 = r2 - r1
__device__ __forceinline__ V3<float> tether_vec(const TermP &p, V3<float> r12, float nat_dist, float *V) {
    float r12_n = norm(r12);
    float dr = r12_n - nat_dist, dr2 = dr * dr;
    float H1 = p.f.tether_H1, H2 = p.f.tether_H2;
    float V_ = 0.5f * dr2 * (H1 + H2 * dr2);
    float dV_dr = dr * (H1 + 2.0f * H2 * dr2);
    *V = clampv<float>(V_, -1.0e3f, 1.0e3f);
    dV_dr = clampv<float>(dV_dr, -1.0e3f, 1.0e3f);
    const float inv = 1.0f / r12_n;
    return dV_dr * V3<float>{r12.x * inv, r12.y * inv, r12.z * inv};
}

// r12, r23: narrowed bond vectors; x12_23: narrowed FP64 cross product.
// hc: heuristic angle coefficients (or null); their polynomial, whose terms
// cancel to ~1e-5 of their size, is summed in FP64
__device__ __forceinline__ void angle_mixed(const TermP &p, V3<float> r12, V3<float> r23, V3<float> x12_23,
                                            float nat_theta, const double *hc, V3<float> *f1, V3<float> *f2,
                                            V3<float> *f3o, float *V) {
    float r12_rn = 1.0f / norm(r12), r23_rn = 1.0f / norm(r23);
    V3<float> d1 = r12_rn * unit(cross(r12, x12_23));
    V3<float> d3 = r23_rn * unit(cross(r23, x12_23));
    V3<float> d2 = (-d1) - d3;
    float theta = atan2f(norm(x12_23), -dot(r12, r23));
    float dV;
    if (hc) {
        const double2 vd = heur_poly_nl(hc, (double)theta);
        *V = (float)vd.x;
        dV = (float)vd.y;
    } else {
        float dtheta = theta - nat_theta;
        float k = p.f.nat_ang_k;
        *V = 0.5f * k * dtheta * dtheta;
        dV = k * dtheta;
    }
    *f1 = -(dV * d1);
    *f2 = -(dV * d2);
    *f3o = -(dV * d3);
}

// narrowed bond vectors and cross products; X = x12_23 . x23_34 and
// T = x12_23 . r34 taken in FP64 by the caller
// (hc: heuristic dihedral coefficients or null, as dihedral_term)
__device__ __forceinline__ void dihedral_mixed(const TermP &p, V3<float> r12, V3<float> r23, V3<float> r34,
                                               V3<float> x12_23, V3<float> x23_34, float X, float T,
                                               float nat_phi, bool cnd, bool snd, const float *hc, V3<float> *f,
                                               float *Vc, float *Vs) {
    float r23_n = norm(r23);
    float phi = atan2f(r23_n * T, X);
    float diff_ = phi - nat_phi;
    float dV = 0.0f;
    *Vc = 0.0f;
    *Vs = 0.0f;
    if (hc) {
        float sp, cp;
        sincosf(phi, &sp, &cp);
        heur_dih_nl<float>(hc, sp, cp, Vc, &dV);
    } else if (cnd) {
        float s1, c1, s3, c3;
        sincosf(diff_, &s1, &c1);
        sincosf(3.0f * diff_, &s3, &c3);
        float CDA = p.f.cnd_CDA, CDB = p.f.cnd_CDB;
        *Vc = CDA * (1.0f - c1) + CDB * (1.0f - c3);
        dV += CDA * s1 + CDB * 3.0f * s3;
    }
    if (snd && !hc) {
        float CDH = p.f.snd_CDH;
        *Vs = 0.5f * CDH * diff_ * diff_;
        dV += CDH * diff_;
    }
    float x12_23_rn = 1.0f / norm(x12_23), x23_34_rn = 1.0f / norm(x23_34);
    V3<float> x12_23_u = x12_23_rn * x12_23, x23_34_u = x23_34_rn * x23_34;
    V3<float> d1 = x12_23_rn * (r23_n * (-x12_23_u));
    V3<float> d4 = x23_34_rn * (r23_n * x23_34_u);
    float k1 = dot(r12, r23), k4 = dot(r23, r34), den = r23_n * r23_n;
    V3<float> df{(-d1.x * k1 + d4.x * k4) / den, (-d1.y * k1 + d4.y * k4) / den, (-d1.z * k1 + d4.z * k4) / den};
    V3<float> d2 = (-d1) + df;
    V3<float> d3 = (-d4) - df;
    f[0] = -(dV * d1);
    f[1] = -(dV * d2);
    f[2] = -(dV * d3);
    f[3] = -(dV * d4);
}

// ---- pair terms: force on the first bead of r12 = r_uv(r_i, r_j) ------------

// lj::operator(): primitives/lj.h:22-30
template <class T>
__device__ __forceinline__ void lj_eval(T depth, T r_min, T r_inv, T *V, T *dV) {
    T s = r_inv * r_min, s6 = ipow6(s), s12 = s6 * s6;
    T V_ = depth * (s12 - T(2) * s6);
    T dV_dr = T(12) * depth * r_inv * (s6 - s12);
    *V = clampv<T>(V_, T(-1.0e3), T(1.0e3));
    *dV = clampv<T>(dV_dr, T(-1.0e3), T(1.0e3));
}

// Go contact: eval_go_forces::iter go.cpp:31-46
template <class T>
__device__ __forceinline__ V3<T> go_pair(const TermP &p, V3<T> r12, T nat_dist, T *V) {
    T r12_rn = ninv(r12);
    V3<T> u = r12_rn * r12;
    T dV;
    lj_eval<T>(tpar<T>(p.go_depth, p.f.go_depth), nat_dist, r12_rn, V, &dV);
    return dV * u;
}

// native disulfide: eval_nat_ssbond_forces::iter native_ss.cpp:27-40,
// harmonic(H1, 0, nat_r) (harmonic.h:18-25) on the bond length
template <class T>
__device__ __forceinline__ V3<T> ss_pair(const TermP &p, V3<T> r12, T *V) {
    const T r12_n = norm(r12);
    const T nat_r = tpar<T>(p.nat_ss_dist, p.f.nat_ss_dist), H1 = tpar<T>(p.nat_ss_H1, p.f.nat_ss_H1);
    const T dr = r12_n - nat_r, dr2 = dr * dr;
    T V_ = T(0.5) * dr2 * (H1 + T(0) * dr2);
    T dV_dr = dr * (H1 + T(2) * T(0) * dr2);
    *V = clampv<T>(V_, T(-1.0e3), T(1.0e3));
    dV_dr = clampv<T>(dV_dr, T(-1.0e3), T(1.0e3));
    const V3<T> u{r12.x / r12_n, r12.y / r12_n, r12.z / r12_n};
    return dV_dr * u;
}

// Pauli exclusion: eval_pauli_exclusion_forces::iter pauli.cpp:32-48,
// shifted_lj::operator() shifted_lj.h:14-21
template <class T>
__device__ __forceinline__ V3<T> pauli_pair(const TermP &p, V3<T> r12, T *V) {
    T r12_rn = ninv(r12);
    T r_excl = tpar<T>(p.pauli_r_excl, p.f.pauli_r_excl);
    if (T(1) < r12_rn * r_excl) {
        V3<T> u = r12_rn * r12;
        T depth = tpar<T>(p.pauli_depth, p.f.pauli_depth);
        T s = r12_rn * r_excl, s6 = ipow6(s), s12 = s6 * s6;
        T V_ = depth * (s12 - T(2) * s6 + T(1));
        T dV_dr = T(12) * depth * r12_rn * (s6 - s12);
        *V = clampv<T>(V_, T(-1.0e3), T(1.0e3));
        dV_dr = clampv<T>(dV_dr, T(-1.0e3), T(1.0e3));
        return dV_dr * u;
    }
    *V = T(0);
    return V3<T>{T(0), T(0), T(0)};
}

// Debye-Hueckel: eval_const_es_forces::iter es/const.cpp:13-32 and
// eval_relative_es_forces::iter es/relative.cpp:13-32
template <class T>
__device__ __forceinline__ V3<T> es_pair(const TermP &p, V3<T> r12, T q1_x_q2, T *V) {
    T r12_n = norm(r12), r12_rn = T(1) / r12_n;
    V3<T> u = r12_rn * r12;
    T sdi = tpar<T>(p.es_sdi, p.f.es_sdi);
    T Vij = tpar<T>(p.es_Vf, p.f.es_Vf) * q1_x_q2 * exp_(-r12_n * sdi) * r12_rn * r12_rn;
    T dVij_dr = p.es_rel ? -Vij * (sdi + T(2) * r12_rn) : -Vij * (sdi + r12_rn);
    *V = Vij;
    return dVij_dr * u;
}

// sink_lj::operator(): primitives/sink_lj.h:24-33
template <class T>
__device__ __forceinline__ void sink_lj_eval(T depth, T r_min, T r_max, T r, T r_inv, T *V, T *dV) {
    T r_eff = (r < r_min ? r_min : (r < r_max ? r : r_max));
    T s = r_inv * r_eff, s6 = ipow6(s), s12 = s6 * s6;
    T V_ = depth * (s12 - T(2) * s6);
    T dV_dr = T(12) * depth * r_inv * (s6 - s12);
    dV_dr = (r_min < r && r < r_max) ? T(0) : dV_dr;
    *V = clampv<T>(V_, T(-1.0e3), T(1.0e3));
    *dV = clampv<T>(dV_dr, T(-1.0e3), T(1.0e3));
}

// ---- generator: rand_gen.h:22-58 ----------------------------------------------
__device__ __forceinline__ uint64_t rng_next(uint64_t &st) {
    uint64_t res = st * 0xd989bcacc137dcd5ull;
    st ^= st >> 11;
    st ^= st << 31;
    st ^= st >> 18;
    return res;
}
// Four draws of one bead (normal_x2 then normal, lang_pc.cpp:15-16)
__device__ __forceinline__ void noise3(uint64_t st, double *nx, double *ny, double *nz) {
    const double inv = 1.0 / 4294967296.0;
    double u1 = (double)(rng_next(st) >> 32) * inv;
    double u2 = (double)(rng_next(st) >> 32) * inv;
    double u3 = (double)(rng_next(st) >> 32) * inv;
    double u4 = (double)(rng_next(st) >> 32) * inv;
    double r = sqrt(-2.0 * log(u1));
    if (isnan(r)) r = 0.0;
    double t = (2.0 * 3.141592653589793) * u2;
    double s, c;
    sincos(t, &s, &c);
    *nx = r * c;
    *ny = r * s;
    double r2 = sqrt(-2.0 * log(u3));
    if (isnan(r2)) r2 = 0.0;
    *nz = r2 * cos((2.0 * 3.141592653589793) * u4);
}
// The same product from 16 nibble tables of 16 entries (entry [q][v] = XOR of
// the columns 4q..4q+3 selected by the bits of v): 16 lookups instead of 64
constexpr int JUMP_WORDS = 256;
__device__ __forceinline__ uint64_t gf2_apply_nib(const uint64_t *__restrict__ tab, uint64_t x) {
    uint64_t y = 0;
#pragma unroll
    for (int q = 0; q < 16; ++q) y ^= __ldg(tab + 16 * q + (int)((x >> (4 * q)) & 15ull));
    return y;
}
// Mixed-path noise: the same four draws per bead, turned into three
// normals without the conversion pipe (which runs at a fraction of the FP64
// rate on GB300).  A uniform in (0, 1) is built from the top 23 bits of a draw
// as a float in [1, 2) minus (1 - 2^-24), which is exact (Sterbenz) and never
// 0 or 1; Box-Muller then uses the hardware log and sine/cosine on
// t - pi in [-pi, pi), whose sine and cosine are those of t negated - the
// same distribution.
__device__ __forceinline__ float u01_bits(uint64_t v) {
    return __uint_as_float(0x3f800000u | (unsigned)(v >> 41)) - __uint_as_float(0x3f7fffffu);
}
__device__ __forceinline__ void noise3m(uint64_t st, float *nx, float *ny, float *nz) {
    const float u1 = u01_bits(rng_next(st)), u2 = u01_bits(rng_next(st));
    const float u3 = u01_bits(rng_next(st)), u4 = u01_bits(rng_next(st));
    const float two_pi = 6.283185307179586f;
    const float r = sqrtf(-2.0f * __logf(u1));
    float s, c;
    __sincosf(two_pi * u2 - 3.141592653589793f, &s, &c);
    *nx = r * c;
    *ny = r * s;
    const float r2 = sqrtf(-2.0f * __logf(u3));
    *nz = r2 * __cosf(two_pi * u4 - 3.141592653589793f);
}
// 64x64 GF(2) matrix (columns) times state: the xorshift jump-ahead
__device__ __forceinline__ uint64_t gf2_apply(const uint64_t *__restrict__ col, uint64_t x) {
    uint64_t y = 0;
#pragma unroll 16
    for (int k = 0; k < 64; ++k) y ^= col[k] & (0ull - ((x >> k) & 1ull));
    return y;
}

// ---- per-bead force accumulation and pair geometry, by path -------------------
// FP64 path: FP64 sums in the reference's term order; r_uv in FP64.
// Mixed path: FP32 terms summed per bead in float-float (each addition exact
// to 2^-47 of the running sum, below the FP32 rounding of the terms by ~10^7)
// and widened once; pair vectors from split positions in FP32 (the minimum
// image subtracted in float-float), with no FP64 instruction per pair.
template <class FT> struct Acc3;
// FP64: every addition rounded on its own (never fused with the product that
// formed the term), so the sums are the same bits whatever code shape the
// compiler gives the loops
template <> struct Acc3<double> {
    double x = 0, y = 0, z = 0;
    __device__ __forceinline__ void add(V3<double> f) { x = __dadd_rn(x, f.x); y = __dadd_rn(y, f.y); z = __dadd_rn(z, f.z); }
    __device__ __forceinline__ void sub(V3<double> f) { x = __dadd_rn(x, -f.x); y = __dadd_rn(y, -f.y); z = __dadd_rn(z, -f.z); }
    __device__ __forceinline__ V3<double> total() const { return V3<double>{x, y, z}; }
};
template <> struct Acc3<float> {
    FF x{0.0f, 0.0f}, y{0.0f, 0.0f}, z{0.0f, 0.0f};
    __device__ __forceinline__ void add(V3<float> f) { ff_acc(x, f.x); ff_acc(y, f.y); ff_acc(z, f.z); }
    __device__ __forceinline__ void sub(V3<float> f) { ff_acc(x, -f.x); ff_acc(y, -f.y); ff_acc(z, -f.z); }
    __device__ __forceinline__ V3<double> total() const { return V3<double>{ff_to_d(x), ff_to_d(y), ff_to_d(z)}; }
};

// w - u of split coordinates along one axis of length L = Lh + Ll (0 when open)
__device__ __forceinline__ float mi_axis(F2 u, F2 w, float Lh, float Ll, float Linv, bool per) {
    if (!per) return __fadd_rn(__fsub_rn(w.h, u.h), __fsub_rn(w.l, u.l));
    const FF dd = ff_diff(u, w);
    const float n = rintf(__fmul_rn(dd.h, Linv));
    const FF q = ff_sub(dd, two_prod(n, Lh));
    return __fadd_rn(q.h, __fsub_rn(q.l, __fmul_rn(n, Ll)));
}

// q_i q_j of the Debye-Hueckel pair (es_pair.cpp:17): an FP64 product on the
// FP64 path; the charges are small integers, so the FP32 product of the
// narrowed charges is the same value on the mixed path
template <class FT> __device__ __forceinline__ FT charge_prod(double qi, double qj);
template <> __device__ __forceinline__ double charge_prod<double>(double qi, double qj) { return qi * qj; }
template <> __device__ __forceinline__ float charge_prod<float>(double qi, double qj) {
    return __fmul_rn(narrow_f(qi), narrow_f(qj));
}

template <class FT> struct PairGeo;
template <> struct PairGeo<double> {
    BoxD bx;
    bool per;
    double4_32a pi;
    __device__ __forceinline__ PairGeo(const BoxD &b, bool periodic, double4_32a p) : bx(b), per(periodic), pi(p) {}
    __device__ __forceinline__ V3<double> to(double4_32a pj) const { return r_uv_p<double>(bx, per, pi, pj); }
    __device__ __forceinline__ V3<double> between(double4_32a a, double4_32a b) const {
        return r_uv_p<double>(bx, per, a, b);
    }
};
template <> struct PairGeo<float> {
    float Lh[3], Ll[3], Li[3];
    bool per;
    P2 si;
    __device__ __forceinline__ PairGeo(const BoxD &b, bool periodic, double4_32a p) : per(periodic), si(split_p(p)) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            Lh[a] = Ll[a] = Li[a] = 0.0f;
            if (periodic) {
                const F2 L = split_d(b.cell[a]);
                Lh[a] = L.h;
                Ll[a] = L.l;
                Li[a] = narrow_f(b.cell_inv[a]);
            }
        }
    }
    __device__ __forceinline__ V3<float> diff2(const P2 &u, const P2 &w) const {
        return V3<float>{mi_axis(u.x, w.x, Lh[0], Ll[0], Li[0], per), mi_axis(u.y, w.y, Lh[1], Ll[1], Li[1], per),
                         mi_axis(u.z, w.z, Lh[2], Ll[2], Li[2], per)};
    }
    __device__ __forceinline__ V3<float> to(double4_32a pj) const { return diff2(si, split_p(pj)); }
    __device__ __forceinline__ V3<float> between(double4_32a a, double4_32a b) const {
        return diff2(split_p(a), split_p(b));
    }
};

}  // namespace xmdg
