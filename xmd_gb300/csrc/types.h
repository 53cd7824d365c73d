// types.h - plain records shared by host code and kernels.
#pragma once
#include <cstdint>

#include "../../include/xmd_gpu.h"

namespace xmdg {

// orthorhombic box (box.h:6-59); cell 0 = open along that axis
struct BoxD {
    double cell[3], cell_inv[3];
};

// ---- parameters shared by all terms (kernel argument, by value) --------------
struct TermP {
    int on[XMD_NUM_TERMS];
    double dt, gamma_factor;
    double dt_inv, dt2_half;     // 1.0 / dt and dt * dt / 2.0, as lang_pc.cpp:8, 21 round them
    double tether_H1, tether_H2;
    double nat_ang_k, cnd_CDA, cnd_CDB, snd_CDH;
    double go_depth;
    double pauli_r_excl, pauli_depth;
    double es_Vf, es_sdi;        // const ES (or relative ES) V_factor, 1/screening distance
    int es_rel;                  // 1: relative ES force law
    double qa_cycle, qa_cycle_inv, qa_factor;
    double lj_bb_r_min, lj_bb_depth, lj_bs_r_min, lj_bs_depth;
    int ss_sinking;
    double chir_e_chi;                       // chirality (chiral.h)
    double nat_ss_H1, nat_ss_dist;           // native ssbonds (native_ss.h: H1, nat_r)
    double vel_afm_H1, vel_afm_H2;           // velocity AFM spring (velocity_afm.h)
    int ext_on;                              // AFM tips or walls: k_ext runs before the step kernel
    int n_solid, n_ljw;                      // wall planes of each kind (0 when the term is off)
    double solid_eps, solid_cutoff;          // walls/solid.h
    double ljw_min_dist, ljw_factor, ljw_cycle, ljw_cycle_inv, ljw_depth;   // walls/lj_attr.h
    int pid_lambda;                          // pid/lambda.h: 0 cosine, 1 algebraic
    double pid_bbp[4], pid_bbm[4], pid_ss[2];   // pid_params (alpha, psi_0, r_min, depth)
    // FP32 copies of the constants the mixed path's FP32 terms use (no
    // FP64-to-FP32 conversion per interaction)
    struct F32 {
        float tether_H1, tether_H2, nat_ang_k, cnd_CDA, cnd_CDB, snd_CDH, go_depth;
        float pauli_r_excl, pauli_depth, es_Vf, es_sdi;
        float chir_e_chi, nat_ss_H1, nat_ss_dist;
    } f;
};

// the constant in the interaction's arithmetic type
template <class T> __host__ __device__ __forceinline__ T tpar(double d, float f);
template <> __host__ __device__ __forceinline__ double tpar<double>(double d, float) { return d; }
template <> __host__ __device__ __forceinline__ float tpar<float>(double, float f) { return f; }

}  // namespace xmdg
