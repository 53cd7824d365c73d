// ref_driver.cpp - drives the reference's OWN hot-path translation units.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/ref/build_ref.sh against the
// reference tree (with `real` set to double for the FP64 oracle) into
// oracle/_ref/, never shipped.  It exposes the same flat API as
// oracle/xmd_oracle.h with an `xr_` prefix, so tests can pin the C
// restatement (xo_*) against the reference's own arithmetic.
//
// The term objects, list filters, QA stages, verify and lang_pc_step are the
// reference's compiled code; this file only wires them together the way
// src/freeform/main.cpp:208-1076 does, restating what cannot run as shipped:
//   - the Verlet list core (src/nl/legacy_update.cpp:6-70: push_back never
//     grows the SoA vector and the native merge never advances) [D1-D3];
//   - update_go_contacts (src/forces/go.cpp:8-23, same push_back bug) [D1];
//   - QA valence initialisation (main.cpp:662-672 appends after n zeros) [D4];
//   - update_free_pairs gets max_formation_min_dist and a copy of the list
//     without pairs already in contact [D5];
//   - process_contacts gets an lj_variants table shifted by one so that its
//     ljs[type] lookup returns the potential of `type` [D6];
//   - process_contacts runs after process_candidates each step [D7];
//   - lang_pc_step gets dt / r / num_particles [D8].
// `particle_pairs` is mapped to `non_native` at compile time [D3].
#include <xmd/types/vec3.h>
#include <xmd/model/box.h>
#include <xmd/random/rand_gen.h>
#include <xmd/forces/tether.h>
#include <xmd/forces/angle/native.h>
#include <xmd/forces/dihedral/complex_native.h>
#include <xmd/forces/dihedral/simple_native.h>
#include <xmd/forces/go.h>
#include <xmd/forces/chiral.h>
#include <xmd/forces/native_ss.h>
#include <xmd/model/model.h>
#include <xmd/forces/angle/heurestic.h>
#include <xmd/forces/velocity_afm.h>
#include <xmd/forces/force_afm.h>
#include <xmd/forces/walls/solid.h>
#include <xmd/forces/walls/lj_attr.h>
#include <xmd/forces/pid/eval_forces.h>
#include <xmd/forces/pid/bundle.h>
#include <xmd/forces/dihedral/heurestic.h>
#include <xmd/forces/pauli.h>
#include <xmd/forces/es/const.h>
#include <xmd/forces/es/relative.h>
#include <xmd/forces/qa/qa.h>
#include <xmd/forces/qa/free_pair.h>
#include <xmd/dynamics/lang_pc.h>
#include <xmd/nl/verify.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <utility>
#include <vector>

#include "../../include/xmd_gpu.h"

using namespace xmd;

namespace {
// amino_acid::all() lives in src/types/amino_acid.cpp, which does not compile
// (it names an undeclared `parsed`, amino_acid.cpp:158); same list, by code.
std::vector<amino_acid> all_aa() {
    std::vector<amino_acid> v;
    for (int k = 0; k < amino_acid::NUM_AA; ++k) v.emplace_back((aa_code)k);
    return v;
}

struct xr_sys {
    xmd_params p;
    int n = 0;
    box bx;
    rand_gen gen{0};
    real t = 0;
    true_real true_t = 0;
    double temperature = 0;

    ::vector<vec3r> r, v, F, n_, h_;
    ::vector<vec3tr> y0, y1, y2, y3, y4, y5;
    ::vector<real> mass, mass_inv, mass_rsqrt;
    ::vector<int> chain, seq, prev, next;
    ::vector<amino_acid> atype;

    ::vector<tether_pair> tethers;
    ::vector<nat_ang> angles;
    ::vector<nat_dih> dihedrals;
    ::vector<nat_cont> all_nat_cont, go_contacts;
    std::vector<std::pair<int, int>> nat_sorted;
    ::vector<chiral_quad> quads;
    ::vector<heur_ang> heur_angles;
    ::vector<heur_dih> heur_dihedrals;
    ::vector<vel_afm_tip> vafm;
    ::vector<force_afm_tip> fafm;
    ::vector<plane> walls[2];
    ::vector<vec3r> wall_F[2];
    ::vector<lj_attr_pair> ljw_pairs;
    ::vector<pid::pid_bundle> pid_bundles;
    ::vector<sink_lj> ss_plain;          // lj_variants::ss, unshifted (PID's ss_ljs)
    real pid_cut = 0;
    ::vector<nat_ss> all_ss, cur_ss;
    std::vector<std::pair<int, int>> ss_sorted;

    nl::nl_data nl, nl_qa;
    bool invalid = true, first_time = true;
    real max_cutoff = 0, pad = 0, req_r = 0, max_form = 0;
    long rebuilds = 0;

    ::vector<pauli_pair> pauli_pairs;
    ::vector<es_pair> es_pairs;
    set<qa::free_pair> free_pairs;
    set<qa::candidate> candidates;
    set<qa::contact> contacts;
    ::vector<qa::sync_data> sync;
    ::vector<sink_lj> ss_shifted;
    real req_min_dist[qa::contact_type::NUM_TYPES];

    double V[XMD_NUM_TERMS];
};

void derive(xr_sys *s) {
    auto &p = s->p;
    real mc = 0;
    if (p.on[XMD_TERM_PAULI]) mc = std::max(mc, (real)p.pauli_r_excl);
    if (p.on[XMD_TERM_NAT_SS]) mc = std::max(mc, harmonic::cutoff((real)p.nat_ss_dist));   // main.cpp:596-597
    if (p.on[XMD_TERM_GO]) {
        real c = 0;
        for (int k = 0; k < s->all_nat_cont.size(); ++k)
            c = std::max(c, lj::cutoff(s->all_nat_cont[k].nat_dist()));
        mc = std::max(mc, c);
    }
    if (p.on[XMD_TERM_CONST_ES]) mc = std::max(mc, (real)(2.0 * p.const_es_screen_dist));
    if (p.on[XMD_TERM_REL_ES]) mc = std::max(mc, (real)(2.0 * p.rel_es_screen_dist));
    for (auto &x : s->req_min_dist) x = 0;
    s->req_min_dist[(short)qa::contact_type::BACK_BACK()] = p.lj_bb_r_min;
    s->req_min_dist[(short)qa::contact_type::BACK_SIDE()] = p.lj_bs_r_min;
    s->req_min_dist[(short)qa::contact_type::SIDE_BACK()] = p.lj_bs_r_min;
    for (auto const &aa1 : all_aa())
        for (auto const &aa2 : all_aa()) {
            int ss_idx = (int)aa1 * amino_acid::NUM_AA + (int)aa2;
            s->req_min_dist[(short)qa::contact_type::SIDE_SIDE(aa1, aa2)] = p.ss_r_max[ss_idx];
        }
    real mf = 0;
    for (int k = 0; k < qa::contact_type::NUM_TYPES; ++k) mf = std::max(mf, s->req_min_dist[k]);
    s->max_form = mf;
    if (p.on[XMD_TERM_QA]) mc = std::max(mc, mf);
    {
        // PID cutoff: main.cpp:801-810
        real c = std::max(lj::cutoff((real)p.lj_bb_r_min), lj::cutoff((real)p.lj_bs_r_min));
        for (int k = 0; k < XMD_NUM_SS; ++k) c = std::max(c, sink_lj::cutoff((real)p.ss_r_max[k]));
        s->pid_cut = c;
        if (p.on[XMD_TERM_PID]) mc = std::max(mc, c);
    }
    if (p.nl_cutoff > 0) mc = p.nl_cutoff;
    s->max_cutoff = mc;
    s->pad = p.nl_skin > 0 ? (real)p.nl_skin : (real)(p.pad_factor * mc);
    s->req_r = mc + s->pad;
}

// restated legacy_update::operator() (legacy_update.cpp:6-70) [D1-D3]
void legacy_update_restated(xr_sys *s) {
    s->nl.native_contacts.clear();
    s->nl.native_ssbonds.clear();
    s->nl.non_native.clear();
    size_t nat_idx = 0, ss_idx = 0;
    for (int i1 = 0; i1 < s->n; ++i1) {
        auto r1 = s->r[i1];
        auto chain1 = s->chain[i1], seq1 = s->seq[i1];
        for (int i2 = i1 + 1; i2 < s->n; ++i2) {
            auto r2 = s->r[i2];
            auto chain2 = s->chain[i2], seq2 = s->seq[i2];
            auto diff = seq1 > seq2 ? seq1 - seq2 : seq2 - seq1;
            if (chain1 == chain2 && diff < 3) continue;
            auto orig_dist = norm(s->bx.r_uv(r1, r2));
            if (orig_dist < s->req_r) {
                bool non_native = true;
                auto key = std::make_pair(i1, i2);
                // all_nat_cont is wired only when native contacts are enabled
                // (main.cpp:504-530); otherwise natives are ordinary pairs
                while (s->p.on[XMD_TERM_GO] && nat_idx < s->nat_sorted.size() && s->nat_sorted[nat_idx] < key) ++nat_idx;
                if (s->p.on[XMD_TERM_GO] && nat_idx < s->nat_sorted.size() && s->nat_sorted[nat_idx] == key) {
                    s->nl.native_contacts.emplace_back(i1, i2, orig_dist);
                    non_native = false;
                }
                // all_nat_ss is wired with native ssbonds enabled (main.cpp:579-580)
                while (s->p.on[XMD_TERM_NAT_SS] && ss_idx < s->ss_sorted.size() && s->ss_sorted[ss_idx] < key) ++ss_idx;
                if (s->p.on[XMD_TERM_NAT_SS] && ss_idx < s->ss_sorted.size() && s->ss_sorted[ss_idx] == key) {
                    s->nl.native_ssbonds.emplace_back(i1, i2, orig_dist);
                    non_native = false;
                }
                if (non_native) s->nl.non_native.emplace_back(i1, i2, orig_dist);
            }
        }
    }
    s->nl.orig_pad = s->pad;
    for (int i = 0; i < s->n; ++i) s->nl.orig_r[i] = s->r[i];
    s->nl.orig_box = s->bx;
    s->nl.ref_t = s->t;
    s->invalid = false;
    s->rebuilds++;
}

void rebuild_lists(xr_sys *s) {
    legacy_update_restated(s);
    auto &p = s->p;
    if (p.on[XMD_TERM_PAULI]) {
        update_pauli_pairs up;
        up.r_excl = p.pauli_r_excl;
        up.r = s->r.data();
        up.box = &s->bx;
        up.nl = &s->nl;
        up.pairs = &s->pauli_pairs;
        up();
    } else {
        s->pauli_pairs.clear();
    }
    if (p.on[XMD_TERM_PID]) {
        pid::update_pid_bundles ub;
        ub.cutoff = s->pid_cut;
        ub.r = s->r.data(); ub.prev = s->prev.data(); ub.next = s->next.data(); ub.atype = s->atype.data();
        ub.box = &s->bx; ub.nl = &s->nl; ub.bundles = &s->pid_bundles;
        ub();
    } else {
        s->pid_bundles.clear();
    }
    if (p.on[XMD_TERM_NAT_SS]) {
        update_nat_ssbonds us;
        us.cutoff = harmonic::cutoff((real)p.nat_ss_dist);   // never set by main.cpp:588-594 [D14]
        us.r = s->r.data();
        us.box = &s->bx;
        us.nl = &s->nl;
        us.all_ssbonds = &s->all_ss;
        us.ssbonds = &s->cur_ss;
        us();
    } else {
        s->cur_ss.clear();
    }
    // restated update_go_contacts::operator() (go.cpp:8-23) [D1]
    s->go_contacts.clear();
    if (p.on[XMD_TERM_GO]) {
        for (int idx = 0; idx < s->all_nat_cont.size(); ++idx) {
            auto nc = s->all_nat_cont.at(idx);
            auto cutoff = lj::cutoff(nc.nat_dist());
            auto r1 = s->r[nc.i1()], r2 = s->r[nc.i2()];
            if (norm(s->bx.r_uv(r1, r2)) < cutoff + s->nl.orig_pad)
                s->go_contacts.emplace_back(nc.i1(), nc.i2(), nc.nat_dist());
        }
    }
    if (p.on[XMD_TERM_CONST_ES] || p.on[XMD_TERM_REL_ES]) {
        update_es_base ue;
        ue.cutoff = p.on[XMD_TERM_CONST_ES] ? 2.0 * p.const_es_screen_dist
                                            : 2.0 * p.rel_es_screen_dist;
        for (auto const &aa : all_aa()) ue.q[(short)aa] = p.charge[(int)aa];
        ue.r = s->r.data();
        ue.box = &s->bx;
        ue.nl = &s->nl;
        ue.pairs = &s->es_pairs;
        ue.atype = s->atype.data();
        ue();
    } else {
        s->es_pairs.clear();
    }
    if (p.on[XMD_TERM_QA]) {
        // [D5]: the list handed to update_free_pairs omits pairs in contact
        std::set<std::pair<int, int>> live;
        for (int k = 0; k < s->contacts.extent(); ++k) {
            auto node = s->contacts.at(k);
            if (node.vacant()) continue;
            live.insert({node.value().i1(), node.value().i2()});
        }
        s->nl_qa.orig_pad = s->nl.orig_pad;
        s->nl_qa.non_native.clear();
        for (int k = 0; k < s->nl.non_native.size(); ++k) {
            auto pr = s->nl.non_native[k];
            if (live.count({pr.i1(), pr.i2()})) continue;
            s->nl_qa.non_native.emplace_back(pr.i1(), pr.i2(), pr.orig_dist());
        }
        qa::update_free_pairs uf;
        uf.max_formation_min_dist = s->max_form;
        uf.r = s->r.data();
        uf.box = &s->bx;
        uf.nl = &s->nl_qa;
        uf.pairs = &s->free_pairs;
        uf();
    }
}

void verify_and_rebuild(xr_sys *s) {
    nl::verify vf;
    vf.r = s->r.data();
    vf.box = &s->bx;
    vf.invalid = &s->invalid;
    vf.first_time = &s->first_time;
    vf.num_particles = s->n;
    vf.data = &s->nl;
    vf();
    if (s->invalid) rebuild_lists(s);
}

lj_variants make_ljs(xr_sys *s) {
    // lj_variants::operator[] counts BB from 0; contact_type counts it from 1.
    // Shift the table by one so ljs[type] is the potential of `type` [D6].
    auto &p = s->p;
    lj_variants ljs;
    ljs.bb = lj(p.lj_bb_depth, p.lj_bb_r_min);     // type 0 (NONE): never used
    ljs.bs = lj(p.lj_bb_depth, p.lj_bb_r_min);     // type 1: BACK_BACK -> bb
    ljs.sb = lj(p.lj_bs_depth, p.lj_bs_r_min);     // type 2: BACK_SIDE -> bs
    s->ss_shifted.clear();
    s->ss_shifted.emplace_back(p.lj_bs_depth, p.lj_bs_r_min, p.lj_bs_r_min);  // type 3: SIDE_BACK -> sb
    for (int k = 0; k < XMD_NUM_SS; ++k) {
        real r_max = p.ss_r_max[k];
        real r_min = p.ss_sinking ? (real)p.lj_bb_r_min : r_max;
        s->ss_shifted.emplace_back((real)p.ss_depth[k], r_min, r_max);
    }
    ljs.ss = s->ss_shifted.view();
    return ljs;
}

void term_forces(xr_sys *s, ::vector<vec3r> &F, real *V) {
    auto &p = s->p;
    for (int i = 0; i < s->n; ++i) F[i] = vec3r::Zero();
    for (int k = 0; k < XMD_NUM_TERMS; ++k) V[k] = 0;
    if (p.on[XMD_TERM_TETHER]) {
        eval_tether_forces e;
        e.H1 = p.tether_H1; e.H2 = p.tether_H2; e.def_length = p.tether_def_length;
        e.r = s->r.data(); e.F = F.data(); e.tethers = s->tethers.view(); e.V = &V[XMD_TERM_TETHER];
        e();
    }
    if (p.on[XMD_TERM_NAT_ANG]) {
        eval_native_angle_forces e;
        e.k = p.nat_ang_k;
        e.r = s->r.data(); e.F = F.data(); e.angles = s->angles.view(); e.V = &V[XMD_TERM_NAT_ANG];
        e();
    }
    if (p.on[XMD_TERM_CND]) {
        eval_cnd_forces e;
        e.CDA = p.cnd_CDA; e.CDB = p.cnd_CDB;
        e.r = s->r.data(); e.F = F.data(); e.dihedrals = s->dihedrals.view(); e.V = &V[XMD_TERM_CND];
        e();
    }
    if (p.on[XMD_TERM_SND]) {
        eval_snd_forces e;
        e.CDH = p.snd_CDH;
        e.r = s->r.data(); e.F = F.data(); e.dihedrals = s->dihedrals.view(); e.V = &V[XMD_TERM_SND];
        e();
    }
    if (p.on[XMD_TERM_PAULI]) {
        eval_pauli_exclusion_forces e;
        e.depth = p.pauli_depth; e.r_excl = p.pauli_r_excl;
        e.r = s->r.data(); e.F = F.data(); e.box = &s->bx; e.pairs = &s->pauli_pairs; e.V = &V[XMD_TERM_PAULI];
        e();
    }
    if (p.on[XMD_TERM_GO]) {
        eval_go_forces e;
        e.depth = p.go_depth;
        e.r = s->r.data(); e.F = F.data(); e.box = &s->bx; e.contacts = &s->go_contacts; e.V = &V[XMD_TERM_GO];
        e();
    }
    if (p.on[XMD_TERM_CONST_ES]) {
        eval_const_es_forces e;
        e.permittivity = p.const_es_permittivity;
        e.V_factor = 1.0 / (4.0 * M_PI * e.permittivity);
        e.screen_dist_inv = 1.0 / p.const_es_screen_dist;
        e.r = s->r.data(); e.F = F.data(); e.box = &s->bx; e.es_pairs = &s->es_pairs; e.V = &V[XMD_TERM_CONST_ES];
        e();
    }
    if (p.on[XMD_TERM_REL_ES]) {
        eval_relative_es_forces e;
        e.factor = p.rel_es_factor;
        e.V_factor = 1.0 / (4.0 * M_PI * e.factor);
        e.screen_dist_inv = 1.0 / p.rel_es_screen_dist;
        e.r = s->r.data(); e.F = F.data(); e.box = &s->bx; e.es_pairs = &s->es_pairs; e.V = &V[XMD_TERM_REL_ES];
        e();
    }
    if (p.on[XMD_TERM_CHIR]) {
        eval_chiral_forces e;
        e.e_chi = p.chir_e_chi;
        e.r = s->r.data(); e.F = F.data(); e.quads = s->quads.view(); e.V = &V[XMD_TERM_CHIR];
        e();
    }
    if (p.on[XMD_TERM_HEUR_ANG]) {
        // main.cpp builds no heuristic term; the kernel gets all 7 table
        // coefficients (freeform/params.cpp:77-80 reads a0..a5 only) [D17]
        eval_heurestic_angle_forces e;
        for (int d = 0; d <= eval_heurestic_angle_forces::POLY_DEG; ++d)
            for (int t = 0; t < eval_heurestic_angle_forces::NUM_TYPES; ++t)
                e.poly_coeffs[d][t] = (real)p.heur_ang_coeffs[t][d];
        e.r = s->r.data(); e.F = F.data(); e.angles = s->heur_angles.view(); e.V = &V[XMD_TERM_HEUR_ANG];
        e();
    }
    if (p.on[XMD_TERM_HEUR_DIH]) {
        // the shipped kernel as it is: phi = cos(cos_phi) and +2 c4 sin cos
        // (dihedral/heurestic.cpp:43, 52-54); the restatement departs [D18]
        eval_heurestic_dihedral_forces e;
        for (int k = 0; k < eval_heurestic_dihedral_forces::NUM_TERMS; ++k)
            for (int t = 0; t < eval_heurestic_dihedral_forces::NUM_TYPES; ++t)
                e.coeffs[k][t] = (real)p.heur_dih_coeffs[t][k];
        e.r = s->r.data(); e.F = F.data(); e.dihedrals = s->heur_dihedrals.view(); e.V = &V[XMD_TERM_HEUR_DIH];
        e();
    }
    if (p.on[XMD_TERM_VEL_AFM]) {
        // afm_force's nat_r is never set (main.cpp:876-879): a zero-length spring [D21]
        eval_velocity_afm_forces e;
        e.afm_force = harmonic((real)p.vel_afm_H1, (real)p.vel_afm_H2, (real)0.0);
        e.r = s->r.data(); e.F = F.data(); e.t = &s->t; e.afm_tips = s->vafm.view();
        e();
    }
    if (p.on[XMD_TERM_FORCE_AFM]) {
        eval_force_afm_forces e;
        e.F = F.data(); e.afm_tips = s->fafm.view();
        e();
    }
    if (p.on[XMD_TERM_PID]) {
        // the shipped kernel leaves dpsi2_* unset (eval_forces.cpp:64-98),
        // so its forces are not compared; its energy is
        pid::eval_pid_forces e;
        auto lv = p.pid_lambda == 1 ? pid::lambda_version::ALGEBRAIC : pid::lambda_version::COSINE;
        e.bb_plus_lam.version() = lv; e.bb_minus_lam.version() = lv; e.ss_lam.version() = lv;
        e.bb_plus_lam.alpha() = p.pid_bbp[0]; e.bb_plus_lam.psi_0() = p.pid_bbp[1];
        e.bb_plus_lj.r_min() = p.pid_bbp[2]; e.bb_plus_lj.depth() = p.pid_bbp[3];
        e.bb_minus_lam.alpha() = p.pid_bbm[0]; e.bb_minus_lam.psi_0() = p.pid_bbm[1];
        e.bb_minus_lj.r_min() = p.pid_bbm[2]; e.bb_minus_lj.depth() = p.pid_bbm[3];
        e.ss_lam.alpha() = p.pid_ss[0]; e.ss_lam.psi_0() = p.pid_ss[1];
        s->ss_plain.clear();
        for (int k = 0; k < XMD_NUM_SS; ++k) {
            real r_max = p.ss_r_max[k];
            real r_min = p.ss_sinking ? (real)p.lj_bb_r_min : r_max;
            s->ss_plain.emplace_back((real)p.ss_depth[k], r_min, r_max);
        }
        e.ss_ljs = s->ss_plain.data();
        ::vector<vec3r> Fd(s->n, vec3r(0, 0, 0));
        e.r = s->r.data(); e.F = Fd.data(); e.box = &s->bx; e.bundles = &s->pid_bundles;
        e.prev = s->prev.data(); e.next = s->next.data(); e.V = &V[XMD_TERM_PID];
        e();
    }
    if (p.on[XMD_TERM_SOLID_WALL]) {
        eval_solid_wall_forces e;
        e.eps = p.solid_wall_depth; e.cutoff = p.solid_wall_cutoff;
        e.r = s->r.data(); e.F = F.data(); e.wall_F = s->wall_F[0].data(); e.box = &s->bx;
        e.walls = s->walls[0].view(); e.V = &V[XMD_TERM_SOLID_WALL]; e.num_particles = s->n;
        e();
    }
    if (p.on[XMD_TERM_LJ_WALL]) {
        // lj_depth is never set by main.cpp:836-843: `depth` [D22]; one state
        // per (wall, bead), wall-major (main.cpp:848-854)
        eval_lj_attr_wall_forces e;
        e.wall_min_dist = p.lj_wall_min_dist; e.lj_depth = p.lj_wall_depth;
        e.cycle_time = p.lj_wall_phase_duration; e.cycle_time_inv = 1.0 / e.cycle_time;
        e.breaking_factor = p.lj_wall_breaking_factor; e.factor = e.breaking_factor * pow(2.0, -1.0 / 6.0);
        e.r = s->r.data(); e.F = F.data(); e.wall_F = s->wall_F[1].data(); e.box = &s->bx;
        e.walls = s->walls[1].view(); e.V = &V[XMD_TERM_LJ_WALL]; e.t = &s->t; e.num_particles = s->n;
        e.pairs = s->ljw_pairs.view();
        e();
    }
    if (p.on[XMD_TERM_NAT_SS]) {
        eval_nat_ssbond_forces e;
        e.H1 = p.nat_ss_H1; e.nat_r = p.nat_ss_dist;
        e.r = s->r.data(); e.F = F.data(); e.box = &s->bx; e.ssbonds = &s->cur_ss; e.V = &V[XMD_TERM_NAT_SS];
        e();
    }
}

void setup_proc_contacts(xr_sys *s, qa::process_contacts &pc, ::vector<vec3r> &F, real *V,
                         set<qa::contact> *contacts, ::vector<qa::sync_data> *sync,
                         set<qa::free_pair> *free_pairs) {
    auto &p = s->p;
    pc.ljs = make_ljs(s);
    pc.cycle_time = p.qa_phase_duration;
    pc.cycle_time_inv = 1.0 / pc.cycle_time;
    pc.breaking_factor = p.qa_breaking_factor;
    pc.factor = pc.breaking_factor * (real)pow(2.0f, -1.0f / 6.0f);   // main.cpp:719-723
    pc.r = s->r.data();
    pc.F = F.data();
    pc.box = &s->bx;
    pc.contacts = contacts;
    pc.V = V;
    pc.t = &s->t;
    pc.sync = sync->data();
    pc.free_pairs = free_pairs;
}

void qa_full(xr_sys *s, ::vector<vec3r> &F, real *V) {
    auto &p = s->p;
    qa::precompute_nh nh;
    nh.r = s->r.data(); nh.n = s->n_.data(); nh.h = s->h_.data(); nh.box = &s->bx;
    nh.prev = s->prev.data(); nh.next = s->next.data(); nh.num_particles = s->n;
    nh();
    qa::sift_candidates sc;
    sc.min_abs_cos_hr = p.qa_min_cos_hr;
    sc.min_abs_cos_hh = p.qa_min_cos_hh;
    sc.max_cos_nr = p.qa_max_cos_nr;
    for (int k = 0; k < qa::contact_type::NUM_TYPES; ++k) sc.req_min_dist[k] = s->req_min_dist[k];
    for (auto const &aa : all_aa())
        sc.ptype[(short)aa] = (polarization_type)p.polarization[(int)aa];
    sc.r = s->r.data(); sc.n = s->n_.data(); sc.h = s->h_.data(); sc.box = &s->bx;
    sc.atype = s->atype.data(); sc.sync = s->sync.data();
    sc.free_pairs = &s->free_pairs; sc.candidates = &s->candidates;
    sc();
    qa::process_candidates pcand;
    pcand.candidates = &s->candidates; pcand.sync = s->sync.data(); pcand.t = &s->t;
    pcand.contacts = &s->contacts; pcand.free_pairs = &s->free_pairs;
    pcand();
    qa::process_contacts pc;
    setup_proc_contacts(s, pc, F, &V[XMD_TERM_QA], &s->contacts, &s->sync, &s->free_pairs);
    pc();
}
}  // namespace

extern "C" {
typedef struct xr_sys_opaque xr_handle;

void *xr_create(const xmd_params *p, int32_t n, const int32_t *chain_idx, const int32_t *seq_idx,
                const uint8_t *atype, const double cell[3], double temperature, uint64_t seed) {
    auto *s = new xr_sys();
    s->p = *p;
    s->n = n;
    s->bx.set_cell(vec3r(cell[0], cell[1], cell[2]));
    s->gen = rand_gen(seed);
    s->temperature = temperature > 0 ? temperature : p->temperature;
    s->r = ::vector<vec3r>(n);
    s->v = ::vector<vec3r>(n);
    s->F = ::vector<vec3r>(n);
    s->n_ = ::vector<vec3r>(n);
    s->h_ = ::vector<vec3r>(n);
    s->y0 = ::vector<vec3tr>(n); s->y1 = ::vector<vec3tr>(n); s->y2 = ::vector<vec3tr>(n);
    s->y3 = ::vector<vec3tr>(n); s->y4 = ::vector<vec3tr>(n); s->y5 = ::vector<vec3tr>(n);
    s->mass = ::vector<real>(n, (real)1.0);       // main.cpp:156
    s->mass_inv = ::vector<real>(n, (real)1.0);
    s->mass_rsqrt = ::vector<real>(n, (real)1.0);
    s->chain = ::vector<int>(n); s->seq = ::vector<int>(n);
    s->prev = ::vector<int>(n, -1); s->next = ::vector<int>(n, -1);
    s->atype = ::vector<amino_acid>(n);
    for (int i = 0; i < n; ++i) {
        s->chain[i] = chain_idx[i];
        s->seq[i] = seq_idx[i];
        s->atype[i] = amino_acid((aa_code)atype[i]);
        if (i > 0 && chain_idx[i - 1] == chain_idx[i] && seq_idx[i - 1] == seq_idx[i] - 1) s->prev[i] = i - 1;
        if (i + 1 < n && chain_idx[i + 1] == chain_idx[i] && seq_idx[i + 1] == seq_idx[i] + 1) s->next[i] = i + 1;
    }
    s->nl.orig_r = ::vector<vec3r>(n);
    for (int i = 0; i < n; ++i) {                                 // [D4]
        int a = atype[i];
        s->sync.emplace_back((int8_t)p->limits[a][0], (int8_t)p->limits[a][1],
                             (int8_t)p->limits[a][2], (int8_t)p->limits[a][3]);
    }
    derive(s);
    return s;
}
void xr_destroy(void *h) { delete (xr_sys *)h; }

int xr_set_tethers(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const double *d) {
    auto *s = (xr_sys *)h;
    s->tethers.clear();
    for (int k = 0; k < n; ++k)
        s->tethers.emplace_back(i1[k], i2[k], (real)((d && d[k] > 0) ? d[k] : s->p.tether_def_length));
    return 0;
}
int xr_set_angles(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                  const double *th) {
    auto *s = (xr_sys *)h;
    s->angles.clear();
    for (int k = 0; k < n; ++k) s->angles.emplace_back(i1[k], i2[k], i3[k], (real)th[k]);
    return 0;
}
int xr_set_dihedrals(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                     const int32_t *i4, const double *ph) {
    auto *s = (xr_sys *)h;
    s->dihedrals.clear();
    for (int k = 0; k < n; ++k) s->dihedrals.emplace_back(i1[k], i2[k], i3[k], i4[k], (real)ph[k]);
    return 0;
}
// chiral quads by field name (main.cpp:391 passes nat_factor where the
// gentype's fifth field is nat_chir, chiral.h:9 [D15])
int xr_set_chirals(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3, const int32_t *i4,
                   const double *nat_factor, const double *nat_chir) {
    auto *s = (xr_sys *)h;
    s->quads.clear();
    for (int k = 0; k < n; ++k) s->quads.emplace_back(i1[k], i2[k], i3[k], i4[k], (real)nat_chir[k], (real)nat_factor[k]);
    return 0;
}
// heuristic angle and dihedral types from the residues (heur_ang_type(a1, a2)
// of the angle's i1, i2; heur_dih_type(a2, a3) of the dihedral's i2, i3)
int xr_set_heuristic_angles(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3) {
    auto *s = (xr_sys *)h;
    s->heur_angles.clear();
    for (int k = 0; k < n; ++k)
        s->heur_angles.emplace_back(i1[k], i2[k], i3[k], heur_ang_type(s->atype[i1[k]], s->atype[i2[k]]));
    return 0;
}
int xr_set_heuristic_dihedrals(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const int32_t *i3,
                               const int32_t *i4) {
    auto *s = (xr_sys *)h;
    s->heur_dihedrals.clear();
    for (int k = 0; k < n; ++k)
        s->heur_dihedrals.emplace_back(i1[k], i2[k], i3[k], i4[k], heur_dih_type(s->atype[i2[k]], s->atype[i3[k]]));
    return 0;
}
// model::morph_into_saw (model.cpp:101-173) on chains of the given lengths
// (positions zero, as seq_file leaves them), with rand_gen(seed); writes the
// positions in residue order and the generator's state afterwards.
// bond <= 0: the optional bond length is absent.
int xr_morph_into_saw(int32_t nchains, const int32_t *lens, double bond, double density, int32_t infer_box,
                      uint64_t seed, double *r_out, uint64_t *state_out, double *cell_out) {
    xmd::model m;
    for (int c = 0; c < nchains; ++c) {
        auto &ch = m.chains.emplace_back(std::make_unique<xmd::model::chain>());
        ch->residues.resize(lens[c]);
        for (int k = 0; k < lens[c]; ++k) {
            auto &res = m.residues.emplace_back(std::make_unique<xmd::model::residue>());
            res->seq_idx = k;
            res->parent = &*ch;
            res->type = amino_acid(GLY);
            res->pos = {0.0, 0.0, 0.0};
            ch->residues[k] = &*res;
        }
    }
    xmd::rand_gen gen(seed);
    std::optional<true_real> bl;
    if (bond > 0) bl = bond;
    m.morph_into_saw(gen, bl, density, infer_box != 0);
    size_t q = 0;
    for (auto const &res : m.residues) {
        r_out[3 * q] = res->pos.x(); r_out[3 * q + 1] = res->pos.y(); r_out[3 * q + 2] = res->pos.z();
        ++q;
    }
    *state_out = gen.state;
    if (cell_out) {
        cell_out[0] = m.model_box.cell.x(); cell_out[1] = m.model_box.cell.y(); cell_out[2] = m.model_box.cell.z();
    }
    return 0;
}
int xr_set_velocity_afm(void *h, int32_t n, const int32_t *bead, const double *orig, const double *vel) {
    auto *s = (xr_sys *)h;
    s->vafm.clear();
    for (int k = 0; k < n; ++k)
        s->vafm.emplace_back(bead[k], vec3r(orig[3 * k], orig[3 * k + 1], orig[3 * k + 2]),
                             vec3r(vel[3 * k], vel[3 * k + 1], vel[3 * k + 2]));
    return 0;
}
int xr_set_force_afm(void *h, int32_t n, const int32_t *bead, const double *F) {
    auto *s = (xr_sys *)h;
    s->fafm.clear();
    for (int k = 0; k < n; ++k) s->fafm.emplace_back(bead[k], vec3r(F[3 * k], F[3 * k + 1], F[3 * k + 2]));
    return 0;
}
int xr_set_walls(void *h, int32_t kind, int32_t n, const double *origin, const double *normal) {
    auto *s = (xr_sys *)h;
    if (kind < 0 || kind > 1) return -1;
    s->walls[kind].clear();
    for (int k = 0; k < n; ++k)
        s->walls[kind].emplace_back(vec3r(origin[3 * k], origin[3 * k + 1], origin[3 * k + 2]),
                                    vec3r(normal[3 * k], normal[3 * k + 1], normal[3 * k + 2]));
    s->wall_F[kind].clear();
    for (int k = 0; k < std::max(n, 1); ++k) s->wall_F[kind].emplace_back(0, 0, 0);
    if (kind == 1) {
        s->ljw_pairs.clear();
        for (int w = 0; w < n; ++w)
            for (int i = 0; i < s->n; ++i) s->ljw_pairs.emplace_back(i, w, FREE, vec3r(0, 0, 0), (real)0);
    }
    return 0;
}
int xr_set_ssbonds(void *h, int32_t n, const int32_t *i1, const int32_t *i2) {
    auto *s = (xr_sys *)h;
    std::vector<std::pair<int, int>> v;
    for (int k = 0; k < n; ++k) v.emplace_back(std::min(i1[k], i2[k]), std::max(i1[k], i2[k]));
    std::sort(v.begin(), v.end());
    s->all_ss.clear();
    s->ss_sorted = v;
    for (auto &[a, b] : v) s->all_ss.emplace_back(a, b);
    s->first_time = true;
    return 0;
}
int xr_set_native_contacts(void *h, int32_t n, const int32_t *i1, const int32_t *i2, const double *d) {
    auto *s = (xr_sys *)h;
    std::vector<std::tuple<int, int, double>> v;
    for (int k = 0; k < n; ++k) v.emplace_back(std::min(i1[k], i2[k]), std::max(i1[k], i2[k]), d[k]);
    std::sort(v.begin(), v.end());
    s->all_nat_cont.clear();
    s->nat_sorted.clear();
    for (auto &[a, b, dd] : v) {
        s->all_nat_cont.emplace_back(a, b, (real)dd);
        s->nat_sorted.emplace_back(a, b);
    }
    derive(s);
    s->first_time = true;
    return 0;
}
int xr_set_state(void *h, const double *r, const double *v) {
    auto *s = (xr_sys *)h;
    for (int i = 0; i < s->n; ++i) {
        s->r[i] = vec3r(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
        s->v[i] = v ? vec3r(v[3 * i], v[3 * i + 1], v[3 * i + 2]) : vec3r();
        s->y0[i] = vec3tr(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
        s->y1[i] = vec3tr(s->v[i].x() * s->p.dt, s->v[i].y() * s->p.dt, s->v[i].z() * s->p.dt);
        s->y2[i] = s->y3[i] = s->y4[i] = s->y5[i] = vec3tr();
    }
    s->t = 0;
    s->true_t = 0;
    s->first_time = true;
    return 0;
}
int xr_set_history(void *h, const double *y, double t, uint64_t rng_state) {
    auto *s = (xr_sys *)h;
    size_t n3 = 3 * (size_t)s->n;
    ::vector<vec3tr> *ys[6] = {&s->y0, &s->y1, &s->y2, &s->y3, &s->y4, &s->y5};
    for (int k = 0; k < 6; ++k)
        for (int i = 0; i < s->n; ++i)
            (*ys[k])[i] = vec3tr(y[k * n3 + 3 * i], y[k * n3 + 3 * i + 1], y[k * n3 + 3 * i + 2]);
    for (int i = 0; i < s->n; ++i) {
        s->r[i] = s->y0[i];
        vec3tr vv = s->y1[i];
        s->v[i] = vec3r(vv.x() * (1.0 / s->p.dt), vv.y() * (1.0 / s->p.dt), vv.z() * (1.0 / s->p.dt));
    }
    s->t = t;
    s->true_t = t;
    s->gen.state = rng_state;
    s->first_time = true;
    return 0;
}
int xr_get_state(void *h, double *r, double *v, double *t) {
    auto *s = (xr_sys *)h;
    for (int i = 0; i < s->n; ++i) {
        if (r) { r[3 * i] = s->r[i].x(); r[3 * i + 1] = s->r[i].y(); r[3 * i + 2] = s->r[i].z(); }
        if (v) { v[3 * i] = s->v[i].x(); v[3 * i + 1] = s->v[i].y(); v[3 * i + 2] = s->v[i].z(); }
    }
    if (t) *t = s->t;
    return 0;
}
int xr_get_history(void *h, double *y, double *t, uint64_t *rng_state) {
    auto *s = (xr_sys *)h;
    size_t n3 = 3 * (size_t)s->n;
    ::vector<vec3tr> *ys[6] = {&s->y0, &s->y1, &s->y2, &s->y3, &s->y4, &s->y5};
    if (y)
        for (int k = 0; k < 6; ++k)
            for (int i = 0; i < s->n; ++i) {
                vec3tr q = (*ys[k])[i];
                y[k * n3 + 3 * i] = q.x(); y[k * n3 + 3 * i + 1] = q.y(); y[k * n3 + 3 * i + 2] = q.z();
            }
    if (t) *t = s->t;
    if (rng_state) *rng_state = s->gen.state;
    return 0;
}

int xr_eval_forces(void *h, double *F, double *V) {
    auto *s = (xr_sys *)h;
    if (s->first_time) verify_and_rebuild(s);
    real Vl[XMD_NUM_TERMS];
    term_forces(s, s->F, Vl);
    if (s->p.on[XMD_TERM_QA]) {
        // force of the current contacts; transitions go to throw-away copies
        set<qa::contact> cc = s->contacts;
        ::vector<qa::sync_data> sy = s->sync;
        set<qa::free_pair> fp = s->free_pairs;
        qa::process_contacts pc;
        setup_proc_contacts(s, pc, s->F, &Vl[XMD_TERM_QA], &cc, &sy, &fp);
        pc();
    }
    for (int i = 0; i < s->n; ++i) {
        if (F) { F[3 * i] = s->F[i].x(); F[3 * i + 1] = s->F[i].y(); F[3 * i + 2] = s->F[i].z(); }
    }
    if (V) for (int k = 0; k < XMD_NUM_TERMS; ++k) V[k] = Vl[k];
    return 0;
}

int xr_step(void *h, int32_t nsteps) {
    auto *s = (xr_sys *)h;
    if (s->first_time) verify_and_rebuild(s);
    lang_pc_step lp;
    lp.gamma_factor = s->p.gamma_factor;
    lp.temperature = s->temperature;
    lp.dt = s->p.dt;                                             // [D8]
    lp.r = s->r.data(); lp.v = s->v.data(); lp.F = s->F.data();
    lp.mass = s->mass.data(); lp.mass_inv = s->mass_inv.data(); lp.mass_rsqrt = s->mass_rsqrt.data();
    lp.t = &s->t;
    lp.y0 = s->y0.data(); lp.y1 = s->y1.data(); lp.y2 = s->y2.data();
    lp.y3 = s->y3.data(); lp.y4 = s->y4.data(); lp.y5 = s->y5.data();
    lp.true_t = &s->true_t;
    lp.num_particles = s->n;
    lp.gen = &s->gen;
    for (int k = 0; k < nsteps; ++k) {
        real V[XMD_NUM_TERMS];
        term_forces(s, s->F, V);
        if (s->p.on[XMD_TERM_QA]) {
            s->candidates.clear();                                 // sift omp_prep
            qa_full(s, s->F, V);
        }
        if (s->p.langevin_on) lp();
        verify_and_rebuild(s);
    }
    return 0;
}

int xr_counts(void *h, int64_t *c) {
    auto *s = (xr_sys *)h;
    int64_t live_fp = 0, live_c = 0;
    for (int k = 0; k < s->free_pairs.extent(); ++k) live_fp += !s->free_pairs.at(k).vacant();
    for (int k = 0; k < s->contacts.extent(); ++k) live_c += !s->contacts.at(k).vacant();
    c[0] = s->go_contacts.size(); c[1] = s->pauli_pairs.size(); c[2] = s->es_pairs.size();
    c[3] = live_fp; c[4] = s->free_pairs.extent(); c[5] = live_c; c[6] = s->contacts.extent();
    c[7] = s->rebuilds;
    return 0;
}
int xr_qa_contacts(void *h, int32_t cap, int32_t *out4, double *ref_time) {
    auto *s = (xr_sys *)h;
    int32_t m = 0;
    for (int k = 0; k < s->contacts.extent(); ++k) {
        auto node = s->contacts.at(k);
        if (node.vacant()) continue;
        auto c = node.value();
        if (m < cap) {
            out4[4 * m] = c.i1(); out4[4 * m + 1] = c.i2();
            out4[4 * m + 2] = (int16_t)c.type(); out4[4 * m + 3] = (int)c.status();
            if (ref_time) ref_time[m] = c.ref_time();
        }
        ++m;
    }
    return m;
}
int xr_nl_pairs(void *h, int64_t cap, int32_t *out2) {
    auto *s = (xr_sys *)h;
    for (int64_t k = 0; k < s->nl.non_native.size() && k < cap; ++k) {
        out2[2 * k] = s->nl.non_native[k].i1();
        out2[2 * k + 1] = s->nl.non_native[k].i2();
    }
    return s->nl.non_native.size();
}
int xr_sync(void *h, int8_t *out) {
    auto *s = (xr_sys *)h;
    for (int i = 0; i < s->n; ++i) {
        auto q = s->sync[i];
        out[4 * i] = q.back(); out[4 * i + 1] = q.side_all();
        out[4 * i + 2] = q.side_polar(); out[4 * i + 3] = q.side_hydrophobic();
    }
    return 0;
}
int xr_cutoffs(void *h, double *out3) {
    auto *s = (xr_sys *)h;
    out3[0] = s->max_cutoff; out3[1] = s->pad; out3[2] = s->req_r;
    return 0;
}
// reference generator, for pinning the restated stream (rand_gen.h:22-58)
uint64_t xr_rng_next(uint64_t *state) {
    rand_gen g(*state);
    auto v = g();
    *state = g.state;
    return v;
}
double xr_rng_normal(uint64_t *state) {
    rand_gen g(*state);
    auto v = g.normal<real>();
    *state = g.state;
    return v;
}
}
