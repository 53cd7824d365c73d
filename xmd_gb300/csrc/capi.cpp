// capi.cpp - the extern "C" boundary (include/xmd_gpu.h).  No exception
// crosses it: every failure becomes a status code plus a thread-local message.
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <memory>
#include <algorithm>

#include "../../include/xmd_gpu.h"
#include "config.h"
#include "engine.h"
#include "server.h"

struct xmd_gpu_ctx {
    xmdg::Engine *eng = nullptr;
};
struct xmd_gpu_server {
    xmdg::Server *srv = nullptr;
};

namespace {
int fail(int code, const std::string &msg) {
    xmdg::last_error() = msg;
    return code;
}
template <class F>
int guard(F &&f) {
    try {
        f();
        xmdg::last_error().clear();
        return XMD_OK;
    } catch (std::length_error &e) {
        return fail(XMD_ERR_CAPACITY, e.what());
    } catch (std::domain_error &e) {
        return fail(XMD_ERR_NUMERIC, e.what());
    } catch (std::invalid_argument &e) {
        return fail(XMD_ERR_ARG, e.what());
    } catch (std::logic_error &e) {
        return fail(XMD_ERR_STATE, e.what());
    } catch (std::runtime_error &e) {
        std::string m = e.what();
        if (m.rfind("CUDA", 0) == 0 || m.find("CUDA device") != std::string::npos)
            return fail(XMD_ERR_CUDA, m);
        return fail(XMD_ERR_CONFIG, m);
    } catch (std::exception &e) {
        return fail(XMD_ERR_STATE, e.what());
    } catch (...) {
        return fail(XMD_ERR_STATE, "unknown error");
    }
}
#define NEED_CTX                                                          \
    if (!ctx || !ctx->eng) return fail(XMD_ERR_ARG, "null context");
}  // namespace

extern "C" {

int xmd_gpu_abi_version(void) { return XMD_GPU_ABI_VERSION; }

int xmd_gpu_params_size(void) { return (int)sizeof(xmd_params); }

uint64_t xmd_gpu_rng_jump(uint64_t state, uint64_t n_draws) { return xmdg::rng_jump(state, n_draws); }

const char *xmd_gpu_last_error(void) { return xmdg::last_error().c_str(); }

int xmd_gpu_parse_params(const char *yaml_text, xmd_params *out) {
    if (!out) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { xmdg::params_from_yaml(yaml_text ? yaml_text : "", out); });
}

int xmd_gpu_create(const char *yaml_text, xmd_gpu_ctx **out) {
    if (!out) return fail(XMD_ERR_ARG, "null output");
    *out = nullptr;
    xmd_params p;
    int rc = guard([&] { xmdg::params_from_yaml(yaml_text ? yaml_text : "", &p); });
    if (rc) return rc;
    return guard([&] {
        auto *c = new xmd_gpu_ctx;
        try {
            c->eng = new xmdg::Engine(p);
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

int xmd_gpu_create_from_file(const char *yaml_path, xmd_gpu_ctx **out) {
    if (!yaml_path) return fail(XMD_ERR_ARG, "null path");
    std::ifstream in(yaml_path);
    if (!in) return fail(XMD_ERR_CONFIG, std::string("cannot open ") + yaml_path);
    std::stringstream ss;
    ss << in.rdbuf();
    return xmd_gpu_create(ss.str().c_str(), out);
}

int xmd_gpu_destroy(xmd_gpu_ctx *ctx) {
    if (!ctx) return XMD_OK;
    int rc = guard([&] { delete ctx->eng; });
    delete ctx;
    return rc;
}

int xmd_gpu_get_params(const xmd_gpu_ctx *ctx, xmd_params *out) {
    NEED_CTX;
    if (!out) return fail(XMD_ERR_ARG, "null output");
    *out = ctx->eng->params;
    return XMD_OK;
}

int xmd_gpu_set_params(xmd_gpu_ctx *ctx, const xmd_params *p) {
    NEED_CTX;
    if (!p) return fail(XMD_ERR_ARG, "null params");
    if (ctx->eng->finalized || !ctx->eng->reps.empty())
        return fail(XMD_ERR_STATE, "parameters are fixed once replicas exist");
    ctx->eng->params = *p;
    return XMD_OK;
}

int xmd_gpu_enable_term(xmd_gpu_ctx *ctx, int term, int on) {
    NEED_CTX;
    if (term < 0 || term >= XMD_NUM_TERMS) return fail(XMD_ERR_ARG, "term out of range");
    if (ctx->eng->finalized) return fail(XMD_ERR_STATE, "terms are fixed after the first eval/step");
    ctx->eng->params.on[term] = on ? 1 : 0;
    return XMD_OK;
}

int xmd_gpu_set_precision(xmd_gpu_ctx *ctx, int precision) {
    NEED_CTX;
    if (precision != XMD_PREC_FP64 && precision != XMD_PREC_MIXED) return fail(XMD_ERR_ARG, "bad precision");
    ctx->eng->params.precision = precision;
    return XMD_OK;
}

int xmd_gpu_add_replica(xmd_gpu_ctx *ctx, int32_t n, const int32_t *chain_idx, const int32_t *seq_idx,
                        const uint8_t *atype, const double cell[3], double temperature, uint64_t seed,
                        int32_t *replica_id) {
    NEED_CTX;
    return guard([&] {
        int id = ctx->eng->add_replica(n, chain_idx, seq_idx, atype, cell, temperature, seed);
        if (replica_id) *replica_id = id;
    });
}

int xmd_gpu_set_tethers(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2,
                        const double *nat_dist) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2))) return fail(XMD_ERR_ARG, "bad tether arrays");
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_tethers(rep, n, i1, i2, nat_dist); });
}

int xmd_gpu_set_angles(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2,
                       const int32_t *i3, const double *nat_theta) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2 || !i3 || !nat_theta))) return fail(XMD_ERR_ARG, "bad angle arrays");
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_angles(rep, n, i1, i2, i3, nat_theta); });
}

int xmd_gpu_set_chirals(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2,
                        const int32_t *i3, const int32_t *i4, const double *nat_factor, const double *nat_chir) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2 || !i3 || !i4 || !nat_factor || !nat_chir)))
        return fail(XMD_ERR_ARG, "set_chirals: null array");
    return guard([&] { ctx->eng->set_chirals(rep, n, i1, i2, i3, i4, nat_factor, nat_chir); });
}

int xmd_gpu_set_heuristic_angles(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2,
                                 const int32_t *i3) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2 || !i3))) return fail(XMD_ERR_ARG, "set_heuristic_angles: null array");
    return guard([&] { ctx->eng->set_heuristic_angles(rep, n, i1, i2, i3); });
}

int xmd_gpu_set_heuristic_dihedrals(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2,
                                    const int32_t *i3, const int32_t *i4) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2 || !i3 || !i4)))
        return fail(XMD_ERR_ARG, "set_heuristic_dihedrals: null array");
    return guard([&] { ctx->eng->set_heuristic_dihedrals(rep, n, i1, i2, i3, i4); });
}

int xmd_gpu_set_velocity_afm(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *bead, const double *orig,
                             const double *vel) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!bead || !orig || !vel))) return fail(XMD_ERR_ARG, "set_velocity_afm: null array");
    return guard([&] { ctx->eng->set_velocity_afm(rep, n, bead, orig, vel); });
}

int xmd_gpu_set_force_afm(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *bead, const double *F) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!bead || !F))) return fail(XMD_ERR_ARG, "set_force_afm: null array");
    return guard([&] { ctx->eng->set_force_afm(rep, n, bead, F); });
}

int xmd_gpu_set_walls(xmd_gpu_ctx *ctx, int32_t kind, int32_t n, const double *origin, const double *normal) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!origin || !normal))) return fail(XMD_ERR_ARG, "set_walls: null array");
    return guard([&] { ctx->eng->set_walls(kind, n, origin, normal); });
}

int xmd_gpu_set_ssbonds(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2))) return fail(XMD_ERR_ARG, "set_ssbonds: null array");
    return guard([&] { ctx->eng->set_ssbonds(rep, n, i1, i2); });
}

int xmd_gpu_set_dihedrals(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1, const int32_t *i2,
                          const int32_t *i3, const int32_t *i4, const double *nat_phi) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2 || !i3 || !i4 || !nat_phi)))
        return fail(XMD_ERR_ARG, "bad dihedral arrays");
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_dihedrals(rep, n, i1, i2, i3, i4, nat_phi); });
}

int xmd_gpu_set_native_contacts(xmd_gpu_ctx *ctx, int32_t rep, int32_t n, const int32_t *i1,
                                const int32_t *i2, const double *nat_dist) {
    NEED_CTX;
    if (n < 0 || (n > 0 && (!i1 || !i2 || !nat_dist))) return fail(XMD_ERR_ARG, "bad native arrays");
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_native(rep, n, i1, i2, nat_dist); });
}

int xmd_gpu_set_state(xmd_gpu_ctx *ctx, int32_t rep, const double *r, const double *v) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_state(rep, r, v); });
}

int xmd_gpu_set_history(xmd_gpu_ctx *ctx, int32_t rep, const double *y, double t, uint64_t rng_state) {
    NEED_CTX;
    if (!y) return fail(XMD_ERR_ARG, "null history");
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_history(rep, y, t, rng_state); });
}

int xmd_gpu_get_state(xmd_gpu_ctx *ctx, int32_t rep, double *r, double *v, double *t) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->get_state(rep, r, v, t); });
}

int xmd_gpu_get_history(xmd_gpu_ctx *ctx, int32_t rep, double *y, double *t, uint64_t *rng_state) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->get_history(rep, y, t, rng_state); });
}

int xmd_gpu_snapshot_size(xmd_gpu_ctx *ctx, int32_t rep, int64_t *bytes) {
    NEED_CTX;
    if (!bytes) return fail(XMD_ERR_ARG, "snapshot_size: null output");
    return guard([&] { ctx->eng->use_device(); *bytes = (int64_t)ctx->eng->snapshot_size(rep); });
}

int xmd_gpu_snapshot(xmd_gpu_ctx *ctx, int32_t rep, void *buf, int64_t bytes) {
    NEED_CTX;
    if (!buf || bytes < 0) return fail(XMD_ERR_ARG, "snapshot: null buffer");
    return guard([&] { ctx->eng->use_device(); ctx->eng->snapshot(rep, buf, (size_t)bytes); });
}

int xmd_gpu_restore(xmd_gpu_ctx *ctx, int32_t rep, const void *buf, int64_t bytes) {
    NEED_CTX;
    if (!buf || bytes < 0) return fail(XMD_ERR_ARG, "restore: null buffer");
    return guard([&] { ctx->eng->use_device(); ctx->eng->restore(rep, buf, (size_t)bytes); });
}

int xmd_gpu_eval_forces(xmd_gpu_ctx *ctx, int32_t rep, double *F, double *V) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->eval_forces(rep, F, V); });
}

int xmd_gpu_step(xmd_gpu_ctx *ctx, int32_t nsteps) {
    NEED_CTX;
    if (nsteps < 0) return fail(XMD_ERR_ARG, "negative step count");
    return guard([&] { ctx->eng->use_device(); ctx->eng->step(nsteps); });
}

int xmd_gpu_observables(xmd_gpu_ctx *ctx, int32_t rep, double *E, double *K, double *Rg, double *Q) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->observables(rep, E, K, Rg, Q); });
}

int xmd_gpu_device_status(xmd_gpu_ctx *ctx, int32_t *status) {
    NEED_CTX;
    return guard([&] {
        int s = ctx->eng->device_status();
        if (status) *status = s;
    });
}

int xmd_gpu_upload_history_all(xmd_gpu_ctx *ctx, const double *y) {
    NEED_CTX;
    if (!y) return fail(XMD_ERR_ARG, "null history");
    return guard([&] { ctx->eng->use_device(); ctx->eng->upload_history_all(y); });
}

int xmd_gpu_download_positions_all(xmd_gpu_ctx *ctx, double *r) {
    NEED_CTX;
    if (!r) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { ctx->eng->use_device(); ctx->eng->download_positions_all(r); });
}

int xmd_gpu_download_history_all(xmd_gpu_ctx *ctx, double *y) {
    NEED_CTX;
    if (!y) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { ctx->eng->use_device(); ctx->eng->download_history_all(y); });
}

int xmd_gpu_get_stream(xmd_gpu_ctx *ctx, void **stream) {
    NEED_CTX;
    if (!stream) return fail(XMD_ERR_ARG, "null output");
    *stream = (void *)ctx->eng->get_stream();
    return XMD_OK;
}

int xmd_gpu_stats(xmd_gpu_ctx *ctx, int64_t *out) {
    NEED_CTX;
    if (!out) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { ctx->eng->use_device(); ctx->eng->stats(out); });
}

int xmd_gpu_set_kernel_timing(xmd_gpu_ctx *ctx, int on) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->set_kernel_timing(on != 0); });
}

int xmd_gpu_autotune(xmd_gpu_ctx *ctx, int32_t steps, int32_t *shape, double *ms_per_step) {
    NEED_CTX;
    return guard([&] {
        ctx->eng->use_device();
        const xmdg::Engine::Tune t = ctx->eng->autotune(steps, ms_per_step);
        if (shape) { shape[0] = t.fb; shape[1] = t.tile_per_sm; shape[2] = t.graph_steps; shape[3] = t.lpb; }
    });
}

int xmd_gpu_set_tuning(xmd_gpu_ctx *ctx, const int32_t *shape) {
    NEED_CTX;
    if (!shape) return XMD_ERR_ARG;
    return guard([&] {
        ctx->eng->use_device();
        xmdg::Engine::Tune t;
        t.fb = shape[0];
        t.tile_per_sm = shape[1];
        t.graph_steps = shape[2];
        t.lpb = shape[3];
        ctx->eng->set_tuning(t);
    });
}

int xmd_gpu_get_tuning(xmd_gpu_ctx *ctx, int32_t *shape) {
    NEED_CTX;
    if (!shape) return XMD_ERR_ARG;
    return guard([&] {
        const xmdg::Engine::Tune t = ctx->eng->tuning();
        shape[0] = t.fb; shape[1] = t.tile_per_sm; shape[2] = t.graph_steps; shape[3] = t.lpb;
    });
}

int xmd_gpu_reserve(xmd_gpu_ctx *ctx, int32_t beads, int32_t replicas, int32_t native_entries) {
    NEED_CTX;
    return guard([&] {
        ctx->eng->use_device();
        ctx->eng->reserve(beads, replicas, native_entries);
    });
}

int xmd_gpu_remove_replica(xmd_gpu_ctx *ctx, int32_t rep) {
    NEED_CTX;
    return guard([&] { ctx->eng->remove_replica(rep); });
}

int xmd_gpu_set_steps(xmd_gpu_ctx *ctx, int32_t rep, int64_t nsteps) {
    NEED_CTX;
    return guard([&] { ctx->eng->set_steps(rep, nsteps); });
}

int xmd_gpu_steps_left(xmd_gpu_ctx *ctx, int64_t *out) {
    NEED_CTX;
    if (!out) return fail(XMD_ERR_ARG, "null output");
    return guard([&] {
        std::vector<long long> v(std::max<size_t>(1, ctx->eng->reps.size()));
        ctx->eng->steps_left(v.data());
        for (size_t k = 0; k < ctx->eng->reps.size(); ++k) out[k] = v[k];
    });
}

#define NEED_SRV \
    if (!srv || !srv->srv) return fail(XMD_ERR_ARG, "null server");

int xmd_gpu_server_create(const char *yaml_text, int64_t hbm_budget_bytes, int32_t max_beads, int32_t chunk_steps,
                          xmd_gpu_server **out) {
    if (!out) return fail(XMD_ERR_ARG, "null output");
    *out = nullptr;
    xmd_params p;
    int rc = guard([&] { xmdg::params_from_yaml(yaml_text ? yaml_text : "", &p); });
    if (rc) return rc;
    return guard([&] {
        auto *h = new xmd_gpu_server;
        try {
            h->srv = new xmdg::Server(p, hbm_budget_bytes, max_beads, chunk_steps);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int xmd_gpu_server_submit(xmd_gpu_server *srv, const xmd_request *q, int64_t *id) {
    NEED_SRV;
    if (!q || !id) return fail(XMD_ERR_ARG, "null request");
    if (q->n <= 0 || !q->chain_idx || !q->seq_idx || !q->atype || !q->r)
        return fail(XMD_ERR_ARG, "request needs n > 0, topology and positions");
    return guard([&] {
        auto r = std::make_unique<xmdg::Request>();
        const int n = q->n;
        r->n = n;
        r->chain.assign(q->chain_idx, q->chain_idx + n);
        r->seq.assign(q->seq_idx, q->seq_idx + n);
        r->atype.assign(q->atype, q->atype + n);
        for (int a = 0; a < 3; ++a) r->cell[a] = q->cell ? q->cell[a] : 0.0;
        r->temperature = q->temperature;
        r->seed = q->seed;
        auto cp = [](std::vector<int32_t> &dst, const int32_t *src, int m) {
            if (m > 0 && !src) throw std::invalid_argument("null topology array");
            dst.assign(src, src + std::max(0, m));
        };
        auto cpd = [](std::vector<double> &dst, const double *src, int m) {
            if (m > 0 && src) dst.assign(src, src + m);
            else dst.assign(std::max(0, m), 0.0);
        };
        cp(r->t1, q->teth_i1, q->n_tethers); cp(r->t2, q->teth_i2, q->n_tethers); cpd(r->td, q->teth_d, q->n_tethers);
        cp(r->a1, q->ang_i1, q->n_angles); cp(r->a2, q->ang_i2, q->n_angles); cp(r->a3, q->ang_i3, q->n_angles);
        if (q->n_angles > 0 && !q->ang_theta) throw std::invalid_argument("null native angles");
        cpd(r->ath, q->ang_theta, q->n_angles);
        cp(r->d1, q->dih_i1, q->n_dihedrals); cp(r->d2, q->dih_i2, q->n_dihedrals);
        cp(r->d3, q->dih_i3, q->n_dihedrals); cp(r->d4, q->dih_i4, q->n_dihedrals);
        if (q->n_dihedrals > 0 && !q->dih_phi) throw std::invalid_argument("null native dihedrals");
        cpd(r->dph, q->dih_phi, q->n_dihedrals);
        cp(r->n1, q->nat_i1, q->n_natives); cp(r->n2, q->nat_i2, q->n_natives);
        if (q->n_natives > 0 && !q->nat_d) throw std::invalid_argument("null native distances");
        cpd(r->nd, q->nat_d, q->n_natives);
        r->r.assign(q->r, q->r + 3 * (size_t)n);
        if (q->v) r->v.assign(q->v, q->v + 3 * (size_t)n);
        r->nsteps = q->nsteps;
        *id = srv->srv->submit(std::move(r));
    });
}

int xmd_gpu_server_poll(xmd_gpu_server *srv, int64_t id, int32_t *state) {
    NEED_SRV;
    if (!state) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { *state = srv->srv->poll(id); });
}

int xmd_gpu_server_result(xmd_gpu_server *srv, int64_t id, double *r, double *v, double *t, double *latency_s) {
    NEED_SRV;
    return guard([&] { srv->srv->result(id, r, v, t, latency_s); });
}

int xmd_gpu_server_wait_all(xmd_gpu_server *srv) {
    NEED_SRV;
    return guard([&] { srv->srv->wait_all(); });
}

int xmd_gpu_server_stats(xmd_gpu_server *srv, double *out) {
    NEED_SRV;
    if (!out) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { srv->srv->stats(out); });
}

int xmd_gpu_server_destroy(xmd_gpu_server *srv) {
    if (!srv) return XMD_OK;
    return guard([&] {
        delete srv->srv;
        delete srv;
    });
}

int xmd_gpu_kernel_times(xmd_gpu_ctx *ctx, double *force_ms, int64_t *force_launches, double *rebuild_ms,
                         int64_t *rebuild_launches) {
    NEED_CTX;
    return guard([&] {
        ctx->eng->use_device();
        ctx->eng->kernel_times(force_ms, force_launches, rebuild_ms, rebuild_launches);
    });
}

int xmd_gpu_qa_contacts(xmd_gpu_ctx *ctx, int32_t rep, int32_t cap, int32_t *out4, double *ref_time,
                        int32_t *count) {
    NEED_CTX;
    if (cap < 0 || (cap > 0 && !out4)) return fail(XMD_ERR_ARG, "bad output buffer");
    return guard([&] {
        ctx->eng->use_device();
        int m = ctx->eng->qa_contacts(rep, cap, out4, ref_time);
        if (count) *count = m;
    });
}

int xmd_gpu_verlet_pairs(xmd_gpu_ctx *ctx, int32_t rep, int32_t cap, int32_t *out2, uint8_t *flags,
                         int32_t *count) {
    NEED_CTX;
    if (cap < 0 || (cap > 0 && !out2)) return fail(XMD_ERR_ARG, "bad output buffer");
    return guard([&] {
        ctx->eng->use_device();
        int m = ctx->eng->verlet_pairs(rep, cap, out2, flags);
        if (count) *count = m;
    });
}

int xmd_gpu_qa_sync(xmd_gpu_ctx *ctx, int32_t rep, int8_t *out) {
    NEED_CTX;
    if (!out) return fail(XMD_ERR_ARG, "null output");
    return guard([&] { ctx->eng->use_device(); ctx->eng->qa_sync(rep, out); });
}

int xmd_gpu_verlet_pairs_noalloc(const double *d_r, const int32_t *d_chain, const int32_t *d_seq, int32_t n,
                                 const double cell[3], double cutoff, int32_t *d_pairs, int32_t cap,
                                 int32_t *d_count, void *stream) {
    if (n < 0) return fail(XMD_ERR_ARG, "negative bead count");
    if (n > XMD_NOALLOC_MAX_BEADS)
        return fail(XMD_ERR_CAPACITY, "xmd_gpu_verlet_pairs_noalloc: " + std::to_string(n) +
                                          " beads exceed the allocation-free scratch (XMD_NOALLOC_MAX_BEADS = " +
                                          std::to_string(XMD_NOALLOC_MAX_BEADS) + ")");
    if (!cell || !d_count || (n > 0 && (!d_r || !d_chain || !d_seq)) || cap < 0 || (cap > 0 && !d_pairs))
        return fail(XMD_ERR_ARG, "null or invalid buffer");
    if (!(cutoff > 0.0)) return fail(XMD_ERR_ARG, "cutoff must be positive");
    for (int a = 0; a < 3; ++a)
        if (!(cell[a] >= 0.0)) return fail(XMD_ERR_ARG, "bad cell");
    return guard([&] { xmdg::verlet_pairs_noalloc(d_r, d_chain, d_seq, n, cell, cutoff, d_pairs, cap, d_count, stream); });
}

int xmd_gpu_synchronize(xmd_gpu_ctx *ctx) {
    NEED_CTX;
    return guard([&] { ctx->eng->use_device(); ctx->eng->sync(); });
}

}  // extern "C"
