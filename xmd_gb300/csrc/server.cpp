// server.cpp - continuous-batching request loop (see server.h).
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <stdexcept>

namespace xmdg {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// native-contact entries reserved per bead slot
constexpr int NATIVES_PER_BEAD = 8;

// Device bytes of a reserved context, fixed part and per bead slot, measured
// on two small probe contexts of these parameters (their allocations at the
// initial Verlet row capacity): the admission budget is enforced against the
// engine's real allocation, not an estimate.
static void reservation_cost(const xmd_params &p, double *fixed, double *per_bead) {
    auto probe = [&](int beads) {
        Engine e(p);
        e.reserve(beads, std::max(16, beads / 30), NATIVES_PER_BEAD * beads);
        return (double)e.device_bytes();
    };
    const int b1 = 4096, b2 = 8192;
    const double m1 = probe(b1), m2 = probe(b2);
    *per_bead = (m2 - m1) / (b2 - b1);
    *fixed = m1 - *per_bead * b1;
}

Server::Server(const xmd_params &p, int64_t hbm_budget, int max_beads, int chunk_steps) : params(p) {
    if (!params.langevin_on) throw std::invalid_argument("server: langevin must be enabled");
    if (params.on[XMD_TERM_QA]) throw std::invalid_argument("server: the quasi-adiabatic term needs a static context");
    if (hbm_budget <= 0 || max_beads <= 0) throw std::invalid_argument("server: bad budget");
    chunk = chunk_steps > 0 ? chunk_steps : 256;
    budget = hbm_budget;
    double fixed = 0.0;
    reservation_cost(params, &fixed, &bytes_per_bead);
    const double fit = ((double)hbm_budget - fixed) / bytes_per_bead;
    cap_beads = (int)std::min<double>(max_beads, std::floor(fit));
    if (cap_beads < 1) throw std::invalid_argument("server: the HBM budget holds no bead");
    // the replica table grows with the bead capacity; shrink until the whole
    // reservation fits the budget
    for (;;) {
        cap_reps = std::min(1024, std::max(16, cap_beads / 30));
        cap_nat = NATIVES_PER_BEAD * cap_beads;
        eng = std::make_unique<Engine>(params);
        // one request whose trajectory diverges fails alone; the others go on
        eng->set_isolate_faults(true);
        eng->reserve(cap_beads, cap_reps, cap_nat);
        if ((int64_t)eng->device_bytes() <= hbm_budget || cap_beads <= 1) break;
        cap_beads = std::max(1, (int)(cap_beads * 0.98));
    }
    if ((int64_t)eng->device_bytes() > hbm_budget) throw std::invalid_argument("server: the HBM budget holds no bead");
    dev_bytes = (int64_t)eng->device_bytes();
    worker = std::thread([this] { loop(); });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
    }
    cv.notify_all();
    if (worker.joinable()) worker.join();
    eng.reset();
}

int64_t Server::submit(std::unique_ptr<Request> req) {
    if (req->n <= 0 || req->nsteps < 0) throw std::invalid_argument("server: empty request");
    if (req->n > cap_beads)
        throw std::length_error("server: the request has more beads than the reserved capacity");
    std::lock_guard<std::mutex> lk(mu);
    if (!fatal.empty()) throw std::runtime_error("server stopped: " + fatal);
    req->id = next_id++;
    req->t_submit = now_s();
    if (t_first < 0) t_first = req->t_submit;
    Request *q = req.get();
    const int64_t id = req->id;
    all[id] = std::move(req);
    queue.push_back(q);
    cv.notify_all();
    return id;
}

int Server::poll(int64_t id) {
    std::lock_guard<std::mutex> lk(mu);
    auto it = all.find(id);
    if (it == all.end()) throw std::invalid_argument("server: unknown request id");
    return it->second->state;
}

void Server::result(int64_t id, double *r, double *v, double *t, double *latency) {
    std::unique_lock<std::mutex> lk(mu);
    auto it = all.find(id);
    if (it == all.end()) throw std::invalid_argument("server: unknown request id");
    Request *q = it->second.get();
    cv_done.wait(lk, [&] { return q->state == XMD_REQ_DONE || q->state == XMD_REQ_FAILED; });
    if (q->state == XMD_REQ_FAILED) {
        std::string e = q->error;
        all.erase(it);
        throw std::runtime_error("request failed: " + e);
    }
    if (r) std::copy(q->r_out.begin(), q->r_out.end(), r);
    if (v) std::copy(q->v_out.begin(), q->v_out.end(), v);
    if (t) *t = q->t_out;
    if (latency) *latency = q->t_done - q->t_submit;
    all.erase(it);
}

void Server::wait_all() {
    std::unique_lock<std::mutex> lk(mu);
    cv_done.wait(lk, [&] { return (queue.empty() && running.empty()) || !fatal.empty(); });
    if (!fatal.empty()) throw std::runtime_error("server stopped: " + fatal);
}

void Server::stats(double *out) {
    std::lock_guard<std::mutex> lk(mu);
    for (int k = 0; k < XMD_SRV_NUM; ++k) out[k] = 0.0;
    std::vector<double> l = latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        // nearest-rank percentile
        size_t k = (size_t)std::ceil(q * l.size());
        return l[std::min(l.size(), std::max<size_t>(1, k)) - 1];
    };
    out[XMD_SRV_P50_S] = pct(0.50);
    out[XMD_SRV_P99_S] = pct(0.99);
    const double span = t_last - t_first;
    out[XMD_SRV_BEAD_STEPS_PER_S] = (span > 0 && !l.empty()) ? bead_steps / span : 0.0;
    out[XMD_SRV_COMPLETED] = (double)l.size();
    out[XMD_SRV_QUEUED] = (double)queue.size();
    out[XMD_SRV_RUNNING] = (double)running.size();
    out[XMD_SRV_CHUNKS] = (double)chunks;
    out[XMD_SRV_PEAK_RUNNING] = (double)peak_running;
    out[XMD_SRV_CAP_BEADS] = (double)cap_beads;
    out[XMD_SRV_BEAD_STEPS] = bead_steps;
    out[XMD_SRV_SPAN_S] = span;
    out[XMD_SRV_FAILED] = (double)failed;
    out[XMD_SRV_DEVICE_BYTES] = (double)dev_bytes;
    out[XMD_SRV_BUDGET_BYTES] = (double)budget;
    out[XMD_SRV_BYTES_PER_BEAD] = bytes_per_bead;
    out[XMD_SRV_ADMIT_S] = admit_s;
    out[XMD_SRV_STEP_S] = step_s;
}

// place a queued request into a free slot; false when the capacity has no
// room for it now (it stays queued)
bool Server::admit(Request *q) {
    Engine &e = *eng;
    int slot;
    try {
        slot = e.add_replica(q->n, q->chain.data(), q->seq.data(), q->atype.data(), q->cell, q->temperature,
                             q->seed);
    } catch (std::length_error &) {
        return false;   // every replica slot is taken
    }
    try {
        e.set_tethers(slot, (int)q->t1.size(), q->t1.data(), q->t2.data(), q->td.data());
        e.set_angles(slot, (int)q->a1.size(), q->a1.data(), q->a2.data(), q->a3.data(), q->ath.data());
        e.set_dihedrals(slot, (int)q->d1.size(), q->d1.data(), q->d2.data(), q->d3.data(), q->d4.data(),
                        q->dph.data());
        e.set_native(slot, (int)q->n1.size(), q->n1.data(), q->n2.data(), q->nd.data());
        e.set_state(slot, q->r.data(), q->v.empty() ? nullptr : q->v.data());
        e.set_steps(slot, q->nsteps);
        // device ranges and uploads on the side stream; live at activation
        e.stage(slot);
    } catch (std::length_error &) {
        e.remove_replica(slot);
        return false;   // no contiguous room in the reserved capacity yet
    } catch (std::exception &ex) {
        e.remove_replica(slot);
        std::lock_guard<std::mutex> lk(mu);
        q->state = XMD_REQ_FAILED;
        q->error = ex.what();
        return true;   // consumed (failed)
    }
    q->slot = slot;
    return true;
}

void Server::retire(Request *q) {
    Engine &e = *eng;
    q->r_out.resize(3 * (size_t)q->n);
    q->v_out.resize(3 * (size_t)q->n);
    e.get_state(q->slot, q->r_out.data(), q->v_out.data(), &q->t_out);
    e.remove_replica(q->slot);
    std::lock_guard<std::mutex> lk(mu);
    q->t_done = now_s();
    q->state = XMD_REQ_DONE;
    latencies.push_back(q->t_done - q->t_submit);
    bead_steps += (double)q->n * (double)q->nsteps;
    t_last = q->t_done;
}

// a request whose replica was frozen by a non-finite force
void Server::fail(Request *q, const char *why) {
    eng->remove_replica(q->slot);
    std::lock_guard<std::mutex> lk(mu);
    q->t_done = now_s();
    q->state = XMD_REQ_FAILED;
    q->error = why;
    ++failed;
}

void Server::loop() {
    // One chunk of steps is in flight while the worker admits the queued
    // requests that fit: their host-side preparation and uploads (side
    // stream, into free device ranges) overlap the chunk.  After the chunk,
    // finished requests are retired, the staged ones are activated on the
    // step stream (ordered after their uploads) and the next chunk starts.
    std::vector<Request *> staged;
    try {
        eng->use_device();
        std::vector<long long> left;
        bool inflight = false;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                if (!inflight) cv.wait(lk, [&] { return stop || !queue.empty() || !running.empty(); });
                if (stop && !inflight) break;
            }
            // admission, first come first served (tried against an idle
            // context when nothing runs, is staged or is in flight)
            const bool idle = !inflight && running.empty() && staged.empty();
            const double ta = now_s();
            for (;;) {
                Request *q;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    if (queue.empty() || stop) break;
                    q = queue.front();
                }
                if (!admit(q)) break;
                std::lock_guard<std::mutex> lk(mu);
                queue.pop_front();
                if (q->state == XMD_REQ_FAILED) {
                    cv_done.notify_all();
                    continue;
                }
                staged.push_back(q);
            }
            const double ts = now_s();
            if (inflight) {
                eng->step_wait();
                inflight = false;
            }
            const double te = now_s();
            // retirement (the staged requests have not stepped yet)
            if (!running.empty()) {
                left.assign(eng->capacity_replicas(), -2);
                eng->steps_left(left.data());
                std::vector<Request *> keep;
                for (Request *q : running) {
                    if (left[q->slot] == -3) fail(q, "non-finite force: the trajectory diverged");
                    else if (left[q->slot] == 0) retire(q);
                    else keep.push_back(q);
                }
                std::lock_guard<std::mutex> lk(mu);
                running.swap(keep);
            }
            eng->activate_staged();
            {
                std::lock_guard<std::mutex> lk(mu);
                const double tn = now_s();
                for (Request *q : staged) {
                    q->state = XMD_REQ_RUNNING;
                    q->t_start = tn;
                    running.push_back(q);
                }
                staged.clear();
                peak_running = std::max(peak_running, (int)running.size());
                if (idle && running.empty() && !queue.empty() && !stop) {
                    // the head of the queue does not fit an empty context: it never will
                    Request *q = queue.front();
                    queue.pop_front();
                    q->state = XMD_REQ_FAILED;
                    q->error = "the request does not fit the reserved capacity";
                }
                // host time outside the chunks' device work: admission and
                // the part of retirement and activation after the wait
                admit_s += (ts - ta) + (now_s() - te);
                step_s += te - ts;
                dev_bytes = (int64_t)eng->device_bytes();
            }
            cv_done.notify_all();
            if (!running.empty() && !stop) {
                eng->step_async(chunk);
                inflight = true;
                ++chunks;
            }
        }
    } catch (std::exception &ex) {
        std::lock_guard<std::mutex> lk(mu);
        fatal = ex.what();
        for (Request *q : running) {
            q->state = XMD_REQ_FAILED;
            q->error = fatal;
        }
        for (Request *q : queue) {
            q->state = XMD_REQ_FAILED;
            q->error = fatal;
        }
        for (Request *q : staged) {
            q->state = XMD_REQ_FAILED;
            q->error = fatal;
        }
        staged.clear();
        running.clear();
        queue.clear();
        cv_done.notify_all();
    }
}

}  // namespace xmdg
