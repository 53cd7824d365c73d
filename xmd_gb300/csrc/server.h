// server.h - continuous-batching request loop over one engine context.
//
// Requests (independent systems of one or more chains, each with its own
// temperature, seed and step count) are queued by any host thread.  A worker
// thread owns the engine.  While a chunk of steps runs on the device it
// admits queued requests into free replica slots while the reserved device
// capacity (sized from the HBM budget) has room: their host-side preparation
// and uploads (a side stream, into free device ranges) overlap the chunk.
// When the chunk ends it retires requests whose step budget is spent (their
// final state is copied out and their slots and device ranges are reused),
// activates the staged requests on the step stream and launches the next
// chunk for every running request together.  A request's trajectory does not
// depend on what else is in the batch.
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/xmd_gpu.h"
#include "engine.h"

namespace xmdg {

struct Request {
    int64_t id = 0;
    int n = 0;
    std::vector<int32_t> chain, seq;
    std::vector<uint8_t> atype;
    double cell[3] = {0, 0, 0};
    double temperature = 0;
    uint64_t seed = 0;
    std::vector<int32_t> t1, t2, a1, a2, a3, d1, d2, d3, d4, n1, n2;
    std::vector<double> td, ath, dph, nd, r, v;
    int64_t nsteps = 0;
    // bookkeeping
    int state = XMD_REQ_QUEUED;
    int slot = -1;
    double t_submit = 0, t_start = 0, t_done = 0;
    std::vector<double> r_out, v_out;
    double t_out = 0;
    std::string error;
};

class Server {
public:
    Server(const xmd_params &p, int64_t hbm_budget, int max_beads, int chunk_steps);
    ~Server();
    int64_t submit(std::unique_ptr<Request> req);
    int poll(int64_t id);
    void result(int64_t id, double *r, double *v, double *t, double *latency);
    void wait_all();
    void stats(double *out);   // XMD_SRV_* slots

private:
    xmd_params params;
    std::unique_ptr<Engine> eng;
    int chunk = 256;
    int cap_beads = 0, cap_reps = 0, cap_nat = 0;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<Request *> queue;
    std::map<int64_t, std::unique_ptr<Request>> all;
    std::vector<Request *> running;
    int64_t next_id = 1;
    bool stop = false;
    std::string fatal;
    std::thread worker;
    // statistics
    double t_first = -1, t_last = 0;
    double bead_steps = 0;
    std::vector<double> latencies;
    int64_t chunks = 0;
    int peak_running = 0;
    int64_t failed = 0;     // requests retired by a diverged trajectory
    int64_t budget = 0, dev_bytes = 0;
    double bytes_per_bead = 0;       // measured device cost of a bead slot
    double admit_s = 0, step_s = 0;  // worker time between chunks and in them

    void loop();
    bool admit(Request *q);
    void retire(Request *q);
    void fail(Request *q, const char *why);
};

double now_s();

}  // namespace xmdg
