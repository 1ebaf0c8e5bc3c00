// nb_serve.cu -- served form: a request loop of galaxy-generation jobs with
// continuous batching.
//
// Jobs wait in a FIFO queue; between rounds finished jobs leave (their final
// state is copied to the host) and queued jobs are admitted while a slot is
// free and the estimated device bytes of the active jobs stay within the
// budget.  When the active set changes, a new batch is built from the active
// jobs -- continuing jobs hand their state over device to device, new jobs
// have their initial conditions generated on the device, straight into the
// batch's arrays (nb_gen.cu) -- and the active jobs are stepped together by
// the batched form for up to steps_per_round steps, never past the nearest
// completion and, when round_seconds is set, for no more steps than fit in
// round_seconds at the batch's measured time per step (the first round of a
// new batch takes one step to measure it), so that jobs arriving meanwhile
// are admitted soon.  Every job's state stays on the device from admission to
// completion; nothing of a job is made on the host.
#include "nb_common.cuh"
#include "nb_internal.hpp"
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <vector>

using namespace nb;

namespace {

// Upper estimate of the batched form's device bytes per body: state and
// compensation (96), sort and topology scratch (~110), tree cells at twice the
// measured count with quadrupoles (~400), direct-sum partials.
constexpr size_t kBytesPerBody = 640;
// Bodies one batch may hold: its octree must stay below 2^27 cells (about
// 1.3 cells per body), the traversal's cell-index range.
constexpr size_t kMaxBatchBodies = (size_t)96 << 20;

struct Job {
    nb_job spec{};
    nb_job_status st{};
    int galaxy = -1;                // index in the current batch
    std::vector<float> res_pos, res_vel;
};

}  // namespace

struct nb_server {
    nb_server_params prm{};
    std::string err;
    std::chrono::steady_clock::time_point t0;
    uint64_t next_id = 1;
    std::map<uint64_t, Job> jobs;
    std::deque<uint64_t> queue;
    std::vector<uint64_t> active;   // in batch galaxy order
    nb_batch* batch = nullptr;
    size_t bytes_used = 0;
    size_t bodies_used = 0;
    bool batch_stale = false;       // the active set changed since the batch was built
    float dt = NAN;                 // dt of the active jobs
    double step_s = 0;              // measured seconds per step of the current batch (0: not yet)
    uint64_t body_steps = 0, rounds = 0;
    uint64_t rebuilds = 0, batch_steps = 0, step_launches = 0;   // where the time went
    double rebuild_s = 0, stepping_s = 0;
};

namespace {

int sfail(nb_server* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}

double now_s(const nb_server* s) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

size_t job_bytes(const nb_job& j) { return j.n * kBytesPerBody; }

// Builds a batch of the active jobs; continuing jobs take their state from
// the previous batch (device to device), new jobs are generated on the device
// at commit.  On failure the previous batch and the jobs' places in it are
// left as they were.
int rebuild(nb_server* s) {
    nb_batch* nb2 = nullptr;
    int rc = nb_batch_create(&s->prm.base, s->prm.bh_threshold, s->prm.base.theta, &nb2);
    if (rc) return sfail(s, rc, "nb_batch_create failed");
    std::vector<int32_t> place(s->active.size(), -1);
    for (size_t a = 0; a < s->active.size(); ++a) {
        const Job& j = s->jobs[s->active[a]];
        int32_t g = -1;
        if (j.galaxy >= 0 && s->batch) {
            const float4 *p, *pc, *v, *vc, *ac;
            size_t n = 0;
            rc = batch_device_state(s->batch, j.galaxy, &p, &pc, &v, &vc, &ac, &n);
            if (!rc) rc = batch_add_device(nb2, p, pc, v, vc, ac, n, &g);
        } else {
            rc = nb_batch_add_generated(nb2, j.spec.model, j.spec.seed, j.spec.n, &g);
        }
        if (rc) {
            std::string m = nb_batch_last_error(nb2);
            nb_batch_destroy(nb2);
            return sfail(s, rc, "batch add: " + m);
        }
        place[a] = g;
    }
    rc = nb_batch_commit(nb2);
    if (rc) {
        std::string m = nb_batch_last_error(nb2);
        nb_batch_destroy(nb2);
        return sfail(s, rc, "batch commit: " + m);
    }
    if (s->batch) nb_batch_destroy(s->batch);
    s->batch = nb2;
    s->step_s = 0;
    for (size_t a = 0; a < s->active.size(); ++a) s->jobs[s->active[a]].galaxy = place[a];
    return NB_OK;
}

}  // namespace

extern "C" {

int nb_server_default_params(nb_server_params* p) {
    try {
        if (!p) return NB_EINVAL;
        std::memset(p, 0, sizeof(*p));
        nb_default_params(&p->base);
        p->base.softening2 = 0.005 * 0.005;
        p->base.theta = 0.5;
        p->memory_budget = (size_t)120 << 30;
        p->max_active = 64;
        p->steps_per_round = 25;
        p->bh_threshold = 1024;
        p->round_seconds = 0.1;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_create(const nb_server_params* p, nb_server** out) {
    try {
        if (!p || !out) return NB_EINVAL;
        *out = nullptr;
        if (p->max_active < 1 || p->steps_per_round < 1 || p->memory_budget == 0 || p->bh_threshold < 2 ||
            !(p->base.theta > 0) || !(p->round_seconds >= 0))
            return NB_EINVAL;
        nb_server* s = new (std::nothrow) nb_server();
        if (!s) return NB_ENOMEM;
        s->prm = *p;
        s->t0 = std::chrono::steady_clock::now();
        *out = s;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_destroy(nb_server* s) {
    try {
        if (!s) return NB_EINVAL;
        if (s->batch) nb_batch_destroy(s->batch);
        delete s;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

const char* nb_server_last_error(const nb_server* s) { return s ? s->err.c_str() : "null handle"; }

double nb_server_clock(nb_server* s) { return s ? now_s(s) : 0.0; }

int nb_server_submit(nb_server* s, const nb_job* job, uint64_t* id) {
    try {
        if (!s || !job) return NB_EINVAL;
        if (job->n < 2 || job->steps < 1 || !(job->dt > 0) || (job->model != 0 && job->model != 1))
            return sfail(s, NB_EINVAL, "bad job");
        Job j;
        j.spec = *job;
        j.st.id = s->next_id++;
        j.st.state = 0;
        j.st.submit_s = now_s(s);
        j.st.bytes = job_bytes(*job);
        if (job->n > kMaxGalaxyBodies || j.st.bytes > s->prm.memory_budget) j.st.state = -1;   // can never fit
        const uint64_t jid = j.st.id;
        const bool queued = j.st.state == 0;
        s->jobs.emplace(jid, std::move(j));
        if (queued) s->queue.push_back(jid);
        if (id) *id = jid;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_tick(nb_server* s, int* active, int* queued) {
    try {
        if (!s) return NB_EINVAL;
        // retire finished jobs (a job whose result cannot be read stays active)
        std::vector<uint64_t> keep;
        int read_rc = NB_OK;
        for (uint64_t id : s->active) {
            Job& j = s->jobs[id];
            if (read_rc == NB_OK && j.st.steps_done >= j.spec.steps) {
                j.res_pos.assign(4 * j.spec.n, 0.f);
                j.res_vel.assign(4 * j.spec.n, 0.f);
                read_rc = nb_batch_read(s->batch, j.galaxy, j.res_pos.data(), j.res_vel.data());
                if (read_rc) {
                    sfail(s, read_rc, std::string("read result: ") + nb_batch_last_error(s->batch));
                    keep.push_back(id);
                    continue;
                }
                j.st.state = 2;
                j.st.done_s = now_s(s);
                j.galaxy = -1;
                s->bytes_used -= j.st.bytes;
                s->bodies_used -= j.spec.n;
                s->batch_stale = true;
            } else {
                keep.push_back(id);
            }
        }
        s->active.swap(keep);
        if (read_rc) return read_rc;
        if (s->active.empty()) s->dt = NAN;
        // admit queued jobs (FIFO) while a slot and the budget allow
        while (!s->queue.empty() && (int)s->active.size() < s->prm.max_active) {
            Job& j = s->jobs[s->queue.front()];
            if (s->bytes_used + j.st.bytes > s->prm.memory_budget) break;
            if (s->bodies_used + j.spec.n > kMaxBatchBodies) break;
            if (!std::isnan(s->dt) && j.spec.dt != s->dt) break;   // waits for a round with its dt
            j.st.state = 1;
            j.st.admit_s = now_s(s);
            j.galaxy = -1;
            s->bytes_used += j.st.bytes;
            s->bodies_used += j.spec.n;
            s->dt = j.spec.dt;
            s->active.push_back(j.st.id);
            s->queue.pop_front();
            s->batch_stale = true;
        }
        // a rebuild that failed is tried again on the next tick: no round runs
        // on a batch that does not hold exactly the active jobs
        if (s->batch_stale && !s->active.empty()) {
            const double t_rb = now_s(s);
            int rc = rebuild(s);
            if (rc) return rc;
            s->rebuild_s += now_s(s) - t_rb;
            ++s->rebuilds;
            s->batch_stale = false;
        } else if (s->active.empty()) {
            if (s->batch) nb_batch_destroy(s->batch);
            s->batch = nullptr;
            s->batch_stale = false;
        }
        // one round
        if (!s->active.empty()) {
            int k = s->prm.steps_per_round;
            for (uint64_t id : s->active) k = std::min(k, s->jobs[id].spec.steps - s->jobs[id].st.steps_done);
            if (s->prm.round_seconds > 0) {
                const double fit = s->step_s > 0 ? s->prm.round_seconds / s->step_s : 1.0;
                if (fit < (double)k) k = (int)fit;
            }
            k = std::max(k, 1);
            const double t_round = now_s(s);
            uint64_t l0 = 0, l1 = 0;
            nb_batch_launch_count(s->batch, &l0);
            int rc = batch_launch_steps(s->batch, s->dt, k);
            nb_batch_launch_count(s->batch, &l1);
            s->step_launches += l1 - l0;
            if (rc) return sfail(s, rc, std::string("step: ") + nb_batch_last_error(s->batch));
            rc = batch_wait(s->batch);
            // a round the batch could not finish (its octree kept outgrowing its
            // arrays) ran its first k - not_run steps: the jobs' counts follow
            const int ran = rc ? k - batch_steps_not_run(s->batch) : k;
            const double t_end = now_s(s);
            if (!rc) s->step_s = (t_end - t_round) / k;
            s->stepping_s += t_end - t_round;
            s->batch_steps += (uint64_t)ran;
            for (uint64_t id : s->active) {
                Job& j = s->jobs[id];
                j.st.steps_done += ran;
                s->body_steps += (uint64_t)ran * j.spec.n;
            }
            ++s->rounds;
            if (rc) return sfail(s, rc, std::string("step: ") + nb_batch_last_error(s->batch));
        }
        if (active) *active = (int)s->active.size();
        if (queued) *queued = (int)s->queue.size();
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_status(nb_server* s, uint64_t id, nb_job_status* out) {
    try {
        if (!s || !out) return NB_EINVAL;
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) return sfail(s, NB_EINVAL, "unknown job");
        *out = it->second.st;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_result(nb_server* s, uint64_t id, float* pos_mass4, float* vel4, size_t n) {
    try {
        if (!s) return NB_EINVAL;
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) return sfail(s, NB_EINVAL, "unknown job");
        const Job& j = it->second;
        if (j.st.state != 2) return sfail(s, NB_EBADSTATE, "job not done");
        if (n != j.spec.n) return sfail(s, NB_EINVAL, "size differs from the job's n");
        if (pos_mass4) std::memcpy(pos_mass4, j.res_pos.data(), 16 * n);
        if (vel4) std::memcpy(vel4, j.res_vel.data(), 16 * n);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_release(nb_server* s, uint64_t id) {
    try {
        if (!s) return NB_EINVAL;
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) return sfail(s, NB_EINVAL, "unknown job");
        if (it->second.st.state != 2 && it->second.st.state != -1)
            return sfail(s, NB_EBADSTATE, "only a finished or rejected job can be released");
        s->jobs.erase(it);
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_timing(nb_server* s, uint64_t* rebuilds, double* rebuild_s, uint64_t* batch_steps, double* step_s,
                     double* generate_s, uint64_t* step_launches) {
    try {
        if (!s) return NB_EINVAL;
        if (rebuilds) *rebuilds = s->rebuilds;
        if (rebuild_s) *rebuild_s = s->rebuild_s;
        if (batch_steps) *batch_steps = s->batch_steps;
        if (step_s) *step_s = s->stepping_s;
        if (generate_s) *generate_s = 0.0;   // initial conditions are made on the device, inside rebuild_s
        if (step_launches) *step_launches = s->step_launches;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

int nb_server_stats(nb_server* s, uint64_t* body_steps, uint64_t* rounds) {
    try {
        if (!s) return NB_EINVAL;
        if (body_steps) *body_steps = s->body_steps;
        if (rounds) *rounds = s->rounds;
        return NB_OK;
    } catch (...) {   // no exception crosses the C-ABI: host allocation failed
        return NB_ENOMEM;
    }
}

}  // extern "C"
