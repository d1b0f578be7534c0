// arap_server.h -- the scheduler behind arap_srv_* (include/arap_gpu.h).
//
// Header-only and templated on its backend B, so the same scheduling code runs
// over the device contexts of the library (arap_server.cpp) and over a host
// model of them in the scheduler's own tests. B provides:
//   using Handle;                                   opaque per-context handle
//   int  create(int V, int F, const int32_t*, Handle*); create_like(Handle, Handle*)
//   void destroy(Handle)
//   int  set_precision(Handle, int, int); set_rest(Handle, const double*)
//   int  set_solve_ctas(Handle, int); set_ordering(Handle, int)
//   int  set_constraints(Handle, int, const int32_t*, const double*)
//   int  set_targets(Handle, int, const double*)
//   int  plan_bytes(Handle, int n_poses, int64_t*); int64_t device_bytes(Handle)
//   int  deform_async(Handle, int iters, double* out)
//   int  deform_poses_async(Handle, int P, const double* targets, int iters, double* out)
//   int  query(Handle, int32_t* done)               non-blocking completion
//   double device_ms(Handle)                        device time of the last launch
//   static constexpr bool kCallbacks; set_done_callback(Handle, void (*)(void*), void*)
//                                                   completion callbacks (else polling)
//   std::string last_error(Handle)
//   void* alloc_host(size_t); void free_host(void*)  staging for results
//   int64_t default_budget()
//
// Threads: one scheduler thread owns every context after its first launch;
// prep_threads workers run the host-side analysis of new constraint sets and
// their first launch; client threads only touch the queues and tickets.
#pragma once

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/arap_gpu.h"

namespace arapsrv {

using Clock = std::chrono::steady_clock;

inline double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Message of the last failed server call on the calling thread.
inline std::string &thread_error() {
    static thread_local std::string e;
    return e;
}

template <class B>
class Server {
    using Handle = typename B::Handle;

    struct MeshRec {
        int V = 0, F = 0;
        std::vector<double> rest;
        Handle proto{};  // topology + rest positions on the device
        int64_t bytes = 0;
    };

    enum class SlotState { Analyzing, Ready, Launching, Busy, Idle };

    struct Slot;
    struct Req {
        int64_t ticket = 0;
        int mesh = 0;
        std::vector<int32_t> idx;  // sorted unique
        std::vector<double> tgt;   // 3 per idx
        int iterations = 0;
        double *out = nullptr;
        Clock::time_point t_submit, t_launch, t_done;
        int status = ARAP_PENDING;
        std::string error;
        int factor_reused = 0, batch = 0;
        uint64_t key = 0;
        Slot *slot = nullptr;      // set once the request waits on a slot
    };

    struct Slot {
        int mesh = 0;
        std::vector<int32_t> idx;
        uint64_t key = 0;
        Handle ctx{};
        bool have_ctx = false;
        SlotState state = SlotState::Analyzing;
        bool built = false;       // a factor exists (first launch done)
        int64_t bytes = 0;        // device bytes held now
        int64_t need = 0;         // device bytes after the next launch
        int64_t reserved = 0;     // bytes reserved for a launch in progress
        Clock::time_point last_used;
        uint64_t order = 0;       // creation order (admission is first come, first served)
        std::vector<Req *> running;
        std::deque<Req *> waiting;  // requests of this constraint set not launched yet, oldest first
        std::vector<double> batch_targets;
        double *staging = nullptr;
        size_t staging_doubles = 0;
        struct Tag {
            Server *srv;
            Slot *slot;
        } tag{nullptr, nullptr};  // completion-callback argument
        int job_rc = ARAP_OK;     // written by a worker, read by the scheduler after the job
        std::string job_err;
        int64_t job_need = 0, job_bytes = 0;
    };

    struct Job {
        enum Kind { Analyze, Launch } kind;
        Slot *slot;
        int P = 1, iterations = 0;
    };

  public:
    Server(B backend, const arap_server_config &cfg) : b_(std::move(backend)), cfg_(cfg) {
        if (cfg_.max_in_flight <= 0) cfg_.max_in_flight = 8;
        if (cfg_.prep_threads <= 0) cfg_.prep_threads = 4;
        if (cfg_.max_batch <= 0) cfg_.max_batch = 64;
        if (cfg_.max_queue <= 0) cfg_.max_queue = 65536;
        if (cfg_.poll_us <= 0) cfg_.poll_us = 20;
        if (cfg_.precision != ARAP_PRECISION_MIXED) cfg_.max_batch = 1;  // multi-pose launches are MIXED only
        budget_ = cfg_.device_budget_bytes > 0 ? cfg_.device_budget_bytes : b_.default_budget();
        sched_ = std::thread([this] { scheduler_loop(); });
        for (int i = 0; i < cfg_.prep_threads; ++i) workers_.emplace_back([this] { worker_loop(); });
    }

    ~Server() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        sched_.join();
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_workers_ = true;
        }
        cv_jobs_.notify_all();
        for (auto &t : workers_) t.join();
        for (auto &kv : slots_) destroy_slot_resources(kv.get());
        slots_.clear();
        for (auto &m : meshes_) b_.destroy(m->proto);
        for (Req *q : pending_) delete q;
        for (auto &kv : tickets_) delete kv.second;
        for (auto &pv : staging_pool_)
            for (double *p : pv.second) b_.free_host(p);
    }


    int add_mesh(int V, int F, const int32_t *faces, const double *rest, int32_t *id) {
        if (V < 0 || F < 0 || !id || (V > 0 && !rest) || (F > 0 && !faces)) return fail("invalid mesh arrays");
        auto m = std::make_unique<MeshRec>();
        m->V = V;
        m->F = F;
        m->rest.assign(rest, rest + (size_t)3 * V);
        int rc = b_.create(V, F, faces, &m->proto);
        if (rc != ARAP_OK) return fail_rc(rc, "mesh context: " + b_.last_error(Handle{}));
        rc = b_.set_precision(m->proto, cfg_.precision, cfg_.refine_steps);
        if (rc == ARAP_OK) rc = b_.set_solve_ctas(m->proto, cfg_.solve_ctas);
        if (rc == ARAP_OK)
            rc = b_.set_ordering(m->proto, cfg_.per_set_ordering ? ARAP_ORDER_PER_CONSTRAINT_SET : ARAP_ORDER_MESH);
        if (rc == ARAP_OK) rc = b_.set_rest(m->proto, rest);
        if (rc != ARAP_OK) {
            const std::string e = b_.last_error(m->proto);
            b_.destroy(m->proto);
            return fail_rc(rc, e);
        }
        m->bytes = b_.device_bytes(m->proto);
        std::lock_guard<std::mutex> lk(mu_);
        meshes_.push_back(std::move(m));
        mesh_bytes_ += meshes_.back()->bytes;
        *id = (int32_t)meshes_.size() - 1;
        return ARAP_OK;
    }

    int submit(const arap_request *r, int64_t *ticket) {
        if (!r || !ticket) return fail("null request");
        const MeshRec *m = nullptr;
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (r->mesh < 0 || r->mesh >= (int)meshes_.size()) return fail("unknown mesh id");
            m = meshes_[r->mesh].get();
        }
        if (r->n_constraints < 0 || r->iterations < 0 || !r->out_xyz ||
            (r->n_constraints > 0 && (!r->indices || !r->targets)))
            return fail("invalid request arrays");
        auto q = std::make_unique<Req>();
        q->mesh = r->mesh;
        q->iterations = r->iterations;
        q->out = r->out_xyz;
        // map semantics of setConstraint: the last target of a vertex wins
        std::vector<std::pair<int32_t, int32_t>> order;
        order.reserve(r->n_constraints);
        for (int i = 0; i < r->n_constraints; ++i) {
            const int32_t v = r->indices[i];
            if (v < 0 || v >= m->V)
                return fail_rc(ARAP_ERR_BAD_INDEX, "constraint index " + std::to_string(v) + " outside [0, " +
                                                       std::to_string(m->V) + ")");
            order.push_back({v, i});
        }
        std::stable_sort(order.begin(), order.end());
        for (size_t i = 0; i < order.size(); ++i) {
            if (i + 1 < order.size() && order[i + 1].first == order[i].first) continue;
            q->idx.push_back(order[i].first);
            const double *t = r->targets + 3 * (size_t)order[i].second;
            q->tgt.insert(q->tgt.end(), t, t + 3);
        }
        q->key = hash_key(q->mesh, q->idx);
        q->t_submit = Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (queued_ >= cfg_.max_queue) {
                ++st_.refused;
                return fail_rc(ARAP_ERR_ADMISSION_REFUSED, "request queue full");
            }
            q->ticket = next_ticket_++;
            *ticket = q->ticket;
            ++st_.submitted;
            ++queued_;
            tickets_[q->ticket] = q.get();
            incoming_.push_back(q.release());
        }
        cv_.notify_all();
        return ARAP_OK;
    }

    int poll(int64_t ticket, arap_request_info *info) { return wait(ticket, 0, info); }

    int wait(int64_t ticket, int timeout_ms, arap_request_info *info) {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = tickets_.find(ticket);
        if (it == tickets_.end()) return fail_locked("unknown ticket " + std::to_string(ticket));
        Req *q = it->second;
        auto done = [&] { return q->status != ARAP_PENDING; };
        if (timeout_ms < 0) cv_done_.wait(lk, done);
        else if (timeout_ms > 0) cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
        if (!done()) return ARAP_PENDING;
        const int rc = q->status;
        if (info) {
            info->status = rc;
            info->factor_reused = q->factor_reused;
            info->batch_size = q->batch;
            info->pad = 0;
            info->queue_ms = ms_between(q->t_submit, q->t_launch);
            info->latency_ms = ms_between(q->t_submit, q->t_done);
        }
        if (rc != ARAP_OK) thread_error() = q->error;
        tickets_.erase(it);
        delete q;
        return rc;
    }

    void stats(arap_server_stats *s) {
        std::lock_guard<std::mutex> lk(mu_);
        *s = st_;
        s->budget_bytes = budget_;
    }

  private:
    // ---- helpers -------------------------------------------------------
    int fail(const std::string &msg) { return fail_rc(ARAP_ERR_INVALID_ARGUMENT, msg); }
    int fail_rc(int rc, const std::string &msg) {
        thread_error() = msg;
        return rc;
    }
    int fail_locked(const std::string &msg) { return fail_rc(ARAP_ERR_INVALID_ARGUMENT, msg); }

    MeshRec *mesh_at(int i) {
        std::lock_guard<std::mutex> lk(mu_);
        return meshes_[i].get();
    }

    static uint64_t hash_key(int mesh, const std::vector<int32_t> &idx) {
        uint64_t h = 1469598103934665603ull ^ (uint64_t)(uint32_t)mesh;
        for (int32_t v : idx) {
            h ^= (uint64_t)(uint32_t)v;
            h *= 1099511628211ull;
        }
        return h;
    }

    Slot *find_slot(const Req *q) {
        auto it = cache_.find(q->key);
        if (it == cache_.end()) return nullptr;
        for (Slot *s : it->second)
            if (s->mesh == q->mesh && s->idx == q->idx) return s;
        return nullptr;
    }

    double *staging_get(size_t doubles) {
        size_t cls = 1024;
        while (cls < doubles) cls <<= 1;
        auto &v = staging_pool_[cls];
        if (!v.empty()) {
            double *p = v.back();
            v.pop_back();
            return p;
        }
        const auto t0 = Clock::now();
        double *p = static_cast<double *>(b_.alloc_host(cls * sizeof(double)));
        std::lock_guard<std::mutex> lk(mu_);
        st_.staging_ms += ms_between(t0, Clock::now());
        return p;
    }
    void staging_put(double *p, size_t doubles) {
        if (!p) return;
        size_t cls = 1024;
        while (cls < doubles) cls <<= 1;
        staging_pool_[cls].push_back(p);
    }

    bool ensure_staging(Slot *s, size_t doubles) {
        if (s->staging && s->staging_doubles >= doubles) return true;
        staging_put(s->staging, s->staging_doubles);
        size_t cls = 1024;
        while (cls < doubles) cls <<= 1;
        s->staging = staging_get(doubles);
        s->staging_doubles = s->staging ? cls : 0;
        return s->staging != nullptr;
    }

    void destroy_slot_resources(Slot *s) {
        if (s->have_ctx) b_.destroy(s->ctx);
        s->have_ctx = false;
        staging_put(s->staging, s->staging_doubles);
        s->staging = nullptr;
    }

    void set_resident() {
        int64_t r = mesh_bytes_, f = 0;
        for (auto &s : slots_) {
            r += s->bytes + s->reserved;
            f += s->built ? 1 : 0;
        }
        resident_ = r;
        std::lock_guard<std::mutex> lk(mu_);
        st_.resident_bytes = r;
        st_.peak_resident_bytes = std::max(st_.peak_resident_bytes, r);
        st_.resident_factors = (int32_t)f;
    }

    void finish(Req *q, int rc, const std::string &err) {
        q->t_done = Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu_);
            q->error = err;
            q->status = rc;
            --queued_;
            if (rc == ARAP_OK) {
                ++st_.completed;
                st_.iterations_done += q->iterations;
            } else if (rc == ARAP_ERR_ADMISSION_REFUSED) {
                ++st_.refused;
            } else {
                ++st_.failed;
            }
        }
        cv_done_.notify_all();
    }

    void remove_slot(Slot *s) {
        auto &v = cache_[s->key];
        v.erase(std::remove(v.begin(), v.end(), s), v.end());
        if (v.empty()) cache_.erase(s->key);
        // destroying the context waits for its stream, so a completion
        // callback of it has run by now: drop any notice it left
        destroy_slot_resources(s);
        notified_.erase(std::remove(notified_.begin(), notified_.end(), s), notified_.end());
        {
            std::lock_guard<std::mutex> lk(mu_);
            done_slots_.erase(std::remove(done_slots_.begin(), done_slots_.end(), s), done_slots_.end());
        }
        for (auto it = slots_.begin(); it != slots_.end(); ++it)
            if (it->get() == s) {
                slots_.erase(it);
                break;
            }
        set_resident();
    }

    void fail_key(Slot *s, int rc, const std::string &err) {
        for (Req *q : s->waiting) {
            q->t_launch = Clock::now();
            finish(q, rc, err);
        }
        s->waiting.clear();
    }

    // ---- launches ----------------------------------------------------------
    // Takes the oldest waiting request of slot s and the others that can share
    // its launch (same iteration count), at most max_p, oldest first.
    std::vector<Req *> take_batch(Slot *s, int max_p) {
        std::vector<Req *> batch;
        const int iters = s->waiting.front()->iterations;
        for (auto it = s->waiting.begin(); it != s->waiting.end() && (int)batch.size() < max_p;) {
            if ((*it)->iterations == iters) {
                batch.push_back(*it);
                it = s->waiting.erase(it);
            } else {
                ++it;
            }
        }
        return batch;
    }

    // requests of slot s that could share a launch with its oldest one
    static int batchable(const Slot *s) {
        if (s->waiting.empty()) return 0;
        const int iters = s->waiting.front()->iterations;
        int n = 0;
        for (const Req *q : s->waiting) n += q->iterations == iters;
        return n;
    }

    // Enqueues the launch of s->running (host work only; the device runs it).
    // Staging and batch targets are prepared by the scheduler (start).
    int launch(Slot *s, std::string &err) {
        const int P = (int)s->running.size();
        const int iters = s->running[0]->iterations;
        const auto t0 = Clock::now();
        int rc;
        if (P == 1) {
            const Req *q = s->running[0];
            rc = b_.set_targets(s->ctx, (int)q->idx.size(), q->tgt.data());
            if (rc == ARAP_OK) rc = b_.deform_async(s->ctx, iters, s->staging);
        } else {
            rc = b_.deform_poses_async(s->ctx, P, s->batch_targets.data(), iters, s->staging);
        }
        if (rc != ARAP_OK) err = b_.last_error(s->ctx);
        double ph[5] = {0, 0, 0, 0, 0};
        if (rc == ARAP_OK) b_.host_timing(s->ctx, ph);
        const double ms = ms_between(t0, Clock::now());
        std::lock_guard<std::mutex> lk(mu_);
        st_.launch_ms += ms;
        for (int i = 0; i < 5; ++i) st_.launch_host_ms[i] += ph[i];
        return rc;
    }

    void start(Slot *s, std::vector<Req *> batch, bool on_worker) {
        const auto now = Clock::now();
        const bool reused = s->built;
        for (Req *q : batch) {
            q->t_launch = now;
            q->factor_reused = reused ? 1 : 0;
            q->batch = (int)batch.size();
        }
        s->running = std::move(batch);
        const int P = (int)s->running.size();
        ++inflight_;
        {
            std::lock_guard<std::mutex> lk(mu_);
            ++st_.launches;
            if (reused) st_.factor_hits += P;
            else st_.factor_misses += P;
            if (P > 1) {
                ++st_.batched_launches;
                st_.batched_requests += P;
            }
            st_.in_flight = inflight_;
        }
        if (!ensure_staging(s, (size_t)P * mesh_at(s->mesh)->V * 3)) {
            if (on_worker) --busy_jobs_;
            launch_failed(s, ARAP_ERR_OUT_OF_MEMORY, "pinned staging allocation failed");
            return;
        }
        s->batch_targets.clear();
        if (P > 1)
            for (const Req *q : s->running) s->batch_targets.insert(s->batch_targets.end(), q->tgt.begin(), q->tgt.end());
        if (on_worker) {
            s->state = SlotState::Launching;
            post_job({Job::Launch, s, P, s->running[0]->iterations});
            return;
        }
        std::string err;
        const int rc = launch(s, err);
        if (rc != ARAP_OK) {
            launch_failed(s, rc, err);
            return;
        }
        s->state = SlotState::Busy;
    }

    void launch_failed(Slot *s, int rc, const std::string &err) {
        for (Req *q : s->running) finish(q, rc, err);
        s->running.clear();
        --inflight_;
        s->reserved = 0;
        fail_key(s, rc, err);
        remove_slot(s);
    }

    // ---- worker threads ----------------------------------------------------
    void post_job(Job j) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            jobs_.push_back(j);
        }
        cv_jobs_.notify_one();
    }

    void worker_loop() {
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_jobs_.wait(lk, [&] { return stop_workers_ || !jobs_.empty(); });
                if (jobs_.empty()) return;
                j = jobs_.front();
                jobs_.pop_front();
            }
            Slot *s = j.slot;
            int rc = ARAP_OK;
            std::string err;
            const auto tw0 = Clock::now();
            if (j.kind == Job::Analyze) {
                const MeshRec &m = *mesh_at(s->mesh);
                Handle h{};
                rc = b_.create_like(m.proto, &h);
                if (rc != ARAP_OK) {
                    err = b_.last_error(Handle{});
                } else {
                    s->ctx = h;
                    s->have_ctx = true;
                    if (B::kCallbacks) {
                        s->tag = {this, s};
                        b_.set_done_callback(h, &Server::on_done, &s->tag);
                    }
                    std::vector<double> tgt(3 * s->idx.size());
                    for (size_t i = 0; i < s->idx.size(); ++i)
                        std::memcpy(&tgt[3 * i], &m.rest[3 * (size_t)s->idx[i]], 3 * sizeof(double));
                    rc = b_.set_constraints(h, (int)s->idx.size(), s->idx.data(), tgt.data());
                    int64_t need = 0;
                    if (rc == ARAP_OK) rc = b_.plan_bytes(h, 0, &need);
                    if (rc != ARAP_OK) err = b_.last_error(h);
                    s->job_need = need;
                    s->job_bytes = b_.device_bytes(h);
                }
            } else {
                rc = launch(s, err);
            }
            s->job_rc = rc;
            s->job_err = err;
            {
                std::lock_guard<std::mutex> lk(mu_);
                st_.worker_busy_ms += ms_between(tw0, Clock::now());
                if (j.kind == Job::Analyze) st_.analyze_ms += ms_between(tw0, Clock::now());
                done_jobs_.push_back(j);
            }
            cv_.notify_all();
        }
    }

    void job_done(const Job &j) {
        Slot *s = j.slot;
        --busy_jobs_;
        if (j.kind == Job::Analyze) {
            s->reserved = 0;
            s->need = s->job_need;
            s->bytes = s->job_bytes;
            if (s->job_rc != ARAP_OK) {
                fail_key(s, s->job_rc, s->job_err);
                remove_slot(s);
                return;
            }
            s->state = SlotState::Ready;
            set_resident();
            return;
        }
        if (s->job_rc != ARAP_OK) {
            launch_failed(s, s->job_rc, s->job_err);
            return;
        }
        s->state = SlotState::Busy;
    }

    // ---- completion ----------------------------------------------------------
    // Completion callback (a CUDA runtime thread): queue the slot for the scheduler.
    static void on_done(void *user) {
        auto *t = static_cast<typename Slot::Tag *>(user);
        {
            std::lock_guard<std::mutex> lk(t->srv->mu_);
            t->srv->done_slots_.push_back(t->slot);
        }
        t->srv->cv_.notify_all();
    }

    // Collects finished launches: the slots the completion callbacks named
    // (a notification that arrives before its launch job is marked done waits
    // for the next round), and every busy slot when there are no callbacks or
    // a full check is due.
    void poll_busy(bool full) {
        std::vector<Slot *> check;
        if (full) {
            for (auto &p : slots_)
                if (p->state == SlotState::Busy) check.push_back(p.get());
            notified_.clear();
        } else {
            std::vector<Slot *> keep;
            for (Slot *s : notified_) {
                if (s->state == SlotState::Busy) check.push_back(s);
                else if (s->state == SlotState::Launching) keep.push_back(s);
            }
            notified_.swap(keep);
        }
        for (Slot *s : check) {
            if (s->state != SlotState::Busy) continue;
            int32_t done = 0;
            const int rc = b_.query(s->ctx, &done);
            if (!done && rc == ARAP_OK) continue;
            const std::string err = rc == ARAP_OK ? std::string() : b_.last_error(s->ctx);
            const int V = mesh_at(s->mesh)->V;
            if (rc == ARAP_OK) {
                const double dms = b_.device_ms(s->ctx);
                std::lock_guard<std::mutex> lk(mu_);
                st_.device_ms += dms;
            }
            for (size_t p = 0; p < s->running.size(); ++p) {
                Req *q = s->running[p];
                if (rc == ARAP_OK)
                    std::memcpy(q->out, s->staging + p * (size_t)V * 3, (size_t)V * 3 * sizeof(double));
                finish(q, rc, err);
            }
            s->running.clear();
            --inflight_;
            s->reserved = 0;
            s->last_used = Clock::now();
            if (rc == ARAP_OK) {
                s->built = true;
                s->state = SlotState::Idle;
                s->bytes = b_.device_bytes(s->ctx);
                set_resident();
            } else {
                // a failed factorisation (or an expired wait) leaves nothing worth keeping
                fail_key(s, rc, err);
                remove_slot(s);
            }
        }
        std::lock_guard<std::mutex> lk(mu_);
        st_.in_flight = inflight_;
    }

    // ---- admission -------------------------------------------------------------
    // Frees idle contexts, least recently used first, that no waiting request
    // needs, until `extra` more bytes fit the budget. True when they fit.
    bool make_room(int64_t extra, const Slot *keep) {
        while (resident_ + extra > budget_) {
            Slot *victim = nullptr;
            for (auto &p : slots_) {
                Slot *s = p.get();
                if (s == keep || s->state != SlotState::Idle || !s->waiting.empty()) continue;
                if (!victim || s->last_used < victim->last_used) victim = s;
            }
            if (!victim) return false;
            {
                std::lock_guard<std::mutex> lk(mu_);
                ++st_.evictions;
            }
            remove_slot(victim);
        }
        return true;
    }

    // Device bytes a launch of P requests on s adds to what s holds now.
    int64_t launch_extra(Slot *s, int P) {
        int64_t need = s->need;
        if (P > 1 && b_.plan_bytes(s->ctx, P, &need) != ARAP_OK) return -1;
        return std::max<int64_t>(0, std::max(need, s->need) - s->bytes);
    }

    void schedule() {
        // attach new requests to their constraint set's slot, creating (and
        // analysing) a slot for a set not seen yet
        for (auto it = pending_.begin(); it != pending_.end();) {
            Req *q = *it;
            const MeshRec &m = *mesh_at(q->mesh);
            if (q->idx.empty()) {
                // deform() without constraints returns without touching the mesh (arap.h:113-114)
                q->t_launch = Clock::now();
                std::memcpy(q->out, m.rest.data(), m.rest.size() * sizeof(double));
                finish(q, ARAP_OK, std::string());
                it = pending_.erase(it);
                continue;
            }
            Slot *s = find_slot(q);
            if (!s) {
                if (unlaunched_slots() >= 2 * cfg_.prep_threads) {
                    ++it;
                    continue;
                }
                // the new context copies the mesh's topology: room for that first
                const int64_t topo = m.bytes;
                if (resident_ + topo > budget_ && !make_room(topo, nullptr)) {
                    if (mesh_bytes_ + topo > budget_ || quiescent()) {
                        q->t_launch = Clock::now();
                        finish(q, ARAP_ERR_ADMISSION_REFUSED, "the mesh's topology alone does not fit the budget");
                        it = pending_.erase(it);
                        continue;
                    }
                    ++it;
                    continue;
                }
                auto ns = std::make_unique<Slot>();
                ns->mesh = q->mesh;
                ns->idx = q->idx;
                ns->key = q->key;
                ns->order = next_order_++;
                ns->state = SlotState::Analyzing;
                ns->reserved = topo;
                s = ns.get();
                cache_[s->key].push_back(s);
                slots_.push_back(std::move(ns));
                set_resident();
                ++busy_jobs_;
                post_job({Job::Analyze, s, 0, 0});
            }
            q->slot = s;
            s->waiting.push_back(q);
            it = pending_.erase(it);
        }
        // resident constraint sets with waiting requests, oldest request first
        std::vector<Slot *> idle;
        for (auto &p : slots_)
            if (p->state == SlotState::Idle && !p->waiting.empty()) idle.push_back(p.get());
        std::sort(idle.begin(), idle.end(),
                  [](const Slot *a, const Slot *b) { return a->waiting.front()->ticket < b->waiting.front()->ticket; });
        for (Slot *s : idle) {
            if (inflight_ >= cfg_.max_in_flight) break;
            int P = std::min(batchable(s), cfg_.max_batch);
            int64_t extra = 0;
            while (P > 1) {
                extra = launch_extra(s, P);
                if (extra >= 0 && (resident_ + extra <= budget_ || make_room(extra, s))) break;
                P /= 2;
                extra = 0;
            }
            if (P <= 1) {
                P = 1;
                extra = 0;
            }
            s->reserved = extra;
            resident_ += extra;
            start(s, take_batch(s, P), false);
        }
        // first launches of analysed constraint sets, first come first served;
        // the oldest one that does not fit holds back the later ones
        std::vector<Slot *> ready;
        for (auto &p : slots_)
            if (p->state == SlotState::Ready) ready.push_back(p.get());
        std::sort(ready.begin(), ready.end(), [](const Slot *a, const Slot *b) { return a->order < b->order; });
        for (Slot *s : ready) {
            if (inflight_ >= cfg_.max_in_flight) break;
            if (s->waiting.empty()) {
                remove_slot(s);
                continue;
            }
            int P = std::min(batchable(s), cfg_.max_batch);
            int64_t extra = launch_extra(s, P);
            if (extra < 0) {
                P = 1;
                extra = launch_extra(s, 1);
            }
            if (resident_ + extra > budget_ && !make_room(extra, s)) {
                if (P > 1) {
                    P = 1;
                    extra = launch_extra(s, 1);
                    if (resident_ + extra <= budget_ || make_room(extra, s)) goto admit;
                }
                if (mesh_bytes_ + s->bytes + extra > budget_ || quiescent()) {
                    // can never fit, or nothing running will free memory
                    fail_key(s, ARAP_ERR_ADMISSION_REFUSED,
                             "planned device footprint of " + std::to_string(s->bytes + extra) +
                                 " bytes does not fit the budget of " + std::to_string(budget_) + " bytes");
                    remove_slot(s);
                    continue;
                }
                break;
            }
        admit:
            s->reserved = extra;
            resident_ += extra;
            ++busy_jobs_;
            start(s, take_batch(s, P), true);
        }
    }

    int unlaunched_slots() const {
        int n = 0;
        for (auto &p : slots_) n += p->state == SlotState::Analyzing || p->state == SlotState::Ready;
        return n;
    }

    // Nothing runs or waits to run that could free device memory later.
    bool quiescent() const {
        if (inflight_ > 0 || busy_jobs_ > 0) return false;
        for (auto &p : slots_)
            if (p->state == SlotState::Idle && !p->waiting.empty()) return false;
        return true;
    }

    bool has_work() const {
        if (!pending_.empty() || inflight_ > 0 || busy_jobs_ > 0) return true;
        for (auto &p : slots_)
            if (!p->waiting.empty()) return true;
        return false;
    }

    void scheduler_loop() {
        for (;;) {
            std::deque<Req *> fresh;
            std::deque<Job> finished;
            bool stopping;
            {
                std::unique_lock<std::mutex> lk(mu_);
                auto ready = [&] {
                    return stop_ || !incoming_.empty() || !done_jobs_.empty() || !done_slots_.empty();
                };
                // with completion callbacks the scheduler sleeps until one
                // arrives (checking every busy slot now and then regardless)
                const auto wait = B::kCallbacks ? std::chrono::microseconds(2000)
                                                : std::chrono::microseconds(cfg_.poll_us);
                if (inflight_ > 0) cv_.wait_for(lk, wait, ready);
                else if (!ready()) cv_.wait(lk, ready);
                fresh.swap(incoming_);
                finished.swap(done_jobs_);
                notified_.insert(notified_.end(), done_slots_.begin(), done_slots_.end());
                done_slots_.clear();
                stopping = stop_;
            }
            const auto t0 = Clock::now();
            for (Req *q : fresh) pending_.push_back(q);
            for (const Job &j : finished) job_done(j);
            const bool full = !B::kCallbacks || t0 - last_full_poll_ > std::chrono::milliseconds(2);
            if (full) last_full_poll_ = t0;
            poll_busy(full);
            schedule();
            {
                int waiting = (int)pending_.size();
                for (auto &p : slots_) waiting += (int)p->waiting.size();
                std::lock_guard<std::mutex> lk(mu_);
                st_.queue_depth = waiting;
                st_.scheduler_busy_ms += ms_between(t0, Clock::now());
            }
            if (stopping && !has_work()) {
                std::lock_guard<std::mutex> lk(mu_);
                if (incoming_.empty()) return;
            }
        }
    }

    B b_;
    arap_server_config cfg_;
    int64_t budget_ = 0;
    // shared with clients and workers (mu_)
    std::mutex mu_;
    std::condition_variable cv_, cv_done_, cv_jobs_;
    bool stop_ = false, stop_workers_ = false;
    std::vector<std::unique_ptr<MeshRec>> meshes_;
    std::deque<Req *> incoming_;
    std::deque<Job> jobs_, done_jobs_;
    std::vector<Slot *> done_slots_;  // named by completion callbacks
    std::unordered_map<int64_t, Req *> tickets_;
    int64_t next_ticket_ = 1;
    int queued_ = 0;
    arap_server_stats st_{};
    // scheduler thread only
    std::list<Req *> pending_;
    std::vector<std::unique_ptr<Slot>> slots_;
    std::unordered_map<uint64_t, std::vector<Slot *>> cache_;
    std::vector<Slot *> notified_;  // finished according to a callback, not collected yet
    Clock::time_point last_full_poll_{};
    std::map<size_t, std::vector<double *>> staging_pool_;
    int64_t resident_ = 0;
    std::atomic<int64_t> mesh_bytes_{0};
    int inflight_ = 0, busy_jobs_ = 0;
    uint64_t next_order_ = 0;
    std::thread sched_;
    std::vector<std::thread> workers_;
};

}  // namespace arapsrv
