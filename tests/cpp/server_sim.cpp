// Scheduler tests of the deform server (mesh-deform_gb300/csrc/arap_server.h)
// over a host model of the device contexts: no GPU, no ARAP arithmetic. The
// model's "deform" finishes after a modelled time and writes the rest pose
// with the constrained vertices at their targets, so the tests can check that
// every request receives its own result. Exit status 0 when all checks pass.
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "arap_server.h"

#ifndef CALLBACKS
#define CALLBACKS 0
#endif

namespace {

using Clock = std::chrono::steady_clock;

struct FakeCtx {
    int V = 0;
    std::vector<double> rest;
    std::vector<int32_t> idx;
    std::vector<double> tgt;
    bool built = false;
    int64_t bytes = 0;
    bool in_flight = false;
    Clock::time_point t_done;
    double *out = nullptr;
    int P = 1;
    std::vector<double> ptgt;
    int pending_rc = ARAP_OK;
    std::string err;
    std::thread notifier;  // completion-callback thread of the last deform
    void (*fn)(void *) = nullptr;
    void *user = nullptr;
};

struct Model {
    std::mutex mu;
    int live = 0, in_flight = 0, max_in_flight = 0;
    int64_t device = 0, peak_device = 0;
};

// Device model: topology 64 B per vertex, a factor of 512 B per vertex, 256 B
// per vertex and pose for multi-pose launches; 50 us per iteration. A
// constraint set whose first vertex is V-1 is singular; 13 iterations make
// the deform fail with an expired wait. CB: completion callbacks from a
// thread of the model (as the CUDA runtime calls them), else polling only.
template <bool CB>
struct FakeBackendT {
    using Handle = FakeCtx *;
    static constexpr bool kCallbacks = CB;
    Model *m;

    void add_bytes(FakeCtx *c, int64_t b) {
        std::lock_guard<std::mutex> lk(m->mu);
        m->device += b - c->bytes;
        c->bytes = b;
        m->peak_device = std::max(m->peak_device, m->device);
    }
    int create(int V, int, const int32_t *, Handle *h) {
        auto *c = new FakeCtx();
        c->V = V;
        {
            std::lock_guard<std::mutex> lk(m->mu);
            ++m->live;
        }
        add_bytes(c, 64LL * V);
        *h = c;
        return ARAP_OK;
    }
    int create_like(Handle src, Handle *h) {
        int rc = create(src->V, 0, nullptr, h);
        (*h)->rest = src->rest;
        return rc;
    }
    void destroy(Handle h) {
        if (!h) return;
        if (h->notifier.joinable()) h->notifier.join();
        add_bytes(h, 0);
        std::lock_guard<std::mutex> lk(m->mu);
        --m->live;
        delete h;
    }
    int set_precision(Handle, int, int) { return ARAP_OK; }
    int set_solve_ctas(Handle, int) { return ARAP_OK; }
    int set_ordering(Handle, int) { return ARAP_OK; }
    int set_done_callback(Handle h, void (*fn)(void *), void *user) {
        h->fn = fn;
        h->user = user;
        return ARAP_OK;
    }
    int set_rest(Handle h, const double *xyz) {
        h->rest.assign(xyz, xyz + 3 * (size_t)h->V);
        return ARAP_OK;
    }
    int set_constraints(Handle h, int n, const int32_t *idx, const double *xyz) {
        h->idx.assign(idx, idx + n);
        h->tgt.assign(xyz, xyz + 3 * (size_t)n);
        h->built = false;
        return ARAP_OK;
    }
    int set_targets(Handle h, int n, const double *xyz) {
        if (n != (int)h->idx.size()) return ARAP_ERR_INVALID_ARGUMENT;
        h->tgt.assign(xyz, xyz + 3 * (size_t)n);
        return ARAP_OK;
    }
    int plan_bytes(Handle h, int P, int64_t *b) {
        if (!h->idx.empty() && h->idx[0] == h->V - 1) {
            h->err = "singular";
            return ARAP_ERR_NOT_SPD;
        }
        *b = 64LL * h->V + 512LL * h->V + 256LL * h->V * P;
        return ARAP_OK;
    }
    int64_t device_bytes(Handle h) { return h->bytes; }
    int begin(Handle h, int P, int iters, double *out) {
        int64_t need = 0;
        int rc = plan_bytes(h, P > 1 ? P : 0, &need);
        if (rc != ARAP_OK) return rc;
        add_bytes(h, std::max(h->bytes, need));
        h->in_flight = true;
        h->t_done = Clock::now() + std::chrono::microseconds(50 * iters + 200);
        h->out = out;
        h->P = P;
        h->pending_rc = iters == 13 ? ARAP_ERR_TIMEOUT : ARAP_OK;
        {
            std::lock_guard<std::mutex> lk(m->mu);
            ++m->in_flight;
            m->max_in_flight = std::max(m->max_in_flight, m->in_flight);
        }
        if (CB && h->fn) {
            if (h->notifier.joinable()) h->notifier.join();
            const auto when = h->t_done;
            auto fn = h->fn;
            void *user = h->user;
            h->notifier = std::thread([when, fn, user] {
                std::this_thread::sleep_until(when);
                fn(user);
            });
        }
        return ARAP_OK;
    }
    void host_timing(Handle, double *ms5) {
        for (int i = 0; i < 5; ++i) ms5[i] = 0.0;
    }
    int deform_async(Handle h, int iters, double *out) {
        h->ptgt = h->tgt;
        return begin(h, 1, iters, out);
    }
    int deform_poses_async(Handle h, int P, const double *tgt, int iters, double *out) {
        h->ptgt.assign(tgt, tgt + 3 * (size_t)P * h->idx.size());
        return begin(h, P, iters, out);
    }
    int query(Handle h, int32_t *done) {
        *done = 1;
        if (!h->in_flight) return ARAP_OK;
        if (Clock::now() < h->t_done) {
            *done = 0;
            return ARAP_OK;
        }
        h->in_flight = false;
        {
            std::lock_guard<std::mutex> lk(m->mu);
            --m->in_flight;
        }
        if (h->pending_rc != ARAP_OK) {
            h->err = "expired wait";
            return h->pending_rc;
        }
        const size_t n = h->idx.size();
        for (int p = 0; p < h->P; ++p) {
            double *o = h->out + (size_t)p * h->V * 3;
            std::copy(h->rest.begin(), h->rest.end(), o);
            for (size_t i = 0; i < n; ++i)
                for (int a = 0; a < 3; ++a) o[3 * (size_t)h->idx[i] + a] = h->ptgt[(p * n + i) * 3 + a];
        }
        h->built = true;
        return ARAP_OK;
    }
    std::string last_error(Handle h) { return h ? h->err : std::string("create failed"); }
    double device_ms(Handle) { return 0.05; }
    void *alloc_host(size_t b) { return ::operator new(b); }
    void free_host(void *p) { ::operator delete(p); }
    int64_t default_budget() { return 1LL << 40; }
};

int failures = 0;
using FakeBackend = FakeBackendT<CALLBACKS>;
#define CHECK(cond, what)                                                        \
    do {                                                                         \
        if (!(cond)) {                                                           \
            std::printf("FAIL %s (line %d): %s\n", what, __LINE__, #cond);       \
            ++failures;                                                          \
        }                                                                        \
    } while (0)

struct MeshData {
    int V;
    std::vector<int32_t> faces;
    std::vector<double> rest;
};

MeshData make_mesh(int V) {
    MeshData m;
    m.V = V;
    for (int i = 0; i + 2 < V; ++i) m.faces.insert(m.faces.end(), {i, i + 1, i + 2});
    for (int i = 0; i < V; ++i) m.rest.insert(m.rest.end(), {double(i), 0.5 * i, -double(i)});
    return m;
}

arap_server_config base_cfg() {
    arap_server_config c{};
    c.precision = ARAP_PRECISION_MIXED;
    c.refine_steps = 1;
    c.max_in_flight = 4;
    c.prep_threads = 2;
    c.poll_us = 10;
    return c;
}

struct Submitted {
    int64_t ticket;
    std::vector<double> out;
    std::vector<int32_t> idx;
    std::vector<double> tgt;
};

// expected output of the model for one request
bool result_ok(const MeshData &m, const Submitted &s) {
    for (int v = 0; v < m.V; ++v) {
        const double *e = &m.rest[3 * (size_t)v];
        double t[3] = {e[0], e[1], e[2]};
        for (size_t i = 0; i < s.idx.size(); ++i)
            if (s.idx[i] == v)
                for (int a = 0; a < 3; ++a) t[a] = s.tgt[3 * i + a];
        for (int a = 0; a < 3; ++a)
            if (s.out[3 * (size_t)v + a] != t[a]) return false;
    }
    return true;
}

int submit(arapsrv::Server<FakeBackend> &srv, int mesh, int V, Submitted &s, int iters, double seed) {
    s.out.assign(3 * (size_t)V, NAN);
    s.tgt.clear();
    for (size_t i = 0; i < s.idx.size(); ++i) s.tgt.insert(s.tgt.end(), {seed + i, seed - i, seed * 2});
    arap_request r{};
    r.mesh = mesh;
    r.n_constraints = (int)s.idx.size();
    r.indices = s.idx.data();
    r.targets = s.tgt.data();
    r.iterations = iters;
    r.out_xyz = s.out.data();
    return srv.submit(&r, &s.ticket);
}

void test_hits_and_results() {
    Model md;
    {
        arapsrv::Server<FakeBackend> srv(FakeBackend{&md}, base_cfg());
        MeshData m = make_mesh(200);
        int32_t id;
        CHECK(srv.add_mesh(m.V, (int)m.faces.size() / 3, m.faces.data(), m.rest.data(), &id) == ARAP_OK, "add_mesh");
        int hits = 0;
        for (int k = 0; k < 10; ++k) {
            Submitted s;
            s.idx = {3, 7, 50, 51};
            CHECK(submit(srv, id, m.V, s, 5, k) == ARAP_OK, "submit");
            arap_request_info info{};
            CHECK(srv.wait(s.ticket, -1, &info) == ARAP_OK, "wait");
            CHECK(result_ok(m, s), "sequential result");
            hits += info.factor_reused;
            CHECK(info.latency_ms >= info.queue_ms, "latency >= queue time");
        }
        CHECK(hits == 9, "first request builds the factor, the other nine reuse it");
        arap_server_stats st;
        srv.stats(&st);
        CHECK(st.completed == 10 && st.factor_misses == 1 && st.factor_hits == 9, "stats counters");
        CHECK(st.resident_factors == 1, "one resident factor");
        CHECK(st.iterations_done == 50, "iterations counted");
    }
    CHECK(md.live == 0 && md.device == 0, "everything released at destroy");
    std::printf("hits_and_results done\n");
}

void test_batching() {
    Model md;
    arap_server_config c = base_cfg();
    c.max_in_flight = 1;
    arapsrv::Server<FakeBackend> srv(FakeBackend{&md}, c);
    MeshData m = make_mesh(100);
    int32_t id;
    srv.add_mesh(m.V, (int)m.faces.size() / 3, m.faces.data(), m.rest.data(), &id);
    // warm the factor, then queue 8 requests while another one occupies the only slot
    std::vector<Submitted> subs(10);
    for (auto &s : subs) s.idx = {1, 2, 3};
    submit(srv, id, m.V, subs[0], 5, 0.0);
    srv.wait(subs[0].ticket, -1, nullptr);
    submit(srv, id, m.V, subs[1], 40, 1.0);  // long one
    std::this_thread::sleep_for(std::chrono::microseconds(300));
    for (int k = 2; k < 10; ++k) submit(srv, id, m.V, subs[k], 5, (double)k);
    int max_batch = 0;
    for (int k = 1; k < 10; ++k) {
        arap_request_info info{};
        CHECK(srv.wait(subs[k].ticket, -1, &info) == ARAP_OK, "batched wait");
        CHECK(result_ok(m, subs[k]), "batched result is the request's own");
        max_batch = std::max(max_batch, info.batch_size);
    }
    CHECK(max_batch == 8, "the eight queued requests ran as one launch");
    arap_server_stats st;
    srv.stats(&st);
    CHECK(st.batched_launches >= 1 && st.batched_requests >= 8, "batch counters");
    std::printf("batching done\n");
}

void test_admission_and_eviction() {
    Model md;
    arap_server_config c = base_cfg();
    const int V = 1000;
    // room for the mesh context and two factors: (64 + 576) B/vertex each
    c.device_budget_bytes = 64LL * V + 2 * (576LL * V) + 1000;
    c.max_batch = 1;
    arapsrv::Server<FakeBackend> srv(FakeBackend{&md}, c);
    MeshData m = make_mesh(V);
    int32_t id;
    srv.add_mesh(m.V, (int)m.faces.size() / 3, m.faces.data(), m.rest.data(), &id);
    for (int k = 0; k < 6; ++k) {
        Submitted s;
        s.idx = {k, k + 10, k + 20};
        submit(srv, id, V, s, 3, k);
        arap_request_info info{};
        CHECK(srv.wait(s.ticket, -1, &info) == ARAP_OK, "admitted after eviction");
        CHECK(result_ok(m, s), "result after eviction");
    }
    arap_server_stats st;
    srv.stats(&st);
    CHECK(st.evictions >= 4, "cold factors evicted to admit new ones");
    CHECK(st.peak_resident_bytes <= c.device_budget_bytes, "resident bytes never above the budget");
    CHECK(md.peak_device <= c.device_budget_bytes, "model device bytes never above the budget");
    // a constraint set on a mesh whose factor alone exceeds the budget is refused
    MeshData big = make_mesh(4000);
    int32_t idb;
    srv.add_mesh(big.V, (int)big.faces.size() / 3, big.faces.data(), big.rest.data(), &idb);
    Submitted s;
    s.idx = {0, 1};
    submit(srv, idb, big.V, s, 3, 1.0);
    CHECK(srv.wait(s.ticket, -1, nullptr) == ARAP_ERR_ADMISSION_REFUSED, "oversized request refused");
    std::printf("admission_and_eviction done\n");
}

void test_errors() {
    Model md;
    arapsrv::Server<FakeBackend> srv(FakeBackend{&md}, base_cfg());
    MeshData m = make_mesh(50);
    int32_t id;
    srv.add_mesh(m.V, (int)m.faces.size() / 3, m.faces.data(), m.rest.data(), &id);
    Submitted bad;
    bad.idx = {3, 99};
    CHECK(submit(srv, id, m.V, bad, 3, 0.0) == ARAP_ERR_BAD_INDEX, "bad index refused at submit");
    Submitted sing;
    sing.idx = {m.V - 1};
    submit(srv, id, m.V, sing, 3, 0.0);
    CHECK(srv.wait(sing.ticket, -1, nullptr) == ARAP_ERR_NOT_SPD, "singular set reported");
    Submitted to;
    to.idx = {4, 5};
    submit(srv, id, m.V, to, 13, 0.0);
    CHECK(srv.wait(to.ticket, -1, nullptr) == ARAP_ERR_TIMEOUT, "device error reported");
    Submitted ok;
    ok.idx = {4, 5};
    submit(srv, id, m.V, ok, 3, 2.0);
    CHECK(srv.wait(ok.ticket, -1, nullptr) == ARAP_OK && result_ok(m, ok), "server keeps working after errors");
    Submitted none;
    submit(srv, id, m.V, none, 3, 0.0);
    CHECK(srv.wait(none.ticket, -1, nullptr) == ARAP_OK && none.out == m.rest, "no constraints: rest pose back");
    CHECK(srv.wait(123456, 0, nullptr) == ARAP_ERR_INVALID_ARGUMENT, "unknown ticket");
    arap_server_config c = base_cfg();
    c.max_queue = 2;
    c.max_in_flight = 1;
    arapsrv::Server<FakeBackend> small(FakeBackend{&md}, c);
    small.add_mesh(m.V, (int)m.faces.size() / 3, m.faces.data(), m.rest.data(), &id);
    std::vector<Submitted> q(3);
    int refused = 0;
    for (auto &s : q) {
        s.idx = {1};
        const int rc = submit(small, id, m.V, s, 40, 1.0);
        refused += rc == ARAP_ERR_ADMISSION_REFUSED;
        if (rc != ARAP_OK) s.ticket = -1;
    }
    CHECK(refused == 1, "queue limit refuses the third waiting request");
    for (auto &s : q)
        if (s.ticket >= 0) CHECK(small.wait(s.ticket, -1, nullptr) == ARAP_OK, "queued requests finish");
    std::printf("errors done\n");
}

void test_concurrent_clients() {
    Model md;
    arap_server_config c = base_cfg();
    c.max_in_flight = 3;
    c.device_budget_bytes = 64LL * 900 + 6 * 576LL * 300;  // a handful of factors
    arapsrv::Server<FakeBackend> srv(FakeBackend{&md}, c);
    std::vector<MeshData> meshes = {make_mesh(300), make_mesh(200), make_mesh(400)};
    std::vector<int32_t> ids(3);
    for (int i = 0; i < 3; ++i)
        srv.add_mesh(meshes[i].V, (int)meshes[i].faces.size() / 3, meshes[i].faces.data(), meshes[i].rest.data(),
                     &ids[i]);
    std::atomic<int> bad{0}, done{0};
    std::vector<std::thread> th;
    for (int t = 0; t < 4; ++t)
        th.emplace_back([&, t] {
            for (int k = 0; k < 40; ++k) {
                const int mi = (t + k) % 3;
                Submitted s;
                s.idx = {k % 5, 10 + k % 3, 20};
                if (submit(srv, ids[mi], meshes[mi].V, s, 2 + k % 4, t * 100 + k) != ARAP_OK) {
                    ++bad;
                    continue;
                }
                if (srv.wait(s.ticket, -1, nullptr) != ARAP_OK || !result_ok(meshes[mi], s)) ++bad;
                ++done;
            }
        });
    for (auto &x : th) x.join();
    CHECK(bad == 0, "every concurrent request got its own result");
    CHECK(done == 160, "all concurrent requests completed");
    CHECK(md.max_in_flight <= 3, "never more launches in flight than max_in_flight");
    arap_server_stats st;
    srv.stats(&st);
    CHECK(st.completed == 160 && st.failed == 0, "stats after concurrent load");
    CHECK(st.peak_resident_bytes <= c.device_budget_bytes, "budget held under concurrent load");
    std::printf("concurrent_clients done (max in flight %d, evictions %lld)\n", md.max_in_flight,
                (long long)st.evictions);
}

}  // namespace

int main() {
    test_hits_and_results();
    test_batching();
    test_admission_and_eviction();
    test_errors();
    test_concurrent_clients();
    std::printf("completion callbacks: %d\n", CALLBACKS);
    std::printf(failures ? "FAILED %d\n" : "ALL PASSED\n", failures);
    return failures ? 1 : 0;
}
