// multi.cu -- many independent scenes stepped together.
//
// One Solver per scene, each with its own stream, device buffers and
// Newton-iteration graph, stepped by a pool of host threads: while one
// thread waits on its scene's status copy the others' scenes run, so the
// scenes' launches overlap on the device (a small scene's PCG runs as one
// thread-block cluster, a few SMs, beside the others'). The reference has no
// counterpart: its backend holds one scene per process.
#include "fatal.cuh"
#include "solver.cuh"
#include "stats.cuh"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

struct PpfMulti {
    std::vector<std::unique_ptr<ppf::gpu::Solver>> solvers;
    unsigned threads = 1;
};

namespace {

// A host that loads the library before it touches CUDA (the solver
// executable, a C program) gets 32 hardware work queues, so that the scenes'
// streams do not share queues (the CUDA default is 8); a value already in the
// environment is kept, and a context created earlier keeps its count.
__attribute__((constructor)) void more_work_queues() {
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

// f(i) for every i in [0, count) on up to `threads` host threads, each
// taking the next index when it is free. The first error any call raised is
// recorded as the library's fatal code and detail; returns 0 or -1.
template <class F> int run_all(unsigned count, unsigned threads, F &&f) {
    std::atomic<unsigned> next{0};
    std::atomic<bool> failed{false};
    std::mutex mu;
    unsigned char code = 0;
    std::string detail;
    auto fail = [&](unsigned char c, const char *d) {
        std::lock_guard<std::mutex> lock(mu);
        if (!failed.exchange(true)) {
            code = c;
            detail = d;
        }
    };
    auto work = [&]() {
        for (unsigned i = next++; i < count && !failed; i = next++) {
            try {
                f(i);
            } catch (const ppf::FatalError &e) {
                fail(e.code, e.what());
            } catch (const std::exception &e) {
                fail(3, e.what());
            }
        }
    };
    std::vector<std::thread> pool;
    const unsigned t = std::max(1u, std::min(threads, count));
    for (unsigned k = 1; k < t; ++k) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    if (!failed) return 0;
    ppf::set_fatal(code, detail.c_str());
    return -1;
}

// The PCG team of a scene stepped beside others: one cluster sized to the
// system (a few SMs each, so several scenes' solves run at once), the whole
// grid above 16,384 vertices.
int team_for(unsigned n) {
    if (n <= 2048) return 2;
    if (n <= 4096) return 4;
    if (n <= 8192) return 8;
    if (n <= 16384) return 16;
    return 0;
}

} // namespace

extern "C" {

PpfMulti *ppf_multi_create(unsigned count, PpfDataSet *const *datasets,
                           PpfParamSet *const *params, unsigned threads) {
    ppf::set_fatal(0, ""); // as initialize: a new handle starts without a fatal report
    if (!count || !datasets || !params) {
        ppf::set_fatal(5, "ppf_multi_create: no scenes");
        return nullptr;
    }
    std::unique_ptr<PpfMulti> m(new PpfMulti);
    m->threads = threads ? threads : 1;
    m->solvers.resize(count);
    for (auto &s : m->solvers) {
        s.reset(new ppf::gpu::Solver);
        s->blocking_sync_ = true;
    }
    const int rc = run_all(count, m->threads, [&](unsigned i) {
        ppf::gpu::Solver &s = *m->solvers[i];
        if (!s.initialize(datasets[i], params[i])) {
            char buf[96];
            snprintf(buf, sizeof(buf), "ppf_multi_create: scene %u did not initialize", i);
            throw ppf::FatalError(g_ppf_fatal_code ? g_ppf_fatal_code : 1, buf);
        }
        const int team = team_for(s.vertices());
        if (!s.set_pcg_team(team)) s.set_pcg_team(-1);
        // 512-thread CTAs: two solves share an SM (6,996 against 6,586
        // Newton iterations/s for the uneven drops with 1024-thread CTAs)
        s.set_pcg_cta_threads(512);
    });
    if (rc != 0) return nullptr;
    return m.release();
}

int ppf_multi_advance(PpfMulti *m, PpfStepResult *results) {
    if (!m) return -1;
    return run_all((unsigned)m->solvers.size(), m->threads, [&](unsigned i) {
        const PpfStepResult r = m->solvers[i]->advance();
        if (results) results[i] = r;
    });
}

int ppf_multi_update_constraint(PpfMulti *m, unsigned i, const PpfConstraint *constraint) {
    if (!m || i >= m->solvers.size()) return -1;
    try {
        m->solvers[i]->update_constraint(constraint);
        return 0;
    } catch (const ppf::FatalError &e) {
        ppf::set_fatal(e.code, e.what());
        return -1;
    }
}

int ppf_multi_fetch(PpfMulti *m, unsigned i) {
    if (!m || i >= m->solvers.size()) return -1;
    try {
        m->solvers[i]->fetch();
        return 0;
    } catch (const ppf::FatalError &e) {
        ppf::set_fatal(e.code, e.what());
        return -1;
    }
}

int ppf_multi_step_stats(PpfMulti *m, unsigned i, PpfStepStats *out) {
    if (!m || i >= m->solvers.size() || !out) return -1;
    ppf::gpu::fill_step_stats(*m->solvers[i], out);
    return 0;
}

int ppf_multi_set_pcg_team(PpfMulti *m, unsigned i, int ctas) {
    if (!m || i >= m->solvers.size()) return -1;
    return m->solvers[i]->set_pcg_team(ctas) ? 0 : -1;
}

int ppf_multi_set_pcg_cta_threads(PpfMulti *m, unsigned i, unsigned threads) {
    if (!m || i >= m->solvers.size()) return -1;
    return m->solvers[i]->set_pcg_cta_threads(threads) ? 0 : -1;
}

int ppf_multi_pcg_team(PpfMulti *m, unsigned i) {
    if (!m || i >= m->solvers.size()) return -1;
    return (int)m->solvers[i]->pcg_team();
}

void ppf_multi_destroy(PpfMulti *m) { delete m; }

} // extern "C"
