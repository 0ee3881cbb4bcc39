// Randomised host simulation of the wavefront step's control loop (wave_control_step in
// elanfmt_gb300/csrc/ewfd_wave_sched.h, the code the device's control warp runs), compiled with
// g++ by tests/test_wave_sched_cpu.py.  CTAs start only while a resident slot is free (fewer
// slots than CTAs, as when other work occupies the GPU), their compute pipelines take random
// times per item, and control passes interleave at random.  Checked: the run ends (no
// deadlock, no wait gives up); every stress and velocity item runs exactly once; a stress item
// is published once, after it was written; a velocity item is handed over only when its ten
// dependencies are published; the compute side sees items in slot order; exactly one CTA draws
// the last ticket.  Prints "ok <runs>" or the first failure.
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <random>
#include <vector>

#include "ewfd_wave_sched.h"

using namespace ewf;

struct Sim;

struct Cta {
    WaveCtrl c;
    int written = 0;           // items completed by the compute side
    std::deque<int> queue;     // handed codes, in order
    int busy = 0;              // remaining work of the front item
    int next_slot = 0;         // slot the compute side expects next
    bool done = false, started = false;
    int dep_idx = -1;
};

struct Sim {
    WaveShape w;
    std::mt19937 rng;
    int ticket = 0;
    std::vector<int> published, ran_s, ran_v, written_s;
    int fails = 0, lasts = 0, last_owner_count = 0;
    const char *err = nullptr;
    int P;
};

struct Env {
    Sim &S;
    Cta &C;
    int draw() { return S.ticket++; }
    bool slot_done(int u) { return u < C.written; }
    void publish(int idx)
    {
        if (!S.written_s[idx]) S.err = "published before written";
        if (S.published[idx]) S.err = "published twice";
        S.published[idx] = 1;
    }
    void fetch_deps(int idx) { C.dep_idx = idx; }
    bool deps_ready()
    {
        for (int d = 0; d < 10; ++d) {
            const int q = wave_dep(S.w, C.dep_idx, d);
            if (q >= 0 && !S.published[q]) return false;
        }
        return true;
    }
    void fail() { S.fails++; }
    bool failed() { return S.fails > 0; }
    void handover(int slot, int code)
    {
        if (code < 0) {
            const int idx = -code - 1;
            for (int d = 0; d < 10; ++d) {
                const int q = wave_dep(S.w, idx, d);
                if (q >= 0 && !S.published[q]) S.err = "velocity handed before its dependencies";
            }
        }
        if (slot != (C.c.handed & 1)) S.err = "slot order";
        C.queue.push_back(code);
    }
    void finish(int, int last)
    {
        if (last == 2 * S.w.n + S.P - 1) S.last_owner_count++;
        if (last < 2 * S.w.n) S.err = "finish with a valid ticket";
        S.lasts++;
    }
};

static const char *run(int nx, int ny, int nz, int K, int lag, int P, int resident, unsigned seed)
{
    Sim S;
    S.w = wave_shape(nx, ny, nz, 32, 8, K, lag);
    S.rng.seed(seed);
    S.P = P;
    const int n = S.w.n;
    S.published.assign(n, 0);
    S.ran_s.assign(n, 0);
    S.ran_v.assign(n, 0);
    S.written_s.assign(n, 0);
    std::vector<Cta> ctas(P);
    int next_start = 0, active = 0, finished_ctas = 0;
    long long idle = 0;
    std::uniform_int_distribution<int> coin(0, 99);
    while (finished_ctas < P) {
        while (active < resident && next_start < P) {
            ctas[next_start++].started = true;
            ++active;
        }
        // a random started, unfinished CTA does one thing
        std::vector<int> live;
        for (int i = 0; i < next_start; ++i)
            if (!ctas[i].done || !ctas[i].queue.empty()) live.push_back(i);
        if (live.empty()) return "no live CTA";
        Cta &C = ctas[live[S.rng() % live.size()]];
        bool progress = false;
        if (coin(S.rng) < 50 && !C.done) {
            Env env{S, C};
            bool moved = false;
            if (wave_control_step(S.w, C.c, env, moved)) {
                C.done = true;
                progress = true;
            }
            progress = progress || moved;
        } else if (!C.queue.empty()) {
            if (C.busy == 0) C.busy = 1 + (int)(S.rng() % 4);
            if (--C.busy == 0) {
                const int code = C.queue.front();
                if (code >= 0) {
                    if (S.ran_s[code]++) return "stress item twice";
                    S.written_s[code] = 1;
                } else {
                    const int idx = -code - 1;
                    if (S.ran_v[idx]++) return "velocity item twice";
                }
                C.queue.pop_front();
                C.written++;
            }
            progress = true;
        }
        if (C.done && C.queue.empty() && C.started) {
            C.started = false;  // leaves its resident slot
            --active;
            ++finished_ctas;
        }
        if (S.err) return S.err;
        idle = progress ? 0 : idle + 1;
        if (idle > 200000) return "deadlock";
    }
    if (S.fails) return "a wait gave up";
    for (int i = 0; i < n; ++i) {
        if (S.ran_s[i] != 1) return "stress item not run once";
        if (S.ran_v[i] != 1) return "velocity item not run once";
        if (!S.published[i]) return "stress item not published";
    }
    if (S.lasts != P || S.last_owner_count != 1) return "end tickets";
    return nullptr;
}

int main()
{
    const int shapes[][3] = {{64, 64, 24}, {96, 40, 17}, {33, 17, 9}, {128, 64, 12}};
    const int ks[] = {3, 4, 6};
    const int lags[] = {0, 3, 20, 100000};
    const int ctas[][2] = {{1, 1}, {3, 2}, {16, 16}, {40, 8}, {200, 50}};
    int runs = 0;
    unsigned seed = 1;
    for (auto &sh : shapes)
        for (int K : ks)
            for (int lag : lags)
                for (auto &pc : ctas) {
                    const char *e = run(sh[0], sh[1], sh[2], K, lag, pc[0], pc[1], seed++);
                    if (e) {
                        printf("FAIL %s shape %dx%dx%d K %d lag %d ctas %d resident %d seed %u\n", e, sh[0], sh[1],
                               sh[2], K, lag, pc[0], pc[1], seed - 1);
                        return 1;
                    }
                    ++runs;
                }
    printf("ok %d\n", runs);
    return 0;
}
