// Randomised host simulation of the tcgen05 GEMM's mbarrier protocol (the parity functions of
// elanfmt_gb300/csrc/ewf_umma.h that the kernel uses), compiled with g++ by
// tests/test_umma_layout_cpu.py.  One CTA: the TMA producer, the MMA issuer and four epilogue
// warps over `tiles` tiles of `nk` k-stages, TMA copies completing in any order, MMA commits in
// issue order, all interleaved at random.  mbarriers are modelled by their completed-phase
// count n; a wait with parity P passes when n % 2 != P (so a fresh barrier passes parity 1).
// Checked: the run ends (no deadlock); the producer fills a slot only after the stage that last
// used it was consumed; the MMA issuer reads stage g exactly when its fill has landed and writes
// an accumulator only after the tile that last used it was drained; the epilogue reads tile i
// exactly when its MMAs are complete.  Prints "ok <runs>" or the first failure.
#include <cstdio>
#include <deque>
#include <random>
#include <vector>

#include "ewf_umma.h"

using namespace ewf_umma;

struct Bar {
    int n = 0;        // completed phases
    int arrived = 0;  // arrivals toward the current phase
    int need = 1;
    void arrive()
    {
        if (++arrived == need) {
            arrived = 0;
            ++n;
        }
    }
    bool pass(uint32_t parity) const { return (uint32_t)(n & 1) != parity; }
};

static const char *run(int tiles, int nk, unsigned seed)
{
    std::mt19937 rng(seed);
    Bar full[STAGES], empty[STAGES], acc_full[2], acc_empty[2];
    for (auto &b : acc_empty) b.need = 4;
    std::vector<int> fills(STAGES, 0), consumed(STAGES, 0);  // per slot: fills landed, stages consumed
    std::vector<int> tma_pending;                            // slots with a copy in flight
    std::deque<std::pair<int, int>> commits;                 // (kind 0 empty / 1 acc_full, index) in issue order
    int drained[2] = {0, 0}, computed[2] = {0, 0};
    // producer
    int p_g = 0, p_total = tiles * nk;
    // MMA issuer
    int m_tile = 0, m_kt = 0, m_g = 0;
    bool m_tile_open = false;
    // epilogue warps
    int e_tile[4] = {0, 0, 0, 0};
    long idle = 0;
    for (;;) {
        bool moved = false;
        const int who = (int)(rng() % 7);
        if (who == 0 && p_g < p_total) {  // producer: wait for a free slot, issue the copy
            const int s = ring_slot(p_g);
            if (!ring_needs_free(p_g) || empty[s].pass(ring_free_parity(p_g))) {
                if (consumed[s] != p_g / STAGES) return "producer refills a slot still in use";
                tma_pending.push_back(s);
                ++p_g;
                moved = true;
            }
        } else if (who == 1 && !tma_pending.empty()) {  // a copy lands (any order)
            const size_t q = rng() % tma_pending.size();
            const int s = tma_pending[q];
            tma_pending.erase(tma_pending.begin() + q);
            ++fills[s];
            full[s].arrive();
            moved = true;
        } else if (who == 2 && m_tile < tiles) {  // MMA issuer
            const int b = acc_buf(m_tile);
            if (!m_tile_open) {
                if (!acc_needs_free(m_tile) || acc_empty[b].pass(acc_free_parity(m_tile))) {
                    if (drained[b] != m_tile / 2) return "accumulator overwritten before it was drained";
                    m_tile_open = true;
                    moved = true;
                }
            } else {
                const int s = ring_slot(m_g);
                if (full[s].pass(ring_full_parity(m_g))) {
                    if (fills[s] != m_g / STAGES + 1) return "stage read before (or after a refill of) its copy";
                    commits.push_back({0, s});
                    ++m_g;
                    moved = true;
                    if (++m_kt == nk) {
                        commits.push_back({1, b});
                        m_kt = 0;
                        m_tile_open = false;
                        ++m_tile;
                    }
                }
            }
        } else if (who == 3 && !commits.empty()) {  // the oldest commit completes (tensor core in order)
            const auto c = commits.front();
            commits.pop_front();
            if (c.first == 0) {
                ++consumed[c.second];
                empty[c.second].arrive();
            } else {
                ++computed[c.second];
                acc_full[c.second].arrive();
            }
            moved = true;
        } else if (who >= 4) {  // an epilogue warp
            const int w = (int)(rng() % 4);
            const int i = e_tile[w];
            if (i < tiles) {
                const int b = acc_buf(i);
                if (acc_full[b].pass(acc_full_parity(i))) {
                    if (computed[b] != i / 2 + 1) return "epilogue read an accumulator before its MMAs completed";
                    ++e_tile[w];
                    // the last warp to drain tile i frees the buffer; count drains when all four arrived
                    const int before = acc_empty[b].n;
                    acc_empty[b].arrive();
                    if (acc_empty[b].n != before) ++drained[b];
                    moved = true;
                }
            }
        }
        const bool done = p_g == p_total && tma_pending.empty() && m_tile == tiles && commits.empty() &&
                          e_tile[0] == tiles && e_tile[1] == tiles && e_tile[2] == tiles && e_tile[3] == tiles;
        if (done) break;
        idle = moved ? 0 : idle + 1;
        if (idle > 100000) return "deadlock";
    }
    return nullptr;
}

int main()
{
    int runs = 0;
    unsigned seed = 1;
    for (int tiles = 1; tiles <= 7; ++tiles)
        for (int nk = 1; nk <= 9; ++nk)
            for (int rep = 0; rep < 20; ++rep) {
                const char *e = run(tiles, nk, seed++);
                if (e) {
                    printf("FAIL %s tiles %d nk %d seed %u\n", e, tiles, nk, seed - 1);
                    return 1;
                }
                ++runs;
            }
    printf("ok %d\n", runs);
    return 0;
}
