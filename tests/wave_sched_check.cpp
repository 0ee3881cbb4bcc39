// Exhaustive host check of the wavefront step's work order (elanfmt_gb300/csrc/ewfd_wave_sched.h),
// compiled with g++ by tests/test_wave_sched_cpu.py.  For each grid shape, slab depth and lag:
//   1. tickets [0, 2n) map one-to-one onto the n stress and n velocity items;
//   2. every dependency of a velocity item holds a smaller ticket (no deadlock);
//   3. stress planes tile [0, nz) once, velocity planes tile [1, nz) once;
//   4. every conflict between a stress item and a velocity item -- the stress item reads old
//      velocities the velocity item overwrites, or writes stresses it reads -- is covered by a
//      dependency.  Footprints follow stress_column / velocity_column at tile x plane
//      granularity: own tile over the z-neighbour planes, the four axis-neighbour tiles over
//      the item's own planes;
//   5. the owner of every source cell is a stress item whose tile and slab hold the cell, or,
//      for cells past the last tile, the item whose dependants read the cell.
// Prints "ok" or the first failure.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ewfd_wave_sched.h"

using namespace ewf;

static int fail(const char *what, int a, int b, int c)
{
    printf("FAIL %s %d %d %d\n", what, a, b, c);
    return 1;
}

struct Box {  // one tile (tx, ty), planes [k0, k1] inclusive
    int tx, ty, k0, k1;
};

static void stress_fp(const WaveShape &w, int nz, int idx, std::vector<Box> &vread, std::vector<Box> &swrite)
{
    const int tx = idx % w.ntx, ty = (idx / w.ntx) % w.nty, s = idx / w.ntx / w.nty;
    int k0, k1;
    wave_stress_planes(w, nz, s, k0, k1);
    vread.clear();
    swrite.clear();
    vread.push_back({tx, ty, k0 - 1, k1});  // Vx, Vy at k-1 and Vz at k+1 of the own column
    const int nb[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
    for (auto &d : nb) {
        const int ux = tx + d[0], uy = ty + d[1];
        if (ux >= 0 && ux < w.ntx && uy >= 0 && uy < w.nty) vread.push_back({ux, uy, k0, k1 - 1});
    }
    swrite.push_back({tx, ty, k0, k1 - 1});
    if (s == 0) swrite.push_back({tx, ty, 1, 1});  // BC1 copy to plane 1
}

static void velocity_fp(const WaveShape &w, int nz, int idx, std::vector<Box> &sread, std::vector<Box> &vwrite)
{
    const int tx = idx % w.ntx, ty = (idx / w.ntx) % w.nty, s = idx / w.ntx / w.nty;
    int kc0, kc1;
    wave_velocity_planes(w, nz, s, kc0, kc1);
    const int k0 = kc0 < 1 ? 1 : kc0, k1 = kc1;
    sread.clear();
    vwrite.clear();
    if (k0 >= k1) return;
    sread.push_back({tx, ty, k0 - 1, k1});  // szz at k-1, sxz / syz at k+1 of the own column
    const int nb[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
    for (auto &d : nb) {
        const int ux = tx + d[0], uy = ty + d[1];
        if (ux >= 0 && ux < w.ntx && uy >= 0 && uy < w.nty) sread.push_back({ux, uy, k0, k1 - 1});
    }
    vwrite.push_back({tx, ty, k0, k1 - 1});
}

static bool overlap(const Box &a, const Box &b)
{
    return a.tx == b.tx && a.ty == b.ty && a.k0 <= b.k1 && b.k0 <= a.k1;
}

static int check(int nx, int ny, int nz, int TXc, int TYc, int K, int lag)
{
    const WaveShape w = wave_shape(nx, ny, nz, TXc, TYc, K, lag);
    const int n = w.n;
    if (!(w.lag > w.ntx || w.lag == n)) return fail("lag", w.lag, w.ntx, n);
    std::vector<int> tk_s(n, -1), tk_v(n, -1);
    for (int t = 0; t < 2 * n; ++t) {
        int idx;
        bool vel;
        wave_decode(w, t, idx, vel);
        if (idx < 0 || idx >= n) return fail("decode range", t, idx, n);
        int &slot = vel ? tk_v[idx] : tk_s[idx];
        if (slot >= 0) return fail("decode twice", t, idx, vel);
        slot = t;
    }
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 10; ++d) {
            const int dep = wave_dep(w, i, d);
            if (dep >= n) return fail("dep range", i, d, dep);
            if (dep >= 0 && tk_s[dep] >= tk_v[i]) return fail("dep ticket", i, dep, tk_v[i]);
        }
    // plane coverage (per tile column: stress once over [0, nz), velocity once over [1, nz))
    std::vector<int> cs(nz + 2, 0), cv(nz + 2, 0);
    for (int s = 0; s < w.nslab; ++s) {
        int a, b;
        wave_stress_planes(w, nz, s, a, b);
        for (int k = a; k < b; ++k) cs[k]++;
        wave_velocity_planes(w, nz, s, a, b);
        for (int k = a < 1 ? 1 : a; k < b; ++k) cv[k]++;
    }
    for (int k = 0; k < nz; ++k) {
        if (cs[k] != 1) return fail("stress planes", k, cs[k], K);
        if (k >= 1 && cv[k] != 1) return fail("velocity planes", k, cv[k], K);
    }
    // conflicts covered by dependencies
    std::vector<Box> vr, sw, sr, vw;
    for (int v = 0; v < n; ++v) {
        velocity_fp(w, nz, v, sr, vw);
        int deps[10];
        for (int d = 0; d < 10; ++d) deps[d] = wave_dep(w, v, d);
        for (int s = 0; s < n; ++s) {
            stress_fp(w, nz, s, vr, sw);
            bool conflict = false;
            for (auto &x : vr)
                for (auto &y : vw) conflict = conflict || overlap(x, y);
            for (auto &x : sw)
                for (auto &y : sr) conflict = conflict || overlap(x, y);
            if (!conflict) continue;
            bool covered = false;
            for (int d = 0; d < 10; ++d) covered = covered || deps[d] == s;
            if (!covered) return fail("uncovered conflict", v, s, K);
        }
    }
    // source owners
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const int o = wave_owner(w, TXc, TYc, i, j, k);
                const int tx = o % w.ntx, ty = (o / w.ntx) % w.nty, s = o / w.ntx / w.nty;
                int k0, k1;
                wave_stress_planes(w, nz, s, k0, k1);
                const bool in_x = i / TXc == tx || (i / TXc >= w.ntx && tx == w.ntx - 1);
                const bool in_y = j / TYc == ty || (j / TYc >= w.nty && ty == w.nty - 1);
                const bool in_z = (k >= k0 && k < k1) || (k >= nz && s == w.nslab - 1);
                if (!(in_x && in_y && in_z)) return fail("owner", i, j, k);
            }
    return 0;
}

int main()
{
    const int shapes[][3] = {{64, 64, 64}, {96, 40, 37}, {33, 17, 9}, {320, 64, 50}, {32, 8, 4}, {40, 24, 130}};
    const int ks[] = {3, 4, 5, 6, 8, 16, 64};
    const int lags[] = {0, 1, 5, 11, 40, 100000};
    int cases = 0;
    for (auto &sh : shapes)
        for (int K : ks)
            for (int lag : lags) {
                if (check(sh[0], sh[1], sh[2], 32, 8, K, lag)) return 1;
                ++cases;
            }
    printf("ok %d\n", cases);
    return 0;
}
