// ewfd_wave_sched.h -- work order of the wavefront step (index arithmetic only; host and device).
//
// The wavefront step runs the stress and velocity updates of one time step in one persistent
// launch.  The grid is cut into items: a tile of TX x TY columns times a slab of K planes.
//   stress item   (s, ty, tx): sigma on planes [sK, min(sK + K, nz)) of the tile (+ its injections)
//   velocity item (s, ty, tx): V on planes [sK - 1, (s + 1)K - 1) of the tile (the last slab: to nz)
// The velocity slab lags one plane behind the stress slab, so velocity item s needs new stresses
// only from stress items s - 1 and s of its tile and its four axis neighbours (V(k) reads sigma
// at k - 1, k, k + 1 and at i - 1, i + 1, j - 1, j + 1).  The same ten stress items are the only
// readers of the old velocities that the item overwrites, so waiting for them is all the
// ordering the in-place update needs; stress items wait for nothing.
//
// Items are numbered idx = (s * nty + ty) * ntx + tx.  CTAs draw tickets from one counter and
// the ticket order interleaves the two kinds with a lag L > ntx:
//   tickets [0, L)                 stress 0 .. L-1
//   tickets [L, L + 2(n - L))      velocity m, stress L + m, alternating (m = 0, 1, ...)
//   tickets [2n - L, 2n)           the remaining velocity items
// Every dependency of velocity item m (stress items up to m + ntx) holds a smaller ticket, and a
// ticket is drawn only by a running CTA, so the smallest unfinished ticket can always proceed:
// the order cannot deadlock, whatever the number of resident CTAs.  L trades waiting (the
// stress items a velocity item needs are still running) against L2 reuse (the new stresses
// and old velocities it reads are still cached).
#pragma once

#if defined(__CUDACC__)
#define EWF_HD __host__ __device__ __forceinline__
#else
#define EWF_HD inline
#endif

namespace ewf {

struct WaveShape {
    int ntx, nty, nslab;  // tiles in x and y, slabs in z
    int n;                // items of each kind
    int lag;              // stress items issued before the first velocity item (ntx < lag <= n)
    int kslab;            // planes per slab (>= 3: slab 0 holds the free-surface planes 0..2)
};

EWF_HD WaveShape wave_shape(int nx, int ny, int nz, int tx, int ty, int kslab, int lag)
{
    WaveShape w;
    w.ntx = (nx + tx - 1) / tx;
    w.nty = (ny + ty - 1) / ty;
    w.kslab = kslab;
    w.nslab = (nz + kslab - 1) / kslab;
    w.n = w.ntx * w.nty * w.nslab;
    int l = lag < w.ntx + 1 ? w.ntx + 1 : lag;
    w.lag = l > w.n ? w.n : l;
    return w;
}

// ticket -> (item index, velocity?)
EWF_HD void wave_decode(const WaveShape &w, int t, int &idx, bool &vel)
{
    if (t < w.lag) {
        idx = t;
        vel = false;
        return;
    }
    const int m = t - w.lag;
    const int paired = 2 * (w.n - w.lag);
    if (m < paired) {
        idx = (m >> 1) + ((m & 1) ? w.lag : 0);
        vel = !(m & 1);
    } else {
        idx = m - paired + (w.n - w.lag);
        vel = true;
    }
}

// The d-th stress item (d in [0, 10)) that velocity item idx waits for, or -1: slabs s and s-1
// times the tile itself and its -x, +x, -y, +y neighbours.
EWF_HD int wave_dep(const WaveShape &w, int idx, int d)
{
    const int tx = idx % w.ntx;
    const int r = idx / w.ntx;
    const int ty = r % w.nty;
    const int s = r / w.nty - d / 5;
    const int nb = d % 5;
    const int ux = tx + (nb == 1 ? -1 : nb == 2 ? 1 : 0);
    const int uy = ty + (nb == 3 ? -1 : nb == 4 ? 1 : 0);
    if (s < 0 || ux < 0 || ux >= w.ntx || uy < 0 || uy >= w.nty) return -1;
    return (s * w.nty + uy) * w.ntx + ux;
}

// planes of the stress and velocity items of slab s
EWF_HD void wave_stress_planes(const WaveShape &w, int nz, int s, int &k0, int &k1)
{
    k0 = s * w.kslab;
    k1 = k0 + w.kslab < nz ? k0 + w.kslab : nz;
}
EWF_HD void wave_velocity_planes(const WaveShape &w, int nz, int s, int &k0, int &k1)
{
    k0 = s * w.kslab - 1 < 0 ? 0 : s * w.kslab - 1;
    k1 = (s == w.nslab - 1) ? nz : (s + 1) * w.kslab - 1;
}

// owning stress item of a point-source entry at cell (i, j, k) (clamped into the item grid)
EWF_HD int wave_owner(const WaveShape &w, int tx, int ty, int i, int j, int k)
{
    int ux = i / tx, uy = j / ty, s = k / w.kslab;
    ux = ux < 0 ? 0 : (ux >= w.ntx ? w.ntx - 1 : ux);
    uy = uy < 0 ? 0 : (uy >= w.nty ? w.nty - 1 : uy);
    s = s < 0 ? 0 : (s >= w.nslab ? w.nslab - 1 : s);
    return (s * w.nty + uy) * w.ntx + ux;
}

constexpr int WAVE_WAIT_LIMIT = 1 << 21;  // dependency polls (an acquire load each, ~1 us) before giving up

// State of one CTA's control loop.  Items pass through two slots: the control hands an item to
// the compute warps (slot handed % 2) once the slot's previous item is written and published and
// the item's dependencies are published; it publishes written stress items in order.
struct WaveCtrl {
    int handed = 0, finished = 0;  // items given to the compute warps / written and published
    int held0 = -1, held1 = -1;    // stress item in slot 0 / 1 (-1: a velocity item)
    bool have = false;             // a drawn item not yet handed over: (idx, vel)
    int idx = 0;
    bool vel = false;
    int last = -1;                 // this CTA's ticket >= 2n once drawn
    int polls = 0;
};

// One pass of the control loop; true once the CTA is done (every item it drew is written and
// published, the end marker handed over).  E supplies the primitives (device: warp collectives
// on shared memory, flags and the ticket counter; host: the simulation in the tests):
//   int  draw()                    next ticket
//   bool slot_done(int u)          has the u-th handed item been written?
//   void publish(int idx)          injections of stress item idx, then its done flag
//   void fetch_deps(int idx)       prepare the dependency test of velocity item idx
//   bool deps_ready()              are all its dependencies published?
//   void fail(); bool failed()     give up waiting (error flag) / has any wait given up?
//   void handover(int slot, int code)   code = idx (stress) or -(idx + 1) (velocity)
//   void finish(int slot, int last)     end marker into `slot`; `last` = the ticket >= 2n
// `moved` reports whether anything changed (the device loop backs off otherwise).
template <class E>
EWF_HD bool wave_control_step(const WaveShape &w, WaveCtrl &c, E &env, bool &moved)
{
    moved = false;
    while (c.finished < c.handed) {
        if (!env.slot_done(c.finished)) break;
        const int held = (c.finished & 1) ? c.held1 : c.held0;
        if (held >= 0) env.publish(held);
        ++c.finished;
        moved = true;
    }
    if (!c.have && c.last < 0 && c.handed - c.finished < 2) {  // at most two items per CTA
        const int t = env.draw();
        if (t >= 2 * w.n) {
            c.last = t;
        } else {
            wave_decode(w, t, c.idx, c.vel);
            c.have = true;
            c.polls = 0;
            if (c.vel) env.fetch_deps(c.idx);
        }
        moved = true;
    }
    if (c.have && c.handed - c.finished < 2) {
        bool ready = !c.vel || env.deps_ready();
        if (!ready && ++c.polls >= WAVE_WAIT_LIMIT) {
            env.fail();
            ready = true;
        }
        if (!ready && (c.polls & 1023) == 0 && env.failed()) ready = true;
        if (ready) {
            const int sl = c.handed & 1;
            env.handover(sl, c.vel ? -(c.idx + 1) : c.idx);
            (sl ? c.held1 : c.held0) = c.vel ? -1 : c.idx;
            ++c.handed;
            c.have = false;
            moved = true;
        }
    }
    if (c.last >= 0 && !c.have && c.finished == c.handed) {
        env.finish(c.handed & 1, c.last);
        return true;
    }
    return false;
}

}  // namespace ewf
