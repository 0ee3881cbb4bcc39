// ewfd_sweep.cuh -- one-pass time step as a lockstep sweep of the whole grid along z.
//
// The two-kernel step (k_stress, then k_velocity) moves 96 + 60 = 156 B per orthorhombic cell:
// the velocity kernel reads back the six stresses the stress kernel just wrote and the three
// velocities it just read.  k_sweep does both updates in one launch and reads each state field
// from DRAM once (120 B per cell, the compulsory traffic); the re-reads come from L2.
//
//   * The state is double-buffered: step n in A (read-only for the whole launch), step n+1
//     written to B.  So no CTA ever waits to read a value another CTA could overwrite.
//   * All CTAs are resident at once (cooperative launch).  CTA c owns a contiguous range of
//     (i, j) columns in row-major order, q = i + j*nx: an exactly balanced share of the grid,
//     one column per compute thread.  Every CTA sweeps the planes k = 0 .. nz-1: at iteration p
//     it writes the new stresses of plane p, then updates the velocities of plane p - L (the lag
//     L >= 2).  The velocity update reads new stresses from planes kv-1 .. kv+1 of its own
//     columns and of the neighbouring columns (i +- 1, j +- 1), which the neighbouring CTAs
//     wrote a few iterations earlier: those reads hit L2.
//   * One control warp per CTA publishes the CTA's progress (stress planes completed, tagged
//     with a launch generation) with a release store after each plane's stores, applies the
//     point sources of that plane first, and checks with acquire loads that the neighbouring
//     CTAs are far enough ahead for the next iteration's velocity plane.  Lockstep progress
//     leaves L - 1 planes of slack, so the check normally passes at the first poll; a lane keeps
//     the highest progress it has seen and polls again only when the target passes it.  It all
//     runs while the compute warps work.  The two roles meet at split named barriers, never at a
//     barrier of the whole CTA: after its stores of plane p each compute warp arrives at
//     "stored(p)" and goes on; the control warp waits there (so its release covers the stores),
//     and after its checks arrives at "cleared(p+1)", where compute warps wait before loading
//     the new stresses of their next velocity plane.  The compute warps do not wait for each
//     other.  The control warp clears planes two iterations ahead, so its fence and checks have a
//     whole iteration of slack; the new stresses of a velocity plane are loaded one iteration
//     before they are used, so the L2 latency hides behind the next plane's stress update.
//     "stored" alternates between two barrier ids, "cleared" between four: no warp can arrive at
//     a barrier again before its previous phase has completed.
//   * The velocity update's inputs from A (old velocities, buoyancy, damping) are loaded before
//     the plane's stress update; only its new-stress loads wait for the barrier.
//   * Every wait is bounded: a wait that gives up sets an error flag (the host reports it), and
//     every later wait of the launch returns at once, so the launch always ends.
//
// The arithmetic is the two-kernel step's (stress_math, vel_math, the same stores and guards),
// so results are bit-identical to it.  Point sources follow k_inject: added after the stress
// update (to the step-n value where the update leaves a cell unchanged), "before BC1" replayed
// exactly (OK4:336-342, BC1 after) or after it (ANISO:533-535).
#pragma once
#include "ewfd_kernels.cuh"

namespace ewf {

struct SweepCtl {
    unsigned gen;    // launch generation: the last CTA of a launch advances it
    unsigned ndone;  // CTAs of the running launch that have finished
    int err;         // a bounded wait gave up (the state of the step is invalid)
    int hold;        // diagnostic: CTA whose progress is never published (-1: none)
};

constexpr int SWEEP_MAX_PF = 28;  // 9 state + 12 materials + 6 weight fields + 1

struct SweepCta {
    int s, e;        // columns [s, e) of the row-major (i, j) order
    int lo, hi;      // CTAs owning the columns [s - nx, e + nx): the velocity stencil's reach
    int src0, src1;  // this CTA's point sources: entries [src0, src1) of the grouped list
};

template <typename T>
struct SweepArgs {
    StepArgs<T> a;               // a.f: state at step n (buffer A); materials, damping, scalars
    T *o[9];                     // state at step n+1 (buffer B)
    const SweepCta *cta;
    const SrcEntry *src;         // grouped by CTA; within a CTA by sweep_src_plane, stable
    const double *stf;
    int nstf;
    const int *it_ptr;
    int order;                   // injection order: 0 before BC1, 1 after
    unsigned long long *flags;   // per CTA: (generation << 32) | stress planes completed
    SweepCtl *ctl;
    int lag;                     // velocity inputs loaded lag planes behind the stress plane, lag >= 3
    int nct;                     // compute threads per CTA (a multiple of 32); one more warp controls
    int pfd;                     // the control warp prefetches input planes this far ahead into L2 (0: off)
    int npf;                     // arrays to prefetch
    int esz;                     // their element size in bytes
    const char *pf[SWEEP_MAX_PF];  // box-layout input arrays, each at its (0,0,0) element
};

// 23 warps: 6 on one of an SM's four register partitions (16384 registers each) -- 80 per thread
constexpr int SWEEP_MAX_THREADS = 736;
constexpr int SWEEP_GRANT = 2;   // the control warp clears velocity planes this many iterations ahead
constexpr int SWEEP_WAIT_POLLS = 1 << 20;

__device__ __forceinline__ unsigned long long sweep_ld_acquire(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void sweep_st_release(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Hint: bring [p, p + bytes) into L2 (p and bytes multiples of 16); no completion to wait for.
__device__ __forceinline__ void l2_prefetch(const void *p, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// The control warp's L2 prefetch of plane k of every input array over this CTA's columns: one
// bulk prefetch per (array, row segment), the segment widened by one cell each side (the x
// neighbours of the stencil) and to 16-byte boundaries.  The rows above and below are other
// CTAs' columns, which those CTAs prefetch.
template <typename T>
__device__ __forceinline__ void sweep_prefetch_plane(const SweepArgs<T> &sa, const SweepCta &me, int k, int lane)
{
    const StepArgs<T> &a = sa.a;
    const int nx = a.nx, r0 = me.s / nx, nrow = (me.e - 1) / nx - r0 + 1;
    for (int t = lane; t < sa.npf * nrow; t += 32) {
        const int f = t / nrow, r = r0 + t % nrow;
        const int ilo = max(me.s - r * nx, 0) - 1, ihi = min(me.e - r * nx, nx) + 1;
        const long long e0 = (long long)ilo + (long long)r * a.sx + (long long)k * a.sy;
        const uintptr_t b0 = (uintptr_t)(sa.pf[f] + e0 * sa.esz) & ~(uintptr_t)15;
        const uintptr_t b1 = ((uintptr_t)(sa.pf[f] + (e0 + (ihi - ilo)) * sa.esz) + 15) & ~(uintptr_t)15;
        l2_prefetch((const void *)b0, (unsigned)(b1 - b0));
    }
}

// named CTA barriers (ids 1-6; 0 is __syncthreads): arrive without waiting / arrive and wait.
// bar.sync / bar.arrive are the warp-aligned forms: every thread of a warp must execute the same
// instruction together, so each call site is one instruction and every caller reconverges its
// warp (__syncwarp) right before it -- the code ahead of a barrier has per-thread branches.
__device__ __forceinline__ void bar_arrive(int id, int count)
{
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ int bar_stored(int p) { return 1 + (p & 1); }
// grants run SWEEP_GRANT = 2 iterations ahead, so up to three "cleared" phases can be open at
// once (four ids); "stored" has at most two open
__device__ __forceinline__ int bar_cleared(int p) { return 3 + (p & 3); }

// Bounded wait until *f >= target: returns the value seen (>= target), or 0 when the wait gave up
// (or another wait of the launch already had).
__device__ __forceinline__ unsigned long long sweep_wait(const unsigned long long *f, unsigned long long target,
                                                         SweepCtl *ctl)
{
    for (int n = 0; n < SWEEP_WAIT_POLLS; ++n) {
        const unsigned long long v = sweep_ld_acquire(f);
        if (v >= target) return v;
        if (*(volatile int *)&ctl->err) return 0;
        if (n >= 8) __nanosleep(100);
    }
    atomicExch(&ctl->err, 1);
    return 0;
}

// Does the stress pass (update, then BC1) write stress component `comp` of cell (i, j, k)?
// The same ranges and guards as stress_math / stress_store.
template <typename T, int MODEL, int DAMP>
__device__ __forceinline__ bool stress_writes(const StepArgs<T> &a, int comp, int i, int j, int k)
{
    if (i >= a.nx || j >= a.ny || k >= a.nz) return false;
    const bool guarded = !(MODEL == MODEL_ISO && DAMP != DAMP_PERCOMP);
    bool w = true;
    if (guarded) {
        if (comp == 6) w = i > 0 && j > 0;
        else if (comp == 7) w = i > 0 && k > 0;
        else if (comp == 8) w = j > 0 && k > 0;
    }
    if (a.bc1 && k == 1 && a.nz > 2) {  // BC1 copies plane 2 into plane 1 (stress_store at k = 2)
        if (comp == 7 && i > 0 && j < a.bc1_rows) w = true;
        if (comp == 8 && j > 0) w = true;
    }
    return w;
}

// The sweep iteration whose stress pass a point-source entry follows: its own plane, except
// that sxz / syz on plane 1 -- which BC1 rewrites from plane 2 while plane 2 is updated -- wait
// for plane 2, and entries beyond the last plane (the extents run to nz) go with plane nz - 1.
// The host groups the entries by this plane too.
__host__ __device__ __forceinline__ int sweep_src_plane(const SrcEntry &q, int nz)
{
    if (q.k == 1 && (q.comp == 7 || q.comp == 8)) return 2;
    return q.k < nz - 1 ? q.k : nz - 1;
}

// One point-source entry on the new state (B), after the stress pass of its plane.  `first`:
// no earlier entry of this plane is on the same cell -- where the stress pass leaves the cell
// unchanged, its step-n value is carried over from A before the first addition.
template <typename T, int MODEL, int DAMP>
__device__ void sweep_inject(const SweepArgs<T> &sa, const SrcEntry &q, T s, bool first)
{
    const StepArgs<T> &a = sa.a;
    const long long c = (long long)q.i + (long long)q.j * a.sx + (long long)q.k * a.sy;
    T *f = sa.o[q.comp];
    if (first && !stress_writes<T, MODEL, DAMP>(a, q.comp, q.i, q.j, q.k)) f[c] = a.f[q.comp][c];
    if (sa.order == 0) {  // inject_entry's replay of "inject, then BC1"
        const bool row_bc = a.bc1 && q.j < a.bc1_rows;
        const bool xz_bc = (q.comp == 7) && q.i > 0 && q.i < a.nx && row_bc;
        const bool yz_bc = a.bc1 && (q.comp == 8) && q.j > 0 && q.j < a.ny && q.i < a.nx;
        if ((q.comp == 5 && q.k == 0 && row_bc) || ((xz_bc || yz_bc) && q.k == 1)) return;
        f[c] = f[c] + (T)q.coef * s;
        if ((xz_bc || yz_bc) && q.k == 2) f[c - a.sy] = a.third * f[c];
    } else {
        f[c] = f[c] + (T)q.coef * s;
    }
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
__global__ void __launch_bounds__(sizeof(T) == 4 ? SWEEP_MAX_THREADS : SWEEP_MAX_THREADS / 2, 1)
    k_sweep(const SweepArgs<T> sa)
{
    const StepArgs<T> &a = sa.a;
    const SweepCta me = sa.cta[blockIdx.x];
    const int nz = a.nz, L = sa.lag;
    const unsigned gen = *(volatile unsigned *)&sa.ctl->gen;
    // iteration p: stress of plane p, velocity of plane p - L - 1 (its inputs loaded at iteration
    // p - 1: the new stresses once the control warp has cleared plane p - 1 - L)
    const int niter = nz + L + 1;
    const int nbar = sa.nct + 32;  // threads at each named barrier: every compute thread and the control warp

    if ((int)threadIdx.x >= sa.nct) {
        // ---------------- control warp ----------------
        const int lane = threadIdx.x & 31;
        const int it = *sa.it_ptr;
        const T sval = (it >= 0 && it < sa.nstf) ? (T)sa.stf[it] : T(0);
        const int hold = sa.ctl->hold;
        unsigned long long seen = 0;  // highest progress seen of neighbour me.lo + lane
        int e = me.src0;
        // grants run SWEEP_GRANT iterations ahead: the first ones need no check (no velocity plane)
        for (int g = 0; g < SWEEP_GRANT && g < niter; ++g) bar_arrive(bar_cleared(g), nbar);
        if (sa.pfd > 0)  // the planes the register prefetch does not cover yet
            for (int k = 1; k < sa.pfd && k <= nz; ++k) sweep_prefetch_plane(sa, me, k, lane);
        for (int p = 0; p < niter; ++p) {
            // while the compute warps work on plane p: input plane p + pfd into L2
            if (sa.pfd > 0 && p + sa.pfd <= nz) sweep_prefetch_plane(sa, me, p + sa.pfd, lane);
            __syncwarp();
            bar_sync(bar_stored(p), nbar);  // every compute warp has stored its stresses of plane p
            if (p < nz && lane == 0) {
                const int e0 = e;
                for (; e < me.src1 && sweep_src_plane(sa.src[e], nz) == p; ++e) {
                    const SrcEntry q = sa.src[e];
                    bool first = true;
                    for (int d = e0; d < e; ++d) {
                        const SrcEntry r = sa.src[d];
                        if (r.comp == q.comp && r.i == q.i && r.j == q.j && r.k == q.k) first = false;
                    }
                    sweep_inject<T, MODEL, DAMP>(sa, q, sval, first);
                }
                // release: the CTA's stores of this plane (ordered before by the barrier) and the
                // injections above become visible before the progress value
                if ((int)blockIdx.x != hold)
                    sweep_st_release(&sa.flags[blockIdx.x], ((unsigned long long)gen << 32) | (unsigned)(p + 1));
            }
            // grant iteration g: its compute warps load the new stresses of velocity plane g - L,
            // which needs planes up to g - L + 1 of the neighbours (and of this CTA: stored and
            // injected by iteration p, as L >= SWEEP_GRANT + 1)
            const int g = p + SWEEP_GRANT;
            const int kl = g - L;
            if (kl >= 1 && kl < nz) {
                const unsigned long long target = ((unsigned long long)gen << 32) | (unsigned)min(kl + 2, nz);
                for (int n = me.lo + lane; n <= me.hi; n += 32) {
                    if (n == (int)blockIdx.x) continue;
                    const bool first = n == me.lo + lane;
                    if (first && seen >= target) continue;
                    const unsigned long long v = sweep_wait(&sa.flags[n], target, sa.ctl);
                    if (first) seen = v;
                }
            }
            __syncwarp();
            if (g < niter) bar_arrive(bar_cleared(g), nbar);
        }
        if (lane == 0) {
            __threadfence();
            if (atomicAdd(&sa.ctl->ndone, 1u) == gridDim.x - 1) {
                sa.ctl->ndone = 0;
                sa.ctl->gen = gen + 1;
            }
        }
        return;
    }

    // ---------------- compute threads: one column each ----------------
    StepArgs<T> out = a;  // stores go to B
    StepArgs<T> mix = a;  // velocity inputs: old velocities (A), new stresses (B)
#pragma unroll
    for (int f = 0; f < 9; ++f) out.f[f] = sa.o[f];
#pragma unroll
    for (int f = 3; f < 9; ++f) mix.f[f] = sa.o[f];
    const int col = me.s + (int)threadIdx.x;
    const bool act = col < me.e;
    const int i = act ? col % a.nx : 0, j = act ? col / a.nx : 0;
    const bool vcol = act && i >= 1 && j >= 1;  // velocity_column's ranges (OK4:358-377)
    const long long sy = a.sy;
    const long long c0 = (long long)i + (long long)j * a.sx;
    ColDamp<T> cd{T(0), T(0), T(0), T(0), T(0)};
    VelDamp<T> vd{T(0), T(0), T(0)};
    const bool row_bc = j < a.bc1_rows;
    T vx_m = T(0), vy_m = T(0), vz_k = T(0), wz_k = T(0);
    StressIn<T, MODEL, DAMP> nxt;
    if (act) {
        cd = col_damp<T, DAMP>(a, i, j);
        vd = vel_damp<T, DAMP>(a, i, j);
        vx_m = lds<0>(a.f[0] + c0 - sy);  // plane -1: the zero halo
        vy_m = lds<0>(a.f[1] + c0 - sy);
        vz_k = lds<0>(a.f[2] + c0);
        if (DAMP == DAMP_PML1D) wz_k = ld(a.w1[2] + 0);
        stress_load<T, MODEL, DAMP, 1>(a, c0, c0, 0, nxt);
    }
    T szz_m = T(0), sxz_k = T(0), syz_k = T(0);  // the velocity march's carried stresses
    VelIn<T, MODEL, DAMP, KAHAN> vq;             // inputs of the next velocity plane

    for (int p = 0; p < niter; ++p) {
        if (p < nz && act) {
            const long long c = c0 + (long long)p * sy;
            const StressIn<T, MODEL, DAMP> q = nxt;
            if (p + 1 < nz) stress_load<T, MODEL, DAMP, 1>(a, c + sy, c + sy, p + 1, nxt);
            T o[6];
            bool w_xy, w_xz, w_yz;
            stress_math<T, MODEL, DAMP>(a, q, cd, i, j, p, vx_m, vy_m, vz_k, wz_k, o, w_xy, w_xz, w_yz);
            stress_store<T>(out, c, sy, p, i, j, row_bc, o, w_xy, w_xz, w_yz);
            if (MODEL == MODEL_ISO && DAMP == DAMP_PML1D) wz_k = q.w;
            vx_m = q.vx;
            vy_m = q.vy;
            vz_k = q.vz_p;
        }
        __syncwarp();
        bar_arrive(bar_stored(p), nbar);  // this warp's stores of plane p come first
        // velocity of plane kc from the inputs loaded last iteration
        const int kc = p - L - 1;
        if (kc >= 1 && kc < nz && vcol) {
            const long long cc = c0 + (long long)kc * sy;
            T v[3], cp[3] = {KAHAN ? vq.cp[0] : T(0), KAHAN ? vq.cp[1] : T(0), KAHAN ? vq.cp[2] : T(0)};
            vel_math<T, MODEL, DAMP, KAHAN>(a, vq, vd, szz_m, sxz_k, syz_k, v, cp);
            vel_store<T, KAHAN>(out, cc, kc, i, j, v, cp);
            szz_m = vq.szz;
            sxz_k = vq.sxz_p;
            syz_k = vq.syz_p;
        }
        // inputs of velocity plane kl: from A now, the new stresses once the control warp clears it
        const int kl = p - L;
        const bool vload = kl >= 1 && kl < nz && vcol;
        const long long cl = c0 + (long long)kl * sy;
        if (vload) {
#pragma unroll
            for (int f = 0; f < 3; ++f) vq.v[f] = lds<0>(a.f[f] + cl);
            vel_load_mat<T, MODEL, DAMP, KAHAN>(a, cl, kl, vq);
            if (KAHAN) {
#pragma unroll
                for (int f = 0; f < 3; ++f) vq.cp[f] = a.comp[f][cl];
            }
        }
        __syncwarp();
        bar_sync(bar_cleared(p), nbar);  // neighbours and this CTA cover velocity plane kl
        if (vload) {
            if (kl == 1) {
                szz_m = lds<2>(mix.f[5] + cl - sy);
                sxz_k = lds<2>(mix.f[7] + cl);
                syz_k = lds<2>(mix.f[8] + cl);
            }
            vel_load_sigma<T, MODEL, DAMP, KAHAN, 1, 2>(mix, cl, vq);
        }
    }
}

}  // namespace ewf
