// ewfd_wave.cuh -- the wavefront step: stress, injection and velocity of one time step in one
// persistent launch, in place, scheduled so that the velocity update reads the new stresses
// and the old velocities back from L2 instead of HBM.
//
// The two-kernel step moves 96 B (stress) + 60 B (velocity) per orthorhombic cell: between the
// two launches the whole grid's new stresses (24 B/cell) and the old velocities (12 B/cell) fall
// out of the 129 MB L2.  Here the work is cut into items (a TX x TY tile times a slab of planes,
// ewfd_wave_sched.h) that CTAs draw in a fixed ticket order; a velocity item runs a short lag
// after the ten stress items it depends on, while their output is still in L2.  The per-cell
// arithmetic is the stress_column / velocity_column code of the two-kernel step, so results are
// bit-identical to it.
//
// Ordering: once the compute warps have written a stress item (named barrier), the control warp
// applies its point-source injections and publishes done[idx] = generation + 1 (fence, release
// store); before a velocity item is handed to the compute warps (named barrier), ten control
// lanes wait for its dependencies (acquire loads).  State fields are read with plain coherent
// loads (never the read-only path).  Waits are bounded: after WAVE_WAIT_LIMIT polls the wait sets
// ctl->err and gives up, later waits return at once, the launch still ends, and the host reports
// the error.  The last CTA to draw a ticket resets the ticket counter and advances the
// generation for the next launch.
#pragma once
#include "ewfd_kernels.cuh"
#include "ewfd_wave_sched.h"

#include <climits>

namespace ewf {

struct WaveCtl {
    int ticket;      // next ticket of the current launch
    int gen;         // launch generation: done flags of this launch read gen + 1
    int err;         // 1: a dependency wait gave up (results of that launch are invalid)
    int pad;
};

struct WaveArgs {
    WaveCtl *ctl;
    int *done;                 // per stress item
    const int *src_off;        // n + 1 offsets into src: point-source entries grouped by owning item
    const SrcEntry *src;       // entries in their original order within each item
    const double *stf;
    int nstf;
    const int *it_ptr;
    int order;                 // injection semantics (k_inject)
    int hold;                  // diagnostic: this stress item never publishes its flag (-1: none)
    WaveShape w;
};

__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ bool reached(int v, int want) { return (int)((unsigned)v - (unsigned)want) >= 0; }

template <int ID>
__device__ __forceinline__ void named_sync(int n) { asm volatile("bar.sync %0, %1;" ::"n"(ID), "r"(n) : "memory"); }
template <int ID>
__device__ __forceinline__ void named_arrive(int n) { asm volatile("bar.arrive %0, %1;" ::"n"(ID), "r"(n) : "memory"); }
// named barrier of slot b (IDs as immediates, so only the barriers used are reserved)
template <int BASE>
__device__ __forceinline__ void slot_sync(int b, int n)
{
    if (b) named_sync<BASE + 1>(n);
    else named_sync<BASE>(n);
}
template <int BASE>
__device__ __forceinline__ void slot_arrive(int b, int n)
{
    if (b) named_arrive<BASE + 1>(n);
    else named_arrive<BASE>(n);
}

// CTA: warps 0..7 compute (one thread per column of the TX x TY tile), warp 8 controls.  Items
// pass through two slots in shared memory.  Control -> compute: a named barrier per slot (the
// control warp arrives once the item's dependencies are met, the compute warps wait).  Compute
// -> control: an mbarrier per slot that every compute thread arrives on after the item; the
// control warp only tests it.  The control warp never blocks: it loops publishing written items
// (injections, fence, release of the done flag), drawing the next ticket and testing that item's
// dependencies, so a written stress item is published while the control warp is still waiting
// for a later item's inputs -- which is what keeps the ticket-order argument (the smallest
// unpublished ticket always progresses) valid -- and the compute warps never wait on a fence.
constexpr int WAVE_THREADS = TX * TY + 32;
constexpr int BAR_FULL = 1;  // + slot; barrier 0 is __syncthreads

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *b, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *b)
{
    unsigned long long state;
    asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(smem_addr(b)) : "memory");
    (void)state;
}
// has the phase of parity `parity` completed?  (non-blocking)
__device__ __forceinline__ bool mbar_test(unsigned long long *b, int parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(b)), "r"(parity)
                 : "memory");
    return ok != 0;
}

template <typename T>
__device__ __forceinline__ void wave_publish(const StepArgs<T> &a, const WaveArgs &wa, int idx, int gen)
{
    const int b = wa.src_off[idx], e = wa.src_off[idx + 1];
    if (b < e) {
        const int it = *wa.it_ptr;
        if (it >= 0 && it < wa.nstf) {  // as k_inject: never read past the source function
            const T sval = (T)wa.stf[it];
            for (int q = b; q < e; ++q) inject_entry(a, wa.src[q], sval, wa.order);
        }
    }
    __threadfence();
    if (idx != wa.hold) st_release_gpu(&wa.done[idx], gen + 1);
}

// MINB: CTAs per SM the register budget is sized for
template <typename T, int MODEL, int DAMP, bool KAHAN, int MINB>
__global__ void __launch_bounds__(WAVE_THREADS, MINB) k_wave(const StepArgs<T> a, const WaveArgs wa)
{
    __shared__ int s_item[2];  // item index, -(index + 1) for a velocity item; INT_MIN: no more items
    __shared__ unsigned long long s_empty[2];
    const WaveShape &w = wa.w;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        mbar_init(&s_empty[0], TX * TY);
        mbar_init(&s_empty[1], TX * TY);
    }
    __syncthreads();
    if (warp == TY) {
        // ---- control warp: wave_control_step over warp-collective primitives ----
        struct Env {
            const StepArgs<T> &a;
            const WaveArgs &wa;
            int *s_item;
            unsigned long long *s_empty;
            int lane, gen, dep;
            __device__ int draw()
            {
                int t = 0;
                if (lane == 0) t = atomicAdd(&wa.ctl->ticket, 1);
                return __shfl_sync(0xffffffffu, t, 0);
            }
            __device__ bool slot_done(int u)
            {
                bool ok = false;
                if (lane == 0) ok = mbar_test(&s_empty[u & 1], (u >> 1) & 1);
                return __shfl_sync(0xffffffffu, ok, 0) != 0;
            }
            __device__ void publish(int idx)
            {
                if (lane == 0) wave_publish(a, wa, idx, gen);
                __syncwarp();
            }
            __device__ void fetch_deps(int idx) { dep = lane < 10 ? wave_dep(wa.w, idx, lane) : -1; }
            __device__ bool deps_ready()
            {
                const bool mine = dep < 0 || reached(ld_acquire_gpu(&wa.done[dep]), gen + 1);
                return __all_sync(0xffffffffu, mine);
            }
            __device__ void fail()
            {
                if (lane == 0) atomicExch(&wa.ctl->err, 1);
                __syncwarp();
            }
            __device__ bool failed()
            {
                int e = 0;
                if (lane == 0) e = ld_acquire_gpu(&wa.ctl->err);
                return __shfl_sync(0xffffffffu, e, 0) != 0;
            }
            __device__ void handover(int slot, int code)
            {
                __threadfence();  // the dependency flags' acquire loads before the compute warps' reads
                if (lane == 0) s_item[slot] = code;
                __syncwarp();
                slot_arrive<BAR_FULL>(slot, WAVE_THREADS);
            }
            __device__ void finish(int slot, int last)
            {
                if (lane == 0) s_item[slot] = INT_MIN;
                __syncwarp();
                slot_arrive<BAR_FULL>(slot, WAVE_THREADS);
                // exactly one ticket >= 2n per CTA: the one drawing the last of them is alone
                if (lane == 0 && last == 2 * wa.w.n + (int)gridDim.x - 1) {
                    atomicExch(&wa.ctl->ticket, 0);
                    __threadfence();
                    atomicAdd(&wa.ctl->gen, 1);  // == gen + 1: every CTA has read gen by now
                }
            }
        };
        int gen = 0;
        if (lane == 0) gen = ld_acquire_gpu(&wa.ctl->gen);  // before this CTA's first ticket
        gen = __shfl_sync(0xffffffffu, gen, 0);
        Env env{a, wa, s_item, s_empty, lane, gen, -1};
        WaveCtrl c;
        bool moved;
        while (!wave_control_step(w, c, env, moved))
            if (!moved) __nanosleep(32);
        return;
    }
    // ---- compute warps ----
    const int X0 = lane, j0 = warp;
    for (int i = 0;; ++i) {
        const int b = i & 1;
        slot_sync<BAR_FULL>(b, WAVE_THREADS);
        const int item = s_item[b];
        if (item == INT_MIN) return;
        const bool vel = item < 0;
        const int idx = vel ? -item - 1 : item;
        const int tx = idx % w.ntx;
        const int r = idx / w.ntx;
        const int ty = r % w.nty;
        const int s = r / w.nty;
        const int X = tx * TX + X0, j = ty * TY + j0;
        int k0, k1;
        if (!vel) {
            wave_stress_planes(w, a.nz, s, k0, k1);
            stress_column<T, MODEL, DAMP, 1, false, true>(a, X, j, k0, k1);
        } else {
            wave_velocity_planes(w, a.nz, s, k0, k1);
            velocity_column<T, MODEL, DAMP, KAHAN, 1, false, true>(a, X, j, k0, k1);
        }
        mbar_arrive(&s_empty[b]);
    }
}

}  // namespace ewf
