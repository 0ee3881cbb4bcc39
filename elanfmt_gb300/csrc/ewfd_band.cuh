// ewfd_band.cuh -- one-pass time step over bands of full-width rows, one thread-block cluster per band.
//
// The two-kernel step moves 156 B per orthorhombic cell-update (the new stresses are written and
// read back, the velocities read twice); the compulsory traffic is 120 B.  k_band reaches it
// without k_step's recomputation of the x halo:
//   * state is double-buffered (step n read from fa.a.f, step n+1 written to fa.o), so no value
//     of step n is overwritten while another CTA may still read it;
//   * a band is BY rows of the whole x extent, split into CTAs of BX = 64 columns that form one
//     thread-block cluster (cluster rank = blockIdx.x); each thread owns one (i, j) column and the
//     cluster marches the band's z-chunk in lockstep: at plane p every CTA computes sigma(p) of
//     its cells, stages the five stress components with x/y neighbours in shared memory, pushes
//     its edge columns into the neighbouring CTAs' halo columns (distributed shared memory: sxx
//     of its last column to the right, sxy and sxz of its first column to the left), arrives on
//     the cluster barrier, updates V(p-1) from the planes staged one barrier earlier, and waits;
//   * the band's y halo -- syy on row j0-1, sxy and syz on row j0+BY -- is recomputed from the
//     step-n state by six warps of the CTA (one component and 32 columns each);
//   * z neighbours stay in registers (szz(p-2..p-1), sxz/syz(p)); one extra sigma plane is
//     recomputed below and above each z-chunk, as in k_step;
//   * the staging buffers rotate over three planes: plane p is staged in buffer p % 3 before
//     barrier p, read by V(p) after it, and restaged (plane p+3) only after barrier p+2, which no
//     CTA passes before every CTA has finished V(p); so one cluster barrier per plane suffices,
//     and its wait overlaps the velocity update;
//   * BC1 (OK4:271-283) and the moment-tensor injection in both reference orders (OK4:336-342
//     before BC1, ANISO:533-535 after) are replayed as in k_step; at plane 2 of the first chunk
//     the plane-1 values BC1 rewrites are staged before the barrier and V(1) waits for it.
// Every thread of every CTA executes the same sequence of barriers (no early exit), and no CTA
// touches another's shared memory before the first barrier or after its last wait.
#pragma once
#include "ewfd_band.h"

namespace ewf {

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }
// Arrival that publishes the whole CTA's earlier shared-memory and distributed-shared-memory
// writes at cluster scope: the CTA barrier orders every thread's writes before thread 0, whose
// release fence makes them visible; the other threads arrive without a fence of their own, so
// they do not wait for their outstanding global stores (a release arrive would, in every thread).
__device__ __forceinline__ void cl_arrive_cta()
{
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) asm volatile("fence.acq_rel.cluster;" ::: "memory");
    asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory");
}
__device__ __forceinline__ unsigned cl_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_nrank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// shared::cluster address of `p` (a variable of this CTA's shared memory) in CTA `rank`
__device__ __forceinline__ unsigned cl_map(const void *p, unsigned rank)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void cl_store(unsigned addr, float v)
{
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void cl_store(unsigned addr, double v)
{
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}

template <typename T, int BY>
struct BandSmem {
    T xx[3][BY][BX + 1];      // own at [ty][tx + 1]; col 0: i0-1 (left CTA's last column)
    T yy[3][BY + 1][BX];      // own at [ty + 1][tx]; row 0: j0-1 (recomputed)
    T xy[3][BY + 1][BX + 1];  // own at [ty][tx]; row BY: j0+BY (recomputed); col BX: i0+BX (right CTA)
    T xz[3][BY][BX + 1];      // own at [ty][tx]; col BX: i0+BX (right CTA)
    T yz[3][BY + 1][BX];      // own at [ty][tx]; row BY: j0+BY (recomputed)
    SrcEntry src[MAXSRC];
    int nsrc;
};

// The inputs of one recomputed stress component (4 syy, 6 sxy, 7 sxz, 8 syz) at (i, j, k), loaded a
// plane ahead of their use so that their latency overlaps a plane of work: v[0] the old value,
// v[1..6] the velocity operands, v[7..9] the moduli, v[10] the 3-D weight.  upd = false where the
// reference does not update the cell (the value is then 0, nothing is loaded).  halo_math computes
// what halo_sigma computes, with the same operations in the same order.
template <typename T>
struct HaloIn {
    T v[11];
    bool upd;
};

template <typename T, int MODEL, int DAMP>
__device__ __forceinline__ void halo_load(const StepArgs<T> &a, int comp, int i, int j, int k, HaloIn<T> &h)
{
    const int nx = a.nx, ny = a.ny;
    if (comp == 3 || comp == 4 || MODEL == MODEL_ISO) h.upd = (i >= 0 && j >= 0 && i < nx && j < ny);
    else if (comp == 6) h.upd = (i > 0 && j > 0 && i < nx && j < ny);
    else if (comp == 7) h.upd = (i > 0 && i < nx && j >= 0 && j < ny && k > 0);
    else h.upd = (j > 0 && j < ny && i >= 0 && i < nx && k > 0);
    if (!h.upd) return;
    const int sx = a.sx;
    const long long sy = a.sy;
    const long long c = (long long)i + (long long)j * sx + (long long)k * sy;
    const T *Vx = a.f[0], *Vy = a.f[1], *Vz = a.f[2];
    h.v[0] = ld(a.f[comp] + c);
    if (comp == 3 || comp == 4) {
        h.v[1] = ld(Vx + c + 1);
        h.v[2] = ld(Vx + c);
        h.v[3] = ld(Vy + c + sx);
        h.v[4] = ld(Vy + c);
        h.v[5] = ld(Vz + c + sy);
        h.v[6] = ld(Vz + c);
        if (MODEL == MODEL_ISO) {
            h.v[7] = ld(a.m[0] + c);
            h.v[8] = ld(a.m[1] + c);
        } else {
            h.v[7] = ld(a.m[comp == 3 ? 0 : 3] + c);
            h.v[8] = ld(a.m[comp == 3 ? 3 : 1] + c);
            h.v[9] = ld(a.m[comp == 3 ? 4 : 5] + c);
        }
    } else {
        if (comp == 6) {
            h.v[1] = ld(Vy + c);
            h.v[2] = ld(Vy + c - 1);
            h.v[3] = ld(Vx + c);
            h.v[4] = ld(Vx + c - sx);
        } else if (comp == 7) {
            h.v[1] = ld(Vz + c);
            h.v[2] = ld(Vz + c - 1);
            h.v[3] = ld(Vx + c);
            h.v[4] = ld(Vx + c - sy);
        } else {
            h.v[1] = ld(Vy + c);
            h.v[2] = ld(Vy + c - sy);
            h.v[3] = ld(Vz + c);
            h.v[4] = ld(Vz + c - sx);
        }
        if (MODEL != MODEL_ISO) h.v[7] = ld(a.m[comp] + c);  // C66 xy, C55 xz, C44 yz
    }
    // the 3-D weight, or the z profile of the separable / 1-D weights (x and y factors: HaloConst)
    if (MODEL != MODEL_ISO && DAMP == DAMP_W3D) h.v[10] = ld(a.w3 + c);
    else h.v[10] = ld(a.w1[2] + k);
}

// The x and y damping factors of a recomputed cell, constant over the z-march.
template <typename T>
struct HaloConst {
    T pxy;   // separable weights: w_x(i) * w_y(j)
    T wx, wy;  // 1-D PML profiles at i, j
    T wav;   // 1-D PML, normal component: 0.5 (w(n+1) + w(n)) along its axis
};

template <typename T, int MODEL, int DAMP>
__device__ __forceinline__ HaloConst<T> halo_const(const StepArgs<T> &a, int comp, int i, int j)
{
    HaloConst<T> hc{T(0), T(0), T(0), T(0)};
    if (i < 0 || j < 0 || i > a.nx || j > a.ny) return hc;
    if (MODEL == MODEL_ISO) {
        hc.wx = ld(a.w1[0] + i);
        hc.wy = ld(a.w1[1] + j);
        if (comp == 3) hc.wav = T(0.5) * (ld(a.w1[0] + i + 1) + hc.wx);
        if (comp == 4) hc.wav = T(0.5) * (ld(a.w1[1] + j + 1) + hc.wy);
    } else if (DAMP == DAMP_SEP) {
        hc.pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
    }
    return hc;
}

template <typename T, int MODEL, int DAMP>
__device__ __forceinline__ T halo_math(const StepArgs<T> &a, int comp, const HaloConst<T> &hk, const HaloIn<T> &h)
{
    if (!h.upd) return T(0);
    const T dt = a.dt, old = h.v[0];
    T W = T(0);
    if (MODEL != MODEL_ISO) W = (DAMP == DAMP_W3D) ? h.v[10] : hk.pxy * h.v[10];
    if (comp == 3 || comp == 4) {
        const T Vxx = (h.v[1] - h.v[2]) * a.rdx;
        const T Vyy = (h.v[3] - h.v[4]) * a.rdy;
        const T Vzz = (h.v[5] - h.v[6]) * a.rdz;
        if (MODEL == MODEL_ISO) {
            const T c11 = h.v[7], c12 = h.v[8];
            if (comp == 3) return nrm_iso(hk.wav, old, dt, c11, c12, c12, Vxx, Vyy, Vzz);
            return nrm_iso(hk.wav, old, dt, c12, c11, c12, Vxx, Vyy, Vzz);
        }
        return nrm_ortho(old, W, dt, h.v[7], h.v[8], h.v[9], Vxx, Vyy, Vzz);
    }
    const T d1 = h.v[1] - h.v[2], d2 = h.v[3] - h.v[4];
    if (MODEL == MODEL_ISO) {
        const T wx = hk.wx, wy = hk.wy, wz = h.v[10];
        const T c66dt = a.c66 * dt;
        if (comp == 6) return shr_iso(wz * wy * wx, old, c66dt, d1, a.rdx, d2, a.rdy);
        if (comp == 7) return shr_iso(wy * wz * wx, old, c66dt, d1, a.rdx, d2, a.rdz);
        return shr_iso(wx * wy * wz, old, c66dt, d1, a.rdz, d2, a.rdy);
    }
    if (comp == 6) return shr_ortho(old, W, dt, h.v[7], d1, a.dx, a.rdx, d2, a.dy, a.rdy, a.fdiv != 0);
    if (comp == 7) return shr_ortho(old, W, dt, h.v[7], d1, a.dx, a.rdx, d2, a.dz, a.rdz, a.fdiv != 0);
    return shr_ortho(old, W, dt, h.v[7], d1, a.dz, a.rdz, d2, a.dy, a.rdy, a.fdiv != 0);
}

template <int BY, typename T>
constexpr int band_min_ctas() { return BY == 4 ? 2 : 1; }

template <typename T, int MODEL, int DAMP, bool KAHAN, int BY>
__global__ void __launch_bounds__(BX *BY, band_min_ctas<BY, T>()) k_band(const FusedArgs<T> fa)
{
    static_assert(BY >= 3, "six y-halo warps need three rows of two warps");
    const StepArgs<T> &a = fa.a;
    __shared__ BandSmem<T, BY> sm;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int lane = tx & 31, warp = (ty * BX + tx) >> 5;
    const unsigned rank = cl_rank(), nrank = cl_nrank();
    const int i0 = blockIdx.x * BX, j0 = blockIdx.y * BY;
    const int i = i0 + tx, j = j0 + ty;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int k0 = blockIdx.z * a.kchunk;
    const int k1 = min(k0 + a.kchunk, nz);
    const int sx = a.sx;
    const long long sy = a.sy;
    const T dt = a.dt, rdx = a.rdx, rdy = a.rdy, rdz = a.rdz;
    const bool in_grid = (i < nx && j < ny);
    const bool row_bc = (j < a.bc1_rows);
    const int ps = (k0 == 0) ? 0 : k0 - 1;

    // sources on the CTA's columns and on its recomputed rows (planes ps..k1)
    if (tx == 0 && ty == 0) {
        int n = 0;
        for (int e = 0; e < fa.nsrc && n < MAXSRC; ++e) {
            const SrcEntry q = fa.src[e];
            if (q.i >= i0 && q.i < i0 + BX && q.j >= j0 - 1 && q.j <= j0 + BY && q.k >= ps && q.k <= k1) sm.src[n++] = q;
        }
        sm.nsrc = n;
    }
    // halo columns the neighbours fill; they stay zero at the ends of the band
    if (tx < 3) {
        sm.xx[tx][ty][0] = T(0);
        sm.xy[tx][ty][BX] = T(0);
        sm.xz[tx][ty][BX] = T(0);
    }
    const int it = *fa.it_ptr;
    const T sval = (fa.nsrc > 0 && it >= 0 && it < fa.nstf) ? (T)fa.stf[it] : T(0);

    // distributed-shared-memory destinations of the edge columns (buffer 0; + b * stride)
    const bool push_r = (tx == BX - 1) && rank + 1 < nrank;
    const bool push_l = (tx == 0) && rank > 0;
    unsigned r_xx = 0, r_xy = 0, r_xz = 0;
    if (push_r) r_xx = cl_map(&sm.xx[0][ty][0], rank + 1);
    if (push_l) {
        r_xy = cl_map(&sm.xy[0][ty][BX], rank - 1);
        r_xz = cl_map(&sm.xz[0][ty][BX], rank - 1);
    }
    constexpr unsigned XX_B = sizeof(T) * BY * (BX + 1), XY_B = sizeof(T) * (BY + 1) * (BX + 1), XZ_B = XX_B;

    // y-halo role: warps 0-5, one component each over 32 columns (uniform per warp)
    const int hk = warp < 6 ? (warp >> 1) : -1;  // 0: syy(j0-1)  1: sxy(j0+BY)  2: syz(j0+BY)
    const int hl = ((warp & 1) << 5) + lane;
    const int hi = i0 + hl, hj = (hk == 0) ? j0 - 1 : j0 + BY;
    const int hcomp = (hk == 0) ? 4 : (hk == 1 ? 6 : 8);
    const bool hin = hk >= 0 && hi <= nx && hj >= -1 && hj <= ny;
    const HaloConst<T> hcst = hin ? halo_const<T, MODEL, DAMP>(a, hcomp, hi, hj) : HaloConst<T>{T(0), T(0), T(0), T(0)};

    // column damping
    T wavx = T(0), wavy = T(0), wxi = T(0), wyj = T(0), pxy = T(0), wxm = T(0), wym = T(0);
    if (in_grid) {
        if (DAMP == DAMP_PML1D) {
            wxi = ld(a.w1[0] + i);
            wyj = ld(a.w1[1] + j);
            wavx = T(0.5) * (ld(a.w1[0] + i + 1) + wxi);
            wavy = T(0.5) * (ld(a.w1[1] + j + 1) + wyj);
            if (i > 0) wxm = ld(a.w1[0] + i - 1);
            if (j > 0) wym = ld(a.w1[1] + j - 1);
        } else if (DAMP == DAMP_SEP) {
            pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
        }
    }
    const bool do_x = in_grid && i >= 1 && j >= 1 && (j < ny - 1);
    const bool do_y = in_grid && i >= 1 && j >= 1 && (i < nx - 1);
    const bool do_z = in_grid && i >= 1 && j >= 1 && (i < nx - 1) && (j < ny - 1);
    const bool bxz = in_grid && i > 0 && row_bc;  // BC1 rewrites sxz(i, j, 1)
    const bool byz = in_grid && j > 0;            // BC1 rewrites syz(i, j, 1)

    long long c = (long long)i + (long long)j * sx + (long long)ps * sy;
    // own column: V(p-1) (vx_m, vy_m, vz_km1) and Vz(p) (vz_k) of the old state, the stress inputs of
    // plane p (nxt), all loaded a plane ahead; the velocity update's own old V comes from them
    T vx_m = T(0), vy_m = T(0), vz_k = T(0), vz_km1 = T(0), wz_k = T(0);
    StressIn<T, MODEL, DAMP> nxt;
    if (in_grid) {
        vx_m = ld(a.f[0] + c - sy);
        vy_m = ld(a.f[1] + c - sy);
        vz_k = ld(a.f[2] + c);
        vz_km1 = ld(a.f[2] + c - sy);
        if (DAMP == DAMP_PML1D) wz_k = ld(a.w1[2] + ps);
        stress_load<T, MODEL, DAMP, 1>(a, c, c, ps, nxt);
    }
    T szz_m = T(0), szz_mm = T(0);  // szz(p-1), szz(p-2) of the own column
    // buoyancy and 3-D weight of the velocity update, loaded a plane ahead (orthorhombic model)
    T bx_n = a.bx, by_n = a.by, bz_n = a.bz, w_n = T(0);
    T wz_prev = T(0);  // separable weights: the z profile at the plane of the last stress update
    // inputs of this warp's recomputed component, loaded a plane ahead (plane ps is never recomputed)
    HaloIn<T> hn;
    hn.upd = false;

    cl_arrive();  // every CTA of the cluster runs; zeroed halo columns and the source list visible
    cl_wait();
    const int nloc = sm.nsrc;

    int b = ps % 3;
    for (int p = ps; p <= k1; ++p, c += sy) {
        const bool compute = (p < nz);
        const bool halo = (p >= max(1, k0)) && (p < k1);
        const bool write = (p >= k0) && (p < k1);
        const bool vplane = (p - 1 >= max(1, k0)) && (p - 1 < k1);
        const bool bc1p = (p == 2 && k0 == 0);  // BC1 rewrites plane 1 from this plane
        const int pb = (b == 0) ? 2 : b - 1;
        T sv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
        T xz1 = T(0), yz1 = T(0);  // plane-1 sxz / syz after BC1 (the BC1 plane only)

        // velocity side of plane p-1: the old V from the own column's registers, buoyancy and weight
        // loaded in the previous iteration; then the loads for plane p (used in the next iteration)
        const long long cv = c - sy;
        const T v0 = vx_m, v1 = vy_m, v2 = vz_km1;
        const T bxv = bx_n, byv = by_n, bzv = bz_n;
        T wv = T(0);
        if (vplane && in_grid) {
            if (MODEL == MODEL_ORTHO) wv = (DAMP == DAMP_W3D) ? w_n : pxy * wz_prev;
            else wv = ld(a.w1[2] + p - 2);
        }
        if (MODEL == MODEL_ORTHO && halo && in_grid) {  // plane p is a velocity plane of this chunk
            bx_n = ld(a.m[9] + c);
            by_n = ld(a.m[10] + c);
            bz_n = ld(a.m[11] + c);
            if (DAMP == DAMP_W3D) w_n = ld(a.w3 + c);
        }
        const HaloIn<T> hc = hn;
        if (hk >= 0 && hin && p + 1 >= max(1, k0) && p + 1 < k1) halo_load<T, MODEL, DAMP>(a, hcomp, hi, hj, p + 1, hn);
        T cp0 = T(0), cp1 = T(0), cp2 = T(0);
        if (vplane && in_grid) {
            if (KAHAN) {
                cp0 = a.comp[0][cv];
                cp1 = a.comp[1][cv];
                cp2 = a.comp[2][cv];
            }
        }

        if (compute) {
            if (in_grid) {
                const StressIn<T, MODEL, DAMP> q = nxt;
                if (p + 1 < nz && p + 1 <= k1) stress_load<T, MODEL, DAMP, 1>(a, c + sy, c + sy, p + 1, nxt);
                const T Vxx = (q.vx_ip - q.vx) * rdx;
                const T Vyy = (q.vy_jp - q.vy) * rdy;
                const T Vzz = (q.vz_p - vz_k) * rdz;
                if (MODEL == MODEL_ISO) {
                    const T c11 = q.c[0], c12 = q.c[1];
                    sv[0] = nrm_iso(wavx, q.s[0], dt, c11, c12, c12, Vxx, Vyy, Vzz);
                    sv[1] = nrm_iso(wavy, q.s[1], dt, c12, c11, c12, Vxx, Vyy, Vzz);
                    sv[2] = nrm_iso(T(0.5) * (q.w + wz_k), q.s[2], dt, c12, c12, c11, Vxx, Vyy, Vzz);
                    const T c66dt = a.c66 * dt;
                    sv[3] = shr_iso(wz_k * wyj * wxi, q.s[3], c66dt, q.vy - q.vy_im, rdx, q.vx - q.vx_jm, rdy);
                    sv[4] = shr_iso(wyj * wz_k * wxi, q.s[4], c66dt, vz_k - q.vz_im, rdx, q.vx - vx_m, rdz);
                    sv[5] = shr_iso(wxi * wyj * wz_k, q.s[5], c66dt, q.vy - vy_m, rdz, vz_k - q.vz_jm, rdy);
                    wz_k = q.w;
                } else {
                    const T W = (DAMP == DAMP_W3D) ? q.w : pxy * q.w;
                    wz_prev = q.w;
                    sv[0] = nrm_ortho(q.s[0], W, dt, q.c[0], q.c[3], q.c[4], Vxx, Vyy, Vzz);
                    sv[1] = nrm_ortho(q.s[1], W, dt, q.c[3], q.c[1], q.c[5], Vxx, Vyy, Vzz);
                    sv[2] = nrm_ortho(q.s[2], W, dt, q.c[4], q.c[5], q.c[2], Vxx, Vyy, Vzz);
                    const T xy = shr_ortho(q.s[3], W, dt, q.c[6], q.vy - q.vy_im, a.dx, a.rdx, q.vx - q.vx_jm, a.dy, a.rdy,
                                           a.fdiv != 0);
                    const T xz = shr_ortho(q.s[4], W, dt, q.c[7], vz_k - q.vz_im, a.dx, a.rdx, q.vx - vx_m, a.dz, a.rdz,
                                           a.fdiv != 0);
                    const T yz = shr_ortho(q.s[5], W, dt, q.c[8], q.vy - vy_m, a.dz, a.rdz, vz_k - q.vz_jm, a.dy, a.rdy,
                                           a.fdiv != 0);
                    sv[3] = (i > 0 && j > 0) ? xy : q.s[3];
                    sv[4] = (i > 0 && p > 0) ? xz : q.s[4];
                    sv[5] = (j > 0 && p > 0) ? yz : q.s[5];
                }
                if (p == 0 && row_bc) sv[2] = T(0);  // BC1 szz (OK4:279)
                vx_m = q.vx;
                vy_m = q.vy;
                vz_km1 = vz_k;
                vz_k = q.vz_p;
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = sm.src[e];
                    if (q2.k == p && q2.i == i && q2.j == j && inject_when(a, q2, fa.order) == 1)
                        sv[q2.comp - 3] = sv[q2.comp - 3] + (T)q2.coef * sval;
                }
            }
            // the recomputed row of this warp
            T h = T(0), h1 = T(0);
            if (halo && hin) {
                h = halo_math<T, MODEL, DAMP>(a, hcomp, hcst, hc);
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = sm.src[e];
                    if (q2.k == p && q2.i == hi && q2.j == hj && q2.comp == hcomp && inject_when(a, q2, fa.order) == 1)
                        h = h + (T)q2.coef * sval;
                }
            }
            // BC1 (OK4:281-282): sxz / syz on plane 1 from plane 2, then the injections that come after it
            if (bc1p) {
                xz1 = a.third * sv[4];
                yz1 = a.third * sv[5];
                const bool hbc = hk == 2 && hin && bc1_plane1(a, 8, hi, hj);
                if (hbc) h1 = a.third * h;
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = sm.src[e];
                    if (inject_when(a, q2, fa.order) != 2) continue;
                    const T add = (T)q2.coef * sval;
                    if (in_grid && q2.i == i && q2.j == j) {
                        if (q2.k == 1) {
                            if (q2.comp == 7) xz1 = xz1 + add;
                            else yz1 = yz1 + add;
                        } else {
                            sv[q2.comp - 3] = sv[q2.comp - 3] + add;
                        }
                    } else if (hbc && q2.i == hi && q2.j == hj && q2.comp == 8) {
                        if (q2.k == 1) h1 = h1 + add;
                        else h = h + add;
                    }
                }
            }
            if (halo) {
                sm.xx[b][ty][tx + 1] = sv[0];
                sm.yy[b][ty + 1][tx] = sv[1];
                sm.xy[b][ty][tx] = sv[3];
                sm.xz[b][ty][tx] = sv[4];
                sm.yz[b][ty][tx] = sv[5];
                if (push_r) cl_store(r_xx + b * XX_B, sv[0]);
                if (push_l) {
                    cl_store(r_xy + b * XY_B, sv[3]);
                    cl_store(r_xz + b * XZ_B, sv[4]);
                }
                if (hk == 0) sm.yy[b][0][hl] = h;
                else if (hk == 1) sm.xy[b][BY][hl] = h;
                else if (hk == 2) sm.yz[b][BY][hl] = h;
                if (bc1p) {  // plane 1 is buffer 1
                    if (bxz) sm.xz[1][ty][tx] = xz1;
                    if (byz) sm.yz[1][ty][tx] = yz1;
                    if (push_l && bxz) cl_store(r_xz + 1 * XZ_B, xz1);
                    if (hk == 2 && hin && bc1_plane1(a, 8, hi, hj)) sm.yz[1][BY][hl] = h1;
                }
            }
        }

        // plane p staged in every CTA of the band (one fence per CTA); the global stores of the new
        // stresses come after it, so that the next fence finds them drained
        cl_arrive_cta();
        if (write && in_grid) {
#pragma unroll
            for (int f = 0; f < 6; ++f) fa.o[3 + f][c] = sv[f];
            if (bc1p) {  // and the plane-1 values BC1 rewrote
                if (bxz) fa.o[7][c - sy] = xz1;
                if (byz) fa.o[8][c - sy] = yz1;
            }
        }
        if (bc1p) cl_wait();      // V(1) reads the plane-1 values staged above

        // velocity of plane p-1 (OK4:346-378 / ANISO:358-389) from the planes staged a barrier ago
        if (vplane && in_grid) {
            const T sxz_p = sv[4], syz_p = sv[5];
            const T dSx = (sm.xx[pb][ty][tx + 1] - sm.xx[pb][ty][tx]) * rdx + (sm.xy[pb][ty + 1][tx] - sm.xy[pb][ty][tx]) * rdy +
                          (sxz_p - sm.xz[pb][ty][tx]) * rdz;
            const T dSy = (sm.yy[pb][ty + 1][tx] - sm.yy[pb][ty][tx]) * rdy + (sm.xy[pb][ty][tx + 1] - sm.xy[pb][ty][tx]) * rdx +
                          (syz_p - sm.yz[pb][ty][tx]) * rdz;
            const T dSz = (szz_m - szz_mm) * rdz + (sm.xz[pb][ty][tx + 1] - sm.xz[pb][ty][tx]) * rdx +
                          (sm.yz[pb][ty + 1][tx] - sm.yz[pb][ty][tx]) * rdy;
            T ax, ay, az;
            if (MODEL == MODEL_ISO) { ax = wxm; ay = wym; az = wv; }
            else { ax = ay = az = wv; }
            const T nvx = vel_update<T, MODEL, KAHAN>(a, v0, dSx, ax, bxv, cp0);
            const T nvy = vel_update<T, MODEL, KAHAN>(a, v1, dSy, ay, byv, cp1);
            const T nvz = vel_update<T, MODEL, KAHAN>(a, v2, dSz, az, bzv, cp2);
            const int kv = p - 1;
            if (do_x && kv < nz - 1) {
                fa.o[0][cv] = nvx;
                if (KAHAN) a.comp[0][cv] = cp0;
            }
            if (do_y && kv < nz - 1) {
                fa.o[1][cv] = nvy;
                if (KAHAN) a.comp[1][cv] = cp1;
            }
            if (do_z) {
                fa.o[2][cv] = nvz;
                if (KAHAN) a.comp[2][cv] = cp2;
            }
        }
        if (!bc1p) cl_wait();     // every CTA has staged plane p (and finished V(p-2))

        szz_mm = szz_m;
        szz_m = sv[2];
        b = (b == 2) ? 0 : b + 1;
    }
}

}  // namespace ewf
