// ewfd_fused.cuh -- one-pass time step: stress and velocity updated in the same z-march.
//
// The two-kernel step (k_stress then k_velocity) moves 96 + 60 = 156 B per orthorhombic cell:
// the new stresses are written and read back, the velocities read twice.  k_step reads each
// state field once and writes it once (120 B per cell, the compulsory traffic):
//   * state is double-buffered (step n in A, step n+1 written to B), so no CTA ever reads a
//     value another CTA has already advanced;
//   * a CTA owns a 32 x 8 column tile and marches its z-chunk; at plane p it computes sigma(p)
//     for the tile plus the 80 halo cells the velocity stencil needs (sxx at i0-1, syy at
//     j0-1, sxy at i1 and j1, sxz at i1, syz at j1 -- recomputed here, not exchanged), stages
//     the five stress planes that have x/y neighbours in shared memory, then updates V(p-1);
//   * the z-neighbours stay in registers (szz(p-2..p-1), sxz/syz(p)); one extra sigma plane is
//     recomputed at each chunk end;
//   * BC1 (OK4:271-283) and the moment-tensor injection in both reference orders (OK4:336-342
//     before BC1, ANISO:533-535 after) are replayed in the march.
// Cells the reference never updates are never read by an updated velocity cell (the velocity
// ranges OK4:358-377 only reach updated stress cells), so halo cells outside the update ranges
// are filled with 0 without loading anything.
#pragma once
#include "ewfd_kernels.cuh"

namespace ewf {

constexpr int FX = 32;                      // tile width (one warp per row)
constexpr int FY = 8;                       // tile height
constexpr int NHALO = 2 * FX + 2 * FY;      // halo positions per plane
constexpr int MAXSRC = 64;                  // point sources per run (checked on the host)

template <typename T>
struct FusedArgs {
    StepArgs<T> a;          // a.f = state at step n (read); materials, damping, scalars
    T *o[9];                // state at step n+1 (written)
    const SrcEntry *src;
    int nsrc;
    const double *stf;
    int nstf;
    const int *it_ptr;
    int order;              // 0: inject before BC1 (OK4), 1: after (ANISO)
};

// ---- arithmetic shared by the tile and the halo cells (same operand order as the reference) ----
template <typename T>
__device__ __forceinline__ T nrm_iso(T wav, T s, T dt, T ca, T cb, T cc, T e1, T e2, T e3)
{
    return wav * (s + dt * (ca * e1 + cb * e2 + cc * e3));   // OK4:307-309
}
template <typename T>
__device__ __forceinline__ T nrm_ortho(T s, T W, T dt, T ca, T cb, T cc, T e1, T e2, T e3)
{
    return s * W + dt * (ca * e1 + cb * e2 + cc * e3);       // ANISO:312-325
}
template <typename T>
__device__ __forceinline__ T shr_iso(T wprod, T s, T c66dt, T d1, T r1, T d2, T r2)
{
    return wprod * (s + c66dt * (d1 * r1 + d2 * r2));        // OK4:323-329
}
template <typename T>
__device__ __forceinline__ T shr_ortho(T s, T W, T dt, T c, T d1, T h1, T r1, T d2, T h2, T r2, bool fd)
{
    return s * W + dt * c * (div_spacing(d1, h1, r1, fd) + div_spacing(d2, h2, r2, fd));  // ANISO:330-351
}

template <typename T, int DAMP>
__device__ __forceinline__ T weight3(const StepArgs<T> &a, long long c, int i, int j, int k)
{
    if (DAMP == DAMP_W3D) return ld(a.w3 + c);
    return ld(a.w1[0] + i) * ld(a.w1[1] + j) * ld(a.w1[2] + k);
}

// One stress component (3 sxx, 4 syy, 6 sxy, 7 sxz, 8 syz) of step n+1 at a halo cell; 0 where
// the reference does not update the cell (never read by an updated velocity cell).
template <typename T, int MODEL, int DAMP>
__device__ T halo_sigma(const StepArgs<T> &a, int comp, int i, int j, int k)
{
    const int nx = a.nx, ny = a.ny;
    bool upd;
    if (comp == 3 || comp == 4 || MODEL == MODEL_ISO) upd = (i >= 0 && j >= 0 && i < nx && j < ny);
    else if (comp == 6) upd = (i > 0 && j > 0 && i < nx && j < ny);
    else if (comp == 7) upd = (i > 0 && i < nx && j >= 0 && j < ny && k > 0);
    else upd = (j > 0 && j < ny && i >= 0 && i < nx && k > 0);
    if (!upd) return T(0);
    const int sx = a.sx;
    const long long sy = a.sy;
    const long long c = (long long)i + (long long)j * sx + (long long)k * sy;
    const T *Vx = a.f[0], *Vy = a.f[1], *Vz = a.f[2];
    const T old = a.f[comp][c];
    const T dt = a.dt;
    if (comp == 3 || comp == 4) {
        const T Vxx = (ld(Vx + c + 1) - ld(Vx + c)) * a.rdx;
        const T Vyy = (ld(Vy + c + sx) - ld(Vy + c)) * a.rdy;
        const T Vzz = (ld(Vz + c + sy) - ld(Vz + c)) * a.rdz;
        if (MODEL == MODEL_ISO) {
            const T c11 = ld(a.m[0] + c), c12 = ld(a.m[1] + c);
            if (comp == 3) return nrm_iso(T(0.5) * (ld(a.w1[0] + i + 1) + ld(a.w1[0] + i)), old, dt, c11, c12, c12, Vxx, Vyy, Vzz);
            return nrm_iso(T(0.5) * (ld(a.w1[1] + j + 1) + ld(a.w1[1] + j)), old, dt, c12, c11, c12, Vxx, Vyy, Vzz);
        }
        const T W = weight3<T, DAMP>(a, c, i, j, k);
        if (comp == 3) return nrm_ortho(old, W, dt, ld(a.m[0] + c), ld(a.m[3] + c), ld(a.m[4] + c), Vxx, Vyy, Vzz);
        return nrm_ortho(old, W, dt, ld(a.m[3] + c), ld(a.m[1] + c), ld(a.m[5] + c), Vxx, Vyy, Vzz);
    }
    T d1, d2;
    if (comp == 6) {
        d1 = ld(Vy + c) - ld(Vy + c - 1);
        d2 = ld(Vx + c) - ld(Vx + c - sx);
    } else if (comp == 7) {
        d1 = ld(Vz + c) - ld(Vz + c - 1);
        d2 = ld(Vx + c) - ld(Vx + c - sy);
    } else {
        d1 = ld(Vy + c) - ld(Vy + c - sy);
        d2 = ld(Vz + c) - ld(Vz + c - sx);
    }
    if (MODEL == MODEL_ISO) {
        const T wx = ld(a.w1[0] + i), wy = ld(a.w1[1] + j), wz = ld(a.w1[2] + k);
        const T c66dt = a.c66 * dt;
        if (comp == 6) return shr_iso(wz * wy * wx, old, c66dt, d1, a.rdx, d2, a.rdy);
        if (comp == 7) return shr_iso(wy * wz * wx, old, c66dt, d1, a.rdx, d2, a.rdz);
        return shr_iso(wx * wy * wz, old, c66dt, d1, a.rdz, d2, a.rdy);
    }
    const T W = weight3<T, DAMP>(a, c, i, j, k);
    if (comp == 6) return shr_ortho(old, W, dt, ld(a.m[6] + c), d1, a.dx, a.rdx, d2, a.dy, a.rdy, a.fdiv != 0);
    if (comp == 7) return shr_ortho(old, W, dt, ld(a.m[7] + c), d1, a.dx, a.rdx, d2, a.dz, a.rdz, a.fdiv != 0);
    return shr_ortho(old, W, dt, ld(a.m[8] + c), d1, a.dz, a.rdz, d2, a.dy, a.rdy, a.fdiv != 0);
}

// Does BC1 (OK4:279-282) overwrite stress component `comp` of cell (i,j) on plane 1?
template <typename T>
__device__ __forceinline__ bool bc1_plane1(const StepArgs<T> &a, int comp, int i, int j)
{
    if (comp == 7) return i > 0 && i < a.nx && j < a.bc1_rows;
    if (comp == 8) return j > 0 && j < a.ny && i < a.nx;
    return false;
}

// Entry applied when sigma of its plane is computed (true) or after the BC1 pass (false).
template <typename T>
__device__ __forceinline__ int inject_when(const StepArgs<T> &a, const SrcEntry &e, int order)
{
    // returns 0 = drop, 1 = immediately, 2 = after the BC1 pass of plane 2
    const bool bcp = (e.k == 1 || e.k == 2) && bc1_plane1(a, e.comp, e.i, e.j);
    if (order == 0) {
        if (e.comp == 5 && e.k == 0 && e.j < a.bc1_rows) return 0;
        if (bcp && e.k == 1) return 0;
        return 1;
    }
    return bcp ? 2 : 1;
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
__global__ void __launch_bounds__(FX * FY, 3) k_step(const FusedArgs<T> fa)
{
    const StepArgs<T> &a = fa.a;
    __shared__ T s_xx[2][FY][FX + 1];      // col 0: i0-1, col tx+1: own
    __shared__ T s_yy[2][FY + 1][FX];      // row 0: j0-1, row ty+1: own
    __shared__ T s_xy[2][FY + 1][FX + 1];  // own at [ty][tx]; row FY: j1; col FX: i1
    __shared__ T s_xz[2][FY][FX + 1];      // own at [ty][tx]; col FX: i1
    __shared__ T s_yz[2][FY + 1][FX];      // own at [ty][tx]; row FY: j1
    __shared__ SrcEntry s_src[MAXSRC];
    __shared__ int s_nsrc;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * FX, j0 = blockIdx.y * FY;
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

    // sources that touch this CTA's cells (tile + halo, planes ps..k1)
    if (tx == 0 && ty == 0) {
        int n = 0;
        for (int e = 0; e < fa.nsrc && n < MAXSRC; ++e) {
            const SrcEntry q = fa.src[e];
            if (q.i >= i0 - 1 && q.i <= i0 + FX && q.j >= j0 - 1 && q.j <= j0 + FY && q.k >= ps && q.k <= k1)
                s_src[n++] = q;
        }
        s_nsrc = n;
    }
    const int it = *fa.it_ptr;
    const T sval = (fa.nsrc > 0 && it >= 0 && it < fa.nstf) ? (T)fa.stf[it] : T(0);

    // halo position of this thread: one kind per warp so its lanes stay convergent
    //   warp 0: syy(i, j0-1)   warp 1: sxy, syz(i, j1)   warp 2: sxx(i0-1, j)   warp 3: sxy, sxz(i1, j)
    const int hk = ty;
    const bool has_halo = (ty < 2) || (ty < 4 && tx < FY);
    const int hr = tx;
    int hi = 0, hj = 0;
    if (hk == 0) { hi = i0 + tx; hj = j0 - 1; }
    else if (hk == 1) { hi = i0 + tx; hj = j0 + FY; }
    else if (hk == 2) { hi = i0 - 1; hj = j0 + tx; }
    else if (hk == 3) { hi = i0 + FX; hj = j0 + tx; }

    // column damping (tile cell)
    T wavx = T(0), wavy = T(0), wxi = T(0), wyj = T(0), pxy = T(0);
    T wxm = T(0), wym = T(0);
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

    long long c = (long long)i + (long long)j * sx + (long long)ps * sy;
    T vx_m = T(0), vy_m = T(0), vz_k = T(0), wz_k = T(0);
    StressIn<T, MODEL, DAMP> nxt;
    if (in_grid) {
        vx_m = ld(a.f[0] + c - sy);
        vy_m = ld(a.f[1] + c - sy);
        vz_k = ld(a.f[2] + c);
        if (DAMP == DAMP_PML1D) wz_k = ld(a.w1[2] + ps);
        stress_load<T, MODEL, DAMP, 1>(a, c, c, ps, nxt);
    }
    T szz_m = T(0), szz_mm = T(0);   // szz(p-1), szz(p-2) of the own column
    __syncthreads();                  // s_src ready
    const int nloc = s_nsrc;

    for (int p = ps; p <= k1; ++p, c += sy) {
        const bool compute = (p < nz);
        const bool halo = (p >= max(1, k0)) && (p < k1);
        const bool write = (p >= k0) && (p < k1);
        const bool vplane = (p - 1 >= max(1, k0)) && (p - 1 < k1);
        const int b = p & 1, pb = (p - 1) & 1;
        T sv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};

        // velocity-side loads of plane p-1 (issued early)
        const long long cv = c - sy;
        T v0 = T(0), v1 = T(0), v2 = T(0), bx = a.bx, by = a.by, bz = a.bz, wv = T(0);
        T cp0 = T(0), cp1 = T(0), cp2 = T(0);
        if (vplane && in_grid) {
            v0 = a.f[0][cv];
            v1 = a.f[1][cv];
            v2 = a.f[2][cv];
            if (MODEL == MODEL_ORTHO) {
                bx = ld(a.m[9] + cv);
                by = ld(a.m[10] + cv);
                bz = ld(a.m[11] + cv);
                wv = (DAMP == DAMP_W3D) ? ld(a.w3 + cv) : pxy * ld(a.w1[2] + p - 1);
            } else {
                wv = ld(a.w1[2] + p - 2);
            }
            if (KAHAN) {
                cp0 = a.comp[0][cv];
                cp1 = a.comp[1][cv];
                cp2 = a.comp[2][cv];
            }
        }

        __syncthreads();  // buffer b was last read by V(p-2)
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
                vz_k = q.vz_p;
                if (nloc > 0) {
                    for (int e = 0; e < nloc; ++e) {
                        const SrcEntry q2 = s_src[e];
                        if (q2.k == p && q2.i == i && q2.j == j && inject_when(a, q2, fa.order) == 1)
                            sv[q2.comp - 3] = sv[q2.comp - 3] + (T)q2.coef * sval;
                    }
                }
            }
            if (halo) {
                s_xx[b][ty][tx + 1] = sv[0];
                s_yy[b][ty + 1][tx] = sv[1];
                s_xy[b][ty][tx] = sv[3];
                s_xz[b][ty][tx] = sv[4];
                s_yz[b][ty][tx] = sv[5];
                if (has_halo) {
                    // kind 0: syy(i, j0-1); 1: sxy, syz(i, j1); 2: sxx(i0-1, j); 3: sxy, sxz(i1, j)
                    const bool hin = hi >= -1 && hi <= nx && hj >= -1 && hj <= ny;
                    T h1 = T(0), h2 = T(0);
                    int c1 = 4, c2 = -1;
                    if (hk == 0) { c1 = 4; }
                    else if (hk == 1) { c1 = 6; c2 = 8; }
                    else if (hk == 2) { c1 = 3; }
                    else { c1 = 6; c2 = 7; }
                    if (hin) {
                        h1 = halo_sigma<T, MODEL, DAMP>(a, c1, hi, hj, p);
                        if (c2 >= 0) h2 = halo_sigma<T, MODEL, DAMP>(a, c2, hi, hj, p);
                        if (nloc > 0) {
                            for (int e = 0; e < nloc; ++e) {
                                const SrcEntry q2 = s_src[e];
                                if (q2.k == p && q2.i == hi && q2.j == hj && inject_when(a, q2, fa.order) == 1) {
                                    if (q2.comp == c1) h1 = h1 + (T)q2.coef * sval;
                                    else if (q2.comp == c2) h2 = h2 + (T)q2.coef * sval;
                                }
                            }
                        }
                    }
                    if (hk == 0) s_yy[b][0][hr] = h1;
                    else if (hk == 1) { s_xy[b][FY][hr] = h1; s_yz[b][FY][hr] = h2; }
                    else if (hk == 2) s_xx[b][hr][0] = h1;
                    else { s_xy[b][hr][FX] = h1; s_xz[b][hr][FX] = h2; }
                }
            }
        }
        __syncthreads();

        // BC1 (OK4:281-282): sxz/syz on plane 1 from plane 2, then injections that come after it
        if (p == 2 && k0 == 0) {
            if (in_grid) {
                if (i > 0 && row_bc) s_xz[1][ty][tx] = a.third * s_xz[0][ty][tx];
                if (j > 0) s_yz[1][ty][tx] = a.third * s_yz[0][ty][tx];
            }
            if (has_halo && (hk == 1 || hk == 3)) {
                if (hk == 3 && hj >= 0 && hj <= ny && bc1_plane1(a, 7, hi, hj)) s_xz[1][hr][FX] = a.third * s_xz[0][hr][FX];
                if (hk == 1 && hi >= -1 && hi <= nx && bc1_plane1(a, 8, hi, hj)) s_yz[1][FY][hr] = a.third * s_yz[0][FY][hr];
            }
            if (nloc > 0) {
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = s_src[e];
                    if (inject_when(a, q2, fa.order) != 2) continue;
                    const int pl = q2.k & 1;  // plane 1 -> buffer 1, plane 2 -> buffer 0
                    const T add = (T)q2.coef * sval;
                    if (in_grid && q2.i == i && q2.j == j) {
                        if (q2.comp == 7) s_xz[pl][ty][tx] = s_xz[pl][ty][tx] + add;
                        else s_yz[pl][ty][tx] = s_yz[pl][ty][tx] + add;
                    } else if (has_halo && q2.i == hi && q2.j == hj) {
                        if (hk == 3 && q2.comp == 7) s_xz[pl][hr][FX] = s_xz[pl][hr][FX] + add;
                        if (hk == 1 && q2.comp == 8) s_yz[pl][FY][hr] = s_yz[pl][FY][hr] + add;
                    }
                }
            }
            __syncthreads();
            if (in_grid) {
                sv[4] = s_xz[0][ty][tx];
                sv[5] = s_yz[0][ty][tx];
                const long long c1 = c - sy;  // plane 1
                if (i > 0 && row_bc) fa.o[7][c1] = s_xz[1][ty][tx];
                if (j > 0) fa.o[8][c1] = s_yz[1][ty][tx];
                // deferred injections on plane 1 outside the BC1 rows cannot exist (not deferred)
            }
        }

        // velocity of plane p-1 (OK4:346-378 / ANISO:358-389)
        if (vplane && in_grid) {
            const int kv = p - 1;
            const T sxz_p = sv[4], syz_p = sv[5];
            const T dSx = (s_xx[pb][ty][tx + 1] - s_xx[pb][ty][tx]) * rdx + (s_xy[pb][ty + 1][tx] - s_xy[pb][ty][tx]) * rdy +
                          (sxz_p - s_xz[pb][ty][tx]) * rdz;
            const T dSy = (s_yy[pb][ty + 1][tx] - s_yy[pb][ty][tx]) * rdy + (s_xy[pb][ty][tx + 1] - s_xy[pb][ty][tx]) * rdx +
                          (syz_p - s_yz[pb][ty][tx]) * rdz;
            const T dSz = (szz_m - szz_mm) * rdz + (s_xz[pb][ty][tx + 1] - s_xz[pb][ty][tx]) * rdx +
                          (s_yz[pb][ty + 1][tx] - s_yz[pb][ty][tx]) * rdy;
            T ax, ay, az;
            if (MODEL == MODEL_ISO) { ax = wxm; ay = wym; az = wv; }
            else { ax = ay = az = wv; }
            const T nvx = vel_update<T, MODEL, KAHAN>(a, v0, dSx, ax, bx, cp0);
            const T nvy = vel_update<T, MODEL, KAHAN>(a, v1, dSy, ay, by, cp1);
            const T nvz = vel_update<T, MODEL, KAHAN>(a, v2, dSz, az, bz, cp2);
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

        // the new stresses of plane p
        if (write && in_grid) {
#pragma unroll
            for (int f = 0; f < 6; ++f) fa.o[3 + f][c] = sv[f];
        }
        szz_mm = szz_m;
        szz_m = sv[2];
    }
}

}  // namespace ewf
