// ewfd_kernels.cuh -- sm_103a kernels of the staggered-grid elastic FDTD time step.
//
// Device layout ("box"): every field -- the 9 staggered state fields, the material fields and
// the 3-D damping field -- lives in one padded geometry shared by all of them:
//   element (i,j,k) at base[i + j*sx + k*sy],  i in [-HX, sx-HX), j in [-1, ny+2), k in [-1, nz+2)
// with HX = 128 B / sizeof(T) so that i = 0 starts a 128-byte line, sx a multiple of 32 and
// the base pointer placed at (0,0,0).  The reference's staggered extents (Vx is (nx+1,ny,nz),
// sxy is (nx+1,ny+1,nz) and so on) all fit inside; cells outside an array's own extent are
// zero and are never written, which makes every neighbour read of the reference stencil an
// in-bounds read of a zero (the reference reads a wrapped neighbour there, e.g. OK4:323-329,
// only for cells whose value is never read back).
//
// One time step (reference order OK4:485-505 / ANISO:519-555):
//   k_stress    stress update + damping, free surface BC1 fused at planes k = 0..2
//   k_inject    moment-tensor point injection (before-BC1 semantics replayed exactly)
//   k_velocity  velocity update + damping (optionally Kahan-compensated)
//   k_record    receiver gather into FP64 traces; advances the device step counter
// Expression order follows the reference so that an FMA-free build is bit-identical to the
// reference's FMA-free build.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ewf {

enum { MODEL_ISO = 0, MODEL_ORTHO = 1 };
enum { DAMP_PML1D = 0, DAMP_W3D = 1, DAMP_SEP = 2 };

// Tile of the z-marching kernels: one thread per (i,j) column, a CTA covers TX x TY columns
// and a chunk of planes.
constexpr int TX = 32;
constexpr int TY = 8;

template <typename T>
struct StepArgs {
    T *f[9];          // Vx Vy Vz sxx syy szz sxy sxz syz
    T *comp[3];       // Kahan compensation of Vx Vy Vz (null unless compensated)
    const T *m[12];   // iso: c11 c12 | ortho: C11 C22 C33 C12 C13 C23 C66xy C55xz C44yz Bx By Bz
    const T *w1[3];   // iso: PML profiles (n+1 each) | separable: per-axis factors (n each)
    const T *w3;      // 3-D damping field (box layout)
    long long sy;     // plane pitch, elements
    int sx;           // row pitch, elements
    int nx, ny, nz;
    int bc1_rows;     // rows j < bc1_rows get the szz / sxz free-surface rule (OK4:279-281)
    int kchunk;       // planes per CTA
    T dt, rdt, dx, dy, dz, rdx, rdy, rdz;
    T c66, bx, by, bz;  // isotropic scalars (OK4:405-407)
    T third;            // (T)1/(T)3 of BC1
};

struct SrcEntry {
    int comp, i, j, k;
    double coef;
};

template <typename T>
__device__ __forceinline__ T ld(const T *p) { return __ldg(p); }

// ---------------------------------------------------------------------------------------------
// Stress update.  Isotropic: OK4:285-331.  Orthorhombic: ANISO:287-356.  BC1: OK4:271-283.
// ---------------------------------------------------------------------------------------------
template <typename T, int MODEL, int DAMP>
__global__ void __launch_bounds__(TX * TY) k_stress(const StepArgs<T> a)
{
    const int i = blockIdx.x * TX + threadIdx.x;
    const int j = blockIdx.y * TY + threadIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    const int k0 = blockIdx.z * a.kchunk;
    const int k1 = min(k0 + a.kchunk, a.nz);
    const int sx = a.sx;
    const long long sy = a.sy;
    const long long c0 = (long long)i + (long long)j * sx + (long long)k0 * sy;

    const T *__restrict__ Vx = a.f[0];
    const T *__restrict__ Vy = a.f[1];
    const T *__restrict__ Vz = a.f[2];
    T *__restrict__ sxx = a.f[3];
    T *__restrict__ syy = a.f[4];
    T *__restrict__ szz = a.f[5];
    T *__restrict__ sxy = a.f[6];
    T *__restrict__ sxz = a.f[7];
    T *__restrict__ syz = a.f[8];
    const T dt = a.dt, rdx = a.rdx, rdy = a.rdy, rdz = a.rdz;

    // damping factors constant along the column
    T wavx = T(0), wavy = T(0), wxi = T(0), wyj = T(0), pxy = T(0);
    if (DAMP == DAMP_PML1D) {
        wxi = ld(a.w1[0] + i);
        wyj = ld(a.w1[1] + j);
        wavx = T(0.5) * (ld(a.w1[0] + i + 1) + wxi);
        wavy = T(0.5) * (ld(a.w1[1] + j + 1) + wyj);
    } else if (DAMP == DAMP_SEP) {
        pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
    }
    const bool row_bc = (j < a.bc1_rows);

    // z-rotation registers
    long long c = c0;
    T vx_m = ld(Vx + c - sy);  // Vx(k-1)
    T vy_m = ld(Vy + c - sy);  // Vy(k-1)
    T vz_k = ld(Vz + c);       // Vz(k)
    T wz_k = T(0);
    if (DAMP == DAMP_PML1D) wz_k = ld(a.w1[2] + k0);

    for (int k = k0; k < k1; ++k, c += sy) {
        const T vx_k = ld(Vx + c);
        const T vy_k = ld(Vy + c);
        const T vz_p = ld(Vz + c + sy);
        const T Vxx = (ld(Vx + c + 1) - vx_k) * rdx;
        const T Vyy = (ld(Vy + c + sx) - vy_k) * rdy;
        const T Vzz = (vz_p - vz_k) * rdz;
        T sxz_new = T(0), syz_new = T(0);
        if (MODEL == MODEL_ISO) {
            const T wz_p = ld(a.w1[2] + k + 1);
            const T c11 = ld(a.m[0] + c), c12 = ld(a.m[1] + c);
            // OK4:307-309
            sxx[c] = wavx * (sxx[c] + dt * (c11 * Vxx + c12 * Vyy + c12 * Vzz));
            syy[c] = wavy * (syy[c] + dt * (c12 * Vxx + c11 * Vyy + c12 * Vzz));
            const T szz_new = T(0.5) * (wz_p + wz_k) * (szz[c] + dt * (c12 * Vxx + c12 * Vyy + c11 * Vzz));
            szz[c] = (k == 0 && row_bc) ? T(0) : szz_new;
            const T c66dt = a.c66 * dt;
            // OK4:323, 326, 329 (no guards: zero-padded neighbours at the low edges)
            sxy[c] = wz_k * wyj * wxi * (sxy[c] + c66dt * ((vy_k - ld(Vy + c - 1)) * rdx + (vx_k - ld(Vx + c - sx)) * rdy));
            sxz_new = wyj * wz_k * wxi * (sxz[c] + c66dt * ((vz_k - ld(Vz + c - 1)) * rdx + (vx_k - vx_m) * rdz));
            sxz[c] = sxz_new;
            syz_new = wxi * wyj * wz_k * (syz[c] + c66dt * ((vy_k - vy_m) * rdz + (vz_k - ld(Vz + c - sx)) * rdy));
            syz[c] = syz_new;
            wz_k = wz_p;
        } else {
            T W;
            if (DAMP == DAMP_W3D) W = ld(a.w3 + c);
            else W = pxy * ld(a.w1[2] + k);
            const T C11 = ld(a.m[0] + c), C22 = ld(a.m[1] + c), C33 = ld(a.m[2] + c);
            const T C12 = ld(a.m[3] + c), C13 = ld(a.m[4] + c), C23 = ld(a.m[5] + c);
            // ANISO:312-325
            sxx[c] = sxx[c] * W + dt * (C11 * Vxx + C12 * Vyy + C13 * Vzz);
            syy[c] = syy[c] * W + dt * (C12 * Vxx + C22 * Vyy + C23 * Vzz);
            const T szz_new = szz[c] * W + dt * (C13 * Vxx + C23 * Vyy + C33 * Vzz);
            szz[c] = (k == 0 && row_bc) ? T(0) : szz_new;
            // ANISO:327-352 (shear derivatives divide by the spacing)
            if (i > 0 && j > 0) {
                const T dVx_dy = (vx_k - ld(Vx + c - sx)) / a.dy;
                const T dVy_dx = (vy_k - ld(Vy + c - 1)) / a.dx;
                sxy[c] = sxy[c] * W + dt * ld(a.m[6] + c) * (dVy_dx + dVx_dy);
            }
            if (i > 0 && k > 0) {
                const T dVx_dz = (vx_k - vx_m) / a.dz;
                const T dVz_dx = (vz_k - ld(Vz + c - 1)) / a.dx;
                sxz_new = sxz[c] * W + dt * ld(a.m[7] + c) * (dVz_dx + dVx_dz);
                sxz[c] = sxz_new;
            }
            if (j > 0 && k > 0) {
                const T dVy_dz = (vy_k - vy_m) / a.dz;
                const T dVz_dy = (vz_k - ld(Vz + c - sx)) / a.dy;
                syz_new = syz[c] * W + dt * ld(a.m[8] + c) * (dVy_dz + dVz_dy);
                syz[c] = syz_new;
            }
        }
        // BC1 plane 1 from the freshly updated plane 2 (OK4:281-282)
        if (k == 2) {
            if (i > 0 && row_bc) sxz[c - sy] = a.third * sxz_new;
            if (j > 0) syz[c - sy] = a.third * syz_new;
        }
        vx_m = vx_k;
        vy_m = vy_k;
        vz_k = vz_p;
    }
}

// ---------------------------------------------------------------------------------------------
// Point injection sigma_c += coef * Src[it], one thread, entries in order.
// order 0 replays "inject, then BC1" (OK4:336-342 run inside the stress kernel, BC1 after it):
// an entry on a cell that BC1 overwrites is dropped, and an entry on the plane BC1 copies from
// refreshes the copy.  order 1 is "BC1, then inject" (ANISO:533-535).
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_inject(const StepArgs<T> a, const SrcEntry *__restrict__ src, int nsrc,
                         const double *__restrict__ stf, int nstf, const int *__restrict__ it_ptr, int order)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int it = *it_ptr;
    if (it < 0 || it >= nstf) return;  // the host validates the step range; never read past Src
    const T s = (T)stf[it];
    for (int e = 0; e < nsrc; ++e) {
        const SrcEntry q = src[e];
        const long long c = (long long)q.i + (long long)q.j * a.sx + (long long)q.k * a.sy;
        T *f = a.f[q.comp];
        if (order == 0) {
            const bool row_bc = q.j < a.bc1_rows;
            const bool xz_bc = (q.comp == 7) && q.i > 0 && q.i < a.nx && row_bc;
            const bool yz_bc = (q.comp == 8) && q.j > 0 && q.j < a.ny && q.i < a.nx;
            if ((q.comp == 5 && q.k == 0 && row_bc) || ((xz_bc || yz_bc) && q.k == 1)) continue;
            f[c] = f[c] + (T)q.coef * s;
            if ((xz_bc || yz_bc) && q.k == 2) f[c - a.sy] = a.third * f[c];
        } else {
            f[c] = f[c] + (T)q.coef * s;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Velocity update.  Isotropic: OK4:346-378.  Orthorhombic: ANISO:358-389.
// KAHAN: V = a*V + inc with the rounding error carried in comp[] (compensated summation).
// ---------------------------------------------------------------------------------------------
template <typename T, int MODEL, int DAMP, bool KAHAN>
__global__ void __launch_bounds__(TX * TY) k_velocity(const StepArgs<T> a)
{
    const int i = blockIdx.x * TX + threadIdx.x;
    const int j = blockIdx.y * TY + threadIdx.y;
    if (i < 1 || j < 1 || i >= a.nx || j >= a.ny) return;
    const int k0 = max(1, (int)blockIdx.z * a.kchunk);
    const int k1 = min((int)blockIdx.z * a.kchunk + a.kchunk, a.nz);
    if (k0 >= k1) return;
    const int sx = a.sx;
    const long long sy = a.sy;
    const int nx = a.nx, ny = a.ny, nz = a.nz;

    T *__restrict__ Vx = a.f[0];
    T *__restrict__ Vy = a.f[1];
    T *__restrict__ Vz = a.f[2];
    const T *__restrict__ sxx = a.f[3];
    const T *__restrict__ syy = a.f[4];
    const T *__restrict__ szz = a.f[5];
    const T *__restrict__ sxy = a.f[6];
    const T *__restrict__ sxz = a.f[7];
    const T *__restrict__ syz = a.f[8];
    const T dt = a.dt, rdt = a.rdt, rdx = a.rdx, rdy = a.rdy, rdz = a.rdz;

    const bool do_x = (j < ny - 1);
    const bool do_y = (i < nx - 1);
    const bool do_z = (i < nx - 1) && (j < ny - 1);

    T wxm = T(0), wym = T(0), pxy = T(0);
    if (DAMP == DAMP_PML1D) {
        wxm = ld(a.w1[0] + i - 1);
        wym = ld(a.w1[1] + j - 1);
    } else if (DAMP == DAMP_SEP) {
        pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
    }

    long long c = (long long)i + (long long)j * sx + (long long)k0 * sy;
    T szz_m = ld(szz + c - sy);
    T sxz_k = ld(sxz + c);
    T syz_k = ld(syz + c);

    for (int k = k0; k < k1; ++k, c += sy) {
        const T szz_k = ld(szz + c);
        const T sxz_p = ld(sxz + c + sy);
        const T syz_p = ld(syz + c + sy);
        T Wc = T(0);
        if (MODEL == MODEL_ORTHO) {
            if (DAMP == DAMP_W3D) Wc = ld(a.w3 + c);
            else Wc = pxy * ld(a.w1[2] + k);
        }
        if (do_x && k < nz - 1) {
            const T sxy_k = ld(sxy + c);
            const T dSx = (ld(sxx + c) - ld(sxx + c - 1)) * rdx + (ld(sxy + c + sx) - sxy_k) * rdy + (sxz_p - sxz_k) * rdz;
            T &V = Vx[c];
            if (!KAHAN) {
                if (MODEL == MODEL_ISO) V = wxm * (V * rdt + a.bx * dSx) * dt;
                else V = (V * rdt * Wc + ld(a.m[9] + c) * dSx) * dt;
            } else {
                const T aa = (MODEL == MODEL_ISO) ? wxm : Wc;
                const T inc = (MODEL == MODEL_ISO) ? aa * (a.bx * dSx) * dt : ld(a.m[9] + c) * dSx * dt;
                T &cp = a.comp[0][c];
                const T y = inc - aa * cp;
                const T av = aa * V;
                const T t = av + y;
                cp = (t - av) - y;
                V = t;
            }
        }
        if (do_y && k < nz - 1) {
            const T dSy = (ld(syy + c) - ld(syy + c - sx)) * rdy + (ld(sxy + c + 1) - ld(sxy + c)) * rdx + (syz_p - syz_k) * rdz;
            T &V = Vy[c];
            if (!KAHAN) {
                if (MODEL == MODEL_ISO) V = wym * (V * rdt + a.by * dSy) * dt;
                else V = (V * rdt * Wc + ld(a.m[10] + c) * dSy) * dt;
            } else {
                const T aa = (MODEL == MODEL_ISO) ? wym : Wc;
                const T inc = (MODEL == MODEL_ISO) ? aa * (a.by * dSy) * dt : ld(a.m[10] + c) * dSy * dt;
                T &cp = a.comp[1][c];
                const T y = inc - aa * cp;
                const T av = aa * V;
                const T t = av + y;
                cp = (t - av) - y;
                V = t;
            }
        }
        if (do_z) {
            const T dSz = (szz_k - szz_m) * rdz + (ld(sxz + c + 1) - sxz_k) * rdx + (ld(syz + c + sx) - syz_k) * rdy;
            T &V = Vz[c];
            T wzm = T(0);
            if (MODEL == MODEL_ISO) wzm = ld(a.w1[2] + k - 1);
            if (!KAHAN) {
                if (MODEL == MODEL_ISO) V = wzm * (V * rdt + a.bz * dSz) * dt;
                else V = (V * rdt * Wc + ld(a.m[11] + c) * dSz) * dt;
            } else {
                const T aa = (MODEL == MODEL_ISO) ? wzm : Wc;
                const T inc = (MODEL == MODEL_ISO) ? aa * (a.bz * dSz) * dt : ld(a.m[11] + c) * dSz * dt;
                T &cp = a.comp[2][c];
                const T y = inc - aa * cp;
                const T av = aa * V;
                const T t = av + y;
                cp = (t - av) - y;
                V = t;
            }
        }
        szz_m = szz_k;
        sxz_k = sxz_p;
        syz_k = syz_p;
    }
}

// ---------------------------------------------------------------------------------------------
// Receiver gather (OK4:383-386, ANISO:254-268): traces[r*len + it] = field value after the
// velocity update, widened to FP64.  One CTA; thread 0 advances the step counter last.
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_record(const StepArgs<T> a, const long long *__restrict__ rec_off, const int *__restrict__ rec_comp,
                         int nrec, double *__restrict__ traces, int trace_len, int *it_ptr)
{
    const int it = *it_ptr;
    if (it >= 0 && it < trace_len)
        for (int r = threadIdx.x; r < nrec; r += blockDim.x)
            traces[(long long)r * trace_len + it] = (double)a.f[rec_comp[r]][rec_off[r]];
    __syncthreads();
    if (threadIdx.x == 0) *it_ptr = it + 1;
}

// ---------------------------------------------------------------------------------------------
// Layout conversion between the reference layout (x fastest, the array's own extents) and the
// box layout, with dtype conversion.
// ---------------------------------------------------------------------------------------------
template <typename TD, typename TS>
__global__ void k_pack(TD *__restrict__ box, const TS *__restrict__ src, int ex, int ey, int ez, int sx, long long sy)
{
    const long long n = (long long)ex * ey * ez;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % ex);
        const long long r = e / ex;
        const int j = (int)(r % ey);
        const int k = (int)(r / ey);
        box[(long long)i + (long long)j * sx + (long long)k * sy] = (TD)src[e];
    }
}

template <typename TD, typename TS>
__global__ void k_unpack(TD *__restrict__ dst, const TS *__restrict__ box, int ex, int ey, int ez, int sx, long long sy)
{
    const long long n = (long long)ex * ey * ez;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % ex);
        const long long r = e / ex;
        const int j = (int)(r % ey);
        const int k = (int)(r / ey);
        dst[e] = (TD)box[(long long)i + (long long)j * sx + (long long)k * sy];
    }
}

}  // namespace ewf
