/*
 * ewf_oracle_body.h -- precision-generic body of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Included twice by ewf_oracle.c, once with OT=float and once with OT=double.  Every
 * expression keeps the operand order of the reference kernels so that, compiled without
 * floating-point contraction (-ffp-contract=off), each operation rounds exactly as the
 * reference's FMA-free build does.
 *
 * Array layout is the reference's: x fastest, idx = i + j*Px + k*Px*Py with each array's
 * own extents (OK4:431-439):
 *   Vx (nx+1,ny,nz)  Vy (nx,ny+1,nz)  Vz (nx,ny,nz+1)  sxx/syy/szz (nx,ny,nz)
 *   sxy (nx+1,ny+1,nz)  sxz (nx+1,ny,nz+1)  syz (nx,ny+1,nz+1)
 */

#define OFN2(a, b) a##_##b
#define OFN1(a, b) OFN2(a, b)
#define OFN(name) OFN1(name, OSUF)

/* Read with zero outside the array: used only for the isotropic shear edge cells, where the
 * reference reads a wrapped neighbour (OK4:323-329).  Those cells are never read back by the
 * velocity update (its ranges start at 1, OK4:358-377), so their value is unobservable. */
static inline OT OFN(at0)(const OT *a, long i, long j, long k, long px, long py, long pz)
{
    if (i < 0 || j < 0 || k < 0 || i >= px || j >= py || k >= pz) return (OT)0;
    return a[i + px * (j + py * k)];
}

/* Isotropic stress update with 1-D PML (OK4:285-331 compute_StressPrf). */
static void OFN(stress_iso)(const orc_grid *g, OT *const *f, const OT *const *m, const OT *const *w)
{
    const long nx = g->nx, ny = g->ny, nz = g->nz;
    const OT dt = (OT)g->dt, rdx = (OT)1.0 / (OT)g->dx, rdy = (OT)1.0 / (OT)g->dy, rdz = (OT)1.0 / (OT)g->dz;
    const OT c66s = (OT)g->c66;
    const OT *Vx = f[0], *Vy = f[1], *Vz = f[2];
    OT *sxx = f[3], *syy = f[4], *szz = f[5], *sxy = f[6], *sxz = f[7], *syz = f[8];
    const OT *c11 = m[0], *c12 = m[1];
    const OT *wx = w[0], *wy = w[1], *wz = w[2];
    long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; k++) {
        for (long j = 0; j < ny; j++) {
            for (long i = 0; i < nx; i++) {
                const long c = i + nx * (j + ny * k);
                /* the diff_BC2_OK3 scheme's c44u: its own value on plane 1, c66 elsewhere */
                const OT c66 = (g->smu > 0.0 && k == 1) ? (OT)g->smu : c66s;
                const OT Vxx = (Vx[(i + 1) + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * (j + ny * k)]) * rdx;
                const OT Vyy = (Vy[i + nx * ((j + 1) + (ny + 1) * k)] - Vy[i + nx * (j + (ny + 1) * k)]) * rdy;
                const OT Vzz = (Vz[i + nx * (j + ny * (k + 1))] - Vz[i + nx * (j + ny * k)]) * rdz;
                /* OK4:307-309 */
                sxx[c] = (OT)0.5 * (wx[i + 1] + wx[i]) * (sxx[c] + dt * (c11[c] * Vxx + c12[c] * Vyy + c12[c] * Vzz));
                syy[c] = (OT)0.5 * (wy[j + 1] + wy[j]) * (syy[c] + dt * (c12[c] * Vxx + c11[c] * Vyy + c12[c] * Vzz));
                szz[c] = (OT)0.5 * (wz[k + 1] + wz[k]) * (szz[c] + dt * (c12[c] * Vxx + c12[c] * Vyy + c11[c] * Vzz));
                /* OK4:323 sxy, no guard: edge cells i==0 / j==0 read outside (never read back) */
                {
                    const long e = i + (nx + 1) * (j + (ny + 1) * k);
                    OT dvy, dvx;
                    if (i > 0 && j > 0) {
                        dvy = Vy[i + nx * (j + (ny + 1) * k)] - Vy[(i - 1) + nx * (j + (ny + 1) * k)];
                        dvx = Vx[i + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * ((j - 1) + ny * k)];
                    } else {
                        dvy = OFN(at0)(Vy, i, j, k, nx, ny + 1, nz) - OFN(at0)(Vy, i - 1, j, k, nx, ny + 1, nz);
                        dvx = OFN(at0)(Vx, i, j, k, nx + 1, ny, nz) - OFN(at0)(Vx, i, j - 1, k, nx + 1, ny, nz);
                    }
                    sxy[e] = wz[k] * wy[j] * wx[i] * (sxy[e] + c66 * dt * (dvy * rdx + dvx * rdy));
                }
                /* OK4:326 sxz */
                {
                    const long e = i + (nx + 1) * (j + ny * k);
                    OT dvz, dvx;
                    if (i > 0 && k > 0) {
                        dvz = Vz[i + nx * (j + ny * k)] - Vz[(i - 1) + nx * (j + ny * k)];
                        dvx = Vx[i + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * (j + ny * (k - 1))];
                    } else {
                        dvz = OFN(at0)(Vz, i, j, k, nx, ny, nz + 1) - OFN(at0)(Vz, i - 1, j, k, nx, ny, nz + 1);
                        dvx = OFN(at0)(Vx, i, j, k, nx + 1, ny, nz) - OFN(at0)(Vx, i, j, k - 1, nx + 1, ny, nz);
                    }
                    sxz[e] = wy[j] * wz[k] * wx[i] * (sxz[e] + c66 * dt * (dvz * rdx + dvx * rdz));
                }
                /* OK4:329 syz */
                {
                    const long e = i + nx * (j + (ny + 1) * k);
                    OT dvy, dvz;
                    if (j > 0 && k > 0) {
                        dvy = Vy[i + nx * (j + (ny + 1) * k)] - Vy[i + nx * (j + (ny + 1) * (k - 1))];
                        dvz = Vz[i + nx * (j + ny * k)] - Vz[i + nx * ((j - 1) + ny * k)];
                    } else {
                        dvy = OFN(at0)(Vy, i, j, k, nx, ny + 1, nz) - OFN(at0)(Vy, i, j, k - 1, nx, ny + 1, nz);
                        dvz = OFN(at0)(Vz, i, j, k, nx, ny, nz + 1) - OFN(at0)(Vz, i, j - 1, k, nx, ny, nz + 1);
                    }
                    syz[e] = wx[i] * wy[j] * wz[k] * (syz[e] + c66 * dt * (dvy * rdz + dvz * rdy));
                }
            }
        }
    }
}

/* Isotropic stress update with a 3-D weight field per component (the DC_Earthquake solver,
 * FastWaveED_GPU3D_v1.cu:298-320): w_c * (sigma_c + ...), each weight in its component's
 * layout (w[0] Vx-, w[1] Vy-, w[2] Vz-, w[3..5] sxy/sxz/syz-shaped), shear moduli c66 (xy),
 * c55 (xz), c44 (yz), shear cells guarded like ANISO. */
static void OFN(stress_iso_percomp)(const orc_grid *g, OT *const *f, const OT *const *m, const OT *const *w)
{
    const long nx = g->nx, ny = g->ny, nz = g->nz;
    const OT dt = (OT)g->dt, rdx = (OT)1.0 / (OT)g->dx, rdy = (OT)1.0 / (OT)g->dy, rdz = (OT)1.0 / (OT)g->dz;
    const OT c66 = (OT)g->c66, c55 = (OT)g->c55, c44 = (OT)g->c44;
    const OT *Vx = f[0], *Vy = f[1], *Vz = f[2];
    OT *sxx = f[3], *syy = f[4], *szz = f[5], *sxy = f[6], *sxz = f[7], *syz = f[8];
    const OT *c11 = m[0], *c12 = m[1];
    long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; k++) {
        for (long j = 0; j < ny; j++) {
            for (long i = 0; i < nx; i++) {
                const long c = i + nx * (j + ny * k);
                const long ex = i + (nx + 1) * (j + ny * k), ey = i + nx * (j + (ny + 1) * k);
                const OT Vxx = (Vx[ex + 1] - Vx[ex]) * rdx;
                const OT Vyy = (Vy[i + nx * ((j + 1) + (ny + 1) * k)] - Vy[ey]) * rdy;
                const OT Vzz = (Vz[i + nx * (j + ny * (k + 1))] - Vz[c]) * rdz;
                /* :313-315 */
                sxx[c] = w[0][ex] * (sxx[c] + dt * (c11[c] * Vxx + c12[c] * Vyy + c12[c] * Vzz));
                syy[c] = w[1][ey] * (syy[c] + dt * (c12[c] * Vxx + c11[c] * Vyy + c12[c] * Vzz));
                szz[c] = w[2][c] * (szz[c] + dt * (c12[c] * Vxx + c12[c] * Vyy + c11[c] * Vzz));
                /* :318 */
                if (i > 0 && j > 0) {
                    const long e = i + (nx + 1) * (j + (ny + 1) * k);
                    const OT dvy = Vy[ey] - Vy[(i - 1) + nx * (j + (ny + 1) * k)];
                    const OT dvx = Vx[ex] - Vx[i + (nx + 1) * ((j - 1) + ny * k)];
                    sxy[e] = w[3][e] * (sxy[e] + c66 * dt * (dvy * rdx + dvx * rdy));
                }
                /* :319 */
                if (i > 0 && k > 0) {
                    const long e = ex;
                    const OT dvz = Vz[c] - Vz[(i - 1) + nx * (j + ny * k)];
                    const OT dvx = Vx[ex] - Vx[i + (nx + 1) * (j + ny * (k - 1))];
                    sxz[e] = w[4][e] * (sxz[e] + c55 * dt * (dvz * rdx + dvx * rdz));
                }
                /* :320 */
                if (j > 0 && k > 0) {
                    const long e = ey;
                    const OT dvy = Vy[ey] - Vy[i + nx * (j + (ny + 1) * (k - 1))];
                    const OT dvz = Vz[c] - Vz[i + nx * ((j - 1) + ny * k)];
                    syz[e] = w[5][e] * (syz[e] + c44 * dt * (dvy * rdz + dvz * rdy));
                }
            }
        }
    }
}

/* Orthorhombic stress update with a 3-D weight field (ANISO:287-356 compute_StressOrtho). */
static void OFN(stress_ortho)(const orc_grid *g, OT *const *f, const OT *const *m, const OT *W)
{
    const long nx = g->nx, ny = g->ny, nz = g->nz;
    const OT dt = (OT)g->dt, dx = (OT)g->dx, dy = (OT)g->dy, dz = (OT)g->dz;
    const OT rdx = (OT)1.0 / dx, rdy = (OT)1.0 / dy, rdz = (OT)1.0 / dz;
    const OT *Vx = f[0], *Vy = f[1], *Vz = f[2];
    OT *sxx = f[3], *syy = f[4], *szz = f[5], *sxy = f[6], *sxz = f[7], *syz = f[8];
    const OT *C11 = m[0], *C22 = m[1], *C33 = m[2], *C12 = m[3], *C13 = m[4], *C23 = m[5];
    const OT *C66 = m[6], *C55 = m[7], *C44 = m[8];
    long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; k++) {
        for (long j = 0; j < ny; j++) {
            for (long i = 0; i < nx; i++) {
                const long c = i + nx * (j + ny * k);
                const OT Vxx = (Vx[(i + 1) + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * (j + ny * k)]) * rdx;
                const OT Vyy = (Vy[i + nx * ((j + 1) + (ny + 1) * k)] - Vy[i + nx * (j + (ny + 1) * k)]) * rdy;
                const OT Vzz = (Vz[i + nx * (j + ny * (k + 1))] - Vz[i + nx * (j + ny * k)]) * rdz;
                const OT Wc = W[c];
                /* ANISO:312-325 */
                sxx[c] = sxx[c] * Wc + dt * (C11[c] * Vxx + C12[c] * Vyy + C13[c] * Vzz);
                syy[c] = syy[c] * Wc + dt * (C12[c] * Vxx + C22[c] * Vyy + C23[c] * Vzz);
                szz[c] = szz[c] * Wc + dt * (C13[c] * Vxx + C23[c] * Vyy + C33[c] * Vzz);
                /* ANISO:327-334 */
                if (i > 0 && j > 0) {
                    const long e = i + (nx + 1) * (j + (ny + 1) * k);
                    const OT dVx_dy = (Vx[i + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * ((j - 1) + ny * k)]) / dy;
                    const OT dVy_dx = (Vy[i + nx * (j + (ny + 1) * k)] - Vy[(i - 1) + nx * (j + (ny + 1) * k)]) / dx;
                    sxy[e] = sxy[e] * Wc + dt * C66[e] * (dVy_dx + dVx_dy);
                }
                /* ANISO:336-343 */
                if (i > 0 && k > 0) {
                    const long e = i + (nx + 1) * (j + ny * k);
                    const OT dVx_dz = (Vx[i + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * (j + ny * (k - 1))]) / dz;
                    const OT dVz_dx = (Vz[i + nx * (j + ny * k)] - Vz[(i - 1) + nx * (j + ny * k)]) / dx;
                    sxz[e] = sxz[e] * Wc + dt * C55[e] * (dVz_dx + dVx_dz);
                }
                /* ANISO:345-352 */
                if (j > 0 && k > 0) {
                    const long e = i + nx * (j + (ny + 1) * k);
                    const OT dVy_dz = (Vy[i + nx * (j + (ny + 1) * k)] - Vy[i + nx * (j + (ny + 1) * (k - 1))]) / dz;
                    const OT dVz_dy = (Vz[i + nx * (j + ny * k)] - Vz[i + nx * ((j - 1) + ny * k)]) / dy;
                    syz[e] = syz[e] * Wc + dt * C44[e] * (dVy_dz + dVz_dy);
                }
            }
        }
    }
}

/* Isotropic stress update with cell c11/c12, edge shear moduli and a 3-D weight field, the 9 km
 * station scheme (9kmst.cu:287-331 compute_StressPrf): ANISO's structure, but the shear
 * derivatives are multiplied by 1/d instead of divided by d.  m[] uses the orthorhombic slots:
 * m[0] c11u_het, m[3] c12u_het, m[6..8] c44u_het xy, xz, yz. */
static void OFN(stress_isohet)(const orc_grid *g, OT *const *f, const OT *const *m, const OT *W)
{
    const long nx = g->nx, ny = g->ny, nz = g->nz;
    const OT dt = (OT)g->dt;
    const OT rdx = (OT)1.0 / (OT)g->dx, rdy = (OT)1.0 / (OT)g->dy, rdz = (OT)1.0 / (OT)g->dz;
    const OT *Vx = f[0], *Vy = f[1], *Vz = f[2];
    OT *sxx = f[3], *syy = f[4], *szz = f[5], *sxy = f[6], *sxz = f[7], *syz = f[8];
    const OT *c11 = m[0], *c12 = m[3], *mxy = m[6], *mxz = m[7], *myz = m[8];
    long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; k++) {
        for (long j = 0; j < ny; j++) {
            for (long i = 0; i < nx; i++) {
                const long c = i + nx * (j + ny * k);
                const OT Vxx = (Vx[(i + 1) + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * (j + ny * k)]) * rdx;
                const OT Vyy = (Vy[i + nx * ((j + 1) + (ny + 1) * k)] - Vy[i + nx * (j + (ny + 1) * k)]) * rdy;
                const OT Vzz = (Vz[i + nx * (j + ny * (k + 1))] - Vz[i + nx * (j + ny * k)]) * rdz;
                const OT Wc = W[c];
                /* 9kmst.cu:316-318 */
                sxx[c] = sxx[c] * Wc + dt * (c11[c] * Vxx + c12[c] * Vyy + c12[c] * Vzz);
                syy[c] = syy[c] * Wc + dt * (c12[c] * Vxx + c11[c] * Vyy + c12[c] * Vzz);
                szz[c] = szz[c] * Wc + dt * (c12[c] * Vxx + c12[c] * Vyy + c11[c] * Vzz);
                /* 9kmst.cu:321 */
                if (i > 0 && j > 0) {
                    const long e = i + (nx + 1) * (j + (ny + 1) * k);
                    const OT dvy = Vy[i + nx * (j + (ny + 1) * k)] - Vy[(i - 1) + nx * (j + (ny + 1) * k)];
                    const OT dvx = Vx[i + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * ((j - 1) + ny * k)];
                    sxy[e] = sxy[e] * Wc + mxy[e] * dt * (dvy * rdx + dvx * rdy);
                }
                /* 9kmst.cu:323 */
                if (i > 0 && k > 0) {
                    const long e = i + (nx + 1) * (j + ny * k);
                    const OT dvz = Vz[i + nx * (j + ny * k)] - Vz[(i - 1) + nx * (j + ny * k)];
                    const OT dvx = Vx[i + (nx + 1) * (j + ny * k)] - Vx[i + (nx + 1) * (j + ny * (k - 1))];
                    sxz[e] = sxz[e] * Wc + mxz[e] * dt * (dvz * rdx + dvx * rdz);
                }
                /* 9kmst.cu:325 */
                if (j > 0 && k > 0) {
                    const long e = i + nx * (j + (ny + 1) * k);
                    const OT dvy = Vy[i + nx * (j + (ny + 1) * k)] - Vy[i + nx * (j + (ny + 1) * (k - 1))];
                    const OT dvz = Vz[i + nx * (j + ny * k)] - Vz[i + nx * ((j - 1) + ny * k)];
                    syz[e] = syz[e] * Wc + myz[e] * dt * (dvy * rdz + dvz * rdy);
                }
            }
        }
    }
}

/* Free surface (OK4:271-283 / ANISO:270-285 BC1), applied after the stress update. */
static void OFN(bc1)(const orc_grid *g, OT *const *f)
{
    const long nx = g->nx, ny = g->ny;
    const long rows = g->bc1_rows;
    OT *szz = f[5], *sxz = f[7], *syz = f[8];
    const OT third = (OT)1.0 / (OT)3.0;
    for (long j = 0; j < rows; j++)
        for (long i = 0; i < nx; i++) szz[i + nx * j] = (OT)0.0;
    for (long j = 0; j < rows; j++)
        for (long i = 1; i < nx; i++)
            sxz[i + (nx + 1) * (j + ny * 1)] = third * sxz[i + (nx + 1) * (j + ny * 2)];
    for (long j = 1; j < ny; j++)
        for (long i = 0; i < nx; i++)
            syz[i + nx * (j + (ny + 1) * 1)] = third * syz[i + nx * (j + (ny + 1) * 2)];
}

/* Extents of field id 0..8 in the reference layout. */
static void OFN(extent)(const orc_grid *g, int id, long *px, long *py)
{
    const long nx = g->nx, ny = g->ny;
    static const int ex[9] = {1, 0, 0, 0, 0, 0, 1, 1, 0};
    static const int ey[9] = {0, 1, 0, 0, 0, 0, 1, 0, 1};
    *px = nx + ex[id];
    *py = ny + ey[id];
}

/* Point injection sigma_c += coef * Src[it] (OK4:336-342, ANISO:228-252). */
static void OFN(inject)(const orc_grid *g, OT *const *f, int nsrc, const int32_t *src, const double *coef,
                        const double *stf, int it)
{
    for (int s = 0; s < nsrc; s++) {
        const int id = src[4 * s + 0];
        long px, py;
        OFN(extent)(g, id, &px, &py);
        const long e = (long)src[4 * s + 1] + px * ((long)src[4 * s + 2] + py * (long)src[4 * s + 3]);
        f[id][e] = f[id][e] + (OT)coef[s] * (OT)stf[it];
    }
}

/* Velocity update (OK4:346-378 update_Qxft; ANISO:358-389 update_VelocityFromStress).
 * comp != NULL selects the compensated (Kahan) form: V = a*V + inc with the rounding error of
 * each step carried in comp[] (a = damping factor, inc = the stress-divergence increment). */
static void OFN(velocity)(const orc_grid *g, OT *const *f, const OT *const *m, const OT *const *w, const OT *W,
                          OT *const *comp)
{
    const long nx = g->nx, ny = g->ny, nz = g->nz;
    const OT dt = (OT)g->dt, rdt = (OT)1.0 / (OT)g->dt;
    const OT rdx = (OT)1.0 / (OT)g->dx, rdy = (OT)1.0 / (OT)g->dy, rdz = (OT)1.0 / (OT)g->dz;
    OT *Vx = f[0], *Vy = f[1], *Vz = f[2];
    const OT *sxx = f[3], *syy = f[4], *szz = f[5], *sxy = f[6], *sxz = f[7], *syz = f[8];
    const int iso = (g->model == 0);
    const int pc = (g->damping == 3);  /* per-component weights, in each velocity's own layout */
    const OT bx = (OT)g->bx, by = (OT)g->by, bz = (OT)g->bz;
    const OT vd = (OT)g->vdamp;  /* 16kmst.cu:337-349: update - vdamp * V_old */
    long k;
#pragma omp parallel for schedule(static)
    for (k = 1; k < nz; k++) {
        for (long j = 1; j < ny; j++) {
            for (long i = 1; i < nx; i++) {
                const long c = i + nx * (j + ny * k);
                /* Vx: 0<k<nz-1, 0<j<ny-1, 0<i<nx (OK4:358) */
                if (k < nz - 1 && j < ny - 1) {
                    const long e = i + (nx + 1) * (j + ny * k);
                    const OT dSx = (sxx[c] - sxx[c - 1]) * rdx
                                 + (sxy[i + (nx + 1) * ((j + 1) + (ny + 1) * k)] - sxy[i + (nx + 1) * (j + (ny + 1) * k)]) * rdy
                                 + (sxz[i + (nx + 1) * (j + ny * (k + 1))] - sxz[i + (nx + 1) * (j + ny * k)]) * rdz;
                    OT a, inc;
                    if (iso) { a = pc ? w[0][e] : w[0][i - 1]; }
                    else     { a = W[c]; }
                    if (!comp) {
                        if (iso) Vx[e] = a * (Vx[e] * rdt + bx * dSx) * dt;
                        else if (vd != (OT)0) Vx[e] = (Vx[e] * rdt * a + m[9][e] * dSx) * dt - vd * Vx[e];
                        else     Vx[e] = (Vx[e] * rdt * a + m[9][e] * dSx) * dt;
                    } else {
                        inc = iso ? a * (bx * dSx) * dt : m[9][e] * dSx * dt;
                        const OT y = inc - a * comp[0][e];
                        const OT av = a * Vx[e];
                        const OT t = av + y;
                        comp[0][e] = (t - av) - y;
                        Vx[e] = t;
                    }
                }
                /* Vy: 0<k<nz-1, 0<j<ny, 0<i<nx-1 (OK4:365) */
                if (k < nz - 1 && i < nx - 1) {
                    const long e = i + nx * (j + (ny + 1) * k);
                    const OT dSy = (syy[c] - syy[c - nx]) * rdy
                                 + (sxy[(i + 1) + (nx + 1) * (j + (ny + 1) * k)] - sxy[i + (nx + 1) * (j + (ny + 1) * k)]) * rdx
                                 + (syz[i + nx * (j + (ny + 1) * (k + 1))] - syz[i + nx * (j + (ny + 1) * k)]) * rdz;
                    OT a, inc;
                    if (iso) { a = pc ? w[1][e] : w[1][j - 1]; }
                    else     { a = W[c]; }
                    if (!comp) {
                        if (iso) Vy[e] = a * (Vy[e] * rdt + by * dSy) * dt;
                        else if (vd != (OT)0) Vy[e] = (Vy[e] * rdt * a + m[10][e] * dSy) * dt - vd * Vy[e];
                        else     Vy[e] = (Vy[e] * rdt * a + m[10][e] * dSy) * dt;
                    } else {
                        inc = iso ? a * (by * dSy) * dt : m[10][e] * dSy * dt;
                        const OT y = inc - a * comp[1][e];
                        const OT av = a * Vy[e];
                        const OT t = av + y;
                        comp[1][e] = (t - av) - y;
                        Vy[e] = t;
                    }
                }
                /* Vz: 0<k<nz, 0<j<ny-1, 0<i<nx-1 (OK4:372) */
                if (j < ny - 1 && i < nx - 1) {
                    const long e = c;
                    const OT dSz = (szz[c] - szz[c - nx * ny]) * rdz
                                 + (sxz[(i + 1) + (nx + 1) * (j + ny * k)] - sxz[i + (nx + 1) * (j + ny * k)]) * rdx
                                 + (syz[i + nx * ((j + 1) + (ny + 1) * k)] - syz[i + nx * (j + (ny + 1) * k)]) * rdy;
                    OT a, inc;
                    if (iso) { a = pc ? w[2][e] : w[2][k - 1]; }
                    else     { a = W[c]; }
                    if (!comp) {
                        if (iso) Vz[e] = a * (Vz[e] * rdt + bz * dSz) * dt;
                        else if (vd != (OT)0) Vz[e] = (Vz[e] * rdt * a + m[11][e] * dSz) * dt - vd * Vz[e];
                        else     Vz[e] = (Vz[e] * rdt * a + m[11][e] * dSz) * dt;
                    } else {
                        inc = iso ? a * (bz * dSz) * dt : m[11][e] * dSz * dt;
                        const OT y = inc - a * comp[2][e];
                        const OT av = a * Vz[e];
                        const OT t = av + y;
                        comp[2][e] = (t - av) - y;
                        Vz[e] = t;
                    }
                }
            }
        }
    }
}

/* Receiver sampling after the velocity update (OK4:383-386, ANISO:254-268). */
static void OFN(record)(const orc_grid *g, OT *const *f, int nrec, const int32_t *rec, double *traces,
                        int trace_len, int it)
{
    for (int r = 0; r < nrec; r++) {
        const int id = rec[4 * r + 3];
        long px, py;
        OFN(extent)(g, id, &px, &py);
        const long e = (long)rec[4 * r + 0] + px * ((long)rec[4 * r + 1] + py * (long)rec[4 * r + 2]);
        traces[(long)r * trace_len + it] = (double)f[id][e];
    }
}

/* One full run of nsteps time steps starting at step it0 (OK4:485-505 / ANISO:519-555). */
int OFN(orc_run)(const orc_grid *g, OT *const *f, OT *const *comp, const OT *const *m, const OT *const *w,
                 const OT *W, int32_t nsrc, const int32_t *src, const double *coef, const double *stf,
                 int32_t nstf, int32_t nrec, const int32_t *rec, double *traces, int32_t trace_len,
                 int32_t it0, int32_t nsteps)
{
    if (!g || !f || g->nx < 3 || g->ny < 3 || g->nz < 3) return -1;
    if (it0 < 0 || nsteps < 0 || it0 + nsteps > nstf) return -2;
    if (nrec > 0 && it0 + nsteps > trace_len) return -3;
    if (g->model == 0 && (!w || !w[0] || !w[1] || !w[2])) return -4;
    if (g->damping == 3 && (g->model != 0 || !w[3] || !w[4] || !w[5])) return -11;
    if (g->model != 0 && !W) return -5;
    if (g->model < 0 || g->model > 2) return -10;
    for (int32_t s = 0; s < nsrc; s++) {
        const int id = src[4 * s];
        long px, py;
        if (id < 3 || id > 8) return -6;
        OFN(extent)(g, id, &px, &py);
        const long pz = g->nz + ((id == 2 || id == 7 || id == 8) ? 1 : 0);
        if (src[4 * s + 1] < 0 || src[4 * s + 2] < 0 || src[4 * s + 3] < 0 || src[4 * s + 1] >= px ||
            src[4 * s + 2] >= py || src[4 * s + 3] >= pz)
            return -7;
    }
    for (int32_t r = 0; r < nrec; r++) {
        const int id = rec[4 * r + 3];
        long px, py;
        if (id < 0 || id > 8) return -8;
        OFN(extent)(g, id, &px, &py);
        const long pz = g->nz + ((id == 2 || id == 7 || id == 8) ? 1 : 0);
        if (rec[4 * r] < 0 || rec[4 * r + 1] < 0 || rec[4 * r + 2] < 0 || rec[4 * r] >= px || rec[4 * r + 1] >= py ||
            rec[4 * r + 2] >= pz)
            return -9;
    }
    for (int32_t s = 0; s < nsteps; s++) {
        const int it = it0 + s;
        if (g->model == 0 && g->damping == 3) OFN(stress_iso_percomp)(g, f, m, w);
        else if (g->model == 0) OFN(stress_iso)(g, f, m, w);
        else if (g->model == 2) OFN(stress_isohet)(g, f, m, W);
        else                    OFN(stress_ortho)(g, f, m, W);
        if (g->src_order == 0) OFN(inject)(g, f, nsrc, src, coef, stf, it);
        if (!g->no_bc1) OFN(bc1)(g, f);
        if (g->src_order != 0) OFN(inject)(g, f, nsrc, src, coef, stf, it);
        OFN(velocity)(g, f, m, w, W, comp);
        OFN(record)(g, f, nrec, rec, traces, trace_len, it);
    }
    return 0;
}

#undef OFN
#undef OFN1
#undef OFN2
