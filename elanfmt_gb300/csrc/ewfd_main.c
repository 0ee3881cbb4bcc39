/*
 * ewfd_main.c -- `ewfd`, the C host driver that takes the place of the reference's a.out/a.exe.
 *
 * The MATLAB drivers write the inputs into the working directory, compile the solver with the
 * grid as -D defines and run `! a.exe` (vizme_FastBiotED_GPU3D_OK_2024_final.m:432-450).  With
 * ewfd the grid is given on the command line instead, in the same NBX/OVERX form
 * (nx = 64*NBX - OVERX, OK4:29-41) or directly as --nx/--ny/--nz; everything else is read from
 * the same files and written to the same 0_infos.inf / 0_0_*.res outputs (OK4:521-532).
 *
 *   ewfd --nbx 12 --nby 12 --nbz 7 [--overx 0 ...] [--model iso|ortho|isohet|dcq] [--nt N] [--vdamp C]
 *        [--precision f32|kahan|f64] [--src i,j,k] [--stencil ok4|aniso] [--mts FILE]
 *        [--free-surface bc1|none] [--surface-mu MU]
 *        [--receivers FILE] [--snap-every N] [--autotune STEPS] [--workdir DIR] [--quiet] [--no-checks]
 *
 * --free-surface none drops BC1 (the diff_BC schemes comment its launch out); --surface-mu MU
 * gives the isotropic scheme's shear modulus MU on plane k = 1 (the diff_BC2_OK3 scheme: 1e-5).
 *
 * Exit status is 0 on success and 1 on any error (the reference returns 0 even after a CUDA
 * failure, OK4:96-99, 558).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ewfd.h"

static int fail(int st, const char *what)
{
    fprintf(stderr, "ewfd: %s: %s (%s)\n", what, ewf_strerror(st), ewf_last_error());
    return 1;
}

static int read_floats(const char *path, float *out, int n)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) return -1;
    const int got = (int)fread(out, 4, (size_t)n, fp);
    fclose(fp);
    return got == n ? 0 : -1;
}

/* receivers file: one "i j k comp" per line, comp 0=Vx 1=Vy 2=Vz */
static int read_receivers(const char *path, int32_t **out, int *n)
{
    FILE *fp = fopen(path, "r");
    if (!fp) return -1;
    int cap = 64, m = 0;
    int32_t *v = (int32_t *)malloc(sizeof(int32_t) * 4 * cap);
    int a, b, c, d;
    while (v && fscanf(fp, "%d %d %d %d", &a, &b, &c, &d) == 4) {
        if (m == cap) {
            cap *= 2;
            int32_t *w = (int32_t *)realloc(v, sizeof(int32_t) * 4 * cap);
            if (!w) { free(v); v = NULL; break; }
            v = w;
        }
        v[4 * m] = a; v[4 * m + 1] = b; v[4 * m + 2] = c; v[4 * m + 3] = d;
        m++;
    }
    fclose(fp);
    if (!v) return -1;
    *out = v;
    *n = m;
    return 0;
}

int main(int argc, char **argv)
{
    ewf_params p;
    ewf_params_default(&p);
    int nbx = 0, nby = 0, nbz = 0, overx = 0, overy = 0, overz = 0;
    int src[3] = {-1, -1, -1}, stencil = -1, snap_every = 0, quiet = 0, percomp = 0, tune = 0;
    const char *mts_file = NULL, *rec_file = NULL;
    p.workdir = ".";
    p.nout = 200;
    for (int a = 1; a < argc; ++a) {
        const char *k = argv[a];
        const char *v = (a + 1 < argc) ? argv[a + 1] : NULL;
#define ARG_INT(name, dst) if (!strcmp(k, name) && v) { dst = atoi(v); ++a; continue; }
        ARG_INT("--nbx", nbx) ARG_INT("--nby", nby) ARG_INT("--nbz", nbz)
        ARG_INT("--overx", overx) ARG_INT("--overy", overy) ARG_INT("--overz", overz)
        ARG_INT("--nx", p.nx) ARG_INT("--ny", p.ny) ARG_INT("--nz", p.nz) ARG_INT("--nt", p.nt)
        ARG_INT("--snap-every", snap_every) ARG_INT("--kchunk", p.kchunk) ARG_INT("--autotune", tune)
#undef ARG_INT
        if (!strcmp(k, "--model") && v) {
            if (!strcmp(v, "ortho")) p.model = EWF_MODEL_ORTHO;
            else if (!strcmp(v, "isohet")) p.model = EWF_MODEL_ISO_HET; /* the 9 km station scheme */
            else if (!strcmp(v, "dcq")) { p.model = EWF_MODEL_ISO; percomp = 1; } /* DC_Earthquake */
            else if (!strcmp(v, "iso")) p.model = EWF_MODEL_ISO;
            else return fail(EWF_ERR_ARG, "--model iso|ortho|isohet|dcq");
            ++a;
            continue;
        }
        if (!strcmp(k, "--vdamp") && v) { p.vdamp = atof(v); ++a; continue; }
        if (!strcmp(k, "--surface-mu") && v) { p.surface_mu = atof(v); ++a; continue; }
        if (!strcmp(k, "--free-surface") && v) {
            if (!strcmp(v, "none")) p.free_surface = EWF_FS_NONE;
            else if (!strcmp(v, "bc1")) p.free_surface = EWF_FS_BC1;
            else return fail(EWF_ERR_ARG, "--free-surface bc1|none");
            ++a;
            continue;
        }
        if (!strcmp(k, "--precision") && v) {
            p.precision = !strcmp(v, "f64") ? EWF_PREC_F64 : !strcmp(v, "kahan") ? EWF_PREC_F32_KAHAN : EWF_PREC_F32;
            ++a;
            continue;
        }
        if (!strcmp(k, "--src") && v) { if (sscanf(v, "%d,%d,%d", &src[0], &src[1], &src[2]) != 3) return fail(EWF_ERR_ARG, "--src i,j,k"); ++a; continue; }
        if (!strcmp(k, "--stencil") && v) { stencil = !strcmp(v, "aniso") ? 1 : 0; ++a; continue; }
        if (!strcmp(k, "--mts") && v) { mts_file = v; ++a; continue; }
        if (!strcmp(k, "--receivers") && v) { rec_file = v; ++a; continue; }
        if (!strcmp(k, "--workdir") && v) { p.workdir = v; ++a; continue; }
        if (!strcmp(k, "--quiet")) { quiet = 1; p.nout = 0; continue; }
        if (!strcmp(k, "--no-checks")) { p.check_finite = 0; continue; }
        fprintf(stderr, "ewfd: unknown or incomplete argument %s\n", k);
        return 1;
    }
    if (p.nx <= 0 && nbx > 0) p.nx = 64 * nbx - overx; /* OK4:26-41 */
    if (p.ny <= 0 && nby > 0) p.ny = 64 * nby - overy;
    if (p.nz <= 0 && nbz > 0) p.nz = 64 * nbz - overz;
    p.over_y = overy;
    p.damping = percomp ? EWF_DAMP_PERCOMP : p.model == EWF_MODEL_ISO ? EWF_DAMP_PML1D : EWF_DAMP_W3D;
    p.src_order = (p.model == EWF_MODEL_ISO && !percomp) ? EWF_SRC_BEFORE_BC1 : EWF_SRC_AFTER_BC1;
    if (p.nx <= 0 || p.ny <= 0 || p.nz <= 0) {
        fprintf(stderr, "ewfd: give the grid as --nbx/--nby/--nbz [--overx..] or --nx/--ny/--nz\n");
        return 1;
    }
    int st = ewf_legacy_params(&p);
    if (st) return fail(st, "reading pa1/pa2/pa3.dat");
    if (!quiet) {
        printf("\n  ewfd: staggered-grid elastic FDTD (%s, %s)\n",
               p.model == EWF_MODEL_ORTHO ? "orthorhombic" : p.model == EWF_MODEL_ISO_HET ? "isotropic, heterogeneous mu/rho" : "isotropic",
               p.precision == EWF_PREC_F64 ? "fp64" : p.precision == EWF_PREC_F32_KAHAN ? "fp32+kahan" : "fp32");
        printf("Local size: %dx%dx%d, %d iterations\n", p.nx, p.ny, p.nz, p.nt);
    }
    ewf_handle *h = NULL;
    if ((st = ewf_create(&p, &h))) return fail(st, "create");
    if ((st = ewf_load_legacy_inputs(h))) { ewf_destroy(h); return fail(st, "loading inputs"); }
    if (src[0] >= 0 || mts_file || stencil >= 0) {
        /* re-place the source: legacy cell unless --src, MTS.dat (iso) unless --mts */
        float m[6] = {0, 0, 0, 0, 0, 0};
        char path[4096];
        snprintf(path, sizeof(path), "%s/%s", p.workdir, mts_file ? mts_file : "MTS.dat");
        if (read_floats(mts_file ? mts_file : path, m, 6)) { ewf_destroy(h); fprintf(stderr, "ewfd: cannot read %s\n", mts_file ? mts_file : path); return 1; }
        double mt[6];
        for (int q = 0; q < 6; ++q) mt[q] = m[q];
        if (src[0] < 0) {
            fprintf(stderr, "ewfd: --mts/--stencil need --src i,j,k\n");
            ewf_destroy(h);
            return 1;
        }
        const int sten = stencil >= 0 ? stencil : (p.model == EWF_MODEL_ISO && !percomp ? 0 : 1);
        if ((st = ewf_set_moment_tensor(h, mt, src[0], src[1], src[2], sten))) { ewf_destroy(h); return fail(st, "source"); }
    }
    if (rec_file) {
        int32_t *r = NULL;
        int n = 0;
        if (read_receivers(rec_file, &r, &n)) { ewf_destroy(h); fprintf(stderr, "ewfd: cannot read %s\n", rec_file); return 1; }
        st = ewf_set_receivers(h, n, r);
        free(r);
        if (st) { ewf_destroy(h); return fail(st, "receivers"); }
    }
    if (tune > 0) {  /* the library's autotuner: launch shapes timed over `tune` steps, state reset after */
        int32_t kc = 0;
        if ((st = ewf_autotune(h, tune, &kc))) { ewf_destroy(h); return fail(st, "autotune"); }
        if (!quiet) printf("autotuned over %d steps: z-chunk %d\n", tune, kc);
    }
    double total_ms = 0.0;
    int isave = 1;
    for (int done = 0; done < p.nt;) {
        int chunk = p.nt - done;
        if (snap_every > 0 && chunk > snap_every) chunk = snap_every;
        if ((st = ewf_run(h, chunk))) { ewf_destroy(h); return fail(st, "run"); }
        double ms = 0;
        ewf_last_run_ms(h, &ms);
        total_ms += ms;
        done += chunk;
        if (snap_every > 0 && done < p.nt) {  /* written by the library while the next chunk runs */
            if ((st = ewf_write_snapshot_async(h, isave++))) { ewf_destroy(h); return fail(st, "snapshot"); }
        }
    }
    if ((st = ewf_snapshot_wait(h))) { ewf_destroy(h); return fail(st, "snapshot"); }
    if (!quiet) {
        const double cells = (double)p.nx * p.ny * p.nz * p.nt;
        printf("\n  time is %.3f s after %d iterations, %.2f Gcell-updates/s\n", total_ms * 1e-3, p.nt,
               total_ms > 0 ? cells / (total_ms * 1e6) : 0.0);
    }
    if ((st = ewf_write_legacy_outputs(h))) { ewf_destroy(h); return fail(st, "writing outputs"); }
    ewf_destroy(h);
    return 0;
}
