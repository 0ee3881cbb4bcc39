// ewfd_legacy.cpp -- the reference's file contract on top of the C ABI.
//
// Inputs are the raw float32 files the MATLAB drivers write into the working directory
// (vizme_FastBiotED_GPU3D_OK_2024_final.m:231-429 for the isotropic solver, vizme_FastWaveED_
// GPU3D_9kmst_ANIS.m:374-533 for the orthorhombic one), read as OK4:401-454 / ANISO:402-487 do.
// Outputs are 0_infos.inf and "0_0_<name>.res" raw arrays (OK4:154-164, 521-532).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ewfd.h"
#include "ewfd_internal.h"

namespace {

std::string join(const char *dir, const char *name)
{
    std::string s = dir ? dir : ".";
    if (!s.empty() && s.back() != '/') s += '/';
    return s + name;
}

// Reads a raw float32 file; exact: size must equal n, else size must be >= n (first n read).
int read_f32(const std::string &path, size_t n, bool exact, std::vector<float> &out)
{
    FILE *fp = fopen(path.c_str(), "rb");
    if (!fp) return ewf_fail(EWF_ERR_IO, "unable to open %s", path.c_str());
    fseek(fp, 0, SEEK_END);
    const long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (sz < 0 || (exact ? (size_t)sz != n * 4 : (size_t)sz < n * 4)) {
        fclose(fp);
        return ewf_fail(EWF_ERR_IO, "%s: %ld bytes, expected %s%zu (float32 x %zu)", path.c_str(), sz, exact ? "" : ">= ", n * 4, n);
    }
    out.resize(n);
    const size_t got = n ? fread(out.data(), 4, n, fp) : 0;
    fclose(fp);
    if (got != n) return ewf_fail(EWF_ERR_IO, "%s: short read", path.c_str());
    return EWF_OK;
}

size_t file_floats(const std::string &path)
{
    FILE *fp = fopen(path.c_str(), "rb");
    if (!fp) return 0;
    fseek(fp, 0, SEEK_END);
    const long sz = ftell(fp);
    fclose(fp);
    return sz > 0 ? (size_t)sz / 4 : 0;
}

int load_field(ewf_handle *h, const char *dir, const char *name, int id, std::vector<float> *keep = nullptr)
{
    std::vector<float> v;
    int st = read_f32(join(dir, name), ewf_field_size(h, id), true, v);
    if (st) return st;
    st = ewf_set_field(h, id, v.data(), v.size(), 4);
    if (!st && keep) keep->swap(v);
    return st;
}

int write_raw(const std::string &path, const void *data, size_t bytes)
{
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) return ewf_fail(EWF_ERR_IO, "unable to open %s for writing", path.c_str());
    const size_t w = bytes ? fwrite(data, 1, bytes, fp) : 0;
    const int c = fclose(fp);
    if (w != bytes || c != 0) return ewf_fail(EWF_ERR_IO, "write %s failed", path.c_str());
    return EWF_OK;
}

// Writes n doubles as the handle's DAT (float32 unless FP64), "<isave>_0_<name>.res" (OK4:159-164).
int save_array(ewf_handle *h, int isave, const char *name, const double *x, size_t n)
{
    char fn[256];
    snprintf(fn, sizeof(fn), "%d_0_%s.res", isave, name);
    const std::string path = join(ewf_workdir(h), fn);
    if (ewf_esz(h) == 8) return write_raw(path, x, n * 8);
    std::vector<float> f(n);
    for (size_t i = 0; i < n; ++i) f[i] = (float)x[i];
    return write_raw(path, f.data(), n * 4);
}

int save_field(ewf_handle *h, int isave, const char *name, int id)
{
    const size_t n = ewf_field_size(h, id);
    const int esz = ewf_esz(h);
    std::vector<char> buf(n * esz);
    int st = ewf_get_field(h, id, buf.data(), n, esz);
    if (st) return st;
    char fn[256];
    snprintf(fn, sizeof(fn), "%d_0_%s.res", isave, name);
    return write_raw(join(ewf_workdir(h), fn), buf.data(), buf.size());
}

}  // namespace

int ewf_write_raw_file(const char *path, const void *data, size_t bytes) { return write_raw(path, data, bytes); }

extern "C" int ewf_load_legacy_inputs(ewf_handle *h)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    ewf_params p;
    ewf_get_params(h, &p);
    const char *dir = ewf_workdir(h);
    std::vector<float> pa1, pa2, pa3;
    int st;
    // pa1 = [dx dy dz dt Lx Ly Lz lamx lamy lamz] (OK4:401, 404)
    if ((st = read_f32(join(dir, "pa1.dat"), 10, false, pa1))) return st;
    // pa2 = [c11u c33u c13u c12u c23u c44u c55u c66u alpha1 alpha2 alpha3 M1 c22u] (OK4:402, 405)
    if ((st = read_f32(join(dir, "pa2.dat"), 13, false, pa2))) return st;
    // pa3 = [vrho_x_11 vrho_y_11 vrho_z_11 ...] (OK4:403, 407); the drivers write 12 values
    if ((st = read_f32(join(dir, "pa3.dat"), 3, false, pa3))) return st;
    const double dx = pa1[0], dy = pa1[1], dz = pa1[2], dt = pa1[3], Ly = pa1[5];
    if (!(dx > 0 && dy > 0 && dz > 0 && dt > 0))
        return ewf_fail(EWF_ERR_IO, "pa1.dat: dx, dy, dz, dt must be > 0 (got %g %g %g %g)", dx, dy, dz, dt);
    // the scalars are kernel arguments fixed at ewf_create: the handle must have been created
    // from these files (ewf_legacy_params)
    if (std::fabs(p.dx - dx) > 0 || std::fabs(p.dy - dy) > 0 || std::fabs(p.dz - dz) > 0 || std::fabs(p.dt - dt) > 0 ||
        (p.model == EWF_MODEL_ISO && (p.c66 != (double)pa2[7] || p.bx != (double)pa3[0] || p.by != (double)pa3[1] ||
                                      p.bz != (double)pa3[2])) ||
        (p.damping == EWF_DAMP_PERCOMP && (p.c44 != (double)pa2[5] || p.c55 != (double)pa2[6])))
        return ewf_fail(EWF_ERR_STATE,
                        "handle parameters differ from pa1/pa2/pa3.dat: create the handle with ewf_legacy_params() first");

    double vmax2 = 0.0;
    if (p.model == EWF_MODEL_ISO) {
        std::vector<float> c11;
        if ((st = load_field(h, dir, "c11u_het.dat", EWF_M_C11, &c11))) return st;
        if ((st = load_field(h, dir, "c12u_het.dat", EWF_M_C12))) return st;
        if (p.damping == EWF_DAMP_PERCOMP) {
            // DC_Earthquake: 3-D weights per component, in the extents its driver writes them
            // (vizme_FastWaveED_GPU3D.m:319-324; the solver itself reads only nx*ny*nz values of
            // the shear ones, FastWaveED_GPU3D_v1.cu:406-410, then indexes them with edge pitches)
            static const struct { const char *file; int id; } wf[] = {
                {"weights_x.dat", EWF_D_PX},   {"weights_y.dat", EWF_D_PY},   {"weights_z.dat", EWF_D_PZ},
                {"weights_xy.dat", EWF_D_PXY}, {"weights_xz.dat", EWF_D_PXZ}, {"weights_yz.dat", EWF_D_PYZ},
            };
            for (const auto &f : wf)
                if ((st = load_field(h, dir, f.file, f.id))) return st;
        } else {
            if ((st = load_field(h, dir, "weights_x.dat", EWF_D_WX))) return st;
            if ((st = load_field(h, dir, "weights_y.dat", EWF_D_WY))) return st;
            if ((st = load_field(h, dir, "weights_z.dat", EWF_D_WZ))) return st;
        }
        double cmax = 0;
        for (float v : c11) cmax = std::max(cmax, (double)v);
        const double bmax = std::max({(double)pa3[0], (double)pa3[1], (double)pa3[2]});
        vmax2 = cmax * bmax;
    } else {
        struct LegacyFile { const char *file; int id; };
        static const LegacyFile ortho_files[] = {
            {"vrho_x_11_hc.dat", EWF_M_BX}, {"vrho_y_11_hc.dat", EWF_M_BY}, {"vrho_z_11_hc.dat", EWF_M_BZ},
            {"C11m.dat", EWF_M_C11},        {"C22m.dat", EWF_M_C22},        {"C33m.dat", EWF_M_C33},
            {"C12m.dat", EWF_M_C12},        {"C13m.dat", EWF_M_C13},        {"C23m.dat", EWF_M_C23},
            {"C44myz.dat", EWF_M_C44YZ},    {"C55mxz.dat", EWF_M_C55XZ},    {"C66mxy.dat", EWF_M_C66XY},
        };
        // the 9 km scheme's inputs (FastWaveED_GPU3D_v1_9kmst.cu:434-452)
        static const LegacyFile isohet_files[] = {
            {"vrho_x_11_hc.dat", EWF_M_BX},    {"vrho_y_11_hc.dat", EWF_M_BY},    {"vrho_z_11_hc.dat", EWF_M_BZ},
            {"c11u_het.dat", EWF_M_C11},       {"c12u_het.dat", EWF_M_C12},       {"c44u_hetxy.dat", EWF_M_C66XY},
            {"c44u_hetxz.dat", EWF_M_C55XZ},   {"c44u_hetyz.dat", EWF_M_C44YZ},
        };
        const bool isohet = p.model == EWF_MODEL_ISO_HET;
        const LegacyFile *files = isohet ? isohet_files : ortho_files;
        const size_t nfiles = isohet ? sizeof(isohet_files) / sizeof(isohet_files[0])
                                     : sizeof(ortho_files) / sizeof(ortho_files[0]);
        double cmax = 0, bmax = 0;
        for (size_t q = 0; q < nfiles; ++q) {
            const LegacyFile &f = files[q];
            std::vector<float> v;
            if ((st = load_field(h, dir, f.file, f.id, &v))) return st;
            double m = 0;
            for (float x : v) m = std::max(m, (double)x);
            if (f.id >= EWF_M_BX && f.id <= EWF_M_BZ) bmax = std::max(bmax, m);
            else if (f.id == EWF_M_C11 || f.id == EWF_M_C22 || f.id == EWF_M_C33) cmax = std::max(cmax, m);
        }
        vmax2 = cmax * bmax;
        if (p.damping == EWF_DAMP_W3D) {
            if ((st = load_field(h, dir, "weights.dat", EWF_D_W3D))) return st;
        } else {
            return ewf_fail(EWF_ERR_UNSUPPORTED, "legacy orthorhombic / 9 km inputs carry a 3-D weights.dat: use damping 1");
        }
    }
    const double courant = std::sqrt(vmax2) * dt * std::sqrt(1.0 / (dx * dx) + 1.0 / (dy * dy) + 1.0 / (dz * dz));
    if (!(courant <= 1.0)) {
        if (p.check_finite)
            return ewf_fail(EWF_ERR_CFL, "Courant number %.4f > 1 (vmax %.1f m/s, dt %g s)", courant, std::sqrt(vmax2), dt);
        fprintf(stderr, "ewfd: warning: Courant number %.4f > 1\n", courant);
    }

    // Src.dat: nt samples (OK4:454)
    std::vector<float> src;
    if ((st = read_f32(join(dir, "Src.dat"), (size_t)p.nt, false, src))) return st;
    std::vector<double> stf(src.begin(), src.end());
    if ((st = ewf_set_stf(h, stf.data(), stf.size()))) return st;

    // source cell and moment tensor (OK4:410-411, 450-452 / ANISO:233-247, 483-485)
    const int ysrc = (int)std::round((Ly - Ly / 2.0) / dy);
    double mt[6];
    int xsrc, zsrc, stencil;
    if (p.model == EWF_MODEL_ISO && p.damping == EWF_DAMP_PERCOMP) {
        // DC_Earthquake's source kernel adds 1.0 Src to sxz and 0.8 Src to syz only, at the
        // ANISO stencil cells (FastWaveED_GPU3D_v1.cu:228-246, 436-438)
        const double c[6] = {0.0, 0.0, 0.0, 0.0, 1.0, (double)0.8f};
        for (int q = 0; q < 6; ++q) mt[q] = c[q];
        xsrc = 234;
        zsrc = 100;
        stencil = 1;
    } else if (p.model == EWF_MODEL_ISO) {
        std::vector<float> mts;
        if ((st = read_f32(join(dir, "MTS.dat"), 6, false, mts))) return st;
        for (int q = 0; q < 6; ++q) mt[q] = mts[q];
        xsrc = 234;
        zsrc = 100;
        stencil = 0;
    } else {
        // ANISO (and the 9 km scheme, 9kmst.cu:228-246) hard-code the tensor in their source
        // kernel (ANISO:233-247): xx yy zz xy xz yz; the 16 km scheme (the 9 km one with vdamp)
        // another one in the same kernel (16kmst.cu:228-252)
        const float c9[6] = {-0.6282f, 0.9437f, 0.2439f, 0.4455f, -0.2709f, -0.2362f};
        const float c16[6] = {-0.7448f, 1.0603f, 0.2439f, -0.0387f, -0.1953f, -0.3017f};
        const bool km16 = p.model == EWF_MODEL_ISO_HET && p.vdamp != 0.0;
        for (int q = 0; q < 6; ++q) mt[q] = km16 ? c16[q] : c9[q];
        xsrc = 180;
        zsrc = 200;
        stencil = 1;
    }
    st = ewf_set_moment_tensor(h, mt, xsrc, ysrc, zsrc, stencil);
    if (st == EWF_ERR_ARG) {
        // the reference has no thread for a cell outside its launch: the source is simply absent
        fprintf(stderr, "ewfd: warning: legacy source cell (%d,%d,%d) outside the grid; no source set\n", xsrc, ysrc, zsrc);
        st = ewf_set_sources(h, 0, nullptr, nullptr);
    }
    if (st) return st;

    // the four legacy traces Rec, Rec_x, Rec_y, Rec_y2 (OK4:383-386 / ANISO:263-266)
    int32_t rec[16];
    if (p.model == EWF_MODEL_ISO && p.damping == EWF_DAMP_PERCOMP) {  // FastWaveED_GPU3D_v1.cu:278-281
        const int32_t r[16] = {504, 129, 1, EWF_F_VZ, 504, 129, 1, EWF_F_VX, 504, 132, 1, EWF_F_VY, 504, 131, 1, EWF_F_VY};
        memcpy(rec, r, sizeof(r));
    } else if (p.model == EWF_MODEL_ISO) {
        const int32_t r[16] = {504, 385, 1, EWF_F_VZ, 504, 385, 1, EWF_F_VX, 504, 388, 1, EWF_F_VY, 504, 387, 1, EWF_F_VY};
        memcpy(rec, r, sizeof(r));
    } else {
        // ANISO:263-266 and 9kmst.cu: cell 631; the 16 km scheme: cell 981 (16kmst.cu:266-269)
        const int32_t ix = (p.model == EWF_MODEL_ISO_HET && p.vdamp != 0.0) ? 981 : 631;
        const int32_t r[16] = {ix, 257, 1, EWF_F_VZ, ix, 257, 1, EWF_F_VX, ix, 257, 1, EWF_F_VY, ix, 257, 1, EWF_F_VY};
        memcpy(rec, r, sizeof(r));
    }
    st = ewf_set_receivers(h, 4, rec);
    if (st == EWF_ERR_ARG) {
        fprintf(stderr, "ewfd: warning: legacy receiver cells lie outside the grid; no receivers set\n");
        st = ewf_set_receivers(h, 0, nullptr);
    }
    return st;
}

extern "C" int ewf_write_legacy_outputs(ewf_handle *h)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    ewf_params p;
    ewf_get_params(h, &p);
    const int esz = ewf_esz(h);
    // 0_infos.inf: PRECIS nx ny nz NB_PARAMS ceil(niter/nout) with niter 10, nout 200 (OK4:154-157)
    {
        char line[128];
        snprintf(line, sizeof(line), "%d %d %d %d %d %d", esz, p.nx, p.ny, p.nz, 1, 1);
        int st = write_raw(std::string(ewf_workdir(h)) + "/0_infos.inf", line, strlen(line));
        if (st) return st;
    }
    std::vector<double> stf;
    ewf_stf_host_copy(h, stf);
    stf.resize((size_t)p.nt, 0.0);
    int st = save_array(h, 0, "Src", stf.data(), (size_t)p.nt);
    if (st) return st;
    const int nrec = ewf_nrec(h);
    std::vector<double> tr((size_t)nrec * p.nt);
    if (nrec && (st = ewf_get_seismograms(h, tr.data(), tr.size()))) return st;
    static const char *names[4] = {"Rec", "Rec_x", "Rec_y", "Rec_y2"};
    std::vector<double> zero((size_t)p.nt, 0.0);
    for (int r = 0; r < 4; ++r) {
        const double *x = r < nrec ? tr.data() + (size_t)r * p.nt : zero.data();
        if ((st = save_array(h, 0, names[r], x, (size_t)p.nt))) return st;
    }
    if (nrec > 4 && (st = save_array(h, 0, "Rec_all", tr.data(), tr.size()))) return st;
    if ((st = save_field(h, 0, "Vx", EWF_F_VX))) return st;
    if ((st = save_field(h, 0, "Vy", EWF_F_VY))) return st;
    return save_field(h, 0, "Vz", EWF_F_VZ);
}

extern "C" int ewf_write_snapshot(ewf_handle *h, int32_t isave)
{
    if (!h || isave < 0) return ewf_fail(EWF_ERR_ARG, "bad argument");
    int st;
    if ((st = save_field(h, isave, "Vx", EWF_F_VX))) return st;
    if ((st = save_field(h, isave, "Vy", EWF_F_VY))) return st;
    return save_field(h, isave, "Vz", EWF_F_VZ);
}

// Fills the scalar parameters of p from workdir/pa1.dat, pa2.dat, pa3.dat and nt from the
// length of Src.dat when p->nt is 0 (the reference's nt is a compile-time constant, OK4:43).
extern "C" int ewf_legacy_params(ewf_params *p)
{
    if (!p) return ewf_fail(EWF_ERR_ARG, "NULL params");
    const char *dir = p->workdir;
    std::vector<float> pa1, pa2, pa3;
    int st;
    if ((st = read_f32(join(dir, "pa1.dat"), 10, false, pa1))) return st;
    if ((st = read_f32(join(dir, "pa2.dat"), 13, false, pa2))) return st;
    if ((st = read_f32(join(dir, "pa3.dat"), 3, false, pa3))) return st;
    p->dx = pa1[0]; p->dy = pa1[1]; p->dz = pa1[2]; p->dt = pa1[3];
    p->c66 = pa2[7];
    p->c44 = pa2[5];
    p->c55 = pa2[6];
    p->bx = pa3[0]; p->by = pa3[1]; p->bz = pa3[2];
    if (p->nt <= 0) {
        const size_t n = file_floats(join(dir, "Src.dat"));
        if (n == 0) return ewf_fail(EWF_ERR_IO, "unable to size %s", join(dir, "Src.dat").c_str());
        p->nt = (int32_t)n;
    }
    return EWF_OK;
}
