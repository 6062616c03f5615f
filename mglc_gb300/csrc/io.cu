// io.cu -- host-side output, checkpoint/restart and the calNuRe statistics
// monitor of the reference drivers, written against the public C-ABI.
//
//   Tecplot binary   mpi_3d_blocked/output.f90:175-296 (lid: X Y Z U V W
//                    Pressure = rho/3), bouyancy3d.F90:1034-1164 (heated: X Y
//                    Z U V W T); node coordinates x_i = i - 0.5
//                    (initial.f90:18-21, bouyancy3d.F90:254-257)
//   profiles         output.f90:318-347 (getVelocity)
//   output_binary    output.f90:350-367 (lid: u, v, rho), bouyancy3d.F90:984-1008
//                    (heated: u, v, w, T)
//   backupData       bouyancy3d.F90:1011-1030 (u, v, w, T, f, g) and its reload
//                    :367-379 with rho = 1 (:289) and up = vp = wp = Tp = 0
//   calNuRe          bouyancy3d.F90:1185-1321 (running means, stationarity and
//                    statistical convergence of Nu and Re per time unit)
//
// Unformatted sequential files use gfortran's record layout: a logical record
// is one or more subrecords of at most 2^31 - 9 bytes, each framed by 4-byte
// little-endian length markers; a negative leading marker means another
// subrecord follows, a negative trailing marker that one precedes.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "mglc.h"

namespace {

constexpr long long DEFAULT_SUBRECORD = 2147483639LL;  // 2^31 - 9

struct File {
    FILE* fp = nullptr;
    explicit File(const char* path, const char* mode) { fp = std::fopen(path, mode); }
    ~File() {
        if (fp) std::fclose(fp);
    }
    bool put(const void* p, size_t n) { return std::fwrite(p, 1, n, fp) == n; }
    bool get(void* p, size_t n) { return std::fread(p, 1, n, fp) == n; }
};

bool put_i32(File& f, int32_t v) { return f.put(&v, 4); }
bool put_f32(File& f, float v) { return f.put(&v, 4); }

// dumpstring (output.f90:298-313): each character as a 4-byte integer, then 0
bool put_tec_string(File& f, const char* s) {
    for (const char* c = s; *c; c++)
        if (!put_i32(f, (int32_t)(unsigned char)*c)) return false;
    return put_i32(f, 0);
}

bool put_record(File& f, const void* data, long long nbytes, long long max_sub) {
    if (max_sub <= 0) max_sub = DEFAULT_SUBRECORD;
    const char* p = (const char*)data;
    long long left = nbytes;
    bool first = true;
    do {
        const long long n = left > max_sub ? max_sub : left;
        const bool more = left > n;
        const int32_t lead = (int32_t)(more ? -n : n), trail = (int32_t)(first ? n : -n);
        if (!put_i32(f, lead) || (n && !f.put(p, (size_t)n)) || !put_i32(f, trail)) return false;
        p += n;
        left -= n;
        first = false;
    } while (left > 0);
    return true;
}

// read one logical record of exactly nbytes (subrecords concatenated)
int get_record(File& f, void* data, long long nbytes) {
    char* p = (char*)data;
    long long got = 0;
    for (;;) {
        int32_t lead, trail;
        if (!f.get(&lead, 4)) return MGLC_ERR_INVALID;
        const long long n = lead < 0 ? -(long long)lead : lead;
        if (got + n > nbytes) return MGLC_ERR_INVALID;
        if (n && !f.get(p + got, (size_t)n)) return MGLC_ERR_INVALID;
        if (!f.get(&trail, 4)) return MGLC_ERR_INVALID;
        if ((trail < 0 ? -(long long)trail : trail) != n) return MGLC_ERR_INVALID;
        got += n;
        if (lead >= 0) break;
    }
    return got == nbytes ? MGLC_OK : MGLC_ERR_INVALID;
}

int geometry(mglc_ctx* c, mglc_info& info) {
    int rc = mglc_get_info(c, &info);
    if (rc) return rc;
    if (info.kind != MGLC_KIND_LID && info.kind != MGLC_KIND_THERMAL) return MGLC_ERR_STATE;
    return MGLC_OK;
}

}  // namespace

extern "C" {

int mglc_tecplot_write_fields(const char* path, int nx, int ny, int nz, const double* u,
                              const double* v, const double* w, const double* s, int thermal) {
    if (!path || nx <= 0 || ny <= 0 || nz <= 0 || !u || !v || !w || !s) return MGLC_ERR_INVALID;
    File f(path, "wb");
    if (!f.fp) return MGLC_ERR_INVALID;
    bool ok = f.put("#!TDV101", 8) && put_i32(f, 1) && put_tec_string(f, "MyFirst") && put_i32(f, 7);
    const char* names[7] = {"X", "Y", "Z", "U", "V", "W", thermal ? "T" : "Pressure"};
    for (int q = 0; q < 7 && ok; q++) ok = put_tec_string(f, names[q]);
    ok = ok && put_f32(f, 299.0f) && put_tec_string(f, "ZONE 001") && put_i32(f, -1) &&
         put_i32(f, 0) && put_i32(f, 1) && put_i32(f, 0) && put_i32(f, 0) && put_i32(f, nx) &&
         put_i32(f, ny) && put_i32(f, nz) && put_i32(f, 0) && put_f32(f, 357.0f) &&
         put_f32(f, 299.0f);
    for (int q = 0; q < 7 && ok; q++) ok = put_i32(f, 1);  // all variables float
    ok = ok && put_i32(f, 0) && put_i32(f, -1);
    // point packing: 7 floats per node, x fastest (the reference writes them one
    // by one; a row is buffered here)
    std::vector<float> row((size_t)nx * 7);
    for (int k = 1; k <= nz && ok; k++)
        for (int j = 1; j <= ny && ok; j++) {
            for (int i = 1; i <= nx; i++) {
                const size_t c = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (k - 1));
                float* r = &row[(size_t)(i - 1) * 7];
                r[0] = (float)((double)i - 0.5);
                r[1] = (float)((double)j - 0.5);
                r[2] = (float)((double)k - 0.5);
                r[3] = (float)u[c];
                r[4] = (float)v[c];
                r[5] = (float)w[c];
                r[6] = (float)(thermal ? s[c] : s[c] / 3.0);
            }
            ok = f.put(row.data(), row.size() * sizeof(float));
        }
    return ok ? MGLC_OK : MGLC_ERR_INVALID;
}

int mglc_write_tecplot(mglc_ctx* c, const char* path) {
    mglc_info info;
    int rc = geometry(c, info);
    if (rc) return rc;
    const size_t n = (size_t)info.nx * info.ny * info.nz;
    const bool th = info.kind == MGLC_KIND_THERMAL;
    std::vector<double> rho(n), u(n), v(n), w(n), T(th ? n : 0);
    if ((rc = mglc_get_macros(c, rho.data(), u.data(), v.data(), w.data(), th ? T.data() : nullptr)))
        return rc;
    return mglc_tecplot_write_fields(path, info.nx, info.ny, info.nz, u.data(), v.data(), w.data(),
                                     th ? T.data() : rho.data(), th ? 1 : 0);
}

int mglc_profiles_write_fields(const char* uz_path, const char* xw_path, int nx, int ny, int nz,
                               const double* u, const double* w, double u0) {
    if (!uz_path || !xw_path || nx <= 0 || ny <= 0 || nz <= 0 || !u || !w || !(u0 != 0.0))
        return MGLC_ERR_INVALID;
    const int ih = (nx - 1) / 2 + 1, jh = (ny - 1) / 2 + 1, kh = (nz - 1) / 2 + 1;  // 1-based
    auto at = [&](const double* a, int i, int j, int k) {
        return a[(size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (k - 1))];
    };
    File a(uz_path, "w"), b(xw_path, "w");
    if (!a.fp || !b.fp) return MGLC_ERR_INVALID;
    // one pair per line, 17 significant digits (the reference uses list-directed
    // output, whose layout is compiler-specific)
    for (int k = 1; k <= nz; k++)
        std::fprintf(a.fp, " %.17E %.17E\n", at(u, ih, jh, k) / u0, ((double)k - 0.5) / (double)nz);
    for (int i = 1; i <= nx; i++)
        std::fprintf(b.fp, " %.17E %.17E\n", ((double)i - 0.5) / (double)nx, at(w, i, jh, kh) / u0);
    return MGLC_OK;
}

int mglc_write_profiles(mglc_ctx* c, const char* uz_path, const char* xw_path, double u0) {
    mglc_info info;
    int rc = geometry(c, info);
    if (rc) return rc;
    const size_t n = (size_t)info.nx * info.ny * info.nz;
    std::vector<double> u(n), w(n);
    if ((rc = mglc_get_macros(c, nullptr, u.data(), nullptr, w.data(), nullptr))) return rc;
    return mglc_profiles_write_fields(uz_path, xw_path, info.nx, info.ny, info.nz, u.data(),
                                      w.data(), u0);
}

int mglc_write_binary(mglc_ctx* c, const char* path) {
    mglc_info info;
    int rc = geometry(c, info);
    if (rc) return rc;
    if (!path) return MGLC_ERR_INVALID;
    const size_t n = (size_t)info.nx * info.ny * info.nz;
    const bool th = info.kind == MGLC_KIND_THERMAL;
    std::vector<double> rho(n), u(n), v(n), w(n), T(th ? n : 0);
    if ((rc = mglc_get_macros(c, rho.data(), u.data(), v.data(), w.data(), th ? T.data() : nullptr)))
        return rc;
    File f(path, "wb");
    if (!f.fp) return MGLC_ERR_INVALID;
    const long long nb = (long long)(n * sizeof(double));
    bool ok = put_record(f, u.data(), nb, 0) && put_record(f, v.data(), nb, 0);
    if (th) ok = ok && put_record(f, w.data(), nb, 0) && put_record(f, T.data(), nb, 0);
    else ok = ok && put_record(f, rho.data(), nb, 0);
    return ok ? MGLC_OK : MGLC_ERR_INVALID;
}

int mglc_backup_write_fields(const char* path, int nx, int ny, int nz, const double* u,
                             const double* v, const double* w, const double* T, const double* f,
                             const double* g, long long max_subrecord) {
    if (!path || nx <= 0 || ny <= 0 || nz <= 0 || !u || !v || !w || !f) return MGLC_ERR_INVALID;
    File fp(path, "wb");
    if (!fp.fp) return MGLC_ERR_INVALID;
    const long long n = (long long)nx * ny * nz, nb = n * (long long)sizeof(double);
    bool ok = put_record(fp, u, nb, max_subrecord) && put_record(fp, v, nb, max_subrecord) &&
              put_record(fp, w, nb, max_subrecord);
    if (T) ok = ok && put_record(fp, T, nb, max_subrecord);
    ok = ok && put_record(fp, f, 19 * nb, max_subrecord);
    if (g) ok = ok && put_record(fp, g, 7 * nb, max_subrecord);
    return ok ? MGLC_OK : MGLC_ERR_INVALID;
}

int mglc_backup_read_fields(const char* path, int nx, int ny, int nz, double* u, double* v,
                            double* w, double* T, double* f, double* g) {
    if (!path || nx <= 0 || ny <= 0 || nz <= 0 || !u || !v || !w || !f) return MGLC_ERR_INVALID;
    File fp(path, "rb");
    if (!fp.fp) return MGLC_ERR_INVALID;
    const long long n = (long long)nx * ny * nz, nb = n * (long long)sizeof(double);
    int rc = get_record(fp, u, nb);
    if (!rc) rc = get_record(fp, v, nb);
    if (!rc) rc = get_record(fp, w, nb);
    if (!rc && T) rc = get_record(fp, T, nb);
    if (!rc) rc = get_record(fp, f, 19 * nb);
    if (!rc && g) rc = get_record(fp, g, 7 * nb);
    return rc;
}

int mglc_backup_save(mglc_ctx* c, const char* path) {
    mglc_info info;
    int rc = geometry(c, info);
    if (rc) return rc;
    const size_t n = (size_t)info.nx * info.ny * info.nz;
    const bool th = info.kind == MGLC_KIND_THERMAL;
    std::vector<double> u(n), v(n), w(n), T(th ? n : 0), f(19 * n), g(th ? 7 * n : 0);
    if ((rc = mglc_get_macros(c, nullptr, u.data(), v.data(), w.data(), th ? T.data() : nullptr)))
        return rc;
    if ((rc = mglc_get_f(c, f.data(), th ? g.data() : nullptr))) return rc;
    return mglc_backup_write_fields(path, info.nx, info.ny, info.nz, u.data(), v.data(), w.data(),
                                    th ? T.data() : nullptr, f.data(), th ? g.data() : nullptr, 0);
}

int mglc_backup_load(mglc_ctx* c, const char* path) {
    mglc_info info;
    int rc = geometry(c, info);
    if (rc) return rc;
    const size_t n = (size_t)info.nx * info.ny * info.nz;
    const bool th = info.kind == MGLC_KIND_THERMAL;
    std::vector<double> rho(n, 1.0), u(n), v(n), w(n), T(th ? n : 0), f(19 * n), g(th ? 7 * n : 0);
    if ((rc = mglc_backup_read_fields(path, info.nx, info.ny, info.nz, u.data(), v.data(), w.data(),
                                      th ? T.data() : nullptr, f.data(), th ? g.data() : nullptr)))
        return rc;
    // the reload keeps rho = 1 (bouyancy3d.F90:289) beside the stored u, v, w, T
    return mglc_load_state(c, f.data(), th ? g.data() : nullptr, rho.data(), u.data(), v.data(),
                           w.data(), th ? T.data() : nullptr);
}

// ------------------------------------------------------------------ calNuRe --
struct mglc_nure_monitor {
    int flow_reversal, flow_reversal_time;
    std::vector<double> nu, re, nu_mean, re_mean;  // index 0 unused (= 0), as in the reference
    int stationary = 0, stationary_time = 0, converged = 0;
};

int mglc_nure_create(int flow_reversal, int flow_reversal_time, mglc_nure_monitor** out) {
    if (!out || (flow_reversal != 0 && flow_reversal != 1)) return MGLC_ERR_INVALID;
    mglc_nure_monitor* m = new mglc_nure_monitor();
    m->flow_reversal = flow_reversal;
    m->flow_reversal_time = flow_reversal_time;
    m->nu.assign(1, 0.0);
    m->re.assign(1, 0.0);
    m->nu_mean.assign(1, 0.0);
    m->re_mean.assign(1, 0.0);
    *out = m;
    return MGLC_OK;
}

void mglc_nure_destroy(mglc_nure_monitor* m) { delete m; }

int mglc_nure_push(mglc_nure_monitor* m, double nu, double re, mglc_nure_status* st) {
    if (!m) return MGLC_ERR_INVALID;
    m->nu.push_back(nu);
    m->re.push_back(re);
    const int t = (int)m->nu.size() - 1;  // dimensionlessTime
    double sn = 0.0, sr = 0.0;
    for (int i = 1; i <= t; i++) sn = sn + m->nu[i];
    for (int i = 1; i <= t; i++) sr = sr + m->re[i];
    m->nu_mean.push_back(sn / (double)t);
    m->re_mean.push_back(sr / (double)t);
    double dnu_half = -1.0, dre_half = -1.0, dnu_mean = -1.0, dre_mean = -1.0;
    if (m->stationary == 1 && (t - m->stationary_time) % 200 == 0) {
        const int t0 = m->stationary_time, half = (t0 + t) / 2;
        double n1 = 0.0, r1 = 0.0, n2 = 0.0, r2 = 0.0;
        for (int i = t0; i <= half; i++) {
            n1 = n1 + m->nu[i];
            r1 = r1 + m->re[i];
        }
        n1 = n1 / (double)(half - t0 + 1);
        r1 = r1 / (double)(half - t0 + 1);
        for (int i = half; i <= t; i++) {
            n2 = n2 + m->nu[i];
            r2 = r2 + m->re[i];
        }
        n2 = n2 / (double)(t - half + 1);
        r2 = r2 / (double)(t - half + 1);
        dnu_half = std::fabs((n1 - n2) / n2);
        dre_half = std::fabs((r1 - r2) / r2);
        if (dnu_half <= 0.01 && dre_half <= 0.01) {
            if (m->flow_reversal == 0) m->converged = 1;
            else if (t >= t0 + m->flow_reversal_time) m->converged = 1;
        }
    }
    if (m->stationary == 0 && t % 100 == 0) {
        dnu_mean = std::fabs((m->nu_mean[t] - m->nu_mean[t - 100]) / m->nu_mean[t]);
        dre_mean = std::fabs((m->re_mean[t] - m->re_mean[t - 100]) / m->re_mean[t]);
        if (dnu_mean <= 0.01 && dre_mean <= 0.01) {
            m->stationary = 1;
            m->stationary_time = t;
        }
    }
    if (st) {
        st->time = t;
        st->nu = nu;
        st->re = re;
        st->nu_mean = m->nu_mean[t];
        st->re_mean = m->re_mean[t];
        st->stationary = m->stationary;
        st->stationary_time = m->stationary_time;
        st->converged = m->converged;
        st->nu_half_change = dnu_half;
        st->re_half_change = dre_half;
        st->nu_mean_change = dnu_mean;
        st->re_mean_change = dre_mean;
    }
    return MGLC_OK;
}

int mglc_nure_sample(mglc_nure_monitor* m, mglc_ctx* c, mglc_nure_status* st) {
    if (!m || !c) return MGLC_ERR_INVALID;
    double nu, re;
    int rc = mglc_nusselt(c, &nu, &re, nullptr, nullptr);
    if (rc) return rc;
    return mglc_nure_push(m, nu, re, st);
}

}  // extern "C"
