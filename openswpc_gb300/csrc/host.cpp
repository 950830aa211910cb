// host.cpp -- host driver layer: the reference's host-side set-up chain
// (src/swpc_3d/main.f90:48-116) rebuilt in C++ with FP64 arithmetic, feeding
// the device library through the C ABI of include/swpc_gpu.h, plus SAC
// output of the receiver traces.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/swpc_gpu.h"
#include "visco.hpp"

namespace swpc {
int set_err(int code, const std::string& msg);
}

namespace {

const double PI = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// input.inf reader (semantics of src/shared/m_readini.f90:29-166): the first
// non-comment line whose text starts with the key followed by '=' wins; the
// value is the first list-directed item; ${VAR} is expanded.
// ---------------------------------------------------------------------------
std::string ltrim(const std::string& s) {
    size_t p = s.find_first_not_of(" \t\r");
    return p == std::string::npos ? std::string() : s.substr(p);
}

struct Inf {
    std::vector<std::string> lines;
    std::string dir;
    bool strict = false;
    explicit Inf(const std::string& path) {
        std::ifstream f(path);
        if (!f) throw std::runtime_error("cannot open " + path);
        for (std::string s; std::getline(f, s);) lines.push_back(s);
        size_t sl = path.find_last_of('/');
        dir = sl == std::string::npos ? "." : path.substr(0, sl);
    }
    static std::string item(const std::string& v0) {
        std::string v = ltrim(v0);
        if (v.empty()) return v;
        if (v[0] == '\'' || v[0] == '"') {
            size_t e = v.find(v[0], 1);
            return v.substr(1, e == std::string::npos ? std::string::npos : e - 1);
        }
        size_t e = v.find_first_of(" \t,/\r");
        return v.substr(0, e);
    }
    bool find(const std::string& key, std::string& out) const {
        for (const auto& l0 : lines) {
            std::string l = ltrim(l0);
            if (l.empty() || l[0] == '#' || l[0] == '!') continue;
            if (l.compare(0, key.size(), key) != 0) continue;
            std::string r = ltrim(l.substr(key.size()));
            if (r.empty() || r[0] != '=') continue;
            out = item(r.substr(1));
            for (size_t p; (p = out.find("${")) != std::string::npos;) {
                size_t e = out.find('}', p);
                if (e == std::string::npos) break;
                const char* ev = std::getenv(out.substr(p + 2, e - p - 2).c_str());
                out = out.substr(0, p) + (ev ? ev : "") + out.substr(e + 1);
            }
            return true;
        }
        if (strict) throw std::runtime_error("key " + key + " is not found (strict_mode)");
        return false;
    }
    static double num(std::string s) {
        for (auto& c : s) if (c == 'd' || c == 'D') c = 'e';
        char* e = nullptr;
        double v = std::strtod(s.c_str(), &e);
        if (e == s.c_str()) throw std::runtime_error("not a number: '" + s + "'");
        return v;
    }
    double r(const std::string& k, double d) const { std::string v; return find(k, v) ? num(v) : d; }
    int i(const std::string& k, int d) const { std::string v; return find(k, v) ? (int)std::lround(num(v)) : d; }
    std::string s(const std::string& k, const std::string& d) const { std::string v; return find(k, v) ? v : d; }
    bool b(const std::string& k, bool d) const {
        std::string v;
        if (!find(k, v)) return d;
        size_t p = (!v.empty() && v[0] == '.') ? 1 : 0;
        if (p >= v.size()) return d;
        char c = (char)std::tolower((unsigned char)v[p]);
        if (c != 't' && c != 'f') throw std::runtime_error("not a logical value for " + k + ": '" + v + "'");
        return c == 't';
    }
    std::string path(const std::string& f) const { return (f.empty() || f[0] == '/') ? f : dir + "/" + f; }
};

std::vector<std::string> table_rows(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<std::string> rows;
    for (std::string s; std::getline(f, s);) {
        std::string t = ltrim(s);
        if (t.empty() || t[0] == '#') continue;
        if (t.find_first_not_of(" \t\r") == std::string::npos) continue;
        rows.push_back(t);
    }
    return rows;
}
std::vector<std::string> split(const std::string& s) {
    std::vector<std::string> v;
    std::string cur;
    bool q = false;
    char qc = 0;
    for (char c : s) {
        if (q) { if (c == qc) q = false; else cur += c; continue; }
        if (c == '\'' || c == '"') { q = true; qc = c; continue; }
        if (c == ' ' || c == '\t' || c == ',' || c == '\r') { if (!cur.empty()) { v.push_back(cur); cur.clear(); } continue; }
        cur += c;
    }
    if (!cur.empty()) v.push_back(cur);
    return v;
}

// ---------------------------------------------------------------------------
// Gauss-Krueger (transverse Mercator, GRS80, scale 0.9999) -- Krueger's
// n-series as published by Karney (2011, J. Geodesy 85:475) and used by the
// Japanese plane rectangular system; x to the north, y to the east, km.
// ---------------------------------------------------------------------------
struct GK {
    double a = 6378137.0, f = 298.257222101, k0 = 0.9999, n;
    double al[6], be[6], de[7], A[6];
    GK() {
        n = 1.0 / (2.0 * f - 1.0);
        const double n2 = n * n, n3 = n2 * n, n4 = n3 * n, n5 = n4 * n, n6 = n5 * n;
        al[1] = n / 2 - 2 * n2 / 3 + 5 * n3 / 16 + 41 * n4 / 180 - 127 * n5 / 288;
        al[2] = 13 * n2 / 48 - 3 * n3 / 5 + 557 * n4 / 1440 + 281 * n5 / 630;
        al[3] = 61 * n3 / 240 - 103 * n4 / 140 + 15061 * n5 / 26880;
        al[4] = 49561 * n4 / 161280 - 179 * n5 / 168;
        al[5] = 34729 * n5 / 80640;
        be[1] = n / 2 - 2 * n2 / 3 + 37 * n3 / 96 - n4 / 360 - 81 * n5 / 512;
        be[2] = n2 / 48 + n3 / 15 - 437 * n4 / 1440 + 46 * n5 / 105;
        be[3] = 17 * n3 / 480 - 37 * n4 / 840 - 209 * n5 / 4480;
        be[4] = 4397 * n4 / 161280 - 11 * n5 / 504;
        be[5] = 4583 * n5 / 161280;
        de[1] = 2 * n - 2 * n2 / 3 - 2 * n3 + 116 * n4 / 45 + 26 * n5 / 45 - 2854 * n6 / 675;
        de[2] = 7 * n2 / 3 - 8 * n3 / 5 - 227 * n4 / 45 + 2704 * n5 / 315 + 2323 * n6 / 945;
        de[3] = 56 * n3 / 15 - 136 * n4 / 35 - 1262 * n5 / 105 + 73814 * n6 / 2835;
        de[4] = 4279 * n4 / 630 - 332 * n5 / 35 - 399572 * n6 / 14175;
        de[5] = 4174 * n5 / 315 - 144838 * n6 / 6237;
        de[6] = 601676 * n6 / 22275;
        A[0] = 1 + n2 / 4 + n4 / 64;
        A[1] = -1.5 * (n - n3 / 8 - n5 / 64);
        A[2] = 15.0 / 16 * (n2 - n4 / 4);
        A[3] = -35.0 / 48 * (n3 - 5 * n5 / 16);
        A[4] = 315.0 / 512 * n4;
        A[5] = -693.0 / 1280 * n5;
    }
    double meridian(double phi0) const {  // scaled meridian arc length to latitude phi0
        double s = A[0] * phi0;
        for (int j = 1; j <= 5; ++j) s += A[j] * std::sin(2 * j * phi0);
        return k0 * a / (1 + n) * s;
    }
    void ll2xy(double lon, double lat, double lon0, double lat0, double& x, double& y) const {
        const double lam = lon * PI / 180, lam0 = lon0 * PI / 180, phi = lat * PI / 180, phi0 = lat0 * PI / 180;
        const double e2n = 2 * std::sqrt(n) / (1 + n);
        const double t = std::sinh(std::atanh(std::sin(phi)) - e2n * std::atanh(e2n * std::sin(phi)));
        const double c = std::sqrt(1 + t * t);
        const double xi = std::atan2(t, std::cos(lam - lam0)), eta = std::atanh(std::sin(lam - lam0) / c);
        double X = xi, Y = eta;
        for (int j = 1; j <= 5; ++j) {
            X += al[j] * std::sin(2 * j * xi) * std::cosh(2 * j * eta);
            Y += al[j] * std::cos(2 * j * xi) * std::sinh(2 * j * eta);
        }
        const double Ab = k0 * a / (1 + n) * A[0];
        x = (Ab * X - meridian(phi0)) / 1000;
        y = Ab * Y / 1000;
    }
    void xy2ll(double x, double y, double lon0, double lat0, double& lon, double& lat) const {
        const double phi0 = lat0 * PI / 180;
        const double Ab = k0 * a / (1 + n) * A[0];
        const double xi = (x * 1000 + meridian(phi0)) / Ab, eta = y * 1000 / Ab;
        double X = xi, Y = eta;
        for (int j = 1; j <= 5; ++j) {
            X -= be[j] * std::sin(2 * j * xi) * std::cosh(2 * j * eta);
            Y -= be[j] * std::cos(2 * j * xi) * std::sinh(2 * j * eta);
        }
        const double chi = std::asin(std::sin(X) / std::cosh(Y));
        double phi = chi;
        for (int j = 1; j <= 6; ++j) phi += de[j] * std::sin(2 * j * chi);
        lon = lon0 + std::atan(std::sinh(Y) / std::cos(X)) * 180 / PI;
        lat = phi * 180 / PI;
    }
};
const GK gk;

// src/shared/m_geomap.f90:16-64: azimuth phi rotates the local frame clockwise
void g2c(double lon, double lat, double lon0, double lat0, double phi, double& x, double& y) {
    double xx, yy, p = phi * PI / 180;
    gk.ll2xy(lon, lat, lon0, lat0, xx, yy);
    x = std::cos(p) * xx + std::sin(p) * yy;
    y = -std::sin(p) * xx + std::cos(p) * yy;
}
void c2g(double x, double y, double lon0, double lat0, double phi, double& lon, double& lat) {
    double p = phi * PI / 180;
    gk.xy2ll(std::cos(p) * x - std::sin(p) * y, std::sin(p) * x + std::cos(p) * y, lon0, lat0, lon, lat);
}

// ---------------------------------------------------------------------------
// Model and set-up state
// ---------------------------------------------------------------------------
struct Params {
    std::string title, odir, abc_type, vmodel_type, stftype, stf_format, fn_stf, sdep_fit, st_format, fn_stloc, wav_format;
    int nx, ny, nz, nt, na, ntdec_w, ntdec_r, ntdec_s, idec, jdec, kdec;
    double dx, dy, dz, dt, xbeg, ybeg, zbeg, tbeg, clon, clat, phi, fq_min, fq_max, fq_ref, vcut, z0_xy, x0_yz, y0_xz;
    bool bf_mode, sw_v, sw_u, sw_stress, sw_strain, munk;
    int snap_sw[5];  // per section xy yz xz fs ob: bit SWPC_SNAPK_* set when <sec>_<kind>%sw is true
    // plane-wave mode (m_source.f90:316-466)
    bool pw_mode = false;
    std::string pw_ps;
    double pw_ztop = 1e30, pw_zlen = -1, pw_strike = 0, pw_dip = 0, pw_rake = 0;
    // Green's-function mode (m_green.f90:100-160)
    bool green_mode = false, green_bforce = false;
    std::string green_stnm, green_cmp, fn_glst, green_fmt;
    double green_trise = 1.0, green_maxdist = 1e30;
};

struct Station { std::string name; double x, y, z, lon, lat; int i, j, k; };

struct Meta {  // what the SAC writer needs after set-up
    Params p;
    std::vector<Station> st;
    double M0 = 0, UC = 1e-15, evlo = 0, evla = 0, evdp = 0, sx0 = 0, sy0 = 0, otim = 0;
    double m6[6] = {0, 0, 0, 0, 0, 0}, f3[3] = {0, 0, 0};
    long long exedate = 0;
    int ntw = 0, flags = 0;
    // snapshot files (m_snap.f90:324-473, 846-892): per section the grid of
    // pixels, the header's first coordinates and spacings, the absorber
    // widths and the medium planes (rho, lam, mu over the section, Fortran
    // order), plus the topography depth of the horizontal sections
    struct SnapSec {
        int sec = 0, kinds = 0, fix = 1, d1 = 1, d2 = 1, n1 = 0, n2 = 0, na1 = 0, na2 = 0;
        float x1 = 0, x2 = 0, dx1 = 0, dx2 = 0;
        std::vector<float> med;
    };
    std::vector<SnapSec> snaps;
    double bd0 = 0;
    // Green's-function mode: the pseudo-source station and the output points
    struct GPoint { double x = 0, y = 0, z = 0, lon = 0, lat = 0; long long gid = 0; int i = 0, j = 0, k = 0; };
    struct Green { bool on = false; Station station; std::vector<GPoint> pts; } green;
    // the numbers of report__setup's banner (src/swpc_3d/m_report.f90:71-85)
    struct Banner {
        int nproc_x = 1, nproc_y = 1;
        float mem_all = 0, mem_node = 0, c = 0, r = 0, vmin = 0, vmax = 0, fmax = 0;
    } banner;
};
std::mutex g_meta_mu;
std::map<swpc_sim*, Meta> g_meta;

struct Grid {  // Fortran halo-array geometry
    int nx, ny, nz;
    size_t n3() const { return (size_t)(nz + 6) * (nx + 6) * (ny + 6); }
    size_t idx(int k, int i, int j) const { return ((size_t)(j + 2) * (nx + 6) + (i + 2)) * (nz + 6) + (k + 2); }
    size_t n2() const { return (size_t)(nx + 6) * (ny + 6); }
    size_t idx2(int i, int j) const { return (size_t)(j + 2) * (nx + 6) + (i + 2); }
};

double seawater_vel(double z, bool munk) {  // src/shared/m_seawater.f90:34-47
    double eps = munk ? 0.00737 : 0.0, zc = 1300.0, zb = 2 * (z * 1000. - zc) / zc;
    return 1.5 * (1.0 + eps * (zb - 1.0 + std::exp(-zb)));
}

// velocity models (m_vmodel_uni.f90:40-149, m_vmodel_lhm.f90:21-169,
// m_vmodel_lgm.f90:21-174); rho, lam, mu, Qp, Qs over the halo grid and
// the topography depth bd0
void vmodel(const Inf& inf, const Params& p, const Grid& G, std::vector<float>& rho, std::vector<float>& lam,
            std::vector<float>& mu, std::vector<float>& qp, std::vector<float>& qs, double& bd0) {
    const size_t n3 = G.n3();
    rho.assign(n3, 0); lam.assign(n3, 0); mu.assign(n3, 0); qp.assign(n3, 0); qs.assign(n3, 0);
    auto zc = [&](int k) { return p.zbeg + (k - 0.5) * p.dz; };
    // these models depend on depth only: build one column (k fastest, as the
    // arrays are laid out) and copy it into every (i, j) column at the end
    const int nk = p.nz + 6;
    std::vector<float> c_rho(nk), c_lam(nk), c_mu(nk), c_qp(nk), c_qs(nk);
    auto fill = [&](int k, double r, double vp, double vs, double q1, double q2) {
        const int q = k + 2;
        c_rho[q] = (float)r; c_mu[q] = (float)(r * vs * vs); c_lam[q] = (float)(r * (vp * vp - 2 * vs * vs));
        c_qp[q] = (float)q1; c_qs[q] = (float)q2;
    };
    auto spread = [&]() {
        std::vector<float>* dst[5] = {&rho, &lam, &mu, &qp, &qs};
        const std::vector<float>* src[5] = {&c_rho, &c_lam, &c_mu, &c_qp, &c_qs};
        for (int j = -2; j <= p.ny + 3; ++j)
            for (int i = -2; i <= p.nx + 3; ++i) {
                const size_t b = G.idx(-2, i, j);
                for (int f = 0; f < 5; ++f) std::copy(src[f]->begin(), src[f]->end(), dst[f]->begin() + b);
            }
    };
    if (inf.b("earth_flattening", false)) throw std::runtime_error("earth_flattening is not supported by openswpc_gb300");
    if (p.vmodel_type == "uni") {
        double vp0 = inf.r("vp0", 5.0), vs0 = inf.r("vs0", vp0 / std::sqrt(3.0)), rho0 = inf.r("rho0", 2.7);
        double qp0 = inf.r("qp0", 1e6), qs0 = inf.r("qs0", 1e6), topo0 = inf.r("topo0", 0.0);
        bd0 = topo0;
        for (int k = -2; k <= p.nz + 3; ++k) {
            double z = zc(k);
            if (z > topo0) fill(k, rho0, vp0, vs0, qp0, qs0);
            else if (z > 0) fill(k, 1.0, seawater_vel(z, p.munk), 0, 1e6, 1e6);
            else fill(k, 0.001, 0, 0, 10, 10);
        }
        spread();
        return;
    }
    if (p.vmodel_type != "lhm" && p.vmodel_type != "lgm")
        throw std::runtime_error("vmodel_type '" + p.vmodel_type + "' is not supported by openswpc_gb300 (uni, lhm, lgm)");
    auto rows = table_rows(inf.path(inf.s("fn_lhm", "")));
    const int nl = (int)rows.size();
    if (nl < 1) throw std::runtime_error("empty layer table");
    std::vector<double> dep(nl), r0(nl), vp(nl), vs(nl), q1(nl), q2(nl);
    for (int l = 0; l < nl; ++l) {
        auto t = split(rows[l]);
        if (t.size() < 6) throw std::runtime_error("bad layer line: " + rows[l]);
        dep[l] = Inf::num(t[0]); r0[l] = Inf::num(t[1]); vp[l] = Inf::num(t[2]);
        vs[l] = Inf::num(t[3]); q1[l] = Inf::num(t[4]); q2[l] = Inf::num(t[5]);
    }
    for (int l = nl - 2; l >= 0; --l)  // velocity cut-off
        if ((vp[l] < p.vcut || vs[l] < p.vcut) && vp[l] > 0 && vs[l] > 0) {
            vp[l] = vp[l + 1]; vs[l] = vs[l + 1]; r0[l] = r0[l + 1]; q1[l] = q1[l + 1]; q2[l] = q2[l + 1];
        }
    bd0 = dep[0];
    for (int k = -2; k <= p.nz + 3; ++k) {
        double z = zc(k);
        if (z < dep[0]) {
            if (z < 0) fill(k, 0.001, 0, 0, 10, 10);
            else fill(k, 1.0, seawater_vel(z, p.munk), 0, 1e6, 1e6);
            continue;
        }
        if (p.vmodel_type == "lhm") {
            int L = 0;
            for (int l = 0; l < nl; ++l) if (z >= dep[l]) L = l;
            fill(k, r0[L], vp[L], vs[L], q1[L], q2[L]);
        } else {
            double R = r0[nl - 1], P = vp[nl - 1], S = vs[nl - 1], A = q1[nl - 1], B = q2[nl - 1];
            for (int l = 0; l < nl - 1; ++l)
                if (dep[l] <= z && z < dep[l + 1]) {
                    double w = (z - dep[l]) / (dep[l + 1] - dep[l]);
                    R = r0[l] + (r0[l + 1] - r0[l]) * w; P = vp[l] + (vp[l + 1] - vp[l]) * w; S = vs[l] + (vs[l + 1] - vs[l]) * w;
                    A = q1[l] + (q1[l + 1] - q1[l]) * w; B = q2[l] + (q2[l + 1] - q2[l]) * w;
                    break;
                }
            fill(k, R, P, S, A, B);
        }
    }
    spread();
}

namespace visco = swpc::visco;
using visco::constq_zeta;
using visco::relaxation_times;

// src/swpc_3d/m_medium.f90:124-394 in FP64: absorber homogenisation,
// tau-method, relaxation of the moduli to fq_ref, surface detection.
void medium_post(int nx, int ny, int nz, int na, double fq_min, double fq_max, double fq_ref, float* rho, float* lam,
                 float* mu, float* qp, float* qs, int* kfs, int* kob, int* kfs_top, int* kfs_bot, int* kob_top,
                 int* kob_bot, double* ts) {
    Grid G{nx, ny, nz};
    float* F[5] = {rho, lam, mu, qp, qs};
    auto cp = [&](int k, int i, int j, int ks, int is, int js) {
        for (auto f : F) f[G.idx(k, i, j)] = f[G.idx(ks, is, js)];
    };
    for (int i = -2; i <= na; ++i)
        for (int j = -2; j <= ny + 3; ++j) for (int k = -2; k <= nz + 3; ++k) cp(k, i, j, k, na + 1, j);
    for (int i = nx - na + 1; i <= nx + 3; ++i)
        for (int j = -2; j <= ny + 3; ++j) for (int k = -2; k <= nz + 3; ++k) cp(k, i, j, k, nx - na, j);
    for (int j = -2; j <= na; ++j)
        for (int i = -2; i <= nx + 3; ++i) for (int k = -2; k <= nz + 3; ++k) cp(k, i, j, k, i, na + 1);
    for (int j = ny - na + 1; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) for (int k = -2; k <= nz + 3; ++k) cp(k, i, j, k, i, ny - na);
    for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) for (int k = nz - na + 1; k <= nz + 3; ++k) cp(k, i, j, nz - na, i, j);
    const int nm = 3;
    relaxation_times(nm, fq_min, fq_max, ts);
    const double zeta = constq_zeta(nm, fq_min, fq_max, ts);
    double cr, ci;
    visco::zener_c(nm, fq_ref, ts, cr, ci);
    const size_t n3 = G.n3();
    // the relaxation factor depends on Q only; media hold few distinct Q
    // values, so remember the last ones
    float lq[2] = {-1.f, -1.f};
    double lrc[2] = {0, 0};
    auto relax = [&](int w, float q, double tau) {
        if (q != lq[w]) { lq[w] = q; lrc[w] = visco::relax_factor(cr, ci, tau); }
        return lrc[w];
    };
    for (size_t q = 0; q < n3; ++q) {
        double tp = nm * zeta / (double)qp[q], tsv = nm * zeta / (double)qs[q];
        double rb2 = mu[q], ra2 = (double)lam[q] + 2.0 * mu[q];
        double m2 = rb2 * relax(0, qs[q], tsv);
        mu[q] = (float)m2;
        lam[q] = (float)(ra2 * relax(1, qp[q], tp) - 2 * m2);
        qp[q] = (float)tp;
        qs[q] = (float)tsv;
    }
    const float eps = 1.1920928955078125e-07f;
    const size_t n2 = G.n2();
    std::fill(kfs, kfs + n2, 0);
    std::fill(kob, kob + n2, 0);
    for (int j = 0; j <= ny + 2; ++j)
        for (int i = 0; i <= nx + 2; ++i)
            for (int k = 1; k <= nz - 1; ++k) {
                if (std::fabs(mu[G.idx(k, i, j)]) < eps && std::fabs(mu[G.idx(k + 1, i, j)]) > eps) kob[G.idx2(i, j)] = k;
                if (std::fabs(lam[G.idx(k, i, j)]) < eps && std::fabs(lam[G.idx(k + 1, i, j)]) > eps) kfs[G.idx2(i, j)] = k;
            }
    std::fill(kfs_top, kfs_top + n2, 0); std::fill(kfs_bot, kfs_bot + n2, 0);
    std::fill(kob_top, kob_top + n2, 0); std::fill(kob_bot, kob_bot + n2, 0);
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            int a = 1 << 30, b = -(1 << 30), c = 1 << 30, d = -(1 << 30);
            for (int jj = j - 2; jj <= j + 3; ++jj)
                for (int ii = i - 2; ii <= i + 3; ++ii) {
                    a = std::min(a, kfs[G.idx2(ii, jj)]); b = std::max(b, kfs[G.idx2(ii, jj)]);
                    c = std::min(c, kob[G.idx2(ii, jj)]); d = std::max(d, kob[G.idx2(ii, jj)]);
                }
            kfs_top[G.idx2(i, j)] = std::max(a - 2, 1); kfs_bot[G.idx2(i, j)] = std::min(b + 2, nz);
            kob_top[G.idx2(i, j)] = std::max(c - 2, 1); kob_bot[G.idx2(i, j)] = std::min(d + 2, nz);
        }
}

// stabilize_absorber (src/swpc_3d/m_medium.f90:273-337), single precision as
// the reference: inside the absorber (k >= the smallest kbeg_a of the 5x5
// neighbourhood) a thin low-velocity layer (at most 20 cells) gets the medium
// of the cell above it at its top cell, and shear velocities below 0.4 of the
// model's largest P velocity are raised to it with Vp = sqrt(3) Vs.
void stabilize_absorber(int nx, int ny, int nz, int na, float* rho, float* lam, float* mu, float* taup, float* taus,
                        const int* kfs) {
    Grid G{nx, ny, nz};
    const float eps = 1.1920928955078125e-07f;
    float vmax = -1;  // velocity_minmax (m_medium.f90:396-427)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
            for (int k = kfs[G.idx2(i, j)] + 1; k <= nz; ++k) {
                const size_t c = G.idx(k, i, j);
                vmax = std::max(vmax, std::sqrt((lam[c] + 2 * mu[c]) / rho[c]));
            }
    const float vmin_pml = vmax * 0.4f;
    const int LV_THICK = 20;
    auto kbeg_a = [&](int i, int j) { return (i <= na || nx - na + 1 <= i || j <= na || ny - na + 1 <= j) ? 1 : nz - na + 1; };
    auto kmin = [&](int i, int j) {
        int m = 1 << 30;
        for (int jj = j - 2; jj <= j + 2; ++jj)
            for (int ii = i - 2; ii <= i + 2; ++ii) m = std::min(m, kbeg_a(ii, jj));
        return m;
    };
    for (int j = 0; j <= ny + 1; ++j)
        for (int i = 0; i <= nx + 1; ++i) {
            int k = kmin(i, j);
            while (k <= nz) {
                const size_t c = G.idx(k, i, j), u = G.idx(k - 1, i, j);
                if (lam[c] < lam[u] || mu[c] < mu[u]) {
                    int k2 = k + 1;
                    for (; k2 <= nz; ++k2)
                        if (lam[G.idx(k2, i, j)] > lam[G.idx(k2 - 1, i, j)] || mu[G.idx(k2, i, j)] > mu[G.idx(k2 - 1, i, j)]) break;
                    if (k2 - k <= LV_THICK) {
                        rho[c] = rho[u]; lam[c] = lam[u]; mu[c] = mu[u]; taup[c] = taup[u]; taus[c] = taus[u];
                        k = k2 - 1;
                    }
                }
                ++k;
            }
        }
    const float gamma = std::sqrt(3.0f);
    for (int j = 0; j <= ny + 1; ++j)
        for (int i = 0; i <= nx + 1; ++i)
            for (int k = kmin(i, j); k <= nz; ++k) {
                const size_t c = G.idx(k, i, j);
                float vs = std::sqrt(mu[c] / rho[c]);
                if (vs < eps) continue;
                if (vs < vmin_pml) {
                    vs = vmin_pml;
                    const float vp = vs * gamma;
                    lam[c] = rho[c] * (vp * vp - 2 * vs * vs);
                    mu[c] = rho[c] * (vs * vs);
                }
            }
}

// src/shared/m_fdtool.f90:307-336
void sdr2moment(double strike, double dip, double rake, double* m6) {
    const double r = PI / 180;
    double sd = std::sin(dip * r), cd = std::cos(dip * r), s2d = std::sin(2 * dip * r), c2d = std::cos(2 * dip * r);
    double sl = std::sin(rake * r), cl = std::cos(rake * r);
    double sf = std::sin(strike * r), cf = std::cos(strike * r), s2f = std::sin(2 * strike * r), c2f = std::cos(2 * strike * r);
    m6[0] = -(sd * cl * s2f + s2d * sl * sf * sf);   // xx
    m6[1] = (sd * cl * s2f - s2d * sl * cf * cf);    // yy
    m6[2] = (s2d * sl);                              // zz
    m6[3] = -(cd * cl * sf - c2d * sl * cf);         // yz
    m6[4] = -(cd * cl * cf + c2d * sl * sf);         // xz
    m6[5] = (sd * cl * c2f + s2d * sl * s2f / 2);    // xy
}

// Source time functions in single precision (src/shared/m_fdtool.f90:339-497)
float momentrate_h(float t, const std::string& type, float ts, float tr) {
    const float pi = 3.14159265358979f;
    if (type == "boxcar") return (ts <= t && t <= ts + tr) ? 1.f / tr : 0.f;
    if (type == "triangle") {
        if (ts <= t && t <= ts + tr / 2) return 4 * (t - ts) / (tr * tr);
        if (ts + tr / 2 < t && t <= ts + tr) return -4 * (t - ts - tr) / (tr * tr);
        return 0.f;
    }
    if (type == "herrmann") {
        const float t1 = ts + tr / 4, t2 = ts + 3 * tr / 4;
        if (ts <= t && t < t1) return 16 * (t - ts) * (t - ts) / (tr * tr * tr);
        if (t1 <= t && t < t2) return -2 * (8 * (t * t + tr * ts + ts * ts - t * tr - 2 * t * ts) + tr * tr) / (tr * tr * tr);
        if (t2 <= t && t <= ts + tr) return 16 * (ts + tr - t) * (ts + tr - t) / (tr * tr * tr);
        return 0.f;
    }
    if (type == "cosine" || type == "scosine")
        return (ts <= t && t <= ts + tr) ? (1 - std::cos(2 * pi * (t - ts) / tr)) / tr : 0.f;
    if (type == "texp") {
        if (ts > t) return 0.f;
        const float tt = t - ts;
        return (2 * pi) * (2 * pi) * tt / (tr * tr) * std::exp(-2 * pi * tt / tr);
    }
    if (ts <= t && t <= ts + tr) {  // kupper
        const float sv = std::sin(pi * (t - ts) / tr);
        return 3 * pi * sv * sv * sv / (4 * tr);
    }
    return 0.f;
}

// pw_setup (src/swpc_3d/m_source.f90:316-466) in single precision: the
// initial velocity and stress of a plane P or S wave over the whole halo grid
// (Vx Vy Vz Sxx Syy Szz Syz Sxz Sxy), and fcut = v / pw_zlen at the centre
// column at depth pw_ztop.
double plane_wave(const Params& p, const Grid& G, const std::vector<float>& rho, const std::vector<float>& lam,
                  const std::vector<float>& mu, std::vector<std::vector<float>>& F) {
    const float d2r = 3.14159265358979f / 180.f;
    const float dipr = (float)p.pw_dip * d2r, strr = (float)p.pw_strike * d2r, rakr = (float)p.pw_rake * d2r;
    const float sd = std::sin(dipr), cd = std::cos(dipr), sf = std::sin(strr), cf = std::cos(strr);
    const float sl = std::sin(rakr), cl = std::cos(rakr), c2d = std::cos(2 * dipr), c2f = std::cos(2 * strr);
    const bool P = p.pw_ps == "p" || p.pw_ps == "P";
    const float xb = (float)p.xbeg, yb = (float)p.ybeg, zb = (float)p.zbeg, dx = (float)p.dx, dy = (float)p.dy;
    const float dz = (float)p.dz, dt = (float)p.dt, zt = (float)p.pw_ztop, zl = (float)p.pw_zlen;
    const std::string& st = p.stftype;
    const float eps = 1.1920928955078125e-07f;
    F.assign(9, std::vector<float>(G.n3(), 0.f));
    for (int j = -2; j <= p.ny + 3; ++j)
        for (int i = -2; i <= p.nx + 3; ++i)
            for (int k = -2; k <= p.nz + 3; ++k) {
                const size_t c = G.idx(k, i, j);
                const float v = P ? std::sqrt((lam[c] + 2 * mu[c]) / rho[c]) : std::sqrt(mu[c] / rho[c]);
                if (v < eps) continue;
                const float x0 = xb + ((float)i - 0.5f) * dx, y0 = yb + ((float)j - 0.5f) * dy;
                const float z0 = zb + ((float)k - 0.5f) * dz - zt;
                const float x1 = x0 + dx / 2.f, y1 = y0 + dy / 2.f, z1 = z0 + dz / 2.f;
                const float sh = dt / 2.f * v;
                auto m = [&](float a) { return momentrate_h(a, st, 0.f, zl); };
                const float s_ii = m(sd * sf * x0 - sd * cf * y0 + cd * z0);
                const float s_vx = m(sd * sf * x1 - sd * cf * y0 + cd * z0 + sh);
                const float s_vy = m(sd * sf * x0 - sd * cf * y1 + cd * z0 + sh);
                const float s_vz = m(sd * sf * x0 - sd * cf * y0 + cd * z1 + sh);
                const float s_yz = m(sd * sf * x0 - sd * cf * y1 + cd * z1);
                const float s_xz = m(sd * sf * x1 - sd * cf * y0 + cd * z1);
                const float s_xy = m(sd * sf * x1 - sd * cf * y1 + cd * z0);
                const float la0 = lam[c], mu0 = mu[c];
                if (P) {
                    F[0][c] = -sd * sf * s_vx;
                    F[1][c] = sd * cf * s_vy;
                    F[2][c] = -cd * s_vz;
                    F[3][c] = -(la0 + 2 * mu0 * sd * sd * sf * sf) * s_ii / v;
                    F[4][c] = -(la0 + 2 * mu0 * sd * sd * cf * cf) * s_ii / v;
                    F[5][c] = -(la0 + 2 * mu0 * cd * cd) * s_ii / v;
                    F[6][c] = 2 * mu0 * sd * cd * cf * s_yz / v;
                    F[7][c] = -2 * mu0 * sd * cd * sf * s_xz / v;
                    F[8][c] = 2 * mu0 * sd * cd * sf * s_xy / v;
                } else {
                    F[0][c] = (cl * cf + sl * cd * sf) * s_vx;
                    F[1][c] = (cl * sf - sl * cd * cf) * s_vy;
                    F[2][c] = -sl * sd * s_vz;
                    F[3][c] = 2 * mu0 * sd * sf * (cl * cf + sl * cd * sf) * s_ii / v;
                    F[4][c] = -2 * mu0 * sd * cf * (cl * sf - sl * cd * cf) * s_ii / v;
                    F[5][c] = -2 * mu0 * cd * sl * sd * s_ii / v;
                    F[6][c] = mu0 * (cl * cd * sf - sl * c2d * cf) * s_yz / v;
                    F[7][c] = mu0 * (cl * cd * cf + sl * c2d * sf) * s_xz / v;
                    F[8][c] = -mu0 * (cl * sd * c2f + 2 * sl * sd * cd * sf * cf) * s_xy / v;
                }
            }
    const float xe = xb + p.nx * dx, ye = yb + p.ny * dy;
    const int ic = (int)std::ceil(((xb + xe) / 2 - xb) / dx), jc = (int)std::ceil(((yb + ye) / 2 - yb) / dy);
    const int kc = (int)std::ceil((zt - zb) / dz);
    if (1 <= ic && ic <= p.nx && 1 <= jc && jc <= p.ny && -2 <= kc && kc <= p.nz + 3) {
        const size_t c = G.idx(kc, ic, jc);
        const float v = P ? std::sqrt((lam[c] + 2 * mu[c]) / rho[c]) : std::sqrt(mu[c] / rho[c]);
        return (double)(v / zl);
    }
    return 0.0;
}

int stf_code(const std::string& s) {
    const char* names[] = {"boxcar", "triangle", "herrmann", "kupper", "cosine", "texp"};
    for (int q = 0; q < 6; ++q) if (s == names[q]) return q;
    if (s == "scosine") return 4;
    return 3;
}

int x2i(double x, double beg, double d) { return (int)std::ceil((x - beg) / d); }

void mkdirs(const std::string& d) {
    std::string cur;
    for (size_t p = 0; p <= d.size(); ++p) {
        if (p == d.size() || d[p] == '/') {
            if (!cur.empty()) mkdir(cur.c_str(), 0755);
        }
        if (p < d.size()) cur += d[p];
    }
}

// SAC header (src/shared/m_sac.f90:267-449, defaults of sac__init :452-562):
// 70 floats, 35 ints, 5 logicals and 192 characters, written before the data.
struct SacHeader {
    float f[70];
    int i[35], l[5];
    char k[192];
    SacHeader() {
        for (auto& v : f) v = -12345.0f;
        for (auto& v : i) v = -12345;
        for (auto& v : l) v = 0;
        for (int q = 0; q < 24; ++q) std::memcpy(k + 8 * q, "-12345  ", 8);
        kset(113, 16, "-12345");  // kevnm is 16 characters
        i[6] = 6;   // nvhdr
        i[15] = 1;  // iftype: time series
        l[0] = 1;   // leven
        l[2] = 1;   // lovrok
    }
    void kset(int word, int len, const std::string& v) {
        std::string t = v.substr(0, len);
        t.resize(len, ' ');
        std::memcpy(k + 4 * (word - 111), t.data(), len);
    }
    void set_time(long long exedate) {  // nzyear .. nzmsec from the run's start time
        time_t tt = (time_t)exedate;
        struct tm lt;
        localtime_r(&tt, &lt);
        i[0] = lt.tm_year + 1900; i[1] = lt.tm_yday + 1; i[2] = lt.tm_hour; i[3] = lt.tm_min; i[4] = lt.tm_sec; i[5] = 0;
    }
    void set_delta(double delta) { f[0] = (float)((long long)(delta * 1e7)) / 1e7f; }
    std::string bytes(const float* dat, int npts) {
        i[9] = npts;
        std::string out;
        out.reserve(632 + (size_t)npts * 4);
        out.append((const char*)f, sizeof f);
        out.append((const char*)i, sizeof i);
        out.append((const char*)l, sizeof l);
        out.append(k, sizeof k);
        out.append((const char*)dat, (size_t)npts * 4);
        return out;
    }
};

// Receiver trace as SAC bytes (headers of m_wav.f90:276-330)
std::string sac_image(const Meta& m, const Station& st, const char* cmp, int idep, double cmpinc, double cmpaz,
                      const float* dat, int npts) {
    SacHeader h;
    const Params& p = m.p;
    h.set_delta(p.ntdec_w * p.dt);
    h.f[5] = (float)p.tbeg;
    h.f[7] = (float)m.otim;
    h.f[31] = (float)st.lat; h.f[32] = (float)st.lon; h.f[34] = (float)(st.z * 1000);
    h.f[35] = (float)m.evla; h.f[36] = (float)m.evlo; h.f[38] = (float)m.evdp;
    h.f[39] = m.M0 < 1.1920928955078125e-07 ? -12345.0f : (float)((std::log10(m.M0) - 9.1) * 2.0 / 3.0);
    if (p.bf_mode) { h.f[40] = (float)m.f3[0]; h.f[41] = (float)m.f3[1]; h.f[42] = (float)m.f3[2]; }
    else {
        h.f[40] = (float)m.m6[0]; h.f[41] = (float)m.m6[1]; h.f[42] = (float)m.m6[2];
        h.f[43] = (float)m.m6[3]; h.f[44] = (float)m.m6[4]; h.f[45] = (float)m.m6[5];
    }
    h.f[46] = (float)p.clon; h.f[47] = (float)p.clat; h.f[48] = (float)p.phi;
    h.f[50] = (float)std::sqrt((m.sx0 - st.x) * (m.sx0 - st.x) + (m.sy0 - st.y) * (m.sy0 - st.y));
    h.f[51] = (float)(std::atan2(st.y - m.sy0, st.x - m.sx0) * 180 / PI);
    h.f[52] = (float)(std::atan2(m.sy0 - st.y, m.sx0 - st.x) * 180 / PI);
    h.f[57] = (float)cmpaz; h.f[58] = (float)cmpinc;
    h.set_time(m.exedate);
    h.i[16] = idep;
    h.kset(111, 8, st.name);
    h.kset(113, 16, p.title.substr(0, 16));
    h.kset(151, 8, cmp);
    return h.bytes(dat, npts);
}

void write_file(const std::string& fn, const std::string& bytes) {
    std::ofstream f(fn, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error("cannot write " + fn);
    f.write(bytes.data(), (std::streamsize)bytes.size());
    if (!f) throw std::runtime_error("short write to " + fn);
}

// One ustar entry as the reference's tar writer lays it out
// (src/shared/m_tar.f90 tar__whdr, tar__wpad; src/shared/m_sac.f90 tarwrite_s):
// numeric fields as 8 or 12 octal digits without terminator, mode 0644,
// uid/gid 0, owner root, magic "ustar" with an empty version field, and the
// data padded with 512 - (size mod 512) zero bytes (a whole block when the
// size is a multiple of 512).
std::string tar_entry(const std::string& name, const std::string& data, long long mtime) {
    char h[512];
    std::memset(h, 0, sizeof h);
    std::memcpy(h, name.data(), std::min<size_t>(name.size(), 99));
    auto oct = [&](int off, int width, long long v) {
        char buf[32];
        std::snprintf(buf, sizeof buf, "%0*llo", width, v);
        std::memcpy(h + off, buf + std::max(0, (int)std::strlen(buf) - width), width);
    };
    oct(100, 8, 420);
    oct(108, 8, 0);
    oct(116, 8, 0);
    oct(124, 12, (long long)data.size());
    oct(136, 12, mtime);
    std::memset(h + 148, ' ', 8);
    h[156] = '0';
    std::memcpy(h + 257, "ustar", 5);
    std::memcpy(h + 265, "root", 4);
    std::memcpy(h + 297, "root", 4);
    long long sum = 0;
    for (unsigned char c : h) sum += c;
    oct(148, 8, sum);
    std::string out(h, sizeof h);
    out += data;
    out.append(512 - data.size() % 512, '\0');
    return out;
}


// report__setup's banner numbers in the reference's single precision
// (src/swpc_3d/m_report.f90:71-73): the memory estimate of memory_size_3d
// (src/shared/m_fdtool.f90:137-187), the stability number c of
// fdm_cond_stability (:81-113) and the wavelength number r of
// fdm_cond_wavelength (:116-134), from the velocity range of the processed
// medium below the free surface (velocity_minmax, m_medium.f90:396-427)
// and fmax = 2 fcut (m_source.f90:184-188).  vel(f, k, i, j) reads the
// processed rho (0), lam (1) or mu (2).
template <class MedV>
void banner_numbers(const Params& p, const Grid& G, const std::vector<int>& kfs, MedV vel, bool colmode, double fcut,
                    int nproc_x, int nproc_y, Meta::Banner& b) {
    b.nproc_x = nproc_x;
    b.nproc_y = nproc_y;
    float vmax = -1.f, vmin = 1e30f;
    const float eps = 1.1920928955078125e-07f;
    const int ie = colmode ? 1 : p.nx, je = colmode ? 1 : p.ny;  // one column stands for every column
    for (int j = 1; j <= je; ++j)
        for (int i = 1; i <= ie; ++i)
            for (int k = kfs[G.idx2(i, j)] + 1; k <= p.nz; ++k) {
                const float r = vel(0, k, i, j), l = vel(1, k, i, j), m = vel(2, k, i, j);
                const float vp = std::sqrt((l + 2 * m) / r), vs = std::sqrt(m / r);
                vmax = std::max(vmax, vp);
                if (vs < eps) continue;
                vmin = std::min(vmin, vs);
            }
    b.vmin = vmin;
    b.vmax = vmax;
    b.fmax = (float)(2 * fcut);
    const float dx = (float)p.dx, dy = (float)p.dy, dz = (float)p.dz;
    const float hh = 1.f / std::sqrt(1 / (dx * dx) + 1 / (dy * dy) + 1 / (dz * dz));
    const float dt2 = 6.f / 7.f * hh / vmax;
    b.c = (float)p.dt / dt2;
    b.r = vmin / b.fmax / std::max(dx, std::max(dy, dz));
    // memory_size_3d: 5 medium words (SP), 3 + 6 state words (DP) over the
    // padded grid of every rank, 6 nm memory variables (SP) over the interior
    // and 18 absorber words (SP) over the shell, as the reference counts them
    const int nxp = (int)std::ceil(p.nx / (float)nproc_x), nyp = (int)std::ceil(p.ny / (float)nproc_y);
    const float rn_com = (float)((nxp + 6) * nproc_x) * (float)((nyp + 6) * nproc_y) * (float)(p.nz + 6);
    const float rn_int = (float)(p.nx - 2 * p.na) * (float)(p.ny - 2 * p.na) * (float)(p.nz - p.na);
    const float rn_abc = (float)p.nx * (float)p.ny * (float)p.nz -
                         (float)(p.nx - 2 * nxp) * (float)(p.ny - 2 * nyp) * (float)(p.nz - p.na);
    const float ba = (5 * 4 + 3 * 8 + 6 * 8) * rn_com + (6 * 3 * 4) * rn_int + (18 * 4) * rn_abc;
    b.mem_all = ba / (1024.f * 1024.f * 1024.f);
    b.mem_node = b.mem_all / (float)(nproc_x * nproc_y);
}

// The banner as report__setup writes it (m_report.f90:64-88).
std::string banner_text(const Meta& m) {
    const Meta::Banner& b = m.banner;
    const Params& p = m.p;
    char buf[1600];
    const char* rule = " ------------------------------------------------------------------------------";
    std::snprintf(buf, sizeof buf,
                  "\n%s\n  SWPC_3D GB300 (openswpc_gb300)\n%s\n\n"
                  "  Grid Size               : %8d x %6d x %6d\n"
                  "  MPI Partitioning        : %8d x %4d\n"
                  "  Total Memory Size       : %15.3f  [GiB]\n"
                  "  Node Memory Size        : %15.3f  [GiB]\n"
                  "  Stability  Condition c  : %15.3f  (c<1)\n"
                  "  Wavelength Condition r  : %15.3f  (r>5-10)\n"
                  "  Minimum velocity        : %15.3f  [km/s]\n"
                  "  Maximum velocity        : %15.3f  [km/s]\n"
                  "  Maximum frequency       : %15.3f  [Hz]\n\n%s\n\n",
                  rule, rule, p.nx, p.ny, p.nz, b.nproc_x, b.nproc_y, b.mem_all, b.mem_node, b.c, b.r, b.vmin, b.vmax,
                  b.fmax, rule);
    return buf;
}

// Everything the host set-up derives from one input.inf, held until the
// simulation is put on a device: the medium, the source and receiver grid
// indices and the device dimensions.
struct Prepared {
    Meta meta;
    swpc_dims d{};
    std::vector<float> rho, lam, mu, tp, tsv;   // full halo arrays, or empty in column mode
    bool colmode = false;
    std::vector<float> col[5];                  // column mode: one processed column per field
    std::vector<int> kfs, kob, kft, kfb, kot, kobb;
    double ts[3] = {0, 0, 0};
    std::vector<int> sijk, rijk;
    std::vector<double> smo, smij, sf3, sprm;
    int stf = 0, bf_mode = 0, flags = 0, ntdec_w = 1, ntdec_s = 10;
    std::vector<int> gijk;  // Green's-function points, 1-based
    std::vector<std::vector<float>> pw_fields;  // plane-wave initial fields (halo arrays), Vx .. Sxy
    bool green_bforce = false;
};

// Host half of the set-up (src/swpc_3d/main.f90:48-117 without the device):
// parse, build the medium, locate sources and stations.  With `dry` set,
// only a JSON summary is produced.
int load(const char* inf_path, Prepared& P, std::string* dry = nullptr) {
    Inf inf(inf_path);
    inf.strict = inf.b("strict_mode", false);
    Params p;
    if (inf.b("benchmark_mode", false)) throw std::runtime_error("benchmark_mode is not supported by openswpc_gb300");
    p.title = inf.s("title", "swpc3d"); p.odir = inf.s("odir", "./out");
    p.nx = inf.i("nx", 256); p.ny = inf.i("ny", 256); p.nz = inf.i("nz", 256); p.nt = inf.i("nt", 1000);
    p.dx = inf.r("dx", 0.5); p.dy = inf.r("dy", 0.5); p.dz = inf.r("dz", 0.5); p.dt = inf.r("dt", 0.01);
    p.na = inf.i("na", 20);
    p.xbeg = inf.r("xbeg", -p.nx / 2 * p.dx); p.ybeg = inf.r("ybeg", -p.ny / 2 * p.dy); p.zbeg = inf.r("zbeg", -30 * p.dz);
    p.tbeg = inf.r("tbeg", 0.0);
    p.clon = inf.r("clon", 139.7604); p.clat = inf.r("clat", 35.7182); p.phi = inf.r("phi", 0.0);
    p.abc_type = inf.s("abc_type", "pml");
    if (p.abc_type != "pml" && p.abc_type != "cerjan") throw std::runtime_error("abc_type must be 'pml' or 'cerjan'");
    p.fq_min = inf.r("fq_min", 0.05); p.fq_max = inf.r("fq_max", 5.0); p.fq_ref = inf.r("fq_ref", 1.0);
    p.vmodel_type = inf.s("vmodel_type", "uni"); p.vcut = inf.r("vcut", 0.0);
    p.munk = inf.b("munk_profile", false);
    p.bf_mode = inf.b("bf_mode", false);
    p.pw_mode = inf.b("pw_mode", false);
    if (p.pw_mode) {
        if (inf.b("green_mode", false)) throw std::runtime_error("pw_mode and green_mode exclude each other");
        p.pw_ztop = inf.r("pw_ztop", 1e30); p.pw_zlen = inf.r("pw_zlen", -1.0);
        p.pw_ps = inf.s("pw_ps", "");
        p.pw_strike = inf.r("pw_strike", 0.0); p.pw_dip = inf.r("pw_dip", 0.0); p.pw_rake = inf.r("pw_rake", 0.0);
        if (!(p.pw_zlen > 0)) throw std::runtime_error("pw_zlen must be positive");
        if (p.pw_ps != "p" && p.pw_ps != "P" && p.pw_ps != "s" && p.pw_ps != "S") throw std::runtime_error("pw_ps must be p or s");
        if (inf.s("abc_type", "pml") != "pml") throw std::runtime_error("pw_mode needs abc_type = pml");
    }
    p.green_mode = inf.b("green_mode", false);
    if (p.green_mode) {
        p.green_stnm = inf.s("green_stnm", ""); p.green_cmp = inf.s("green_cmp", "");
        p.green_trise = inf.r("green_trise", 1.0); p.green_bforce = inf.b("green_bforce", false);
        p.green_maxdist = inf.r("green_maxdist", 1e30); p.fn_glst = inf.s("fn_glst", "");
        p.green_fmt = inf.s("green_fmt", "xyz");
        if (!(p.green_maxdist > 0)) throw std::runtime_error("green_maxdist must be positive");
        if (p.green_fmt != "xyz" && p.green_fmt != "llz") throw std::runtime_error("green_fmt must be xyz or llz");
        if (p.green_cmp != "x" && p.green_cmp != "y" && p.green_cmp != "z") throw std::runtime_error("no matching green_cmp");
        // m_wav.f90:76-82: no station recording in this mode
        p.sw_v = p.sw_u = p.sw_stress = p.sw_strain = false;
    }

    p.stftype = inf.s("stftype", "kupper"); p.stf_format = inf.s("stf_format", "xym0ij");
    p.fn_stf = inf.s("fn_stf", ""); p.sdep_fit = inf.s("sdep_fit", "asis");
    p.ntdec_w = inf.i("ntdec_w", 10); p.st_format = inf.s("st_format", "xy"); p.fn_stloc = inf.s("fn_stloc", "");
    p.wav_format = inf.s("wav_format", "sac");
    p.sw_v = inf.b("sw_wav_v", false); p.sw_u = inf.b("sw_wav_u", false);
    p.sw_stress = inf.b("sw_wav_stress", false); p.sw_strain = inf.b("sw_wav_strain", false);
    p.ntdec_r = inf.i("ntdec_r", 10);  // m_report.f90:47
    // snapshot switches and planes (m_snap.f90:105-127)
    {
        const char* secs[5] = {"xy", "yz", "xz", "fs", "ob"};
        const char* kinds[3] = {"v", "u", "ps"};
        for (int q = 0; q < 5; ++q) {
            p.snap_sw[q] = 0;
            for (int c = 0; c < 3; ++c)
                if (inf.b(std::string(secs[q]) + "_" + kinds[c] + "%sw", false)) p.snap_sw[q] |= 1 << c;
        }
    }
    double zend = p.zbeg + p.nz * p.dz, xend = p.xbeg + p.nx * p.dx, yend = p.ybeg + p.ny * p.dy;
    p.z0_xy = inf.r("z0_xy", std::max(std::min(10.0, zend), p.zbeg));
    p.x0_yz = inf.r("x0_yz", std::max(std::min(0.0, xend), p.xbeg));
    p.y0_xz = inf.r("y0_xz", std::max(std::min(0.0, yend), p.ybeg));
    p.idec = inf.i("idec", 1); p.jdec = inf.i("jdec", 1); p.kdec = inf.i("kdec", 1); p.ntdec_s = inf.i("ntdec_s", 10);
    if (p.idec < 1 || p.jdec < 1 || p.kdec < 1 || p.ntdec_s < 1)
        throw std::runtime_error("idec, jdec, kdec and ntdec_s must be positive");
    if (inf.s("snp_format", "native") != "native")
        std::fprintf(stderr, "swpc: snp_format other than native is written as native by openswpc_gb300\n");
    if (p.nt < 1) throw std::runtime_error("nt must be positive");

    Grid G{p.nx, p.ny, p.nz};
    std::vector<float> rho, lam, mu, tp, tsv;
    double bd0 = 0;
    std::vector<int> kfs(G.n2()), kob(G.n2()), kft(G.n2()), kfb(G.n2()), kot(G.n2()), kobb(G.n2());
    double ts[3];
    // Depth-only models (uni, lhm, lgm) give the same processed column at
    // every (i, j): the medium set-up runs on a small grid of the same depth,
    // one column of it goes to the device, which spreads it over the grid
    // (swpc_gpu_upload_medium_column).  Models that vary laterally, the
    // absorber conditioning and the plane-wave set-up keep full host arrays.
    const bool stabilize = inf.b("stabilize_pml", false);
    const bool colmode = (p.vmodel_type == "uni" || p.vmodel_type == "lhm" || p.vmodel_type == "lgm") && !stabilize &&
                         !p.pw_mode;
    std::vector<float> col[5];  // processed column k = -2 .. nz+3: rho lam mu taup taus
    if (colmode) {
        const int nr = 2 * p.na + 6, ic = p.na + 3;
        Params pr = p;
        pr.nx = pr.ny = nr;
        Grid Gr{nr, nr, p.nz};
        std::vector<float> r5[5];
        vmodel(inf, pr, Gr, r5[0], r5[1], r5[2], r5[3], r5[4], bd0);
        std::vector<int> m6[6];
        for (auto& m : m6) m.assign(Gr.n2(), 0);
        medium_post(nr, nr, p.nz, p.na, p.fq_min, p.fq_max, p.fq_ref, r5[0].data(), r5[1].data(), r5[2].data(),
                    r5[3].data(), r5[4].data(), m6[0].data(), m6[1].data(), m6[2].data(), m6[3].data(), m6[4].data(),
                    m6[5].data(), ts);
        for (int f = 0; f < 5; ++f) {
            col[f].resize(p.nz + 6);
            for (int k = -2; k <= p.nz + 3; ++k) col[f][k + 2] = r5[f][Gr.idx(k, ic, ic)];
        }
        // the maps as the surface detection fills them over the full grid
        const int v_fs = m6[0][Gr.idx2(ic, ic)], v_ob = m6[1][Gr.idx2(ic, ic)];
        for (int j = 0; j <= p.ny + 2; ++j)
            for (int i = 0; i <= p.nx + 2; ++i) { kfs[G.idx2(i, j)] = v_fs; kob[G.idx2(i, j)] = v_ob; }
        for (int j = 1; j <= p.ny; ++j)
            for (int i = 1; i <= p.nx; ++i) {
                const size_t q = G.idx2(i, j), r = Gr.idx2(ic, ic);
                kft[q] = m6[2][r]; kfb[q] = std::min(m6[3][r], p.nz); kot[q] = m6[4][r]; kobb[q] = std::min(m6[5][r], p.nz);
            }
    } else {
        vmodel(inf, p, G, rho, lam, mu, tp, tsv, bd0);
        medium_post(p.nx, p.ny, p.nz, p.na, p.fq_min, p.fq_max, p.fq_ref, rho.data(), lam.data(),
                    mu.data(), tp.data(), tsv.data(), kfs.data(), kob.data(), kft.data(), kfb.data(), kot.data(), kobb.data(), ts);
        if (stabilize)  // m_medium.f90:218-222, after surface detection
            stabilize_absorber(p.nx, p.ny, p.nz, p.na, rho.data(), lam.data(), mu.data(), tp.data(), tsv.data(), kfs.data());
    }
    // medium value f (0 rho, 1 lam, 2 mu) at cell (k, i, j) in either form
    auto medv = [&](int f, int k, int i, int j) -> float {
        if (colmode) return col[f][k + 2];
        const std::vector<float>& a = f == 0 ? rho : f == 1 ? lam : mu;
        return a[G.idx(k, i, j)];
    };

    // sources (src/swpc_3d/m_source.f90:41-314, 468-774)
    Meta meta;
    meta.p = p;
    meta.exedate = (long long)std::time(nullptr);
    // m_source.f90:84-91: no regular source grid in Green's-function mode
    auto rows = (p.green_mode || p.pw_mode) ? std::vector<std::string>() : table_rows(inf.path(p.fn_stf));
    const std::string& f = p.stf_format;
    struct S0 { double x, y, z, t0, tr, mo, m6[6], f3[3]; };
    std::vector<S0> srcs;
    for (size_t r = 0; r < rows.size(); ++r) {
        auto t = split(rows[r]);
        auto R = [&](size_t q) { if (q >= t.size()) throw std::runtime_error("short source line: " + rows[r]); return Inf::num(t[q]); };
        S0 s{};
        bool ll = f.size() >= 2 && f.compare(0, 2, "ll") == 0;
        if (f == "psmeca") {
            double lon = R(0), lat = R(1);
            s.z = R(2);
            double mzz = R(3), mxx = R(4), myy = R(5), mxz = R(6), myz = -R(7), mxy = -R(8);
            int iex = (int)R(9);
            g2c(lon, lat, p.clon, p.clat, p.phi, s.x, s.y);
            double m0 = std::sqrt(mxx * mxx + myy * myy + mzz * mzz + 2 * (mxz * mxz + myz * myz + mxy * mxy)) / std::sqrt(2.0);
            s.mo = m0 * std::pow(10.0, iex);
            s.t0 = 0; s.tr = 2 * 1.05e-8 * std::pow(s.mo, 1.0 / 3.0);
            s.mo *= 1e-7;
            double m6[6] = {mxx, myy, mzz, myz, mxz, mxy};
            for (int c = 0; c < 6; ++c) s.m6[c] = m6[c] / m0;
        } else {
            if (ll) { g2c(R(0), R(1), p.clon, p.clat, p.phi, s.x, s.y); }
            else { s.x = R(0); s.y = R(1); }
            s.z = R(2); s.t0 = R(3); s.tr = R(4);
            if (p.bf_mode) {
                if (!(f.compare(0, 2, "xy") == 0 || ll)) throw std::runtime_error("unknown body-force stf_format " + f);
                s.f3[0] = R(5); s.f3[1] = R(6); s.f3[2] = R(7);
            } else if (f == "xym0ij" || f == "llm0ij" || f == "xymwij" || f == "llmwij") {
                s.mo = R(5);
                if (f[2] == 'm' && f[3] == 'w') s.mo = std::pow(10.0, 1.5 * s.mo + 9.05);
                for (int c = 0; c < 6; ++c) s.m6[c] = R(6 + c);
            } else if (f == "xym0dc" || f == "llm0dc" || f == "xymwdc" || f == "llmwdc") {
                s.mo = R(5);
                if (f[2] == 'm' && f[3] == 'w') s.mo = std::pow(10.0, 1.5 * s.mo + 9.05);
                sdr2moment(R(6) - p.phi, R(7), R(8), s.m6);
            } else if (f == "xydsdc" || f == "lldsdc") {
                double D = R(5), Sa = R(6);
                sdr2moment(R(7) - p.phi, R(8), R(9), s.m6);
                int is = x2i(s.x, p.xbeg, p.dx), js = x2i(s.y, p.ybeg, p.dy), ks = x2i(s.z, p.zbeg, p.dz);
                s.mo = (is >= -2 && is <= p.nx + 3 && js >= -2 && js <= p.ny + 3 && ks >= -2 && ks <= p.nz + 3)
                           ? 1e9 * medv(2, ks, is, js) * D * Sa : 0.0;
            } else {
                throw std::runtime_error("invalid source type " + f);
            }
        }
        if (srcs.empty()) {
            c2g(s.x, s.y, p.clon, p.clat, p.phi, meta.evlo, meta.evla);
            meta.sx0 = s.x; meta.sy0 = s.y; meta.evdp = s.z; meta.otim = s.t0;
            for (int c = 0; c < 6; ++c) meta.m6[c] = s.m6[c];
            for (int c = 0; c < 3; ++c) meta.f3[c] = s.f3[c];
        }
        srcs.push_back(s);
    }
    if (srcs.empty() && !p.green_mode && !p.pw_mode) throw std::runtime_error("no source grid in " + p.fn_stf);
    double fcut = 0, M0 = 0;
    for (auto& s : srcs) fcut = std::max(fcut, 1.0 / s.tr);
    double UC = 1e-15;
    std::vector<std::vector<float>> pw_fields;
    if (p.green_mode) {
        M0 = 1;  // m_green.f90:127; fcut stays 0, source__setup never sets it
    } else if (p.pw_mode) {
        M0 = (double)(1.0f / (float)UC);  // fictitious moment for output, single precision (m_source.f90:77)
        fcut = plane_wave(p, G, rho, lam, mu, pw_fields);
    } else if (p.bf_mode) {
        for (auto& s : srcs) M0 += s.f3[0] * s.f3[0] + s.f3[1] * s.f3[1] + s.f3[2] * s.f3[2];
        M0 = std::sqrt(M0);
        UC *= 1e3;
    } else {
        for (auto& s : srcs) M0 += s.mo;
    }
    std::vector<int> sijk;
    std::vector<double> smo, smij, sf3, sprm;
    for (auto& s : srcs) {
        int is = x2i(s.x, p.xbeg, p.dx), js = x2i(s.y, p.ybeg, p.dy), ks = x2i(s.z, p.zbeg, p.dz);
        if (p.sdep_fit.size() == 3 && p.sdep_fit.compare(0, 2, "bd") == 0 && p.sdep_fit[2] == '0') ks = x2i(bd0, p.zbeg, p.dz);
        if (!(is >= -1 && is <= p.nx + 3 && js >= -1 && js <= p.ny + 3 && ks >= -1 && ks <= p.nz + 3)) continue;
        if (!(p.xbeg <= s.x && s.x <= xend && p.ybeg <= s.y && s.y <= yend && p.zbeg <= s.z && s.z <= zend))
            throw std::runtime_error("source outside the model space");
        sijk.insert(sijk.end(), {is, js, ks});
        smo.push_back(M0 > 0 ? s.mo / M0 : 0.0);
        smij.insert(smij.end(), s.m6, s.m6 + 6);
        for (int c = 0; c < 3; ++c) sf3.push_back(M0 > 0 ? s.f3[c] / M0 : 0.0);
        sprm.insert(sprm.end(), {s.t0, s.tr});
    }

    // stations (src/swpc_3d/m_wav.f90:141-271)
    int flags = (p.sw_v ? SWPC_WAV_V : 0) | (p.sw_u ? SWPC_WAV_U : 0) | (p.sw_stress ? SWPC_WAV_STRESS : 0) |
                (p.sw_strain ? SWPC_WAV_STRAIN : 0);
    std::vector<Station> all_st;
    if (flags || p.green_mode) {
        std::vector<std::string> srows;
        try { srows = table_rows(inf.path(p.fn_stloc)); }
        catch (...) { std::fprintf(stderr, "swpc: no station location file found\n"); }
        for (auto& r : srows) {
            auto t = split(r);
            if (t.size() < 5) throw std::runtime_error("bad station line: " + r);
            Station st;
            if (p.st_format == "xy") {
                st.x = Inf::num(t[0]); st.y = Inf::num(t[1]);
                c2g(st.x, st.y, p.clon, p.clat, p.phi, st.lon, st.lat);
            } else if (p.st_format == "ll") {
                st.lon = Inf::num(t[0]); st.lat = Inf::num(t[1]);
                g2c(st.lon, st.lat, p.clon, p.clat, p.phi, st.x, st.y);
            } else throw std::runtime_error("unknown st_format " + p.st_format);
            st.z = Inf::num(t[2]);
            st.name = t[3].substr(0, 8);
            std::string zsw = t[4].substr(0, 3);
            st.i = x2i(st.x, p.xbeg, p.dx); st.j = x2i(st.y, p.ybeg, p.dy); st.k = x2i(st.z, p.zbeg, p.dz);
            double x1 = p.xbeg + 0.5 * p.dx, xn = p.xbeg + (p.nx - 0.5) * p.dx;
            double y1 = p.ybeg + 0.5 * p.dy, yn = p.ybeg + (p.ny - 0.5) * p.dy;
            if (!(x1 < st.x && st.x < xn && y1 < st.y && st.y < yn && 1 < st.k && st.k < p.nz)) {
                std::fprintf(stderr, "swpc: station %s is out of the region\n", st.name.c_str());
                continue;
            }
            if (zsw == "fsb") st.k = kfs[G.idx2(st.i, st.j)] + 1;
            else if (zsw == "obb") st.k = kob[G.idx2(st.i, st.j)] + 1;
            else if (zsw == "oba") st.k = kob[G.idx2(st.i, st.j)] - 1;
            else if (zsw == "bd0") st.k = x2i(bd0, p.zbeg, p.dz);
            if (st.k > p.nz) st.k = p.nz - 1;
            if (st.k < 1) st.k = 2;
            all_st.push_back(st);
        }
    }
    if (flags) meta.st = all_st;

    // Green's-function mode: the pseudo source at station green_stnm and
    // the grid points of fn_glst (m_green.f90:145-404)
    std::vector<int> gijk;
    if (p.green_mode) {
        const Station* gs = nullptr;
        for (const auto& st : all_st)
            if (st.name == p.green_stnm.substr(0, 8)) gs = &st;
        if (!gs) throw std::runtime_error("green_stnm " + p.green_stnm + " is not a station inside the model");
        Meta::Green& g = meta.green;
        g.on = true;
        g.station = *gs;
        sijk.insert(sijk.end(), {gs->i, gs->j, gs->k});
        smo.push_back(0.0);
        smij.insert(smij.end(), 6, 0.0);
        sf3.push_back(p.green_cmp == "x" ? 1.0 : 0.0);
        sf3.push_back(p.green_cmp == "y" ? 1.0 : 0.0);
        sf3.push_back(p.green_cmp == "z" ? 1.0 : 0.0);
        sprm.insert(sprm.end(), {0.0, p.green_trise});
        for (auto& r : table_rows(inf.path(p.fn_glst))) {
            auto t = split(r);
            if (t.size() < 4) throw std::runtime_error("bad Green's-function point: " + r);
            Meta::GPoint q;
            if (p.green_fmt == "xyz") {
                q.x = Inf::num(t[0]); q.y = Inf::num(t[1]);
                c2g(q.x, q.y, p.clon, p.clat, p.phi, q.lon, q.lat);
            } else {
                q.lon = Inf::num(t[0]); q.lat = Inf::num(t[1]);
                g2c(q.lon, q.lat, p.clon, p.clat, p.phi, q.x, q.y);
            }
            q.z = Inf::num(t[2]);
            q.gid = (long long)Inf::num(t[3]);
            if (q.gid < 0 || q.gid > 99999999) throw std::runtime_error("Green's-function id outside 0..99999999");
            const double dd = std::sqrt((q.x - gs->x) * (q.x - gs->x) + (q.y - gs->y) * (q.y - gs->y));
            if (dd > p.green_maxdist) continue;
            q.i = x2i(q.x, p.xbeg, p.dx); q.j = x2i(q.y, p.ybeg, p.dy); q.k = x2i(q.z, p.zbeg, p.dz);
            if (!(1 <= q.i && q.i <= p.nx && 1 <= q.j && q.j <= p.ny)) continue;
            if (!(kob[G.idx2(q.i, q.j)] <= q.k && q.k <= p.nz)) continue;  // the solid part only
            g.pts.push_back(q);
            gijk.insert(gijk.end(), {q.i, q.j, q.k});
        }
    }

    banner_numbers(p, G, kfs, medv, colmode, fcut, std::max(1, inf.i("nproc_x", 1)), std::max(1, inf.i("nproc_y", 1)),
                   meta.banner);
    if (dry) {  // set-up summary only, no device
        char buf[1024];
        std::string src_s, st_s;
        for (size_t q = 0; q < smo.size(); ++q)
            src_s += (q ? ";" : "") + std::to_string(sijk[3 * q]) + "," + std::to_string(sijk[3 * q + 1]) + "," + std::to_string(sijk[3 * q + 2]);
        for (size_t q = 0; q < meta.st.size(); ++q)
            st_s += (q ? ";" : "") + std::to_string(meta.st[q].i) + "," + std::to_string(meta.st[q].j) + "," + std::to_string(meta.st[q].k);
        const Meta::Banner& bn = meta.banner;
        auto jn = [](double v) {  // JSON number, null when not finite (e.g. r without a source frequency)
            char t[40];
            if (std::isfinite(v)) std::snprintf(t, sizeof t, "%.9g", v);
            else std::snprintf(t, sizeof t, "null");
            return std::string(t);
        };
        const std::string bj = "\"banner\": {\"mem_total_gib\": " + jn(bn.mem_all) + ", \"mem_node_gib\": " + jn(bn.mem_node) +
                               ", \"c\": " + jn(bn.c) + ", \"r\": " + jn(bn.r) + ", \"vmin\": " + jn(bn.vmin) +
                               ", \"vmax\": " + jn(bn.vmax) + ", \"fmax\": " + jn(bn.fmax) + ", \"nproc\": [" +
                               std::to_string(bn.nproc_x) + ", " + std::to_string(bn.nproc_y) + "]}, ";
        std::snprintf(buf, sizeof buf, "{\"nx\": %d, \"ny\": %d, \"nz\": %d, \"nt\": %d, \"na\": %d, \"M0\": %.9g, \"UC\": %.9g, "
                      "\"fcut\": %.9g, \"nsrc\": %d, \"nst\": %d, \"ts\": [%.9g, %.9g, %.9g], ",
                      p.nx, p.ny, p.nz, p.nt, p.na, M0, UC, fcut, (int)smo.size(), (int)meta.st.size(), ts[0], ts[1], ts[2]);
        *dry = std::string(buf) + bj + "\"src\": \"" + src_s + "\", \"sta\": \"" + st_s + "\"}";
        return 0;
    }

    swpc_dims& d = P.d;
    d = swpc_dims{};
    d.nx = p.nx; d.ny = p.ny; d.nz = p.nz; d.nt = p.nt; d.na = p.na; d.nm = 3;
    d.abc_type = p.abc_type == "pml" ? SWPC_ABC_PML : p.abc_type == "cerjan" ? SWPC_ABC_CERJAN : -1;
    if (d.abc_type < 0) throw std::runtime_error("abc_type must be 'pml' or 'cerjan'");
    std::string store = inf.s("gpu_store", "fp32");
    d.store = store == "fp16" ? SWPC_STORE_FP16 : store == "bf16" ? SWPC_STORE_BF16 : SWPC_STORE_FP32;
    d.dx = p.dx; d.dy = p.dy; d.dz = p.dz; d.dt = p.dt;
    d.xbeg = p.xbeg; d.ybeg = p.ybeg; d.zbeg = p.zbeg; d.tbeg = p.tbeg;
    d.fcut = fcut; d.M0 = M0; d.UC = UC; d.ntdec_r = p.ntdec_r;
    meta.M0 = M0; meta.UC = UC;
    meta.flags = flags;

    P.rho = std::move(rho); P.lam = std::move(lam); P.mu = std::move(mu); P.tp = std::move(tp); P.tsv = std::move(tsv);
    P.colmode = colmode;
    for (int f = 0; f < 5; ++f) P.col[f] = std::move(col[f]);
    P.kfs = std::move(kfs); P.kob = std::move(kob); P.kft = std::move(kft); P.kfb = std::move(kfb);
    P.kot = std::move(kot); P.kobb = std::move(kobb);
    for (int m = 0; m < 3; ++m) P.ts[m] = ts[m];
    P.sijk = std::move(sijk); P.smo = std::move(smo); P.smij = std::move(smij); P.sf3 = std::move(sf3);
    P.sprm = std::move(sprm);
    P.stf = stf_code(p.stftype);
    P.bf_mode = p.bf_mode || p.green_mode;  // the Green's-function pseudo source is a body force
    P.gijk = std::move(gijk);
    P.pw_fields = std::move(pw_fields);
    P.green_bforce = p.green_bforce;
    P.rijk.clear();
    for (auto& st : meta.st) P.rijk.insert(P.rijk.end(), {st.i, st.j, st.k});
    P.flags = flags;
    P.ntdec_w = std::max(1, p.ntdec_w);
    P.ntdec_s = p.ntdec_s;
    meta.bd0 = bd0;
    // the medium now lives in P: read it there
    auto pmedv = [&](int f, int k, int i, int j) -> float {
        if (P.colmode) return P.col[f][k + 2];
        const std::vector<float>& a = f == 0 ? P.rho : f == 1 ? P.lam : P.mu;
        return a[G.idx(k, i, j)];
    };
    {  // snap__setup and newfile_* (m_snap.f90:131-160, 324-473)
        const int idec = p.idec, jdec = p.jdec, kdec = p.kdec;
        const int nxs = (p.nx + idec / 2) / idec, nys = (p.ny + jdec / 2) / jdec, nzs = (p.nz + kdec / 2) / kdec;
        // section coordinates in single precision as i2x/j2y/k2z compute them
        // (m_fdtool.f90:639-680)
        auto c2f = [](int i, double b, double d) { const float t = ((float)i - 0.5f) * (float)d; return (float)b + t; };
        const int k0 = x2i(p.z0_xy, p.zbeg, p.dz), i0 = x2i(p.x0_yz, p.xbeg, p.dx), j0 = x2i(p.y0_xz, p.ybeg, p.dy);
        for (int sec = 0; sec < 5; ++sec) {
            if (!p.snap_sw[sec]) continue;
            Meta::SnapSec S;
            S.sec = sec;
            S.kinds = p.snap_sw[sec];
            const bool horiz = sec == SWPC_SEC_XY || sec == SWPC_SEC_FS || sec == SWPC_SEC_OB;
            int dd1 = idec, dd2 = jdec;
            double b1 = p.xbeg, b2 = p.ybeg, h1 = p.dx, h2 = p.dy;
            if (sec == SWPC_SEC_YZ) { dd1 = jdec; dd2 = kdec; b1 = p.ybeg; b2 = p.zbeg; h1 = p.dy; h2 = p.dz; }
            if (sec == SWPC_SEC_XZ) { dd1 = idec; dd2 = kdec; b2 = p.zbeg; h2 = p.dz; }
            S.d1 = dd1; S.d2 = dd2;
            S.n1 = sec == SWPC_SEC_YZ ? nys : nxs;
            S.n2 = horiz ? nys : nzs;
            S.na1 = p.na / dd1; S.na2 = p.na / dd2;
            S.fix = sec == SWPC_SEC_XY ? k0 : sec == SWPC_SEC_YZ ? i0 : sec == SWPC_SEC_XZ ? j0 : 1;
            if (!horiz || sec == SWPC_SEC_XY) {
                const int lim = sec == SWPC_SEC_XY ? p.nz : sec == SWPC_SEC_YZ ? p.nx : p.ny;
                if (S.fix < 1 || S.fix > lim) throw std::runtime_error("snapshot section outside the model");
            }
            S.x1 = c2f(dd1 - dd1 / 2, b1, h1);
            S.x2 = c2f(dd2 - dd2 / 2, b2, h2);
            S.dx1 = c2f(2 * dd1 - dd1 / 2, b1, h1) - S.x1;
            S.dx2 = c2f(2 * dd2 - dd2 / 2, b2, h2) - S.x2;
            const size_t pl = (size_t)S.n1 * S.n2;
            S.med.assign(3 * pl, 0.f);
            for (int b = 1; b <= S.n2; ++b)
                for (int a = 1; a <= S.n1; ++a) {
                    const int ca = a * dd1 - dd1 / 2, cb = b * dd2 - dd2 / 2;
                    int i, j, k;
                    if (sec == SWPC_SEC_YZ) { i = S.fix; j = ca; k = cb; }
                    else if (sec == SWPC_SEC_XZ) { i = ca; j = S.fix; k = cb; }
                    else {
                        i = ca; j = cb;
                        k = sec == SWPC_SEC_XY ? S.fix : (sec == SWPC_SEC_FS ? P.kfs : P.kob)[G.idx2(i, j)] + 1;
                    }
                    const size_t q = (size_t)(b - 1) * S.n1 + (a - 1);
                    S.med[q] = pmedv(0, k, i, j);
                    S.med[pl + q] = pmedv(1, k, i, j);
                    S.med[2 * pl + q] = pmedv(2, k, i, j);
                }
            meta.snaps.push_back(std::move(S));
        }
    }
    P.meta = std::move(meta);
    return 0;
}

// Device half of the set-up: create the simulation, upload the medium,
// sources, receivers and snapshot plan.
int materialize(const Prepared& P, swpc_sim** out) {
    swpc_sim* sim = nullptr;
    int rc = swpc_gpu_create(&P.d, &sim);
    if (rc) return rc;
    auto bail = [&](int code) { swpc_gpu_destroy(sim); return code; };
    if (P.colmode)
        rc = swpc_gpu_upload_medium_column(sim, P.col[0].data(), P.col[1].data(), P.col[2].data(), P.col[3].data(),
                                           P.col[4].data(), P.kfs.data(), P.kob.data(), P.kft.data(), P.kfb.data(),
                                           P.kot.data(), P.kobb.data(), P.ts);
    else
        rc = swpc_gpu_upload_medium(sim, P.rho.data(), P.lam.data(), P.mu.data(), P.tp.data(), P.tsv.data(),
                                    P.kfs.data(), P.kob.data(), P.kft.data(), P.kfb.data(), P.kot.data(),
                                    P.kobb.data(), P.ts);
    if (rc) return bail(rc);
    if ((rc = swpc_gpu_set_sources(sim, (int)P.smo.size(), P.sijk.data(), P.smo.data(), P.smij.data(), P.sf3.data(),
                                   P.sprm.data(), P.stf, P.bf_mode)))
        return bail(rc);
    if ((rc = swpc_gpu_set_receivers(sim, (int)P.meta.st.size(), P.rijk.data(), P.ntdec_w, P.flags)))
        return bail(rc);
    for (int w = 0; w < (int)P.pw_fields.size(); ++w)
        if ((rc = swpc_gpu_set_field(sim, w, P.pw_fields[w].data()))) return bail(rc);
    if (!P.pw_fields.empty() && (rc = swpc_gpu_set_plane_wave(sim, 1))) return bail(rc);
    if (!P.gijk.empty() &&
        (rc = swpc_gpu_set_green(sim, (int)P.gijk.size() / 3, P.gijk.data(), P.ntdec_w, P.green_bforce ? 1 : 0)))
        return bail(rc);
    for (const auto& S : P.meta.snaps)
        for (int kind = 0; kind < 3; ++kind)
            if ((S.kinds >> kind & 1) && (rc = swpc_gpu_add_snapshot(sim, S.sec, kind, S.fix, S.d1, S.d2, P.ntdec_s)))
                return bail(rc);
    Meta meta = P.meta;
    swpc_gpu_query(sim, &meta.ntw, nullptr, nullptr, nullptr, nullptr);
    {
        std::lock_guard<std::mutex> lk(g_meta_mu);
        g_meta[sim] = std::move(meta);
    }
    *out = sim;
    return 0;
}

int prepare(const char* inf_path, swpc_sim** out, std::string* dry = nullptr) {
    Prepared P;
    int rc = load(inf_path, P, dry);
    if (rc || dry) return rc;
    return materialize(P, out);
}

}  // namespace

extern "C" {

int swpc_host_medium(int nx, int ny, int nz, int na, double fq_min, double fq_max, double fq_ref, float* rho, float* lam,
                     float* mu, float* qp_taup, float* qs_taus, int* kfs, int* kob, int* kfs_top, int* kfs_bot,
                     int* kob_top, int* kob_bot, double* ts) {
    if (!rho || !lam || !mu || !qp_taup || !qs_taus || !kfs || !kob || !kfs_top || !kfs_bot || !kob_top || !kob_bot || !ts)
        return swpc::set_err(SWPC_E_ARG, "null argument to swpc_host_medium");
    if (nx <= 2 * na || ny <= 2 * na || nz <= na || na < 0) return swpc::set_err(SWPC_E_ARG, "bad grid / absorber size");
    medium_post(nx, ny, nz, na, fq_min, fq_max, fq_ref, rho, lam, mu, qp_taup, qs_taus, kfs, kob, kfs_top, kfs_bot,
                kob_top, kob_bot, ts);
    return 0;
}

int swpc_host_prepare(const char* inf_path, swpc_sim** out) {
    if (!inf_path || !out) return swpc::set_err(SWPC_E_ARG, "null argument");
    *out = nullptr;
    try {
        return prepare(inf_path, out);
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

struct swpc_request {
    Prepared P;
};

int swpc_host_load(const char* inf_path, swpc_request** out) {
    if (!inf_path || !out) return swpc::set_err(SWPC_E_ARG, "null argument");
    *out = nullptr;
    try {
        auto* r = new swpc_request();
        int rc = load(inf_path, r->P);
        if (rc) { delete r; return rc; }
        *out = r;
        return 0;
    } catch (const std::bad_alloc&) {
        return swpc::set_err(SWPC_E_NOMEM, "host memory exhausted while loading " + std::string(inf_path));
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

long long swpc_host_request_bytes(const swpc_request* req) {
    if (!req) return swpc::set_err(SWPC_E_ARG, "null request");
    return (long long)swpc_gpu_required_bytes(&req->P.d);
}

int swpc_host_request_dims(const swpc_request* req, swpc_dims* out) {
    if (!req || !out) return swpc::set_err(SWPC_E_ARG, "null argument");
    *out = req->P.d;
    return 0;
}

int swpc_host_materialize(const swpc_request* req, swpc_sim** out) {
    if (!req || !out) return swpc::set_err(SWPC_E_ARG, "null argument");
    *out = nullptr;
    try {
        return materialize(req->P, out);
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

int swpc_host_request_free(swpc_request* req) {
    delete req;
    return 0;
}

int swpc_host_check(const char* inf_path, char* summary, size_t n) {
    if (!inf_path) return swpc::set_err(SWPC_E_ARG, "null argument");
    try {
        std::string s;
        int rc = prepare(inf_path, nullptr, &s);
        if (summary && n) {
            size_t m = std::min(n - 1, s.size());
            std::memcpy(summary, s.data(), m);
            summary[m] = 0;
        }
        return rc ? rc : (int)s.size();
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

int swpc_host_banner(swpc_sim* sim, char* buf, size_t n) {
    std::string t;
    {
        std::lock_guard<std::mutex> lk(g_meta_mu);
        auto it = g_meta.find(sim);
        if (it == g_meta.end()) return swpc::set_err(SWPC_E_STATE, "simulation was not made by swpc_host_prepare");
        t = banner_text(it->second);
    }
    if (buf && n) {
        size_t m = std::min(n - 1, t.size());
        std::memcpy(buf, t.data(), m);
        buf[m] = 0;
    }
    return (int)t.size();
}

int swpc_host_ntdec_r(swpc_sim* sim) {
    std::lock_guard<std::mutex> lk(g_meta_mu);
    auto it = g_meta.find(sim);
    return it == g_meta.end() ? 0 : it->second.p.ntdec_r;
}

int swpc_host_nt(swpc_sim* sim) {
    std::lock_guard<std::mutex> lk(g_meta_mu);
    auto it = g_meta.find(sim);
    return it == g_meta.end() ? 0 : it->second.p.nt;
}

int swpc_host_write_snp(swpc_sim* sim, const char* odir) {
    Meta m;
    {
        std::lock_guard<std::mutex> lk(g_meta_mu);
        auto it = g_meta.find(sim);
        if (it == g_meta.end()) return swpc::set_err(SWPC_E_STATE, "simulation was not prepared by swpc_host_prepare");
        m = it->second;
    }
    if (m.snaps.empty()) return 0;
    try {
        const Params& p = m.p;
        std::string dir = (odir && *odir) ? std::string(odir) : p.odir;
        mkdirs(dir);
        const char* secname[5] = {"xy", "yz", "xz", "fs", "ob"};
        const char* kindname[3] = {"v", "u", "ps"};
        const char* typname[3] = {"v3", "u3", "ps"};
        for (const auto& S : m.snaps) {
            const bool horiz = S.sec == SWPC_SEC_XY || S.sec == SWPC_SEC_FS || S.sec == SWPC_SEC_OB;
            const size_t pl = (size_t)S.n1 * S.n2;
            for (int kind = 0; kind < 3; ++kind) {
                if (!(S.kinds >> kind & 1)) continue;
                int n1 = 0, n2 = 0, nframes = 0;
                int rc = swpc_gpu_query_snapshot(sim, S.sec, kind, &n1, &n2, &nframes);
                if (rc) return rc;
                if (n1 != S.n1 || n2 != S.n2) return swpc::set_err(SWPC_E_STATE, "snapshot geometry differs from the set-up");
                const int nc = kind == SWPC_SNAPK_PS ? 4 : 3;
                const std::string fn = dir + "/" + p.title + ".3d." + secname[S.sec] + "." + kindname[kind] + ".snp";
                std::ofstream f(fn, std::ios::binary | std::ios::trunc);
                if (!f) throw std::runtime_error("cannot write " + fn);
                auto wi = [&](int32_t x) { f.write((const char*)&x, 4); };
                auto wf = [&](float x) { f.write((const char*)&x, 4); };
                auto ws = [&](const std::string& t, size_t n) {
                    std::string u = t.substr(0, n);
                    u.resize(n, ' ');
                    f.write(u.data(), (std::streamsize)n);
                };
                // write_snp_header (m_snap.f90:846-892), header version 6
                ws("STREAMIO", 8); ws("SWPC_3D ", 8); wi(6); ws(p.title, 80); wi((int32_t)m.exedate);
                ws(secname[S.sec], 2); ws(typname[kind], 2); wi(S.n1); wi(S.n2);
                wf(S.x1); wf(S.x2); wf(S.dx1); wf(S.dx2);
                wf((float)p.dt * (float)p.ntdec_s);
                wi(S.na1); wi(S.na2);
                wi(horiz ? 6 : 3); wi(nc);  // nmed, nsnp (m_snap.f90:200-207)
                wf((float)p.clon); wf((float)p.clat); wf((float)p.phi);
                wf(1.f); wf(1.f); wf(1.f);
                // medium planes rho, lam, mu, and the topography of the
                // horizontal sections (newfile_yz/xz/xy)
                f.write((const char*)S.med.data(), (std::streamsize)(S.med.size() * 4));
                if (horiz) {
                    std::vector<float> tp(pl, -(float)m.bd0 * 1000.f);
                    f.write((const char*)tp.data(), (std::streamsize)(pl * 4));
                }
                // nc planes of (n1, n2) per frame (wbuf_*)
                std::vector<float> frame(pl * nc);
                for (int q = 0; q < nframes; ++q) {
                    if ((rc = swpc_gpu_fetch_section(sim, S.sec, kind, q, frame.data()))) return rc;
                    f.write((const char*)frame.data(), (std::streamsize)(frame.size() * 4));
                }
                if (!f) throw std::runtime_error("short write to " + fn);
            }
        }
        return 0;
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

int swpc_host_write_green(swpc_sim* sim, const char* odir) {
    Meta m;
    {
        std::lock_guard<std::mutex> lk(g_meta_mu);
        auto it = g_meta.find(sim);
        if (it == g_meta.end()) return swpc::set_err(SWPC_E_STATE, "simulation was not prepared by swpc_host_prepare");
        m = it->second;
    }
    if (!m.green.on || m.green.pts.empty()) return 0;
    try {
        const Params& p = m.p;
        const int ng = (int)m.green.pts.size();
        int ncmp = 0, ntw = 0;
        int rc = swpc_gpu_fetch_green(sim, nullptr, nullptr, &ncmp, &ntw);
        if (rc) return rc;
        std::vector<float> gf((size_t)ntw * ncmp * ng);
        if ((rc = swpc_gpu_fetch_green(sim, gf.data(), nullptr, nullptr, nullptr))) return rc;
        if (p.green_cmp == "z")  // m_green.f90:566-568: positive upward force
            for (auto& v : gf) v = -v;
        const Station& st = m.green.station;
        const std::string dir = ((odir && *odir) ? std::string(odir) : p.odir) + "/green/" + st.name;
        mkdirs(dir);
        const char* cmp[9] = {"mxx", "myy", "mzz", "myz", "mxz", "mxy", "fx_", "fy_", "fz_"};
        const std::string V = p.green_cmp == "x" ? "G_Vx_" : p.green_cmp == "y" ? "G_Vy_" : "G_Vz_";
        const float inc = p.green_cmp == "z" ? 0.f : 90.f;
        const float az = p.green_cmp == "x" ? (float)(0.0 + p.phi) : p.green_cmp == "y" ? (float)(90.0 + p.phi) : 0.f;
        // SAC images of every point and component (m_green.f90:318-398)
        auto image = [&](int n, int c) {
            const Meta::GPoint& q = m.green.pts[n];
            char cid8[16];
            std::snprintf(cid8, sizeof cid8, "%08lld", q.gid);
            SacHeader h;
            h.f[31] = (float)st.lat; h.f[32] = (float)st.lon; h.f[34] = (float)(st.z * 1000);  // stla stlo stdp
            h.kset(151, 8, V + cmp[c]);
            h.f[58] = inc; h.f[57] = az;
            h.kset(113, 16, cid8);
            h.kset(111, 8, st.name);
            h.f[36] = (float)q.lon; h.f[35] = (float)q.lat; h.f[38] = (float)q.z;  // evlo evla evdp
            h.set_time(m.exedate);
            h.i[16] = c < 6 ? 7 : 6;
            h.f[5] = (float)p.tbeg;
            h.set_delta(p.ntdec_w * p.dt);
            h.f[40] = (float)q.x; h.f[41] = (float)q.y; h.f[42] = (float)q.z;  // user0-2: location asked for
            const float xb = (float)p.xbeg, yb = (float)p.ybeg, zb = (float)p.zbeg;
            auto c2f = [](int i, float b, float d) { const float t = ((float)i - 0.5f) * d; return b + t; };
            h.f[43] = c2f(q.i, xb, (float)p.dx); h.f[44] = c2f(q.j, yb, (float)p.dy); h.f[45] = c2f(q.k, zb, (float)p.dz);
            h.f[46] = (float)p.clon; h.f[47] = (float)p.clat; h.f[48] = (float)p.phi;  // user6-8
            return h.bytes(&gf[((size_t)n * ncmp + c) * ntw], ntw);
        };
        if (p.wav_format == "csf") {  // m_green.f90:577-585
            std::string b = "CSFD";
            const int32_t ntr = ng * ncmp, np = ntw;
            b.append((const char*)&ntr, 4);
            b.append((const char*)&np, 4);
            for (int n = 0; n < ng; ++n)
                for (int c = 0; c < ncmp; ++c) b += image(n, c);
            write_file(dir + "/" + p.title + "__" + st.name + "__" + p.green_cmp + "__000000__.csf", b);
        } else if (p.wav_format == "sac") {  // m_green.f90:571-576, file names :326-331
            for (int n = 0; n < ng; ++n) {
                char cid8[16];
                std::snprintf(cid8, sizeof cid8, "%08lld", m.green.pts[n].gid);
                for (int c = 0; c < ncmp; ++c)
                    write_file(dir + "/" + p.title + "__" + cid8 + "__" + st.name + "__" + p.green_cmp + "__" + cmp[c] + "__.sac",
                               image(n, c));
            }
        } else {
            return swpc::set_err(SWPC_E_ARG, "Green's-function output is written as sac or csf by openswpc_gb300");
        }
        return 0;
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

int swpc_host_write_sac(swpc_sim* sim, const char* odir) {
    Meta m;
    {
        std::lock_guard<std::mutex> lk(g_meta_mu);
        auto it = g_meta.find(sim);
        if (it == g_meta.end()) return swpc::set_err(SWPC_E_STATE, "simulation was not prepared by swpc_host_prepare");
        m = it->second;
    }
    try {
        std::string dir = (odir && *odir) ? std::string(odir) : m.p.odir;
        mkdirs(dir + "/wav");
        const int nst = (int)m.st.size(), ntw = m.ntw;
        struct K { int kind, nc, idep; const char* names[6]; };
        const K kinds[4] = {{SWPC_WAV_V, 3, 7, {"Vx", "Vy", "Vz"}}, {SWPC_WAV_U, 3, 6, {"Ux", "Uy", "Uz"}},
                            {SWPC_WAV_STRESS, 6, 5, {"Sxx", "Syy", "Szz", "Syz", "Sxz", "Sxy"}},
                            {SWPC_WAV_STRAIN, 6, 5, {"Exx", "Eyy", "Ezz", "Eyz", "Exz", "Exy"}}};
        // traces of every recorded kind, (ntw, ncmp, nst) Fortran order
        std::vector<std::vector<float>> wav(4);
        for (int q = 0; q < 4; ++q) {
            const K& k = kinds[q];
            if (!(m.flags & k.kind)) continue;
            wav[q].resize((size_t)ntw * k.nc * nst);
            int rc = swpc_gpu_fetch_waveforms(sim, k.kind, wav[q].data());
            if (rc) return rc;
        }
        // SAC image of station s, component c of kind q (m_wav.f90:276-330)
        auto image = [&](int q, int s, int c) {
            const K& k = kinds[q];
            double inc = -12345, az = -12345;
            if (k.nc == 3) { inc = 90.0; az = c == 0 ? 0.0 + m.p.phi : c == 1 ? 90.0 + m.p.phi : 0.0; }
            return sac_image(m, m.st[s], k.names[c], k.idep, inc, az, &wav[q][((size_t)s * k.nc + c) * ntw], ntw);
        };
        const std::string& fmt = m.p.wav_format;
        if (fmt == "csf") {
            // one CSF file per kind, the last kind written wins as in the
            // reference, whose file name does not name the kind
            // (m_wav.f90:707-712, 795-808; m_sac.f90 wcsf_s)
            for (int q = 0; q < 4; ++q) {
                if (wav[q].empty()) continue;
                std::string b = "CSFD";
                const int32_t ntr = nst * kinds[q].nc, np = ntw;
                b.append((const char*)&ntr, 4);
                b.append((const char*)&np, 4);
                for (int st = 0; st < nst; ++st)
                    for (int c = 0; c < kinds[q].nc; ++c) b += image(q, st, c);
                write_file(dir + "/wav/" + m.p.title + "__00000__.csf", b);
            }
        } else if (fmt == "tar_st" || fmt == "tar_node") {
            // tar archives of SAC entries named <title>.<station>.3d.<cmp>.sac,
            // one per station or one for the whole run (m_wav.f90:714-779)
            std::string node;
            for (int st = 0; st < nst; ++st) {
                std::string arc;
                for (int q = 0; q < 4; ++q) {
                    if (wav[q].empty()) continue;
                    for (int c = 0; c < kinds[q].nc; ++c)
                        arc += tar_entry(m.p.title + "." + m.st[st].name + ".3d." + kinds[q].names[c] + ".sac",
                                         image(q, st, c), m.exedate);
                }
                if (fmt == "tar_st")
                    write_file(dir + "/wav/" + m.p.title + ".3d." + m.st[st].name + ".sac.tar", arc + std::string(1024, '\0'));
                else
                    node += arc;
            }
            if (fmt == "tar_node") write_file(dir + "/wav/" + m.p.title + ".3d.000000.sac.tar", node + std::string(1024, '\0'));
        } else {
            for (int q = 0; q < 4; ++q) {
                if (wav[q].empty()) continue;
                for (int st = 0; st < nst; ++st)
                    for (int c = 0; c < kinds[q].nc; ++c)
                        write_file(dir + "/wav/" + m.p.title + ".3d." + m.st[st].name + "." + kinds[q].names[c] + ".sac",
                                   image(q, st, c));
            }
        }
        return 0;
    } catch (const std::exception& e) {
        return swpc::set_err(SWPC_E_IO, e.what());
    }
}

}  // extern "C"
