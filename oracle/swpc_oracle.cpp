// swpc_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A plain CPU restatement of OpenSWPC's swpc_3d time-stepping path, against
// which the tests compare the CUDA implementation in openswpc_gb300/.  Nothing in the
// product links or calls this file; only tests/, __graft_entry__.smoke() and
// bench.py's CPU baseline (and its --impl reference arm) load it.
//
// Parity status: the reference is Fortran 2008 + MPI + NetCDF and cannot be
// compiled in this environment, and it ships no tests or golden vectors for
// this path (its only known-answer artifact is the console log
// example/example.out).  This restatement is therefore checked by its own
// known-answer tests (operator exactness, coefficient closed forms, source
// time function integrals, reciprocity, analytic far field, cross-precision
// agreement) in tests/test_oracle.py, and held to its own committed traces
// (tests/golden/, regenerated by tests/golden/make_golden.py) -- parity
// against the reference's own binary is UNPINNED.
//
// Three precision modes mirror the reference's build variants:
//   mode 0  fp32   MP = SP = float            (reference rebuilt with MP = SP)
//   mode 1  mixed  MP = double, SP = float    (reference default, MP = DP)
//   mode 2  fp64   MP = SP = double           (an all-FP64 build)
// MP is the velocity/stress type, SP the memory-variable, medium and
// intermediate type (src/swpc_3d/m_global.f90:30,34-41).
//
// Array layout follows the reference: A(k,i,j), k fastest, with a 3-cell halo
// k,i,j in [-2, n+3] (src/swpc_3d/m_global.f90:295-300 with one MPI rank).
// The loop order of every routine is the reference's (j outer, i, k inner),
// parallelised over j with OpenMP as the reference's CPU build does.

#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

static const double PI_D = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// input.inf reader: restates src/shared/m_readini.f90:29-100.  A key matches
// when a (left-adjusted, non-comment) line starts with the key and the rest,
// left-adjusted, starts with '='.  The value is the first list-directed item.
// ---------------------------------------------------------------------------
struct Ini {
    std::vector<std::string> lines;
    explicit Ini(const std::string& path) {
        std::ifstream f(path);
        if (!f) throw std::runtime_error("cannot open parameter file " + path);
        std::string s;
        while (std::getline(f, s)) lines.push_back(s);
    }
    static std::string ltrim(const std::string& s) {
        size_t p = 0;
        while (p < s.size() && (s[p] == ' ' || s[p] == '\t' || s[p] == '\r')) ++p;
        return s.substr(p);
    }
    // first list-directed item of the value text
    static std::string first_item(const std::string& v) {
        std::string s = ltrim(v);
        if (s.empty()) return s;
        if (s[0] == '\'' || s[0] == '"') {
            char q = s[0];
            size_t e = s.find(q, 1);
            return s.substr(1, e == std::string::npos ? std::string::npos : e - 1);
        }
        size_t e = 0;
        while (e < s.size() && s[e] != ' ' && s[e] != '\t' && s[e] != ',' && s[e] != '/' && s[e] != '\r') ++e;
        return s.substr(0, e);
    }
    bool raw(const std::string& key, std::string& out) const {
        for (const auto& l0 : lines) {
            std::string l = ltrim(l0);
            if (l.empty() || l[0] == '#' || l[0] == '!') continue;
            if (l.compare(0, key.size(), key) != 0) continue;
            std::string rest = ltrim(l.substr(key.size()));
            if (rest.empty() || rest[0] != '=') continue;
            out = first_item(rest.substr(1));
            // ${VAR} expansion (src/shared/m_system.f90:75)
            size_t p;
            while ((p = out.find("${")) != std::string::npos) {
                size_t e = out.find('}', p);
                if (e == std::string::npos) break;
                const char* ev = std::getenv(out.substr(p + 2, e - p - 2).c_str());
                out = out.substr(0, p) + (ev ? ev : "") + out.substr(e + 1);
            }
            return true;
        }
        return false;
    }
    static double to_real(std::string s) {
        for (auto& c : s) if (c == 'd' || c == 'D') c = 'e';
        return std::strtod(s.c_str(), nullptr);
    }
    double real(const std::string& k, double def) const { std::string v; return raw(k, v) ? to_real(v) : def; }
    int integer(const std::string& k, int def) const { std::string v; return raw(k, v) ? (int)std::strtol(v.c_str(), nullptr, 10) : def; }
    std::string str(const std::string& k, const std::string& def) const { std::string v; return raw(k, v) ? v : def; }
    bool logical(const std::string& k, bool def) const {
        std::string v;
        if (!raw(k, v)) return def;
        size_t p = (!v.empty() && v[0] == '.') ? 1 : 0;
        return p < v.size() && (v[p] == 't' || v[p] == 'T');
    }
};

// Fortran-ordered 3-D array A(k,i,j) with arbitrary lower bounds.
template <class T>
struct F3 {
    int kb = 0, ke = -1, ib = 0, ie = -1, jb = 0, je = -1;
    long nk = 0, nki = 0;
    std::vector<T> d;
    void alloc(int kb_, int ke_, int ib_, int ie_, int jb_, int je_) {
        kb = kb_; ke = ke_; ib = ib_; ie = ie_; jb = jb_; je = je_;
        nk = ke - kb + 1; nki = nk * (ie - ib + 1);
        d.assign((size_t)nki * (je - jb + 1), T(0));
    }
    T& operator()(int k, int i, int j) { return d[(size_t)(j - jb) * nki + (size_t)(i - ib) * nk + (k - kb)]; }
    const T& operator()(int k, int i, int j) const { return d[(size_t)(j - jb) * nki + (size_t)(i - ib) * nk + (k - kb)]; }
    bool empty() const { return d.empty(); }
};

// 2-D integer map M(i,j)
struct I2 {
    int ib = 0, ie = -1, jb = 0, je = -1;
    std::vector<int> d;
    void alloc(int ib_, int ie_, int jb_, int je_, int v) { ib = ib_; ie = ie_; jb = jb_; je = je_; d.assign((size_t)(ie - ib + 1) * (je - jb + 1), v); }
    int& operator()(int i, int j) { return d[(size_t)(j - jb) * (ie - ib + 1) + (i - ib)]; }
    int operator()(int i, int j) const { return d[(size_t)(j - jb) * (ie - ib + 1) + (i - ib)]; }
};

static inline int fsign1(long x) { return x >= 0 ? 1 : -1; }  // Fortran sign(1, x): sign(1,0) = +1

// Source time functions: src/shared/m_fdtool.f90:339-497
template <class S>
static S momentrate(S t, int stf, S ts, S tr) {
    const S pi = (S)PI_D;
    switch (stf) {
    case 0:  // boxcar :399-416
        return (ts <= t && t <= ts + tr) ? S(1.0) / tr : S(0);
    case 1:  // triangle :419-438
        if (ts <= t && t <= ts + tr / 2) return 4 * (t - ts) / (tr * tr);
        if (ts + tr / 2 < t && t <= ts + tr) return -4 * (t - ts - tr) / (tr * tr);
        return 0;
    case 2: {  // herrmann :441-468
        S t1 = ts + tr / 4, t2 = ts + 3 * tr / 4;
        if (ts <= t && t < t1) return 16 * (t - ts) * (t - ts) / (tr * tr * tr);
        if (t1 <= t && t < t2) return -2 * (8 * (t * t + tr * ts + ts * ts - t * tr - 2 * t * ts) + tr * tr) / (tr * tr * tr);
        if (t2 <= t && t <= ts + tr) return 16 * (ts + tr - t) * (ts + tr - t) / (tr * tr * tr);
        return 0;
    }
    case 4:  // cosine :379-396
        return (ts <= t && t <= ts + tr) ? (1 - std::cos(2 * pi * (t - ts) / tr)) / tr : S(0);
    case 5: {  // texp :356-376
        if (ts <= t) { S tt = t - ts; return (2 * pi) * (2 * pi) * tt / (tr * tr) * std::exp(-2 * pi * tt / tr); }
        return 0;
    }
    default: {  // kupper :339-353
        if (ts <= t && t <= ts + tr) { S s = std::sin(pi * (t - ts) / tr); return 3 * pi * s * s * s / (4 * tr); }
        return 0;
    }
    }
}

static int stf_code(const std::string& s) {
    if (s == "boxcar") return 0;
    if (s == "triangle") return 1;
    if (s == "herrmann") return 2;
    if (s == "kupper") return 3;
    if (s == "cosine" || s == "scosine") return 4;
    if (s == "texp") return 5;
    return 3;
}

static std::vector<std::string> data_lines(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<std::string> out;
    std::string s;
    while (std::getline(f, s)) {
        std::string t = Ini::ltrim(s);
        if (t.empty() || t[0] == '#') continue;
        bool blank = true;
        for (char c : t) if (!std::isspace((unsigned char)c)) blank = false;
        if (blank) continue;
        out.push_back(t);
    }
    return out;
}
static std::vector<std::string> tokens(const std::string& s) {
    std::vector<std::string> v;
    std::string cur;
    bool inq = false; char q = 0;
    for (char c : s) {
        if (inq) { if (c == q) inq = false; else cur += c; continue; }
        if (c == '\'' || c == '"') { inq = true; q = c; continue; }
        if (c == ' ' || c == '\t' || c == ',' || c == '\r') { if (!cur.empty()) { v.push_back(cur); cur.clear(); } continue; }
        cur += c;
    }
    if (!cur.empty()) v.push_back(cur);
    return v;
}

// ---------------------------------------------------------------------------
// The simulation state and the reference routines, templated on precision.
// ---------------------------------------------------------------------------
struct Params {
    std::string title, odir, abc_type, vmodel_type, fn_lhm, stftype, stf_format, fn_stf, sdep_fit, st_format, fn_stloc;
    int nx, ny, nz, nt, na, ntdec_w, ntdec_r, ntdec_s, idec, jdec, kdec;
    double dx, dy, dz, dt, xbeg, ybeg, zbeg, tbeg, clon, clat, phi, fq_min, fq_max, fq_ref, vcut;
    double vp0, vs0, rho0, qp0, qs0, topo0, z0_xy, x0_yz, y0_xz;
    int snap_sw[5];  // sections xy yz xz fs ob; bits: 1 v, 2 u, 4 ps
    // Green's-function mode (src/swpc_3d/m_green.f90:67-160)
    std::string green_stnm, green_cmp, fn_glst, green_fmt;
    double green_trise, green_maxdist;
    bool green_bforce, stabilize_pml;
    // plane-wave mode (src/swpc_3d/m_source.f90:316-466)
    double pw_ztop, pw_zlen, pw_strike, pw_dip, pw_rake;
    std::string pw_ps;
    bool bf_mode, pw_mode, green_mode, sw_wav_v, sw_wav_u, sw_wav_stress, sw_wav_strain, munk, xy_v, xy_u;
};

// src/swpc_3d/m_global.f90:124-177
static Params read_params(const Ini& ini) {
    Params p;
    p.title = ini.str("title", "swpc3d");
    p.odir = ini.str("odir", "./out");
    p.nx = ini.integer("nx", 256); p.ny = ini.integer("ny", 256); p.nz = ini.integer("nz", 256);
    p.nt = ini.integer("nt", 1000);
    if (ini.logical("benchmark_mode", false)) throw std::runtime_error("benchmark_mode is not supported by the oracle");
    p.dx = ini.real("dx", 0.5); p.dy = ini.real("dy", 0.5); p.dz = ini.real("dz", 0.5);
    p.dt = ini.real("dt", 0.01);
    p.na = ini.integer("na", 20);
    p.xbeg = ini.real("xbeg", -p.nx / 2 * (float)p.dx);
    p.ybeg = ini.real("ybeg", -p.ny / 2 * (float)p.dy);
    p.zbeg = ini.real("zbeg", -30 * (float)p.dz);
    p.tbeg = ini.real("tbeg", 0.0);
    p.clon = ini.real("clon", 139.7604); p.clat = ini.real("clat", 35.7182); p.phi = ini.real("phi", 0.0);
    p.abc_type = ini.str("abc_type", "pml");
    p.fq_min = ini.real("fq_min", 0.05); p.fq_max = ini.real("fq_max", 5.0); p.fq_ref = ini.real("fq_ref", 1.0);
    p.vmodel_type = ini.str("vmodel_type", "uni");
    p.vcut = ini.real("vcut", 0.0);
    p.fn_lhm = ini.str("fn_lhm", "");
    p.munk = ini.logical("munk_profile", false);
    p.vp0 = ini.real("vp0", 5.0); p.vs0 = ini.real("vs0", p.vp0 / std::sqrt(3.0f)); p.rho0 = ini.real("rho0", 2.7);
    p.qp0 = ini.real("qp0", 1000000.0); p.qs0 = ini.real("qs0", 1000000.0); p.topo0 = ini.real("topo0", 0.0);
    p.pw_mode = ini.logical("pw_mode", false);
    p.green_mode = ini.logical("green_mode", false);
    p.bf_mode = ini.logical("bf_mode", false);
    if (p.pw_mode) {
        p.pw_ztop = ini.real("pw_ztop", 1e30f); p.pw_zlen = ini.real("pw_zlen", -1.0f);
        p.pw_ps = ini.str("pw_ps", "");
        p.pw_strike = ini.real("pw_strike", 0.0f); p.pw_dip = ini.real("pw_dip", 0.0f); p.pw_rake = ini.real("pw_rake", 0.0f);
        if (!(p.pw_zlen > 0)) throw std::runtime_error("pw_zlen must be positive");
    }
    if (p.green_mode) {
        p.green_stnm = ini.str("green_stnm", ""); p.green_cmp = ini.str("green_cmp", "");
        p.green_trise = ini.real("green_trise", 1.0); p.green_bforce = ini.logical("green_bforce", false);
        p.green_maxdist = ini.real("green_maxdist", 1e30); p.fn_glst = ini.str("fn_glst", "");
        p.green_fmt = ini.str("green_fmt", "xyz");
        if (p.green_fmt != "xyz") throw std::runtime_error("only green_fmt = xyz is supported by the oracle");
        if (p.green_cmp != "x" && p.green_cmp != "y" && p.green_cmp != "z") throw std::runtime_error("no matching green_cmp");
    }
    if (ini.logical("earth_flattening", false)) throw std::runtime_error("earth_flattening is not supported by the oracle");
    p.stabilize_pml = ini.logical("stabilize_pml", false);
    p.fn_stf = ini.str("fn_stf", "");
    p.stftype = ini.str("stftype", "kupper");
    p.stf_format = ini.str("stf_format", "xym0ij");
    p.sdep_fit = ini.str("sdep_fit", "asis");
    p.ntdec_w = ini.integer("ntdec_w", 10);
    p.sw_wav_v = ini.logical("sw_wav_v", false); p.sw_wav_u = ini.logical("sw_wav_u", false);
    p.sw_wav_stress = ini.logical("sw_wav_stress", false); p.sw_wav_strain = ini.logical("sw_wav_strain", false);
    p.st_format = ini.str("st_format", "xy");
    p.fn_stloc = ini.str("fn_stloc", "");
    p.ntdec_r = ini.integer("ntdec_r", 100);
    // src/swpc_3d/m_snap.f90:105-127
    {
        const char* secs[5] = {"xy", "yz", "xz", "fs", "ob"};
        const char* kinds[3] = {"v", "u", "ps"};
        for (int q = 0; q < 5; ++q) {
            p.snap_sw[q] = 0;
            for (int c = 0; c < 3; ++c)
                if (ini.logical(std::string(secs[q]) + "_" + kinds[c] + "%sw", false)) p.snap_sw[q] |= 1 << c;
        }
    }
    p.xy_v = p.snap_sw[0] & 1; p.xy_u = (p.snap_sw[0] & 2) != 0;
    float zend = (float)p.zbeg + p.nz * (float)p.dz;
    float xend = (float)p.xbeg + p.nx * (float)p.dx, yend = (float)p.ybeg + p.ny * (float)p.dy;
    p.z0_xy = ini.real("z0_xy", std::max(std::min(10.0f, zend), (float)p.zbeg));
    p.x0_yz = ini.real("x0_yz", std::max(std::min(0.0f, xend), (float)p.xbeg));
    p.y0_xz = ini.real("y0_xz", std::max(std::min(0.0f, yend), (float)p.ybeg));
    p.idec = ini.integer("idec", 1); p.jdec = ini.integer("jdec", 1); p.kdec = ini.integer("kdec", 1);
    p.ntdec_s = ini.integer("ntdec_s", 10);
    return p;
}

struct Src {  // one source grid point after setup (src/swpc_3d/m_source.f90:41-314)
    int i, j, k;
    double mo, mxx, myy, mzz, myz, mxz, mxy, fx, fy, fz;
    double tbeg, trise;
};
struct Sta { int i, j, k; std::string name; };

struct SimBase {
    virtual ~SimBase() {}
    virtual int get_sources(int* ijk, double* vals) = 0;
    virtual void step(int it) = 0;
    virtual void get_field(int which, double* out) = 0;
    virtual void set_field(int which, const float* halo) = 0;
    virtual void get_medium(int which, float* out) = 0;
    virtual int green_out(int* ng_ncmp_ntw, float* out) = 0;
    virtual int coefs(double* out) = 0;
    Params p;
    int nt_done = 0;
    int nst = 0, ntw = 0;
    std::vector<float> wav_vel, wav_disp, wav_stress, wav_strain;  // (ntw, ncmp, nst) Fortran order
    std::vector<float> vmax_log;  // (it, vx, vy, vz) every ntdec_r
    // snapshot planes: section (0 xy, 1 yz, 2 xz, 3 fs, 4 ob), kind (0 v,
    // 1 u, 2 ps), pixel grid and decimation, fixed index; frames stacked as
    // (nc, n2, n1) each
    struct OSnap {
        int sec, kind, n1, n2, d1, d2, fix;
        std::vector<double> ubuf;   // running displacement (u), FP32 values as the reference sums them
        std::vector<float> frames;
    };
    std::vector<OSnap> snaps;
    float M0 = 0, UC = 1e-15f, fcut = 0;
    int nxs = 0, nys = 0, k0_xy = 0;
    std::vector<Sta> sta;
};

template <class MP, class SP>
struct Sim : SimBase {
    int nx, ny, nz, na, nm = 3;
    int ibeg, iend, jbeg, jend, kbeg, kend, ibeg_m, iend_m, jbeg_m, jend_m, kbeg_m, kend_m;
    int ibeg_k, iend_k, jbeg_k, jend_k, kbeg_k, kend_k;
    MP dx, dy, dz;
    SP dt, xbeg, ybeg, zbeg, tbeg, xend, yend, zend;
    bool pml;
    std::vector<SP> xc, yc, zc;  // indexed from *_m
    F3<MP> Vx, Vy, Vz, Sxx, Syy, Szz, Syz, Sxz, Sxy;
    F3<SP> rho, lam, mu, taup, taus;
    std::vector<F3<SP>> Rxx, Ryy, Rzz, Ryz, Rxz, Rxy;  // per m: R(m,k,i,j) stored as nm arrays
    I2 kfs, kob, kfs_top, kfs_bot, kob_top, kob_bot, kbeg_a;
    std::vector<SP> ts, c1, c2, d1;
    SP d2 = 0;
    MP rc40x, rc41x, rc40y, rc41y, rc40z, rc41z, rd40x, rd41x, rd40y, rd41y, rd40z, rd41z;
    // PML
    std::vector<SP> gxc, gxe, gyc, gye, gzc, gze;  // (4, n) flattened: g[4*(i-ibeg)+l]
    F3<SP> axVx, ayVx, azVx, axVy, ayVy, azVy, axVz, ayVz, azVz;
    F3<SP> axSxx, aySxy, azSxz, axSxy, aySyy, azSyz, axSxz, aySyz, azSzz;
    MP r20x, r20y, r20z;
    // Cerjan
    std::vector<SP> gx_c, gx_b, gy_c, gy_b, gz_c, gz_b;
    // sources
    std::vector<Src> src;
    int stf = 3;
    MP dt_dxyz;
    // receivers
    std::vector<SP> ux, uy, uz, exx, eyy, ezz, eyz, exz, exy;
    MP r40x, r40y, r40z, r41x, r41y, r41z;

    SP& gx(std::vector<SP>& g, int l, int i, int b) { return g[4 * (i - b) + (l - 1)]; }

    // i2x etc: src/shared/m_fdtool.f90:639-675
    static SP i2x(int i, SP beg, SP d) { return beg + (SP)(i - (SP)0.5) * d; }
    static int x2i(SP x, SP beg, SP d) { return (int)std::ceil((x - beg) / d); }

    Sim(const Params& pp, const std::string& inf_dir, const float* vm5) {
        p = pp;
        nx = p.nx; ny = p.ny; nz = p.nz; na = p.na;
        dx = (MP)p.dx; dy = (MP)p.dy; dz = (MP)p.dz;
        dt = (SP)p.dt; xbeg = (SP)p.xbeg; ybeg = (SP)p.ybeg; zbeg = (SP)p.zbeg; tbeg = (SP)p.tbeg;
        // global__setup derived parameters: m_global.f90:203-206
        xend = xbeg + nx * (SP)dx; yend = ybeg + ny * (SP)dy; zend = zbeg + nz * (SP)dz;
        setup_regions();
        setup_medium(inf_dir, vm5);
        kernel_setup();
        if (p.pw_mode) pw_setup();
        else if (!p.green_mode) source_setup(inf_dir);  // m_source.f90:84-91: no regular source grid
        if (p.green_mode || p.pw_mode) dt_dxyz = (MP)dt / (dx * dy * dz);
        absorb_setup();
        wav_setup(inf_dir);
        if (p.green_mode) green_setup(inf_dir);
        snap_setup();
    }

    // ------------------------------------------------------------------
    // Green's-function mode (src/swpc_3d/m_green.f90): a unit body force at
    // the station green_stnm, strain (and displacement) recorded at the grid
    // points of fn_glst
    // ------------------------------------------------------------------
    struct GPt { int i, j, k, gid; SP x, y, z; };
    std::vector<GPt> gpts;
    std::vector<SP> gacc;         // (12, ng): dxUx dxUy dxUz dyUx dyUy dyUz dzUx dzUy dzUz Ux Uy Uz
    std::vector<float> gf;        // (ntw, ncmp * ng), Fortran order
    int gncmp = 6, gsrc_i = 0, gsrc_j = 0, gsrc_k = 0;
    SP gfx = 0, gfy = 0, gfz = 0;

    // m_green.f90:67-404
    void green_setup(const std::string& inf_dir) {
        int q = 0;
        while (q < (int)sta_all.size() && sta_all[q].name != p.green_stnm.substr(0, 8)) ++q;
        if (q == (int)sta_all.size()) throw std::runtime_error("green_stnm not in the station list");
        gsrc_i = sta_all[q].i; gsrc_j = sta_all[q].j; gsrc_k = sta_all[q].k;
        const SP xsrc = sta_all[q].x, ysrc = sta_all[q].y;
        gfx = p.green_cmp == "x" ? 1 : 0; gfy = p.green_cmp == "y" ? 1 : 0; gfz = p.green_cmp == "z" ? 1 : 0;
        M0 = 1;
        fcut = 0;  // never set by source__setup in this mode
        stf = stf_code(p.stftype);
        ntw = (int)std::floor((float)(p.nt - 1) / (float)p.ntdec_w + 1.0f);
        std::string fn = p.fn_glst;
        if (!fn.empty() && fn[0] != '/') fn = inf_dir + "/" + fn;
        for (auto& r : data_lines(fn)) {
            auto t = tokens(r);
            if (t.size() < 4) throw std::runtime_error("bad Green's function point: " + r);
            const SP xg = (SP)Ini::to_real(t[0]), yg = (SP)Ini::to_real(t[1]), zg = (SP)Ini::to_real(t[2]);
            const int gid = (int)Ini::to_real(t[3]);
            const SP dd = std::sqrt((xg - xsrc) * (xg - xsrc) + (yg - ysrc) * (yg - ysrc));
            if (dd > (SP)p.green_maxdist) continue;
            const int ii = x2i(xg, xbeg, (SP)dx), jj = x2i(yg, ybeg, (SP)dy), kk = x2i(zg, zbeg, (SP)dz);
            if (ibeg <= ii && ii <= iend && jbeg <= jj && jj <= jend && kob(ii, jj) <= kk && kk <= kend)
                gpts.push_back(GPt{ii, jj, kk, gid, xg, yg, zg});
        }
        gncmp = p.green_bforce ? 9 : 6;
        gacc.assign(12 * gpts.size(), 0);
        gf.assign((size_t)ntw * gncmp * gpts.size(), 0.f);
        r40x = MP(9.0) / MP(8.0) / dx; r40y = MP(9.0) / MP(8.0) / dy; r40z = MP(9.0) / MP(8.0) / dz;
        r41x = MP(1.0) / MP(24.0) / dx; r41y = MP(1.0) / MP(24.0) / dy; r41z = MP(1.0) / MP(24.0) / dz;
        r20x = (MP)1.0 / dx; r20y = (MP)1.0 / dy; r20z = (MP)1.0 / dz;
    }

    int green_out(int* v, float* out) override {
        if (!p.green_mode) return -1;
        v[0] = (int)gpts.size(); v[1] = gncmp; v[2] = ntw;
        if (out) std::copy(gf.begin(), gf.end(), out);
        return 0;
    }

    // m_green.f90:406-551
    void green_store(int it) {
        if (!p.green_mode) return;
        const SP UC_BF = (SP)1e-12, UC_DERIV = (SP)1e-15;
        const int ng = (int)gpts.size();
        for (int n = 0; n < ng; ++n) {
            const int ii = gpts[n].i, jj = gpts[n].j, kk = gpts[n].k;
            auto D = [&](F3<MP>& V, int k1, int i1, int j1, int k0, int i0, int j0, int k2, int i2, int j2, int k3, int i3,
                         int j3, MP r0, MP r1) { return (V(k1, i1, j1) - V(k0, i0, j0)) * r0 - (V(k2, i2, j2) - V(k3, i3, j3)) * r1; };
            const MP dxVx = D(Vx, kk, ii, jj, kk, ii - 1, jj, kk, ii + 1, jj, kk, ii - 2, jj, r40x, r41x);
            const MP dyVy = D(Vy, kk, ii, jj, kk, ii, jj - 1, kk, ii, jj + 1, kk, ii, jj - 2, r40y, r41y);
            const MP dzVz = D(Vz, kk, ii, jj, kk - 1, ii, jj, kk + 1, ii, jj, kk - 2, ii, jj, r40z, r41z);
            // four-point averages of the staggered off-diagonal derivatives
            auto dxq = [&](F3<MP>& V, int k, int j) {
                return D(V, k, ii + 1, j, k, ii, j, k, ii + 2, j, k, ii - 1, j, r40x, r41x);
            };
            auto dxp = [&](F3<MP>& V, int k, int j) {
                return D(V, k, ii, j, k, ii - 1, j, k, ii + 1, j, k, ii - 2, j, r40x, r41x);
            };
            auto dyq = [&](F3<MP>& V, int k, int i) {
                return D(V, k, i, jj + 1, k, i, jj, k, i, jj + 2, k, i, jj - 1, r40y, r41y);
            };
            auto dyp = [&](F3<MP>& V, int k, int i) {
                return D(V, k, i, jj, k, i, jj - 1, k, i, jj + 1, k, i, jj - 2, r40y, r41y);
            };
            auto dzq = [&](F3<MP>& V, int i, int j) {
                return D(V, kk + 1, i, j, kk, i, j, kk + 2, i, j, kk - 1, i, j, r40z, r41z);
            };
            auto dzp = [&](F3<MP>& V, int i, int j) {
                return D(V, kk, i, j, kk - 1, i, j, kk + 1, i, j, kk - 2, i, j, r40z, r41z);
            };
            const MP dxVy = (dxq(Vy, kk, jj) + dxq(Vy, kk, jj - 1) + dxp(Vy, kk, jj) + dxp(Vy, kk, jj - 1)) * (MP)0.25;
            const MP dxVz = (dxq(Vz, kk, jj) + dxq(Vz, kk - 1, jj) + dxp(Vz, kk, jj) + dxp(Vz, kk - 1, jj)) * (MP)0.25;
            const MP dyVx = (dyq(Vx, kk, ii) + dyq(Vx, kk, ii - 1) + dyp(Vx, kk, ii) + dyp(Vx, kk, ii - 1)) * (MP)0.25;
            const MP dyVz = (dyq(Vz, kk, ii) + dyq(Vz, kk - 1, ii) + dyp(Vz, kk, ii) + dyp(Vz, kk - 1, ii)) * (MP)0.25;
            const MP dzVx = (dzq(Vx, ii, jj) + dzq(Vx, ii - 1, jj) + dzp(Vx, ii, jj) + dzp(Vx, ii - 1, jj)) * (MP)0.25;
            const MP dzVy = (dzq(Vy, ii, jj) + dzq(Vy, ii, jj - 1) + dzp(Vy, ii, jj) + dzp(Vy, ii, jj - 1)) * (MP)0.25;
            SP* a = &gacc[12 * n];
            const MP g9[9] = {dxVx, dxVy, dxVz, dyVx, dyVy, dyVz, dzVx, dzVy, dzVz};
            for (int c = 0; c < 9; ++c) a[c] = a[c] + (SP)(g9[c] * (MP)dt);
            if (p.green_bforce) {
                a[9] = a[9] + (SP)0.5 * (SP)(Vx(kk, ii, jj) + Vx(kk, ii - 1, jj)) * dt;
                a[10] = a[10] + (SP)0.5 * (SP)(Vy(kk, ii, jj) + Vy(kk, ii, jj - 1)) * dt;
                a[11] = a[11] + (SP)0.5 * (SP)(Vz(kk, ii, jj) + Vz(kk - 1, ii, jj)) * dt;
            }
        }
        if ((it - 1) % p.ntdec_w != 0) return;
        const int itw = (it - 1) / p.ntdec_w;
        const SP sd = UC_DERIV * (SP)1e9, sb = UC_BF * (SP)1e9;
        for (int n = 0; n < ng; ++n) {
            const SP* a = &gacc[12 * n];
            float* g = &gf[(size_t)gncmp * n * ntw + itw];
            auto put = [&](int c, SP v) { g[(size_t)c * ntw] = (float)v; };
            put(0, a[0] * sd); put(1, a[4] * sd); put(2, a[8] * sd);
            put(3, (a[5] + a[7]) * sd); put(4, (a[2] + a[6]) * sd); put(5, (a[1] + a[3]) * sd);
            if (p.green_bforce) { put(6, a[9] * sb); put(7, a[10] * sb); put(8, a[11] * sb); }
        }
    }

    // m_green.f90:614-649
    void green_source(int it) {
        if (!p.green_mode) return;
        const SP st = momentrate<SP>(tbeg + it * dt, stf, (SP)0, (SP)p.green_trise);
        const SP dtd = (SP)dt_dxyz;
        const SP fx = gfx * dtd * st, fy = gfy * dtd * st, fz = gfz * dtd * st;
        const int ii = gsrc_i, jj = gsrc_j, kk = gsrc_k;
        const SP two = 2.0;
        Vx(kk, ii, jj) = Vx(kk, ii, jj) + (MP)((two / (rho(kk, ii, jj) + rho(kk, ii + 1, jj))) * fx / 2);
        Vx(kk, ii - 1, jj) = Vx(kk, ii - 1, jj) + (MP)((two / (rho(kk, ii, jj) + rho(kk, ii - 1, jj))) * fx / 2);
        Vy(kk, ii, jj) = Vy(kk, ii, jj) + (MP)((two / (rho(kk, ii, jj) + rho(kk, ii, jj + 1))) * fy / 2);
        Vy(kk, ii, jj - 1) = Vy(kk, ii, jj - 1) + (MP)((two / (rho(kk, ii, jj) + rho(kk, ii, jj - 1))) * fy / 2);
        Vz(kk, ii, jj) = Vz(kk, ii, jj) + (MP)((two / (rho(kk, ii, jj) + rho(kk + 1, ii, jj))) * fz / 2);
        Vz(kk - 1, ii, jj) = Vz(kk - 1, ii, jj) + (MP)((two / (rho(kk, ii, jj) + rho(kk - 1, ii, jj))) * fz / 2);
    }

    // m_global.f90:219-376 for a single rank
    void setup_regions() {
        ibeg = 1; iend = nx; jbeg = 1; jend = ny; kbeg = 1; kend = nz;
        ibeg_m = ibeg - 3; iend_m = iend + 3; jbeg_m = jbeg - 3; jend_m = jend + 3; kbeg_m = kbeg - 3; kend_m = kend + 3;
        xc.resize(iend_m - ibeg_m + 1); yc.resize(jend_m - jbeg_m + 1); zc.resize(kend_m - kbeg_m + 1);
        for (int i = ibeg_m; i <= iend_m; ++i) xc[i - ibeg_m] = i2x(i, xbeg, (SP)dx);
        for (int j = jbeg_m; j <= jend_m; ++j) yc[j - jbeg_m] = i2x(j, ybeg, (SP)dy);
        for (int k = kbeg_m; k <= kend_m; ++k) zc[k - kbeg_m] = i2x(k, zbeg, (SP)dz);
        kbeg_a.alloc(ibeg_m, iend_m, jbeg_m, jend_m, 0);
        for (int j = jbeg_m; j <= jend_m; ++j)
            for (int i = ibeg_m; i <= iend_m; ++i)
                kbeg_a(i, j) = (i <= na || nx - na + 1 <= i || j <= na || ny - na + 1 <= j) ? kbeg : kend - na + 1;
        ibeg_k = ibeg; iend_k = iend; jbeg_k = jbeg; jend_k = jend; kbeg_k = kbeg; kend_k = kend;
        pml = (p.abc_type == "pml");
        if (!pml && p.abc_type != "cerjan") throw std::runtime_error("unknown abc_type " + p.abc_type);
        if (pml) {
            if (iend <= na) ibeg_k = iend + 1; else if (ibeg <= na) ibeg_k = na + 1;
            if (ibeg >= nx - na + 1) iend_k = ibeg - 1; else if (iend >= nx - na + 1) iend_k = nx - na;
            if (jend <= na) jbeg_k = jend + 1; else if (jbeg <= na) jbeg_k = na + 1;
            if (jbeg >= ny - na + 1) jend_k = jbeg - 1; else if (jend >= ny - na + 1) jend_k = ny - na;
            kend_k = nz - na;
        }
        auto a3 = [&](F3<MP>& a) { a.alloc(kbeg_m, kend_m, ibeg_m, iend_m, jbeg_m, jend_m); };
        a3(Vx); a3(Vy); a3(Vz); a3(Sxx); a3(Syy); a3(Szz); a3(Syz); a3(Sxz); a3(Sxy);
    }

    // seawater: src/shared/m_seawater.f90:34-47
    SP seawater_vel(SP z) const {
        double eps = p.munk ? 0.00737 : 0.0;
        double zcc = 1300.0, zb = 2 * ((double)z * 1000. - zcc) / zcc;
        return (SP)(1.5 * (1.0 + eps * (zb - 1.0 + std::exp(-zb))));
    }

    // m_vmodel_uni.f90:40-149, m_vmodel_lhm.f90:21-169, m_vmodel_lgm.f90:21-174
    void vmodel(const std::string& inf_dir, F3<SP>& qp, F3<SP>& qs) {
        const std::string& vt = p.vmodel_type;
        if (vt == "uni") {
            SP vp0 = (SP)p.vp0, vs0 = (SP)p.vs0, rho0 = (SP)p.rho0, topo0 = (SP)p.topo0;
            for (int j = jbeg_m; j <= jend_m; ++j)
                for (int i = ibeg_m; i <= iend_m; ++i)
                    for (int k = kbeg_m; k <= kend_m; ++k) {
                        SP z = zc[k - kbeg_m], r, vp1, vs1, q1, q2;
                        if (z > topo0) { vp1 = vp0; vs1 = vs0; r = rho0; q1 = (SP)p.qp0; q2 = (SP)p.qs0; }
                        else if (z > 0) { vp1 = seawater_vel(z); vs1 = 0; r = 1; q1 = q2 = (SP)1000000.0; }
                        else { vp1 = vs1 = 0; r = (SP)0.001; q1 = q2 = 10; }
                        rho(k, i, j) = r; mu(k, i, j) = r * vs1 * vs1; lam(k, i, j) = r * (vp1 * vp1 - 2 * vs1 * vs1);
                        qp(k, i, j) = q1; qs(k, i, j) = q2;
                    }
            return;
        }
        if (vt != "lhm" && vt != "lgm") throw std::runtime_error("vmodel_type not supported by the oracle: " + vt);
        std::string fn = p.fn_lhm;
        if (!fn.empty() && fn[0] != '/') fn = inf_dir + "/" + fn;
        auto rows = data_lines(fn);
        int nl = (int)rows.size();
        std::vector<SP> dep(nl), rho0(nl), vp0(nl), vs0(nl), qp0(nl), qs0(nl);
        for (int l = 0; l < nl; ++l) {
            auto t = tokens(rows[l]);
            if (t.size() < 6) throw std::runtime_error("bad layer line in " + fn);
            dep[l] = (SP)Ini::to_real(t[0]); rho0[l] = (SP)Ini::to_real(t[1]); vp0[l] = (SP)Ini::to_real(t[2]);
            vs0[l] = (SP)Ini::to_real(t[3]); qp0[l] = (SP)Ini::to_real(t[4]); qs0[l] = (SP)Ini::to_real(t[5]);
        }
        SP vcut = (SP)p.vcut;
        for (int l = nl - 2; l >= 0; --l)
            if ((vp0[l] < vcut || vs0[l] < vcut) && (vp0[l] > 0 && vs0[l] > 0)) {
                vp0[l] = vp0[l + 1]; vs0[l] = vs0[l + 1]; rho0[l] = rho0[l + 1]; qp0[l] = qp0[l + 1]; qs0[l] = qs0[l + 1];
            }
        for (int k = kbeg_m; k <= kend_m; ++k) {
            SP z = zc[k - kbeg_m], r, vp1, vs1, q1, q2;
            if (z < dep[0]) {
                if (z < 0) { r = (SP)0.001; vp1 = vs1 = 0; q1 = q2 = 10; }
                else { r = 1; vp1 = seawater_vel(z); vs1 = 0; q1 = q2 = (SP)1000000.0; }
            } else if (vt == "lhm") {
                r = vp1 = vs1 = q1 = q2 = 0;
                for (int l = 0; l < nl; ++l)
                    if (z >= dep[l]) { r = rho0[l]; vp1 = vp0[l]; vs1 = vs0[l]; q1 = qp0[l]; q2 = qs0[l]; }
            } else {
                r = rho0[nl - 1]; vp1 = vp0[nl - 1]; vs1 = vs0[nl - 1]; q1 = qp0[nl - 1]; q2 = qs0[nl - 1];
                for (int l = 0; l < nl - 1; ++l)
                    if (dep[l] <= z && z < dep[l + 1]) {
                        SP f = (z - dep[l]);
                        SP h = (dep[l + 1] - dep[l]);
                        r = rho0[l] + (rho0[l + 1] - rho0[l]) / h * f;
                        vp1 = vp0[l] + (vp0[l + 1] - vp0[l]) / h * f;
                        vs1 = vs0[l] + (vs0[l + 1] - vs0[l]) / h * f;
                        q1 = qp0[l] + (qp0[l + 1] - qp0[l]) / h * f;
                        q2 = qs0[l] + (qs0[l + 1] - qs0[l]) / h * f;
                        break;
                    }
            }
            SP m1 = r * vs1 * vs1, l1 = r * (vp1 * vp1 - 2 * vs1 * vs1);
            for (int j = jbeg_m; j <= jend_m; ++j)
                for (int i = ibeg_m; i <= iend_m; ++i) {
                    rho(k, i, j) = r; mu(k, i, j) = m1; lam(k, i, j) = l1; qp(k, i, j) = q1; qs(k, i, j) = q2;
                }
        }
    }

    // src/shared/m_fdtool.f90:691-727
    void visco_set_relaxtime(SP fmin, SP fmax) {
        ts.assign(nm, 0);
        SP oa = (SP)(2 * PI_D * fmin), ob = (SP)(2 * PI_D * fmax);
        if (nm == 1) { ts[0] = (SP)(1.0 / std::sqrt(oa * ob)); return; }
        for (int im = 1; im <= nm; ++im) {
            SP om = (SP)((double)oa * std::pow((double)(SP)(ob / oa), (double)(im - 1) / (double)(nm - 1)));
            ts[im - 1] = (SP)1.0 / om;
        }
    }
    // src/shared/m_fdtool.f90:756-812 (tau-method zeta of Blanch et al.)
    SP visco_constq_zeta(SP fmin, SP fmax) {
        SP oa = (SP)(2 * PI_D * fmin), ob = (SP)(2 * PI_D * fmax);
        SP i0s = 0, i1s = 0, i2s = 0;
        for (int m = 0; m < nm; ++m) {
            SP t = ts[m];
            i0s += (std::log((SP)1.0 + ob * ob * t * t) - std::log((SP)1.0 + oa * oa * t * t)) / (2 * t);
            i1s += ((std::atan(ob * t) - ob * t / (1 + ob * ob * t * t)) - (std::atan(oa * t) - oa * t / (1 + oa * oa * t * t))) / (2 * t);
        }
        for (int im = 0; im < nm - 1; ++im)
            for (int km = im + 1; km < nm; ++km) {
                SP wk1 = std::atan(ob * ts[im]) / ts[im] - std::atan(ob * ts[km]) / ts[km];
                SP wk2 = std::atan(oa * ts[im]) / ts[im] - std::atan(oa * ts[km]) / ts[km];
                i2s += ts[im] * ts[km] / (ts[km] * ts[km] - ts[im] * ts[im]) * (wk1 - wk2);
            }
        return i0s / (i1s + 2 * i2s);
    }

    // src/swpc_3d/m_medium.f90:36-229
    void setup_medium(const std::string& inf_dir, const float* vm5) {
        auto a3 = [&](F3<SP>& a) { a.alloc(kbeg_m, kend_m, ibeg_m, iend_m, jbeg_m, jend_m); };
        a3(rho); a3(lam); a3(mu); a3(taup); a3(taus);
        if (vm5) {
            // caller-provided rho, lam, mu, qp, qs over the halo grid (a stand-in for a model file)
            size_t n = rho.d.size();
#pragma omp parallel for schedule(static)
            for (size_t q = 0; q < n; ++q) {
                rho.d[q] = (SP)vm5[q]; lam.d[q] = (SP)vm5[n + q]; mu.d[q] = (SP)vm5[2 * n + q];
                taup.d[q] = (SP)vm5[3 * n + q]; taus.d[q] = (SP)vm5[4 * n + q];
            }
        } else {
            vmodel(inf_dir, taup, taus);  // taup/taus hold Qp/Qs until the tau-method below
        }
        // homogenize absorber region :124-190
        auto cp = [&](int kd, int id, int jd, int ks, int is, int js) {
            rho(kd, id, jd) = rho(ks, is, js); lam(kd, id, jd) = lam(ks, is, js); mu(kd, id, jd) = mu(ks, is, js);
            taup(kd, id, jd) = taup(ks, is, js); taus(kd, id, jd) = taus(ks, is, js);
        };
        for (int i = ibeg_m; i <= na; ++i)
            for (int j = jbeg_m; j <= jend_m; ++j) for (int k = kbeg_m; k <= kend_m; ++k) cp(k, i, j, k, na + 1, j);
        for (int i = nx - na + 1; i <= iend_m; ++i)
            for (int j = jbeg_m; j <= jend_m; ++j) for (int k = kbeg_m; k <= kend_m; ++k) cp(k, i, j, k, nx - na, j);
        for (int j = jbeg_m; j <= na; ++j)
            for (int i = ibeg_m; i <= iend_m; ++i) for (int k = kbeg_m; k <= kend_m; ++k) cp(k, i, j, k, i, na + 1);
        for (int j = ny - na + 1; j <= jend_m; ++j)
            for (int i = ibeg_m; i <= iend_m; ++i) for (int k = kbeg_m; k <= kend_m; ++k) cp(k, i, j, k, i, ny - na);
        for (int j = jbeg_m; j <= jend_m; ++j)
            for (int i = ibeg_m; i <= iend_m; ++i) for (int k = nz - na + 1; k <= kend_m; ++k) cp(k, i, j, nz - na, i, j);
        // tau-method :192-207
        SP fmin = (SP)p.fq_min, fmax = (SP)p.fq_max, fref = (SP)p.fq_ref;
        visco_set_relaxtime(fmin, fmax);
        SP zeta = visco_constq_zeta(fmin, fmax);
        // (every point on its own: the set-up loops of this restatement run
        // in parallel to keep large grids' set-up short; the values are the
        // same as in serial order)
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < taup.d.size(); ++q) { taup.d[q] = nm * zeta / taup.d[q]; taus.d[q] = nm * zeta / taus.d[q]; }
        // relaxed_medium :231-271
        {
            typedef std::complex<SP> C;
            SP omega = (SP)(2 * PI_D * fref);
            C cc(0, 0);
            for (int m = 0; m < nm; ++m) {
                std::complex<double> ei(0.0, 1.0);
                std::complex<double> v = (ei * (double)omega * (double)ts[m]) / (1.0 - ei * (double)omega * (double)ts[m]);
                cc += C((SP)v.real(), (SP)v.imag());
            }
            cc = cc / (SP)nm;
#pragma omp parallel for schedule(static)
            for (size_t q = 0; q < mu.d.size(); ++q) {
                SP rb2 = mu.d[q], ra2 = lam.d[q] + 2 * mu.d[q];
                SP chi_mu = (SP)1.0 / (((SP)1.0) / std::sqrt(C(1, 0) - cc * taus.d[q])).real();
                SP chi_lam = (SP)1.0 / (((SP)1.0) / std::sqrt(C(1, 0) - cc * taup.d[q])).real();
                mu.d[q] = rb2 / (chi_mu * chi_mu);
                lam.d[q] = ra2 / (chi_lam * chi_lam) - 2 * mu.d[q];
            }
        }
        // surface_detection :339-394
        SP epsl = std::numeric_limits<float>::epsilon();
        kfs.alloc(ibeg_m, iend_m, jbeg_m, jend_m, kbeg - 1);
        kob.alloc(ibeg_m, iend_m, jbeg_m, jend_m, kbeg - 1);
        for (int j = jbeg - 1; j <= jend + 2; ++j)
            for (int i = ibeg - 1; i <= iend + 2; ++i)
                for (int k = kbeg; k <= kend - 1; ++k) {
                    if (std::abs(mu(k, i, j)) < epsl && std::abs(mu(k + 1, i, j)) > epsl) kob(i, j) = k;
                    if (std::abs(lam(k, i, j)) < epsl && std::abs(lam(k + 1, i, j)) > epsl) kfs(i, j) = k;
                }
        kfs_top.alloc(ibeg_m, iend_m, jbeg_m, jend_m, 0); kfs_bot = kfs_top; kob_top = kfs_top; kob_bot = kfs_top;
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i) {
                int fmn = 1 << 30, fmx = -(1 << 30), omn = 1 << 30, omx = -(1 << 30);
                for (int jj = j - 2; jj <= j + 3; ++jj)
                    for (int ii = i - 2; ii <= i + 3; ++ii) {
                        fmn = std::min(fmn, kfs(ii, jj)); fmx = std::max(fmx, kfs(ii, jj));
                        omn = std::min(omn, kob(ii, jj)); omx = std::max(omx, kob(ii, jj));
                    }
                kfs_top(i, j) = std::max(fmn - 2, kbeg); kfs_bot(i, j) = std::min(fmx + 2, kend);
                kob_top(i, j) = std::max(omn - 2, kbeg); kob_bot(i, j) = std::min(omx + 2, kend);
            }
        if (p.stabilize_pml) stabilize_absorber();
    }

    // src/swpc_3d/m_medium.f90:273-337 (with velocity_minmax :396-427)
    void stabilize_absorber() {
        float vmax = -1;
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i)
                for (int k = kfs(i, j) + 1; k <= kend; ++k)
                    vmax = std::max(vmax, (float)std::sqrt((lam(k, i, j) + 2 * mu(k, i, j)) / rho(k, i, j)));
        const float V_DYNAMIC_RANGE = 0.4f, vmin_pml = vmax * V_DYNAMIC_RANGE;
        const int LV_THICK = 20;
        auto ka = [&](int i, int j) { return (i <= na || nx - na + 1 <= i || j <= na || ny - na + 1 <= j) ? kbeg : kend - na + 1; };
        auto kmin = [&](int i, int j) {
            int m = 1 << 30;
            for (int jj = j - 2; jj <= j + 2; ++jj)
                for (int ii = i - 2; ii <= i + 2; ++ii) m = std::min(m, ka(ii, jj));
            return m;
        };
        for (int j = jbeg - 1; j <= jend + 1; ++j)
            for (int i = ibeg - 1; i <= iend + 1; ++i) {
                int k = kmin(i, j);
                while (k <= kend) {
                    if (lam(k, i, j) < lam(k - 1, i, j) || mu(k, i, j) < mu(k - 1, i, j)) {
                        int k2;
                        for (k2 = k + 1; k2 <= kend; ++k2)
                            if (lam(k2, i, j) > lam(k2 - 1, i, j) || mu(k2, i, j) > mu(k2 - 1, i, j)) break;
                        if (k2 - k <= LV_THICK) {
                            rho(k, i, j) = rho(k - 1, i, j); lam(k, i, j) = lam(k - 1, i, j); mu(k, i, j) = mu(k - 1, i, j);
                            taup(k, i, j) = taup(k - 1, i, j); taus(k, i, j) = taus(k - 1, i, j);
                            k = k2 - 1;
                        }
                    }
                    k = k + 1;
                }
            }
        const SP eps = std::numeric_limits<float>::epsilon(), gamma = std::sqrt((SP)3.0);
        for (int j = jbeg - 1; j <= jend + 1; ++j)
            for (int i = ibeg - 1; i <= iend + 1; ++i)
                for (int k = kmin(i, j); k <= kend; ++k) {
                    SP vs = std::sqrt(mu(k, i, j) / rho(k, i, j));
                    if (vs < eps) continue;
                    if (vs < (SP)vmin_pml) {
                        vs = (SP)vmin_pml;
                        const SP vp = vs * gamma;
                        lam(k, i, j) = rho(k, i, j) * (vp * vp - 2 * vs * vs);
                        mu(k, i, j) = rho(k, i, j) * (vs * vs);
                    }
                }
    }

    // src/swpc_3d/m_kernel.f90:30-73
    void kernel_setup() {
        rc40x = MP(17.0) / MP(16.0) / dx; rc40y = MP(17.0) / MP(16.0) / dy; rc40z = MP(17.0) / MP(16.0) / dz;
        rc41x = MP(1.0) / MP(48.0) / dx; rc41y = MP(1.0) / MP(48.0) / dy; rc41z = MP(1.0) / MP(48.0) / dz;
        rd40x = MP(-1.0) / MP(16.0) / dx; rd40y = MP(-1.0) / MP(16.0) / dy; rd40z = MP(-1.0) / MP(16.0) / dz;
        rd41x = MP(-1.0) / MP(48.0) / dx; rd41y = MP(-1.0) / MP(48.0) / dy; rd41z = MP(-1.0) / MP(48.0) / dz;
        int nk = kend_k - kbeg_k + 1, ni = iend_k - ibeg_k + 1, nj = jend_k - jbeg_k + 1;
        (void)nk; (void)ni; (void)nj;
        auto a4 = [&](std::vector<F3<SP>>& R) {
            R.resize(nm);
            for (auto& r : R) r.alloc(kbeg_k, kend_k, ibeg_k, iend_k, jbeg_k, jend_k);
        };
        a4(Rxx); a4(Ryy); a4(Rzz); a4(Ryz); a4(Rxz); a4(Rxy);
        c1.resize(nm); c2.resize(nm); d1.resize(nm);
        d2 = 0;
        for (int m = 0; m < nm; ++m) {
            c1[m] = (2 * ts[m] - dt) / (2 * ts[m] + dt);
            c2[m] = (SP)2 / (2 * ts[m] + dt) / (SP)nm;
        }
        for (int m = 0; m < nm; ++m) d2 += dt / (2 * ts[m] - dt);
        d2 = d2 / (SP)nm;
        for (int m = 0; m < nm; ++m) d1[m] = 2 * ts[m] / (2 * ts[m] - dt);
    }

    // src/swpc_3d/m_source.f90:41-314, 468-774 (xy formats)
    void source_setup(const std::string& inf_dir) {
        stf = stf_code(p.stftype);
        std::string fn = p.fn_stf;
        if (!fn.empty() && fn[0] != '/') fn = inf_dir + "/" + fn;
        auto rows = data_lines(fn);
        const std::string& f = p.stf_format;
        std::vector<SP> sx, sy, sz, mo, mxx, myy, mzz, myz, mxz, mxy, fx, fy, fz, t0, tr;
        SP phi = (SP)p.phi;
        for (auto& r : rows) {
            auto t = tokens(r);
            auto R = [&](size_t q) -> SP { if (q >= t.size()) throw std::runtime_error("short source line: " + r); return (SP)Ini::to_real(t[q]); };
            sx.push_back(R(0)); sy.push_back(R(1)); sz.push_back(R(2)); t0.push_back(R(3)); tr.push_back(R(4));
            if (p.bf_mode) {
                if (f.substr(0, 2) != "xy") throw std::runtime_error("only xy body-force sources are supported by the oracle");
                fx.push_back(R(5)); fy.push_back(R(6)); fz.push_back(R(7));
                continue;
            }
            SP m6[6] = {0, 0, 0, 0, 0, 0};  // xx yy zz yz xz xy
            SP m0v = 0;
            if (f == "xym0ij" || f == "xymwij") {
                m0v = R(5);
                for (int q = 0; q < 6; ++q) m6[q] = R(6 + q);
                if (f == "xymwij") m0v = (SP)std::pow((SP)10, (SP)1.5 * m0v + (SP)9.05);
            } else if (f == "xym0dc" || f == "xymwdc" || f == "xydsdc") {
                SP strike, dip, rake;
                if (f == "xydsdc") { strike = R(7); dip = R(8); rake = R(9); }
                else { m0v = R(5); strike = R(6); dip = R(7); rake = R(8); }
                if (f == "xymwdc") m0v = (SP)std::pow((SP)10, (SP)1.5 * m0v + (SP)9.05);
                sdr2moment(strike - phi, dip, rake, m6);
                if (f == "xydsdc") {
                    int is0 = x2i(sx.back(), xbeg, (SP)dx), js0 = x2i(sy.back(), ybeg, (SP)dy), ks0 = x2i(sz.back(), zbeg, (SP)dz);
                    SP D = R(5), S = R(6);
                    if (ibeg - 2 <= is0 && is0 <= iend + 3 && jbeg - 2 <= js0 && js0 <= jend + 3 && kbeg - 2 <= ks0 && ks0 <= kend + 3)
                        m0v = (SP)(((SP)1e9 * mu(ks0, is0, js0)) * (double)D * (double)S);
                    else m0v = 0;
                }
            } else {
                throw std::runtime_error("stf_format not supported by the oracle: " + f);
            }
            mo.push_back(m0v); mxx.push_back(m6[0]); myy.push_back(m6[1]); mzz.push_back(m6[2]);
            myz.push_back(m6[3]); mxz.push_back(m6[4]); mxy.push_back(m6[5]);
        }
        int ns = (int)sx.size();
        fcut = 0;
        for (int q = 0; q < ns; ++q) fcut = std::max(fcut, (float)((SP)1 / tr[q]));
        if (p.bf_mode) {
            SP s = 0;
            for (int q = 0; q < ns; ++q) s += fx[q] * fx[q] + fy[q] * fy[q] + fz[q] * fz[q];
            M0 = (float)std::sqrt(s);
            UC = UC * (float)std::pow(10.0f, 3);
        } else {
            SP s = 0;
            for (int q = 0; q < ns; ++q) s += mo[q];
            M0 = (float)s;
        }
        for (int q = 0; q < ns; ++q) {
            int is = x2i(sx[q], xbeg, (SP)dx), js = x2i(sy[q], ybeg, (SP)dy), ks = x2i(sz[q], zbeg, (SP)dz);
            if (!(ibeg - 2 <= is && is <= iend + 3 && jbeg - 2 <= js && js <= jend + 3 && kbeg - 2 <= ks && ks <= kend + 3)) continue;
            if (!(xbeg <= sx[q] && sx[q] <= xend && ybeg <= sy[q] && sy[q] <= yend && zbeg <= sz[q] && sz[q] <= zend))
                throw std::runtime_error("source outside the model space");
            Src s{};
            s.i = is; s.j = js; s.k = ks; s.tbeg = t0[q]; s.trise = tr[q];
            if (p.bf_mode) { s.fx = (MP)fx[q] / (MP)(SP)M0; s.fy = (MP)fy[q] / (MP)(SP)M0; s.fz = (MP)fz[q] / (MP)(SP)M0; }
            else {
                s.mo = (MP)mo[q] / (MP)(SP)M0;
                s.mxx = mxx[q]; s.myy = myy[q]; s.mzz = mzz[q]; s.myz = myz[q]; s.mxz = mxz[q]; s.mxy = mxy[q];
            }
            src.push_back(s);
        }
        dt_dxyz = (MP)dt / (dx * dy * dz);
    }

    // src/shared/m_fdtool.f90:307-336
    static void sdr2moment(SP strike, SP dip, SP rake, SP m6[6]) {
        auto d2r = [](SP d) { return (SP)(PI_D / 180.0 * (double)d); };
        SP sind = std::sin(d2r(dip)), cosd = std::cos(d2r(dip)), sin2d = std::sin(d2r(2 * dip)), cos2d = std::cos(d2r(2 * dip));
        SP sinl = std::sin(d2r(rake)), cosl = std::cos(d2r(rake));
        SP sinf = std::sin(d2r(strike)), cosf = std::cos(d2r(strike)), sin2f = std::sin(d2r(2 * strike)), cos2f = std::cos(d2r(2 * strike));
        m6[0] = -(sind * cosl * sin2f + sin2d * sinl * sinf * sinf);
        m6[5] = (sind * cosl * cos2f + sin2d * sinl * sin2f / 2);
        m6[4] = -(cosd * cosl * cosf + cos2d * sinl * sinf);
        m6[1] = (sind * cosl * sin2f - sin2d * sinl * cosf * cosf);
        m6[3] = -(cosd * cosl * sinf - cos2d * sinl * cosf);
        m6[2] = (sin2d * sinl);
    }

    // src/swpc_3d/m_absorb_p.f90:533-573
    void damping_profile(SP x, SP H, SP xb, SP xe, SP* g) {
        SP R0 = std::pow((SP)10, -(std::log10((SP)na) - 1) / std::log10((SP)2.0) - (SP)3.0);
        SP d0 = -((SP)1.0 / ((SP)2.0 * H)) * (SP)2 * (SP)6.0 * std::log(R0);
        SP b0 = 7.0, a0 = (SP)(PI_D * (double)(SP)fcut);
        SP xx;
        if (x <= xb + H) xx = (xb + H) - x;
        else if (x >= xe - H) xx = x - (xe - H);
        else xx = 0;
        SP r = std::abs(xx / H);
        SP d = d0 * r, a = a0 * (1 - r), b = 1 + (b0 - 1) * (r * r);
        SP h = dt / (SP)2.0;
        g[0] = ((1 + h * a) / b) / (1 + h * (a + d / b));
        g[1] = ((SP)-1.0 / b) / (1 + h * (a + d / b));
        g[2] = (1 - h * (a + d / b)) / (1 + h * (a + d / b));
        g[3] = (d / b) / (1 + h * (a + d / b));
    }

    // m_absorb_p.f90:60-124 / m_absorb_c.f90:27-111
    void absorb_setup() {
        if (pml) {
            r20x = (MP)1.0 / dx; r20y = (MP)1.0 / dy; r20z = (MP)1.0 / dz;
            gxc.assign(4 * nx, 0); gxe.assign(4 * nx, 0); gyc.assign(4 * ny, 0); gye.assign(4 * ny, 0); gzc.assign(4 * nz, 0); gze.assign(4 * nz, 0);
            SP hx = na * (SP)dx, hy = na * (SP)dy, hz = na * (SP)dz;
            for (int i = 1; i <= nx; ++i) {
                damping_profile(xc[i - ibeg_m], hx, xbeg, xend, &gxc[4 * (i - 1)]);
                damping_profile(xc[i - ibeg_m] + (SP)dx / (SP)2.0, hx, xbeg, xend, &gxe[4 * (i - 1)]);
            }
            for (int j = 1; j <= ny; ++j) {
                damping_profile(yc[j - jbeg_m], hy, ybeg, yend, &gyc[4 * (j - 1)]);
                damping_profile(yc[j - jbeg_m] + (SP)dy / (SP)2.0, hy, ybeg, yend, &gye[4 * (j - 1)]);
            }
            for (int k = 1; k <= nz; ++k) {
                damping_profile(zc[k - kbeg_m], hz, zbeg, zend, &gzc[4 * (k - 1)]);
                damping_profile(zc[k - kbeg_m] + (SP)dz / (SP)2.0, hz, zbeg, zend, &gze[4 * (k - 1)]);
            }
            int kmin = 1 << 30;
            for (int v : kbeg_a.d) kmin = std::min(kmin, v);
            for (F3<SP>* a : {&axVx, &ayVx, &azVx, &axVy, &ayVy, &azVy, &axVz, &ayVz, &azVz,
                              &axSxx, &aySxy, &azSxz, &axSxy, &aySyy, &azSyz, &axSxz, &aySyz, &azSzz})
                a->alloc(kmin, kend, ibeg, iend, jbeg, jend);
        } else {
            const SP alpha = (SP)0.09;
            gx_c.assign(nx + 7, 1); gx_b.assign(nx + 7, 1); gy_c.assign(ny + 7, 1); gy_b.assign(ny + 7, 1); gz_c.assign(nz + 7, 1); gz_b.assign(nz + 7, 1);
            SP Lx = na * (SP)dx, Ly = na * (SP)dy, Lz = na * (SP)dz;
            auto sq = [](SP v) { return v * v; };
            for (int i = 1; i <= nx; ++i) {
                SP* c = &gx_c[i + 3]; SP* b = &gx_b[i + 3];
                if (i <= na) {
                    *c = std::exp(-alpha * sq(1 - i2x(i, 0, (SP)dx) / Lx));
                    *b = std::exp(-alpha * sq(1 - (i2x(i, 0, (SP)dx) + (SP)dx / 2) / Lx));
                } else if (i >= nx - na + 1) {
                    *c = std::exp(-alpha * sq(1 - (i2x(i, nx * (SP)dx, -(SP)dx) + (SP)dx / 2) / Lx));
                    *b = std::exp(-alpha * sq(1 - i2x(i, nx * (SP)dx, -(SP)dx) / Lx));
                }
            }
            for (int j = 1; j <= ny; ++j) {
                SP* c = &gy_c[j + 3]; SP* b = &gy_b[j + 3];
                if (j <= na) {
                    *c = std::exp(-alpha * sq(1 - i2x(j, 0, (SP)dy) / Ly));
                    *b = std::exp(-alpha * sq(1 - (i2x(j, 0, (SP)dy) + (SP)dy / 2) / Ly));
                } else if (j >= ny - na + 1) {
                    *c = std::exp(-alpha * sq(1 - (i2x(j, ny * (SP)dy, -(SP)dy) + (SP)dy / 2) / Ly));
                    *b = std::exp(-alpha * sq(1 - i2x(j, ny * (SP)dy, -(SP)dy) / Ly));
                }
            }
            for (int k = 1; k <= nz; ++k) {
                SP* c = &gz_c[k + 3]; SP* b = &gz_b[k + 3];
                if (k >= nz - na + 1) {
                    *c = std::exp(-alpha * sq(1 - (i2x(k, nz * (SP)dz, -(SP)dz) + (SP)dz / 2) / Lz));
                    *b = std::exp(-alpha * sq(1 - i2x(k, nz * (SP)dz, -(SP)dz) / Lz));
                }
            }
        }
    }

    // src/swpc_3d/m_wav.f90:54-271 (xy station format)
    struct StaPos { int i, j, k; std::string name; SP x, y; };
    std::vector<StaPos> sta_all;  // every station inside the model (the green_stnm look-up)

    void wav_setup(const std::string& inf_dir) {
        const bool rec = p.sw_wav_v || p.sw_wav_u || p.sw_wav_stress || p.sw_wav_strain;
        if (!rec && !p.green_mode) { nst = 0; return; }
        ntw = (int)std::floor((float)(p.nt - 1) / (float)p.ntdec_w + 1.0f);
        std::string fn = p.fn_stloc;
        if (!fn.empty() && fn[0] != '/') fn = inf_dir + "/" + fn;
        std::vector<std::string> rows;
        try { rows = data_lines(fn); } catch (...) { nst = 0; return; }
        if (p.st_format != "xy") throw std::runtime_error("only xy station files are supported by the oracle");
        for (auto& r : rows) {
            auto t = tokens(r);
            if (t.size() < 5) throw std::runtime_error("bad station line: " + r);
            SP xs = (SP)Ini::to_real(t[0]), ys = (SP)Ini::to_real(t[1]), zs = (SP)Ini::to_real(t[2]);
            std::string nm8 = t[3].substr(0, 8), zsw = t[4].substr(0, 3);
            int is = x2i(xs, xbeg, (SP)dx), js = x2i(ys, ybeg, (SP)dy), ks = x2i(zs, zbeg, (SP)dz);
            if (i2x(1, xbeg, (SP)dx) < xs && xs < i2x(nx, xbeg, (SP)dx) && i2x(1, ybeg, (SP)dy) < ys && ys < i2x(ny, ybeg, (SP)dy) &&
                kbeg < ks && ks < kend) {
                if (zsw == "dep") ks = x2i(zs, zbeg, (SP)dz);
                else if (zsw == "fsb") ks = kfs(is, js) + 1;
                else if (zsw == "obb") ks = kob(is, js) + 1;
                else if (zsw == "oba") ks = kob(is, js) - 1;
                else ks = x2i(zs, zbeg, (SP)dz);
                if (ks > kend) ks = kend - 1;
                if (ks < kbeg) ks = kbeg + 1;
                sta_all.push_back(StaPos{is, js, ks, nm8, xs, ys});
                if (rec) sta.push_back(Sta{is, js, ks, nm8});
            }
        }
        nst = (int)sta.size();
        if (!rec) return;
        if (p.sw_wav_v) wav_vel.assign((size_t)ntw * 3 * nst, 0);
        if (p.sw_wav_u) wav_disp.assign((size_t)ntw * 3 * nst, 0);
        if (p.sw_wav_stress) wav_stress.assign((size_t)ntw * 6 * nst, 0);
        if (p.sw_wav_strain) wav_strain.assign((size_t)ntw * 6 * nst, 0);
        ux.assign(nst, 0); uy.assign(nst, 0); uz.assign(nst, 0);
        exx.assign(nst, 0); eyy.assign(nst, 0); ezz.assign(nst, 0); eyz.assign(nst, 0); exz.assign(nst, 0); exy.assign(nst, 0);
        r40x = MP(9.0) / MP(8.0) / dx; r40y = MP(9.0) / MP(8.0) / dy; r40z = MP(9.0) / MP(8.0) / dz;
        r41x = MP(1.0) / MP(24.0) / dx; r41y = MP(1.0) / MP(24.0) / dy; r41z = MP(1.0) / MP(24.0) / dz;
    }

    // src/swpc_3d/m_snap.f90:95-207
    void snap_setup() {
        nxs = (nx + p.idec / 2) / p.idec;
        nys = (ny + p.jdec / 2) / p.jdec;
        const int nzs = (nz + p.kdec / 2) / p.kdec;
        k0_xy = x2i((SP)p.z0_xy, zbeg, (SP)dz);
        const int i0 = x2i((SP)p.x0_yz, xbeg, (SP)dx), j0 = x2i((SP)p.y0_xz, ybeg, (SP)dy);
        for (int sec = 0; sec < 5; ++sec)
            for (int kind = 0; kind < 3; ++kind) {
                if (!(p.snap_sw[sec] >> kind & 1)) continue;
                OSnap o;
                o.sec = sec; o.kind = kind;
                if (sec == 1) { o.n1 = nys; o.n2 = nzs; o.d1 = p.jdec; o.d2 = p.kdec; o.fix = i0; }
                else if (sec == 2) { o.n1 = nxs; o.n2 = nzs; o.d1 = p.idec; o.d2 = p.kdec; o.fix = j0; }
                else { o.n1 = nxs; o.n2 = nys; o.d1 = p.idec; o.d2 = p.jdec; o.fix = k0_xy; }
                if (kind == 1) o.ubuf.assign((size_t)3 * o.n1 * o.n2, 0.0);
                snaps.push_back(std::move(o));
            }
    }

    // ------------------------------------------------------------------
    // time step (src/swpc_3d/main.f90:119-139)
    // ------------------------------------------------------------------
    void step(int it) override {
        if (p.ntdec_r > 0 && it % p.ntdec_r == 0) vmax(it);
        green_store(it);
        wav_store(it);
        snap_write(it);
        update_stress();
        if (pml) pml_stress(); else cerjan_stress();
        stressglut(it);
        comm_stress();
        update_vel();
        if (pml) pml_vel(); else cerjan_vel();
        bodyforce(it);
        green_source(it);
        comm_vel();
        nt_done = it;
    }

    MP coef_sel(int isign, MP rc, MP rd) const { return rc + isign * rd; }
    int band_sign(int k, int i, int j) const {
        long a = (long)(k - kfs_top(i, j)) * (kfs_bot(i, j) - k);
        long b = (long)(k - kob_top(i, j)) * (kob_bot(i, j) - k);
        return fsign1(std::max(a, b));
    }

    // src/swpc_3d/m_kernel.f90:75-140
    void update_vel() {
#pragma omp parallel for schedule(static, 1)
        for (int j = jbeg_k; j <= jend_k; ++j)
            for (int i = ibeg_k; i <= iend_k; ++i)
                for (int k = kbeg_k; k <= kend_k; ++k) {
                    int s = band_sign(k, i, j);
                    MP e40x = coef_sel(s, rc40x, rd40x), e41x = coef_sel(s, rc41x, rd41x);
                    MP e40y = coef_sel(s, rc40y, rd40y), e41y = coef_sel(s, rc41y, rd41y);
                    MP e40z = coef_sel(s, rc40z, rd40z), e41z = coef_sel(s, rc41z, rd41z);
                    MP d3Sx3 = (Sxx(k, i + 1, j) - Sxx(k, i, j)) * e40x - (Sxx(k, i + 2, j) - Sxx(k, i - 1, j)) * e41x
                             + (Sxy(k, i, j) - Sxy(k, i, j - 1)) * e40y - (Sxy(k, i, j + 1) - Sxy(k, i, j - 2)) * e41y
                             + (Sxz(k, i, j) - Sxz(k - 1, i, j)) * e40z - (Sxz(k + 1, i, j) - Sxz(k - 2, i, j)) * e41z;
                    MP d3Sy3 = (Sxy(k, i, j) - Sxy(k, i - 1, j)) * e40x - (Sxy(k, i + 1, j) - Sxy(k, i - 2, j)) * e41x
                             + (Syy(k, i, j + 1) - Syy(k, i, j)) * e40y - (Syy(k, i, j + 2) - Syy(k, i, j - 1)) * e41y
                             + (Syz(k, i, j) - Syz(k - 1, i, j)) * e40z - (Syz(k + 1, i, j) - Syz(k - 2, i, j)) * e41z;
                    MP d3Sz3 = (Sxz(k, i, j) - Sxz(k, i - 1, j)) * e40x - (Sxz(k, i + 1, j) - Sxz(k, i - 2, j)) * e41x
                             + (Syz(k, i, j) - Syz(k, i, j - 1)) * e40y - (Syz(k, i, j + 1) - Syz(k, i, j - 2)) * e41y
                             + (Szz(k + 1, i, j) - Szz(k, i, j)) * e40z - (Szz(k + 2, i, j) - Szz(k - 1, i, j)) * e41z;
                    SP two = 2.0;
                    Vx(k, i, j) = Vx(k, i, j) + (MP)(two / (rho(k, i, j) + rho(k, i + 1, j))) * d3Sx3 * (MP)dt;
                    Vy(k, i, j) = Vy(k, i, j) + (MP)(two / (rho(k, i, j) + rho(k, i, j + 1))) * d3Sy3 * (MP)dt;
                    Vz(k, i, j) = Vz(k, i, j) + (MP)(two / (rho(k, i, j) + rho(k + 1, i, j))) * d3Sz3 * (MP)dt;
                }
    }

    // src/swpc_3d/m_kernel.f90:142-348
    void update_stress() {
        const SP epsl = std::numeric_limits<float>::epsilon();
#pragma omp parallel for schedule(static, 1)
        for (int j = jbeg_k; j <= jend_k; ++j)
            for (int i = ibeg_k; i <= iend_k; ++i)
                for (int k = kbeg_k; k <= kend_k; ++k) {
                    int s = band_sign(k, i, j);
                    MP e40x = coef_sel(s, rc40x, rd40x), e41x = coef_sel(s, rc41x, rd41x);
                    MP e40y = coef_sel(s, rc40y, rd40y), e41y = coef_sel(s, rc41y, rd41y);
                    MP e40z = coef_sel(s, rc40z, rd40z), e41z = coef_sel(s, rc41z, rd41z);
                    MP dxVx = (Vx(k, i, j) - Vx(k, i - 1, j)) * e40x - (Vx(k, i + 1, j) - Vx(k, i - 2, j)) * e41x;
                    MP dyVy = (Vy(k, i, j) - Vy(k, i, j - 1)) * e40y - (Vy(k, i, j + 1) - Vy(k, i, j - 2)) * e41y;
                    MP dzVz = (Vz(k, i, j) - Vz(k - 1, i, j)) * e40z - (Vz(k + 1, i, j) - Vz(k - 2, i, j)) * e41z;
                    SP mu2 = 2 * mu(k, i, j), lam2mu = lam(k, i, j) + mu2;
                    SP taup1 = taup(k, i, j), taus1 = taus(k, i, j);
                    SP d3v3 = (SP)(dxVx + dyVy + dzVz);
                    SP dyVy_dzVz = (SP)(dyVy + dzVz), dxVx_dzVz = (SP)(dxVx + dzVz), dxVx_dyVy = (SP)(dxVx + dyVy);
                    SP Rxx_n = 0, Ryy_n = 0, Rzz_n = 0;
                    for (int m = 0; m < nm; ++m) {
                        SP& rxx = Rxx[m](k, i, j); SP& ryy = Ryy[m](k, i, j); SP& rzz = Rzz[m](k, i, j);
                        rxx = c1[m] * rxx - c2[m] * (lam2mu * taup1 * d3v3 - mu2 * taus1 * dyVy_dzVz) * dt;
                        ryy = c1[m] * ryy - c2[m] * (lam2mu * taup1 * d3v3 - mu2 * taus1 * dxVx_dzVz) * dt;
                        rzz = c1[m] * rzz - c2[m] * (lam2mu * taup1 * d3v3 - mu2 * taus1 * dxVx_dyVy) * dt;
                        Rxx_n = Rxx_n + d1[m] * rxx; Ryy_n = Ryy_n + d1[m] * ryy; Rzz_n = Rzz_n + d1[m] * rzz;
                    }
                    SP tp1 = 1 + taup1 * (1 + d2), ts1 = 1 + taus1 * (1 + d2);
                    Sxx(k, i, j) = Sxx(k, i, j) + (MP)((lam2mu * tp1 * d3v3 - mu2 * ts1 * dyVy_dzVz + Rxx_n) * dt);
                    Syy(k, i, j) = Syy(k, i, j) + (MP)((lam2mu * tp1 * d3v3 - mu2 * ts1 * dxVx_dzVz + Ryy_n) * dt);
                    Szz(k, i, j) = Szz(k, i, j) + (MP)((lam2mu * tp1 * d3v3 - mu2 * ts1 * dxVx_dyVy + Rzz_n) * dt);
                }
#pragma omp parallel for schedule(static, 1)
        for (int j = jbeg_k; j <= jend_k; ++j)
            for (int i = ibeg_k; i <= iend_k; ++i)
                for (int k = kbeg_k; k <= kend_k; ++k) {
                    int s = band_sign(k, i, j);
                    MP e40x = coef_sel(s, rc40x, rd40x), e41x = coef_sel(s, rc41x, rd41x);
                    MP e40y = coef_sel(s, rc40y, rd40y), e41y = coef_sel(s, rc41y, rd41y);
                    MP e40z = coef_sel(s, rc40z, rd40z), e41z = coef_sel(s, rc41z, rd41z);
                    MP dxVy_dyVx = (Vy(k, i + 1, j) - Vy(k, i, j)) * e40x - (Vy(k, i + 2, j) - Vy(k, i - 1, j)) * e41x
                                 + (Vx(k, i, j + 1) - Vx(k, i, j)) * e40y - (Vx(k, i, j + 2) - Vx(k, i, j - 1)) * e41y;
                    MP dxVz_dzVx = (Vz(k, i + 1, j) - Vz(k, i, j)) * e40x - (Vz(k, i + 2, j) - Vz(k, i - 1, j)) * e41x
                                 + (Vx(k + 1, i, j) - Vx(k, i, j)) * e40z - (Vx(k + 2, i, j) - Vx(k - 1, i, j)) * e41z;
                    MP dyVz_dzVy = (Vz(k, i, j + 1) - Vz(k, i, j)) * e40y - (Vz(k, i, j + 2) - Vz(k, i, j - 1)) * e41y
                                 + (Vy(k + 1, i, j) - Vy(k, i, j)) * e40z - (Vy(k + 2, i, j) - Vy(k - 1, i, j)) * e41z;
                    SP muxz, muxy, muyz;
                    hmeans(k, i, j, epsl, muxz, muxy, muyz);
                    SP taus1 = taus(k, i, j);
                    SP ryz_n = 0, rxz_n = 0, rxy_n = 0;
                    for (int m = 0; m < nm; ++m) {
                        SP& ryz = Ryz[m](k, i, j); SP& rxz = Rxz[m](k, i, j); SP& rxy = Rxy[m](k, i, j);
                        ryz = (SP)(c1[m] * ryz - (MP)(c2[m] * muyz * taus1) * dyVz_dzVy * (MP)dt);
                        rxz = (SP)(c1[m] * rxz - (MP)(c2[m] * muxz * taus1) * dxVz_dzVx * (MP)dt);
                        rxy = (SP)(c1[m] * rxy - (MP)(c2[m] * muxy * taus1) * dxVy_dyVx * (MP)dt);
                        ryz_n = ryz_n + d1[m] * ryz; rxz_n = rxz_n + d1[m] * rxz; rxy_n = rxy_n + d1[m] * rxy;
                    }
                    SP ts1 = 1 + taus1 * (1 + d2);
                    Syz(k, i, j) = Syz(k, i, j) + ((MP)(muyz * ts1) * dyVz_dzVy + (MP)ryz_n) * (MP)dt;
                    Sxz(k, i, j) = Sxz(k, i, j) + ((MP)(muxz * ts1) * dxVz_dzVx + (MP)rxz_n) * (MP)dt;
                    Sxy(k, i, j) = Sxy(k, i, j) + ((MP)(muxy * ts1) * dxVy_dyVx + (MP)rxy_n) * (MP)dt;
                }
    }

    // harmonic averages of mu: m_kernel.f90:293-309 (identical in m_absorb_p.f90:486-502)
    void hmeans(int k, int i, int j, SP epsl, SP& muxz, SP& muxy, SP& muyz) const {
        SP a = mu(k, i, j), b = mu(k + 1, i, j), c = mu(k, i + 1, j), d = mu(k + 1, i + 1, j);
        muxz = 4 * a * b * c * d / (a * b * c + a * b * d + a * c * d + b * c * d + epsl);
        SP e = mu(k, i, j + 1), f = mu(k, i + 1, j + 1);
        muxy = 4 * a * c * e * f / (a * c * e + a * c * f + a * e * f + c * e * f + epsl);
        SP g = mu(k + 1, i, j + 1);
        muyz = 4 * a * b * e * g / (a * b * e + a * b * g + a * e * g + b * e * g + epsl);
    }

    // src/swpc_3d/m_absorb_p.f90:126-317 (pw_mode ghost extrapolation excluded)
    // m_absorb_p.f90:137-244 / 332-427: lateral ghost planes extrapolated
    // linearly in plane-wave mode (x sides for j = 1..ny, then y sides for
    // i = 1..nx, k = 1..nz)
    void pw_ghosts(std::initializer_list<F3<MP>*> fs) {
        for (F3<MP>* f : fs) {
            F3<MP>& A = *f;
            for (int j = jbeg; j <= jend; ++j)
                for (int k = 1; k <= nz; ++k) {
                    A(k, 0, j) = 2 * A(k, 1, j) - A(k, 2, j);
                    A(k, nx + 1, j) = 2 * A(k, nx, j) - A(k, nx - 1, j);
                }
            for (int i = ibeg; i <= iend; ++i)
                for (int k = 1; k <= nz; ++k) {
                    A(k, i, 0) = 2 * A(k, i, 1) - A(k, i, 2);
                    A(k, i, ny + 1) = 2 * A(k, i, ny) - A(k, i, ny - 1);
                }
        }
    }

    // m_source.f90:316-466
    void pw_setup() {
        const SP d2r = (SP)(PI_D / 180.0);
        const SP dipr = (SP)p.pw_dip * d2r, strr = (SP)p.pw_strike * d2r, rakr = (SP)p.pw_rake * d2r;
        const SP sd = std::sin(dipr), cd = std::cos(dipr), sf = std::sin(strr), cf = std::cos(strr);
        const SP sl = std::sin(rakr), cl = std::cos(rakr), c2d = std::cos(2 * dipr), c2f = std::cos(2 * strr);
        const bool P = p.pw_ps == "p" || p.pw_ps == "P";
        const int stt = stf_code(p.stftype);
        const SP zt = (SP)p.pw_ztop, zl = (SP)p.pw_zlen, eps = std::numeric_limits<float>::epsilon();
        for (int j = jbeg_m; j <= jend_m; ++j)
            for (int i = ibeg_m; i <= iend_m; ++i)
                for (int k = kbeg_m; k <= kend_m; ++k) {
                    const SP v = P ? std::sqrt((lam(k, i, j) + 2 * mu(k, i, j)) / rho(k, i, j)) : std::sqrt(mu(k, i, j) / rho(k, i, j));
                    if (v < eps) continue;
                    const SP x0 = xbeg + (SP)(i - (SP)0.5) * (SP)dx, y0 = ybeg + (SP)(j - (SP)0.5) * (SP)dy;
                    const SP z0 = zbeg + (SP)(k - (SP)0.5) * (SP)dz - zt;
                    const SP x1 = x0 + (SP)dx / (SP)2, y1 = y0 + (SP)dy / (SP)2, z1 = z0 + (SP)dz / (SP)2;
                    const SP sh = dt / (SP)2 * v;
                    auto m = [&](SP a) { return momentrate<SP>(a, stt, (SP)0, zl); };
                    const SP s_ii = m(sd * sf * x0 - sd * cf * y0 + cd * z0);
                    const SP s_vx = m(sd * sf * x1 - sd * cf * y0 + cd * z0 + sh);
                    const SP s_vy = m(sd * sf * x0 - sd * cf * y1 + cd * z0 + sh);
                    const SP s_vz = m(sd * sf * x0 - sd * cf * y0 + cd * z1 + sh);
                    const SP s_yz = m(sd * sf * x0 - sd * cf * y1 + cd * z1);
                    const SP s_xz = m(sd * sf * x1 - sd * cf * y0 + cd * z1);
                    const SP s_xy = m(sd * sf * x1 - sd * cf * y1 + cd * z0);
                    const SP la0 = lam(k, i, j), mu0 = mu(k, i, j);
                    if (P) {
                        Vx(k, i, j) = -sd * sf * s_vx; Vy(k, i, j) = sd * cf * s_vy; Vz(k, i, j) = -cd * s_vz;
                        Sxx(k, i, j) = -(la0 + 2 * mu0 * sd * sd * sf * sf) * s_ii / v;
                        Syy(k, i, j) = -(la0 + 2 * mu0 * sd * sd * cf * cf) * s_ii / v;
                        Szz(k, i, j) = -(la0 + 2 * mu0 * cd * cd) * s_ii / v;
                        Syz(k, i, j) = 2 * mu0 * sd * cd * cf * s_yz / v;
                        Sxz(k, i, j) = -2 * mu0 * sd * cd * sf * s_xz / v;
                        Sxy(k, i, j) = 2 * mu0 * sd * cd * sf * s_xy / v;
                    } else {
                        Vx(k, i, j) = (cl * cf + sl * cd * sf) * s_vx; Vy(k, i, j) = (cl * sf - sl * cd * cf) * s_vy;
                        Vz(k, i, j) = -sl * sd * s_vz;
                        Sxx(k, i, j) = 2 * mu0 * sd * sf * (cl * cf + sl * cd * sf) * s_ii / v;
                        Syy(k, i, j) = -2 * mu0 * sd * cf * (cl * sf - sl * cd * cf) * s_ii / v;
                        Szz(k, i, j) = -2 * mu0 * cd * sl * sd * s_ii / v;
                        Syz(k, i, j) = mu0 * (cl * cd * sf - sl * c2d * cf) * s_yz / v;
                        Sxz(k, i, j) = mu0 * (cl * cd * cf + sl * c2d * sf) * s_xz / v;
                        Sxy(k, i, j) = -mu0 * (cl * sd * c2f + 2 * sl * sd * cd * sf * cf) * s_xy / v;
                    }
                }
        const int ic = x2i((xbeg + xend) / 2, xbeg, (SP)dx), jc = x2i((ybeg + yend) / 2, ybeg, (SP)dy);
        const int kc = x2i(zt, zbeg, (SP)dz);
        fcut = 0;
        if (ibeg <= ic && ic <= iend && jbeg <= jc && jc <= jend)
            fcut = (float)((P ? std::sqrt((lam(kc, ic, jc) + 2 * mu(kc, ic, jc)) / rho(kc, ic, jc))
                              : std::sqrt(mu(kc, ic, jc) / rho(kc, ic, jc))) / zl);
        M0 = 1.0f / UC;  // fictitious moment for output
    }

    void pml_vel() {
        if (p.pw_mode) pw_ghosts({&Sxx, &Syy, &Szz, &Syz, &Sxz, &Sxy});
#pragma omp parallel for schedule(dynamic)
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i)
                for (int k = kbeg_a(i, j); k <= kend; ++k) {
                    MP dxSxx = (Sxx(k, i + 1, j) - Sxx(k, i, j)) * r20x;
                    MP dySyy = (Syy(k, i, j + 1) - Syy(k, i, j)) * r20y;
                    MP dzSzz = (Szz(k + 1, i, j) - Szz(k, i, j)) * r20z;
                    MP dySyz = (Syz(k, i, j) - Syz(k, i, j - 1)) * r20y;
                    MP dzSyz = (Syz(k, i, j) - Syz(k - 1, i, j)) * r20z;
                    MP dxSxz = (Sxz(k, i, j) - Sxz(k, i - 1, j)) * r20x;
                    MP dzSxz = (Sxz(k, i, j) - Sxz(k - 1, i, j)) * r20z;
                    MP dxSxy = (Sxy(k, i, j) - Sxy(k, i - 1, j)) * r20x;
                    MP dySxy = (Sxy(k, i, j) - Sxy(k, i, j - 1)) * r20y;
                    SP two = 2.0;
                    SP bx = two / (rho(k, i, j) + rho(k, i + 1, j));
                    SP by = two / (rho(k, i, j) + rho(k, i, j + 1));
                    SP bz = two / (rho(k, i, j) + rho(k + 1, i, j));
                    SP* gxe_ = &gxe[4 * (i - 1)]; SP* gxc_ = &gxc[4 * (i - 1)];
                    SP* gye_ = &gye[4 * (j - 1)]; SP* gyc_ = &gyc[4 * (j - 1)];
                    SP* gze_ = &gze[4 * (k - 1)]; SP* gzc_ = &gzc[4 * (k - 1)];
                    Vx(k, i, j) = Vx(k, i, j) + (MP)(bx * (SP)(gxe_[0] * dxSxx + gyc_[0] * dySxy + gzc_[0] * dzSxz
                                     + (MP)(gxe_[1] * axSxx(k, i, j)) + (MP)(gyc_[1] * aySxy(k, i, j)) + (MP)(gzc_[1] * azSxz(k, i, j))) * dt);
                    Vy(k, i, j) = Vy(k, i, j) + (MP)(by * (SP)(gxc_[0] * dxSxy + gye_[0] * dySyy + gzc_[0] * dzSyz
                                     + (MP)(gxc_[1] * axSxy(k, i, j)) + (MP)(gye_[1] * aySyy(k, i, j)) + (MP)(gzc_[1] * azSyz(k, i, j))) * dt);
                    Vz(k, i, j) = Vz(k, i, j) + (MP)(bz * (SP)(gxc_[0] * dxSxz + gyc_[0] * dySyz + gze_[0] * dzSzz
                                     + (MP)(gxc_[1] * axSxz(k, i, j)) + (MP)(gyc_[1] * aySyz(k, i, j)) + (MP)(gze_[1] * azSzz(k, i, j))) * dt);
                    axSxx(k, i, j) = gxe_[2] * axSxx(k, i, j) + gxe_[3] * (SP)dxSxx * dt;
                    aySxy(k, i, j) = gyc_[2] * aySxy(k, i, j) + gyc_[3] * (SP)dySxy * dt;
                    azSxz(k, i, j) = gzc_[2] * azSxz(k, i, j) + gzc_[3] * (SP)dzSxz * dt;
                    axSxy(k, i, j) = gxc_[2] * axSxy(k, i, j) + gxc_[3] * (SP)dxSxy * dt;
                    aySyy(k, i, j) = gye_[2] * aySyy(k, i, j) + gye_[3] * (SP)dySyy * dt;
                    azSyz(k, i, j) = gzc_[2] * azSyz(k, i, j) + gzc_[3] * (SP)dzSyz * dt;
                    axSxz(k, i, j) = gxc_[2] * axSxz(k, i, j) + gxc_[3] * (SP)dxSxz * dt;
                    aySyz(k, i, j) = gyc_[2] * aySyz(k, i, j) + gyc_[3] * (SP)dySyz * dt;
                    azSzz(k, i, j) = gze_[2] * azSzz(k, i, j) + gze_[3] * (SP)dzSzz * dt;
                }
    }

    // src/swpc_3d/m_absorb_p.f90:319-531
    void pml_stress() {
        if (p.pw_mode) pw_ghosts({&Vx, &Vy, &Vz});
        const SP epsl = std::numeric_limits<float>::epsilon();
#pragma omp parallel for schedule(dynamic)
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i) {
                SP* gxe_ = &gxe[4 * (i - 1)]; SP* gxc_ = &gxc[4 * (i - 1)];
                SP* gye_ = &gye[4 * (j - 1)]; SP* gyc_ = &gyc[4 * (j - 1)];
                for (int k = kbeg_a(i, j); k <= kend; ++k) {
                    SP* gzc_ = &gzc[4 * (k - 1)];
                    MP dxVx = (Vx(k, i, j) - Vx(k, i - 1, j)) * r20x;
                    MP dyVy = (Vy(k, i, j) - Vy(k, i, j - 1)) * r20y;
                    MP dzVz = (Vz(k, i, j) - Vz(k - 1, i, j)) * r20z;
                    SP lam2mu_R = lam(k, i, j) + 2 * mu(k, i, j);
                    SP lam_R = lam2mu_R - 2 * mu(k, i, j);
                    SP dxVx_ade = gxc_[0] * (SP)dxVx + gxc_[1] * axVx(k, i, j);
                    SP dyVy_ade = gyc_[0] * (SP)dyVy + gyc_[1] * ayVy(k, i, j);
                    SP dzVz_ade = gzc_[0] * (SP)dzVz + gzc_[1] * azVz(k, i, j);
                    Sxx(k, i, j) = Sxx(k, i, j) + (MP)((lam2mu_R * dxVx_ade + lam_R * (dyVy_ade + dzVz_ade)) * dt);
                    Syy(k, i, j) = Syy(k, i, j) + (MP)((lam2mu_R * dyVy_ade + lam_R * (dxVx_ade + dzVz_ade)) * dt);
                    Szz(k, i, j) = Szz(k, i, j) + (MP)((lam2mu_R * dzVz_ade + lam_R * (dxVx_ade + dyVy_ade)) * dt);
                    axVx(k, i, j) = gxc_[2] * axVx(k, i, j) + gxc_[3] * (SP)dxVx * dt;
                    ayVy(k, i, j) = gyc_[2] * ayVy(k, i, j) + gyc_[3] * (SP)dyVy * dt;
                    azVz(k, i, j) = gzc_[2] * azVz(k, i, j) + gzc_[3] * (SP)dzVz * dt;
                }
                for (int k = kbeg_a(i, j); k <= kend; ++k) {
                    SP* gze_ = &gze[4 * (k - 1)];
                    MP dxVy = (Vy(k, i + 1, j) - Vy(k, i, j)) * r20x;
                    MP dxVz = (Vz(k, i + 1, j) - Vz(k, i, j)) * r20x;
                    MP dyVx = (Vx(k, i, j + 1) - Vx(k, i, j)) * r20y;
                    MP dyVz = (Vz(k, i, j + 1) - Vz(k, i, j)) * r20y;
                    MP dzVx = (Vx(k + 1, i, j) - Vx(k, i, j)) * r20z;
                    MP dzVy = (Vy(k + 1, i, j) - Vy(k, i, j)) * r20z;
                    SP muxz, muxy, muyz;
                    hmeans(k, i, j, epsl, muxz, muxy, muyz);
                    Syz(k, i, j) = Syz(k, i, j) + (MP)muyz * (gye_[0] * dyVz + gze_[0] * dzVy + (MP)(gye_[1] * ayVz(k, i, j)) + (MP)(gze_[1] * azVy(k, i, j))) * (MP)dt;
                    Sxz(k, i, j) = Sxz(k, i, j) + (MP)muxz * (gxe_[0] * dxVz + gze_[0] * dzVx + (MP)(gxe_[1] * axVz(k, i, j)) + (MP)(gze_[1] * azVx(k, i, j))) * (MP)dt;
                    Sxy(k, i, j) = Sxy(k, i, j) + (MP)muxy * (gxe_[0] * dxVy + gye_[0] * dyVx + (MP)(gxe_[1] * axVy(k, i, j)) + (MP)(gye_[1] * ayVx(k, i, j))) * (MP)dt;
                    ayVx(k, i, j) = gye_[2] * ayVx(k, i, j) + gye_[3] * (SP)dyVx * dt;
                    azVx(k, i, j) = gze_[2] * azVx(k, i, j) + gze_[3] * (SP)dzVx * dt;
                    axVy(k, i, j) = gxe_[2] * axVy(k, i, j) + gxe_[3] * (SP)dxVy * dt;
                    azVy(k, i, j) = gze_[2] * azVy(k, i, j) + gze_[3] * (SP)dzVy * dt;
                    axVz(k, i, j) = gxe_[2] * axVz(k, i, j) + gxe_[3] * (SP)dxVz * dt;
                    ayVz(k, i, j) = gye_[2] * ayVz(k, i, j) + gye_[3] * (SP)dyVz * dt;
                }
            }
    }

    // src/swpc_3d/m_absorb_c.f90:113-198
    void cerjan_stress() {
#pragma omp parallel for schedule(dynamic)
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i)
                for (int k = kbeg; k <= kend_k; ++k) {
                    SP gcc = gx_c[i + 3] * gy_c[j + 3] * gz_c[k + 3];
                    Sxx(k, i, j) = Sxx(k, i, j) * (MP)gcc; Syy(k, i, j) = Syy(k, i, j) * (MP)gcc; Szz(k, i, j) = Szz(k, i, j) * (MP)gcc;
                }
#pragma omp parallel for schedule(dynamic)
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i)
                for (int k = kbeg; k <= kend_k; ++k) {
                    Syz(k, i, j) = Syz(k, i, j) * (MP)gx_c[i + 3] * (MP)gy_b[j + 3] * (MP)gz_b[k + 3];
                    Sxz(k, i, j) = Sxz(k, i, j) * (MP)gx_b[i + 3] * (MP)gy_c[j + 3] * (MP)gz_b[k + 3];
                    Sxy(k, i, j) = Sxy(k, i, j) * (MP)gx_b[i + 3] * (MP)gy_b[j + 3] * (MP)gz_c[k + 3];
                }
    }
    void cerjan_vel() {
#pragma omp parallel for schedule(dynamic)
        for (int j = jbeg; j <= jend; ++j)
            for (int i = ibeg; i <= iend; ++i)
                for (int k = kbeg; k <= kend; ++k) {
                    Vx(k, i, j) = Vx(k, i, j) * (MP)gx_b[i + 3] * (MP)gy_c[j + 3] * (MP)gz_c[k + 3];
                    Vy(k, i, j) = Vy(k, i, j) * (MP)gx_c[i + 3] * (MP)gy_b[j + 3] * (MP)gz_c[k + 3];
                    Vz(k, i, j) = Vz(k, i, j) * (MP)gx_c[i + 3] * (MP)gy_c[j + 3] * (MP)gz_b[k + 3];
                }
    }

    // src/swpc_3d/m_source.f90:776-848
    void stressglut(int it) {
        if (p.bf_mode) return;
        for (auto& s : src) {
            SP t = tbeg + (SP)(it - (SP)0.5) * dt;
            SP st = momentrate<SP>(t, stf, (SP)s.tbeg, (SP)s.trise);
            MP sdrop = (MP)s.mo * (MP)st * dt_dxyz;
            int ii = s.i, jj = s.j, kk = s.k;
            Sxx(kk, ii, jj) -= (MP)s.mxx * sdrop; Syy(kk, ii, jj) -= (MP)s.myy * sdrop; Szz(kk, ii, jj) -= (MP)s.mzz * sdrop;
            MP qxy = (MP)s.mxy * sdrop / 4, qxz = (MP)s.mxz * sdrop / 4, qyz = (MP)s.myz * sdrop / 4;
            Sxy(kk, ii, jj) -= qxy; Sxy(kk, ii, jj - 1) -= qxy; Sxy(kk, ii - 1, jj) -= qxy; Sxy(kk, ii - 1, jj - 1) -= qxy;
            Sxz(kk, ii, jj) -= qxz; Sxz(kk - 1, ii, jj) -= qxz; Sxz(kk, ii - 1, jj) -= qxz; Sxz(kk - 1, ii - 1, jj) -= qxz;
            Syz(kk, ii, jj) -= qyz; Syz(kk - 1, ii, jj) -= qyz; Syz(kk, ii, jj - 1) -= qyz; Syz(kk - 1, ii, jj - 1) -= qyz;
        }
    }

    // src/swpc_3d/m_source.f90:850-898
    void bodyforce(int it) {
        if (!p.bf_mode) return;
        for (auto& s : src) {
            SP st = momentrate<SP>(tbeg + it * dt, stf, (SP)s.tbeg, (SP)s.trise);
            int ii = s.i, jj = s.j, kk = s.k;
            SP two = 2.0;
            auto add = [&](F3<MP>& V, int k, int i, int j, SP b, MP f) { V(k, i, j) = V(k, i, j) + (MP)b * f * (MP)st * dt_dxyz / 2; };
            add(Vx, kk, ii, jj, two / (rho(kk, ii, jj) + rho(kk, ii + 1, jj)), s.fx);
            add(Vx, kk, ii - 1, jj, two / (rho(kk, ii, jj) + rho(kk, ii - 1, jj)), s.fx);
            add(Vy, kk, ii, jj, two / (rho(kk, ii, jj) + rho(kk, ii, jj + 1)), s.fy);
            add(Vy, kk, ii, jj - 1, two / (rho(kk, ii, jj) + rho(kk, ii, jj - 1)), s.fy);
            add(Vz, kk, ii, jj, two / (rho(kk, ii, jj) + rho(kk + 1, ii, jj)), s.fz);
            add(Vz, kk - 1, ii, jj, two / (rho(kk, ii, jj) + rho(kk - 1, ii, jj)), s.fz);
        }
    }

    // Halo exchange with a single rank: every neighbour is MPI_PROC_NULL, so
    // the receive buffers stay zero and the unpack writes zeros into the
    // ghost planes (src/swpc_3d/m_global.f90:500-607, 391-494).
    void comm_stress() {
        for (int j = 1; j <= ny; ++j) for (int k = 1; k <= nz; ++k) {
            Sxx(k, 0, j) = 0; Sxy(k, -1, j) = 0; Sxy(k, 0, j) = 0; Sxz(k, -1, j) = 0; Sxz(k, 0, j) = 0;
            Sxx(k, nx + 1, j) = 0; Sxx(k, nx + 2, j) = 0; Sxy(k, nx + 1, j) = 0; Sxz(k, nx + 1, j) = 0;
        }
        for (int i = 1; i <= nx; ++i) for (int k = 1; k <= nz; ++k) {
            Syy(k, i, 0) = 0; Sxy(k, i, -1) = 0; Sxy(k, i, 0) = 0; Syz(k, i, -1) = 0; Syz(k, i, 0) = 0;
            Syy(k, i, ny + 1) = 0; Syy(k, i, ny + 2) = 0; Sxy(k, i, ny + 1) = 0; Syz(k, i, ny + 1) = 0;
        }
    }
    void comm_vel() {
        for (int j = 1; j <= ny; ++j) for (int k = 1; k <= nz; ++k) {
            Vx(k, -1, j) = 0; Vx(k, 0, j) = 0; Vy(k, 0, j) = 0; Vz(k, 0, j) = 0;
            Vx(k, nx + 1, j) = 0; Vy(k, nx + 1, j) = 0; Vy(k, nx + 2, j) = 0; Vz(k, nx + 1, j) = 0; Vz(k, nx + 2, j) = 0;
        }
        for (int i = 1; i <= nx; ++i) for (int k = 1; k <= nz; ++k) {
            Vx(k, i, 0) = 0; Vy(k, i, -1) = 0; Vy(k, i, 0) = 0; Vz(k, i, 0) = 0;
            Vx(k, i, ny + 1) = 0; Vx(k, i, ny + 2) = 0; Vy(k, i, ny + 1) = 0; Vz(k, i, ny + 1) = 0; Vz(k, i, ny + 2) = 0;
        }
    }

    // src/swpc_3d/m_wav.f90:397-625
    void wav_store(int it) {
        if (nst == 0) return;
        SP hdt = (SP)0.5 * dt;
        if (p.sw_wav_u)
            for (int n = 0; n < nst; ++n) {
                int i = sta[n].i, j = sta[n].j, k = sta[n].k;
                ux[n] = ux[n] + (SP)(Vx(k, i, j) + Vx(k, i - 1, j)) * (SP)0.5 * dt;
                uy[n] = uy[n] + (SP)(Vy(k, i, j) + Vy(k, i, j - 1)) * (SP)0.5 * dt;
                uz[n] = uz[n] - (SP)(Vz(k, i, j) + Vz(k - 1, i, j)) * (SP)0.5 * dt;
            }
        (void)hdt;
        if (p.sw_wav_strain)
            for (int n = 0; n < nst; ++n) strain_tap(n);
        if ((it - 1) % p.ntdec_w != 0) return;
        int itw = (it - 1) / p.ntdec_w;  // 0-based
        SP M0s = (SP)M0, UCs = (SP)UC;
        auto W = [&](std::vector<float>& w, int nc, int c, int n) -> float& { return w[(size_t)n * nc * ntw + (size_t)c * ntw + itw]; };
        for (int n = 0; n < nst; ++n) {
            int i = sta[n].i, j = sta[n].j, k = sta[n].k;
            if (p.sw_wav_v) {
                W(wav_vel, 3, 0, n) = (float)((SP)(Vx(k, i, j) + Vx(k, i - 1, j)) / (SP)2.0 * M0s * UCs * (SP)1e9);
                W(wav_vel, 3, 1, n) = (float)((SP)(Vy(k, i, j) + Vy(k, i, j - 1)) / (SP)2.0 * M0s * UCs * (SP)1e9);
                W(wav_vel, 3, 2, n) = (float)(-(SP)(Vz(k, i, j) + Vz(k - 1, i, j)) / (SP)2.0 * M0s * UCs * (SP)1e9);
            }
            if (p.sw_wav_u) {
                W(wav_disp, 3, 0, n) = (float)(ux[n] * M0s * UCs * (SP)1e9);
                W(wav_disp, 3, 1, n) = (float)(uy[n] * M0s * UCs * (SP)1e9);
                W(wav_disp, 3, 2, n) = (float)(uz[n] * M0s * UCs * (SP)1e9);
            }
            if (p.sw_wav_stress) {
                SP f = M0s * UCs * (SP)1e6;
                W(wav_stress, 6, 0, n) = (float)((SP)Sxx(k, i, j) * M0s * UCs * (SP)1e6);
                W(wav_stress, 6, 1, n) = (float)((SP)Syy(k, i, j) * M0s * UCs * (SP)1e6);
                W(wav_stress, 6, 2, n) = (float)((SP)Szz(k, i, j) * M0s * UCs * (SP)1e6);
                W(wav_stress, 6, 3, n) = (float)((SP)(Syz(k, i, j) + Syz(k, i, j - 1) + Syz(k - 1, i, j) + Syz(k - 1, i, j - 1)) / (SP)4.0 * M0s * UCs * (SP)1e6);
                W(wav_stress, 6, 4, n) = (float)((SP)(Sxz(k, i, j) + Sxz(k, i - 1, j) + Sxz(k - 1, i, j) + Sxz(k - 1, i - 1, j)) / (SP)4.0 * M0s * UCs * (SP)1e6);
                W(wav_stress, 6, 5, n) = (float)((SP)(Sxy(k, i, j) + Sxy(k, i, j - 1) + Sxy(k, i - 1, j) + Sxy(k, i - 1, j - 1)) / (SP)4.0 * M0s * UCs * (SP)1e6);
                (void)f;
            }
            if (p.sw_wav_strain) {
                SP f = M0s * UCs;
                SP e6[6] = {exx[n], eyy[n], ezz[n], eyz[n], exz[n], exy[n]};
                for (int c = 0; c < 6; ++c) W(wav_strain, 6, c, n) = (float)(e6[c] * f * (SP)1e-3);
            }
        }
    }

    // 4th-order strain at a receiver: m_wav.f90:465-504
    void strain_tap(int n) {
        int i = sta[n].i, j = sta[n].j, k = sta[n].k;
        auto D = [&](F3<MP>& V, int k1, int i1, int j1, int k0, int i0, int j0, int k2, int i2, int j2, int k3, int i3, int j3, MP r40, MP r41) {
            return (V(k1, i1, j1) - V(k0, i0, j0)) * r40 - (V(k2, i2, j2) - V(k3, i3, j3)) * r41;
        };
        MP dxVx = D(Vx, k, i, j, k, i - 1, j, k, i + 1, j, k, i - 2, j, r40x, r41x);
        MP dyVy = D(Vy, k, i, j, k, i, j - 1, k, i, j + 1, k, i, j - 2, r40y, r41y);
        MP dzVz = D(Vz, k, i, j, k - 1, i, j, k + 1, i, j, k - 2, i, j, r40z, r41z);
        MP dxVy = (D(Vy, k, i + 1, j, k, i, j, k, i + 2, j, k, i - 1, j, r40x, r41x) + D(Vy, k, i + 1, j - 1, k, i, j - 1, k, i + 2, j - 1, k, i - 1, j - 1, r40x, r41x)
                 + D(Vy, k, i, j, k, i - 1, j, k, i + 1, j, k, i - 2, j, r40x, r41x) + D(Vy, k, i, j - 1, k, i - 1, j - 1, k, i + 1, j - 1, k, i - 2, j - 1, r40x, r41x)) / (MP)4.0;
        MP dxVz = (D(Vz, k, i + 1, j, k, i, j, k, i + 2, j, k, i - 1, j, r40x, r41x) + D(Vz, k - 1, i + 1, j, k - 1, i, j, k - 1, i + 2, j, k - 1, i - 1, j, r40x, r41x)
                 + D(Vz, k, i, j, k, i - 1, j, k, i + 1, j, k, i - 2, j, r40x, r41x) + D(Vz, k - 1, i, j, k - 1, i - 1, j, k - 1, i + 1, j, k - 1, i - 2, j, r40x, r41x)) / (MP)4.0;
        MP dyVx = (D(Vx, k, i, j + 1, k, i, j, k, i, j + 2, k, i, j - 1, r40y, r41y) + D(Vx, k, i - 1, j + 1, k, i - 1, j, k, i - 1, j + 2, k, i - 1, j - 1, r40y, r41y)
                 + D(Vx, k, i, j, k, i, j - 1, k, i, j + 1, k, i, j - 2, r40y, r41y) + D(Vx, k, i - 1, j, k, i - 1, j - 1, k, i - 1, j + 1, k, i - 1, j - 2, r40y, r41y)) / (MP)4.0;
        MP dyVz = (D(Vz, k, i, j + 1, k, i, j, k, i, j + 2, k, i, j - 1, r40y, r41y) + D(Vz, k - 1, i, j + 1, k - 1, i, j, k - 1, i, j + 2, k - 1, i, j - 1, r40y, r41y)
                 + D(Vz, k, i, j, k, i, j - 1, k, i, j + 1, k, i, j - 2, r40y, r41y) + D(Vz, k - 1, i, j, k - 1, i, j - 1, k - 1, i, j + 1, k - 1, i, j - 2, r40y, r41y)) / (MP)4.0;
        MP dzVx = (D(Vx, k + 1, i, j, k, i, j, k + 2, i, j, k - 1, i, j, r40z, r41z) + D(Vx, k + 1, i - 1, j, k, i - 1, j, k + 2, i - 1, j, k - 1, i - 1, j, r40z, r41z)
                 + D(Vx, k, i, j, k - 1, i, j, k + 1, i, j, k - 2, i, j, r40z, r41z) + D(Vx, k, i - 1, j, k - 1, i - 1, j, k + 1, i - 1, j, k - 2, i - 1, j, r40z, r41z)) / (MP)4.0;
        MP dzVy = (D(Vy, k + 1, i, j, k, i, j, k + 2, i, j, k - 1, i, j, r40z, r41z) + D(Vy, k + 1, i, j - 1, k, i, j - 1, k + 2, i, j - 1, k - 1, i, j - 1, r40z, r41z)
                 + D(Vy, k, i, j, k - 1, i, j, k + 1, i, j, k - 2, i, j, r40z, r41z) + D(Vy, k, i, j - 1, k - 1, i, j - 1, k + 1, i, j - 1, k - 2, i, j - 1, r40z, r41z)) / (MP)4.0;
        exx[n] = exx[n] + (SP)dxVx * dt;
        eyy[n] = eyy[n] + (SP)dyVy * dt;
        ezz[n] = ezz[n] + (SP)dzVz * dt;
        eyz[n] = eyz[n] + (SP)(dyVz + dzVy) / (SP)2.0 * dt;
        exz[n] = exz[n] + (SP)(dxVz + dzVx) / (SP)2.0 * dt;
        exy[n] = exy[n] + (SP)(dxVy + dyVx) / (SP)2.0 * dt;
    }

    // wbuf_{xy,yz,xz,fs,ob}_{v,u,ps} (src/swpc_3d/m_snap.f90:981-2205),
    // native buffers only.  v: V * UC * M0 at frame steps; u: V * UC * M0 * dt
    // summed every step; ps: the
    // divergence and rotation of V with the lam and |S| masks, * UC * M0 * 1e-3.
    // The u sums are rounded to single precision after every step, as the
    // reference's real buffers are.
    void snap_write(int it) {
        if (snaps.empty()) return;
        const SP UCs = (SP)UC, M0s = (SP)M0;
        const bool frame = (it - 1) % p.ntdec_s == 0;
        const SP eps = std::numeric_limits<float>::epsilon();
        for (auto& o : snaps) {
            if (o.kind != 1 && !frame) continue;
            const size_t pl = (size_t)o.n1 * o.n2, nc = o.kind == 2 ? 4 : 3;
            size_t base = 0;
            if (frame) {
                base = o.frames.size();
                o.frames.resize(base + nc * pl);
            }
            for (int b = 1; b <= o.n2; ++b)
                for (int a = 1; a <= o.n1; ++a) {
                    const int ca = a * o.d1 - o.d1 / 2, cb = b * o.d2 - o.d2 / 2;
                    int i, j, k;
                    if (o.sec == 1) { i = o.fix; j = ca; k = cb; }
                    else if (o.sec == 2) { i = ca; j = o.fix; k = cb; }
                    else {
                        i = ca; j = cb;
                        k = o.sec == 0 ? o.fix : (o.sec == 3 ? kfs(i, j) : kob(i, j)) + 1;
                    }
                    const size_t q = (size_t)(b - 1) * o.n1 + (a - 1);
                    if (o.kind == 0) {
                        o.frames[base + q] = (float)(Vx(k, i, j) * (MP)UCs * (MP)M0s);
                        o.frames[base + pl + q] = (float)(Vy(k, i, j) * (MP)UCs * (MP)M0s);
                        o.frames[base + 2 * pl + q] = (float)(Vz(k, i, j) * (MP)UCs * (MP)M0s);
                    } else if (o.kind == 1) {
                        const MP v3[3] = {Vx(k, i, j), Vy(k, i, j), Vz(k, i, j)};
                        for (int c = 0; c < 3; ++c) {
                            const float u = (float)o.ubuf[c * pl + q] + (float)(v3[c] * (MP)UCs * (MP)M0s * (MP)dt);
                            o.ubuf[c * pl + q] = u;
                            if (frame) o.frames[base + c * pl + q] = u;
                        }
                    } else {
                        SP div = (SP)((Vx(k, i, j) - Vx(k, i - 1, j)) * r20x + (Vy(k, i, j) - Vy(k, i, j - 1)) * r20y +
                                      (Vz(k, i, j) - Vz(k - 1, i, j)) * r20z);
                        SP rx = (SP)((Vz(k, i, j + 1) - Vz(k, i, j)) * r20y - (Vy(k + 1, i, j) - Vy(k, i, j)) * r20z);
                        SP ry = (SP)((Vx(k + 1, i, j) - Vx(k, i, j)) * r20z - (Vz(k, i + 1, j) - Vz(k, i, j)) * r20x);
                        SP rz = (SP)((Vy(k, i + 1, j) - Vy(k, i, j)) * r20x - (Vx(k, i, j + 1) - Vx(k, i, j)) * r20y);
                        const SP l = lam(k, i, j);
                        const SP syz = (SP)Syz(k, i, j), sxz = (SP)Sxz(k, i, j), sxy = (SP)Sxy(k, i, j);
                        div = div * l / std::abs(l + eps);
                        if (o.sec == 1) {  // m_snap.f90:1027-1030
                            rx = rx * std::abs(syz) / std::abs(syz + eps);
                            ry = ry * std::abs(sxz) / std::abs(sxz + eps);
                            rz = rz * std::abs(sxy) / std::abs(sxy + eps);
                        } else {
                            rx = rx * std::abs(syz) / (std::abs(syz) + eps);
                            ry = ry * std::abs(sxz) / (std::abs(sxz) + eps);
                            rz = rz * std::abs(sxy) / (std::abs(sxy) + eps);
                        }
                        const SP f = (SP)1e-3;
                        o.frames[base + q] = (float)(div * UCs * M0s * f);
                        o.frames[base + pl + q] = (float)(rx * UCs * M0s * f);
                        o.frames[base + 2 * pl + q] = (float)(ry * UCs * M0s * f);
                        o.frames[base + 3 * pl + q] = (float)(rz * UCs * M0s * f);
                    }
                }
        }
    }

    // src/swpc_3d/m_kernel.f90:350-374 with the report (m_report.f90:120-185)
    void vmax(int it) {
        const int margin = 5;
        SP mx = 0, my = 0, mz = 0;
        for (int j = std::max(na + margin + 1, jbeg_k); j <= std::min(ny - na - margin, jend_k); ++j)
            for (int i = std::max(na + margin + 1, ibeg_k); i <= std::min(nx - na - margin, iend_k); ++i) {
                int k = kob(i, j) + 1;
                mx = std::max(mx, (SP)std::abs(Vx(k, i, j)));
                my = std::max(my, (SP)std::abs(Vy(k, i, j)));
                mz = std::max(mz, (SP)std::abs(Vz(k, i, j)));
            }
        vmax_log.push_back((float)it); vmax_log.push_back((float)mx); vmax_log.push_back((float)my); vmax_log.push_back((float)mz);
    }

    // source grid points: ijk (3n, 1-based); vals 11n: mo mxx myy mzz myz mxz mxy fx fy fz tbeg trise ... (12 per source)
    int get_sources(int* ijk, double* vals) override {
        int n = (int)src.size();
        if (ijk)
            for (int q = 0; q < n; ++q) {
                ijk[3 * q] = src[q].i; ijk[3 * q + 1] = src[q].j; ijk[3 * q + 2] = src[q].k;
                double* v = vals + 12 * q;
                v[0] = src[q].mo; v[1] = src[q].mxx; v[2] = src[q].myy; v[3] = src[q].mzz; v[4] = src[q].myz; v[5] = src[q].mxz;
                v[6] = src[q].mxy; v[7] = src[q].fx; v[8] = src[q].fy; v[9] = src[q].fz; v[10] = src[q].tbeg; v[11] = src[q].trise;
            }
        return n;
    }
    int stf_type() const { return stf; }

    // fields over the physical grid [1..nz]x[1..nx]x[1..ny], k fastest
    void get_field(int which, double* out) override {
        F3<MP>* f[9] = {&Vx, &Vy, &Vz, &Sxx, &Syy, &Szz, &Syz, &Sxz, &Sxy};
        if (which < 0 || which >= 9) throw std::runtime_error("bad field id");
        F3<MP>& A = *f[which];
        size_t q = 0;
        for (int j = 1; j <= ny; ++j) for (int i = 1; i <= nx; ++i) for (int k = 1; k <= nz; ++k) out[q++] = (double)A(k, i, j);
    }
    // Zener coefficients c1, c2, d1 (nm each), d2, then with the PML the
    // damping profiles gxc, gxe (4 x nx), gyc, gye (4 x ny), gzc, gze
    // (4 x nz), l fastest; returns the number of values written
    int coefs(double* out) override {
        int q = 0;
        for (const std::vector<SP>* v : {&c1, &c2, &d1})
            for (SP x : *v) out[q++] = (double)x;
        out[q++] = (double)d2;
        if (pml)
            for (const std::vector<SP>* v : {&gxc, &gxe, &gyc, &gye, &gzc, &gze})
                for (SP x : *v) out[q++] = (double)x;
        return q;
    }
    // overwrite one state field from a halo-grid array A(k,i,j) (k fastest):
    // every cell of the physical columns i in [1,nx], j in [1,ny] including
    // the z halo planes; the x/y ghost columns stay zero, as after a halo
    // exchange on a single rank
    void set_field(int which, const float* halo) override {
        F3<MP>* f[9] = {&Vx, &Vy, &Vz, &Sxx, &Syy, &Szz, &Syz, &Sxz, &Sxy};
        if (which < 0 || which >= 9) throw std::runtime_error("bad field id");
        F3<MP>& A = *f[which];
        const long hk = nz + 6, hki = hk * (nx + 6);
        for (int j = A.jb; j <= A.je; ++j)
            for (int i = A.ib; i <= A.ie; ++i)
                for (int k = A.kb; k <= A.ke; ++k) {
                    const bool phys = i >= 1 && i <= nx && j >= 1 && j <= ny && k >= -2 && k <= nz + 3;
                    A(k, i, j) = phys ? (MP)halo[(size_t)(j + 2) * hki + (size_t)(i + 2) * hk + (k + 2)] : MP(0);
                }
    }
    // medium / maps over the halo grid [-2..nz+3]x[-2..nx+3]x[-2..ny+3]
    void get_medium(int which, float* out) override {
        F3<SP>* f[5] = {&rho, &lam, &mu, &taup, &taus};
        if (which >= 0 && which < 5) {
            for (size_t q = 0; q < f[which]->d.size(); ++q) out[q] = (float)f[which]->d[q];
            return;
        }
        I2* m[6] = {&kfs, &kob, &kfs_top, &kfs_bot, &kob_top, &kob_bot};
        if (which >= 5 && which < 11) {
            I2& M = *m[which - 5];
            for (size_t q = 0; q < M.d.size(); ++q) out[q] = (float)M.d[q];
            return;
        }
        if (which == 11) { for (int m2 = 0; m2 < nm; ++m2) out[m2] = (float)ts[m2]; return; }
        throw std::runtime_error("bad medium id");
    }
};

static std::string g_err;

}  // namespace orc

using namespace orc;

extern "C" {

// Build an oracle simulation from an input.inf file.
//   mode     0 = fp32, 1 = mixed (reference default), 2 = fp64
//   vm5      optional rho, lam, mu, qp, qs over the halo grid (5 x (nz+6)(nx+6)(ny+6),
//            k fastest); when given it replaces the velocity model file
int oracle_create(const char* inf_path, int mode, int nthreads, const float* vm5, void** out) {
    try {
#ifdef _OPENMP
        if (nthreads > 0) omp_set_num_threads(nthreads);
#else
        (void)nthreads;
#endif
        std::string path(inf_path);
        std::string dir = ".";
        size_t sl = path.find_last_of('/');
        if (sl != std::string::npos) dir = path.substr(0, sl);
        Ini ini(path);
        Params p = read_params(ini);
        SimBase* s = nullptr;
        if (mode == 0) s = new Sim<float, float>(p, dir, vm5);
        else if (mode == 1) s = new Sim<double, float>(p, dir, vm5);
        else if (mode == 2) s = new Sim<double, double>(p, dir, vm5);
        else throw std::runtime_error("bad precision mode");
        *out = s;
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

const char* oracle_last_error() { return g_err.c_str(); }

// advance n steps (it = nt_done+1 .. nt_done+n)
int oracle_run(void* h, int n) {
    try {
        SimBase* s = (SimBase*)h;
        for (int q = 0; q < n; ++q) s->step(s->nt_done + 1);
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// ints: nx ny nz nt na nst ntw nt_done nxs nys k0_xy nvmax ; reals: M0 UC fcut
void oracle_info(void* h, int* ints, double* reals) {
    SimBase* s = (SimBase*)h;
    ints[0] = s->p.nx; ints[1] = s->p.ny; ints[2] = s->p.nz; ints[3] = s->p.nt; ints[4] = s->p.na;
    ints[5] = s->nst; ints[6] = s->ntw; ints[7] = s->nt_done; ints[8] = s->nxs; ints[9] = s->nys; ints[10] = s->k0_xy;
    ints[11] = (int)(s->vmax_log.size() / 4);
    ints[12] = 0;
    for (auto& o : s->snaps)
        if (o.sec == 0 && o.kind == 0) ints[12] = (int)o.frames.size();
    reals[0] = s->M0; reals[1] = s->UC; reals[2] = s->fcut;
    reals[3] = s->p.dx; reals[4] = s->p.dy; reals[5] = s->p.dz; reals[6] = s->p.dt;
    reals[7] = s->p.xbeg; reals[8] = s->p.ybeg; reals[9] = s->p.zbeg; reals[10] = s->p.tbeg;
    ints[13] = s->p.ntdec_w; ints[14] = s->p.ntdec_r; ints[15] = s->p.bf_mode ? 1 : 0;
}

// kind: 0 vel (ntw,3,nst), 1 disp, 2 stress (ntw,6,nst), 3 strain
int oracle_waveforms(void* h, int kind, float* out) {
    SimBase* s = (SimBase*)h;
    std::vector<float>* w[4] = {&s->wav_vel, &s->wav_disp, &s->wav_stress, &s->wav_strain};
    if (kind < 0 || kind > 3) return -1;
    std::copy(w[kind]->begin(), w[kind]->end(), out);
    return (int)w[kind]->size();
}

void oracle_stations(void* h, int* ijk) {
    SimBase* s = (SimBase*)h;
    for (int n = 0; n < s->nst; ++n) { ijk[3 * n] = s->sta[n].i; ijk[3 * n + 1] = s->sta[n].j; ijk[3 * n + 2] = s->sta[n].k; }
}

int oracle_field(void* h, int which, double* out) {
    try { ((SimBase*)h)->get_field(which, out); return 0; } catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int oracle_coefs(void* h, double* out) {
    try { return ((SimBase*)h)->coefs(out); } catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int oracle_set_field(void* h, int which, const float* halo) {
    try { ((SimBase*)h)->set_field(which, halo); return 0; } catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int oracle_medium(void* h, int which, float* out) {
    try { ((SimBase*)h)->get_medium(which, out); return 0; } catch (const std::exception& e) { g_err = e.what(); return -1; }
}
void oracle_vmax(void* h, float* out) { SimBase* s = (SimBase*)h; std::copy(s->vmax_log.begin(), s->vmax_log.end(), out); }
void oracle_snap_xy_v(void* h, float* out) {
    SimBase* s = (SimBase*)h;
    for (auto& o : s->snaps)
        if (o.sec == 0 && o.kind == 0) std::copy(o.frames.begin(), o.frames.end(), out);
}
// Green's-function traces (ntw, ncmp * ng) in Fortran order and the layout
// ints: ng, ncmp, ntw; returns 0, or -1 outside green mode
int oracle_green(void* h, int* ng_ncmp_ntw, float* out) {
    SimBase* s = (SimBase*)h;
    return s->green_out(ng_ncmp_ntw, out);
}
// stacked frames of one snapshot (section, kind); returns the float count,
// -1 when that snapshot was not requested; out may be null to query
long long oracle_snap(void* h, int sec, int kind, float* out) {
    SimBase* s = (SimBase*)h;
    for (auto& o : s->snaps)
        if (o.sec == sec && o.kind == kind) {
            if (out) std::copy(o.frames.begin(), o.frames.end(), out);
            return (long long)o.frames.size();
        }
    return -1;
}

void oracle_destroy(void* h) { delete (SimBase*)h; }

int oracle_sources(void* h, int* ijk, double* vals) { return ((SimBase*)h)->get_sources(ijk, vals); }
int oracle_stf(void* h) { return stf_code(((SimBase*)h)->p.stftype); }

// ---------------------------------------------------------------------------
// Small known-answer helpers exposed for the oracle's own tests
// ---------------------------------------------------------------------------
float oracle_momentrate(float t, int stf, float ts, float tr) { return momentrate<float>(t, stf, ts, tr); }
void oracle_sdr2moment(float strike, float dip, float rake, float* m6) { Sim<float, float>::sdr2moment(strike, dip, rake, m6); }

}  // extern "C"
