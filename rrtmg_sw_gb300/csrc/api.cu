// api.cu -- host side of the GB300 RRTMG_SW library: table loading and
// upload (rrtmg_sw_ini), the per-call solar-source setup of inatm_sw, the
// device workspace and the C-ABI entry points of include/rrtmg_sw_gb300.h.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rrtmg_sw_gb300.h"
#include "launch.h"

using namespace rrsw;

namespace {

const int kNG[14] = {6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12};
const int kNSPA[14] = {9, 9, 9, 9, 1, 9, 9, 1, 9, 1, 0, 1, 9, 1};  // rrtmg_sw_init.f90:194
const int kNSPB[14] = {1, 5, 1, 1, 1, 5, 1, 0, 1, 0, 0, 1, 5, 1};  // rrtmg_sw_init.f90:195

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

struct State {
    std::mutex mu;
    bool init = false;
    int device = 0, num_sms = 0;
    DevTables tabs{};
    std::vector<double> blob64;
    double mgavgcyc[134], sbavgcyc[134];
    double cpdair = 1.004e3;
    DevBuf d_tab64, d_tab32, scratch, errw, bounds;
    std::map<std::string, DevBuf> stage;  // host-API staging buffers
    int* h_err = nullptr;                  // pinned: [0] error word, [1] tiled-kernel overflow count
    unsigned long long* h_stats = nullptr;  // pinned: the FP32 form's counters of the last solve
    DevBuf statsw;                         // their device copy
    long long last_stats[4] = {0, 0, 0, 0};
    // from the environment at each rrtmg_sw_ini_c: RRTMG_SW_TILED=0 keeps the
    // FP32 form on the scratch-based kernel (the tiled kernel is the default
    // where it applies); RRTMG_SW_TILE_QCAP=n
    // lowers the tiled kernel's capacity of FP64 cells per column pair (tests
    // of its fallback)
    bool no_tiled = false;
    int tile_qcap = 0;
    int batch_tile = 0;  // batch plans: 0 = tile chosen by the autotuner, else 2 or 4 columns only
    // host-array calls run on this non-blocking stream (not the legacy
    // default stream, which would serialise against every stream of the host)
    cudaStream_t host_stream = nullptr;
    int form = RRTMG_SW_FORM_FP64;
    int last_launches = 0;
    int last_kernel = -1;  // RRTMG_SW_KERNEL_* of the most recent solve's main launch
    int last_tile_slots = 0;  // pair slots of the most recent tiled launch (0: not tiled)
    int last_ad_store = -1;  // checkpointing choice of the last adjoint / tangent-linear call
    std::string last_cuda;
};

State& S() {
    static State s;
    return s;
}

int cuda_fail(cudaError_t e) {
    S().last_cuda = cudaGetErrorString(e);
    return RRTMG_SW_ECUDA;
}
#define CK(x)                                 \
    do {                                      \
        cudaError_t e_ = (x);                 \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)

// Every entry point that touches the device first checks that the tables
// were loaded (rrtmg_sw_ini_c) and that the current device is the one they
// were loaded on: the tables and the workspace live on that GPU, and a
// kernel launched on another would read them from the wrong device.
int ready(const State& st) {
    if (!st.init) return RRTMG_SW_ENOTINIT;
    int dev = -1;
    CK(cudaGetDevice(&dev));
    return dev == st.device ? RRTMG_SW_OK : RRTMG_SW_ENOTINIT;
}

std::string table_path() {
    if (const char* env = std::getenv("RRTMG_SW_TABLES")) return env;
    Dl_info info;
    if (dladdr((void*)&table_path, &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        const std::string dir = so.substr(0, so.find_last_of('/'));
        for (const char* rel : {"/rrtmg_sw_tables.bin", "/../data/rrtmg_sw_tables.bin", "/data/rrtmg_sw_tables.bin"}) {
            const std::string p = dir + rel;
            if (FILE* f = std::fopen(p.c_str(), "rb")) {
                std::fclose(f);
                return p;
            }
        }
    }
    return "rrtmg_sw_tables.bin";
}

bool read_tables(const std::string& path, std::map<std::string, std::vector<double>>& rec) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[8];
    uint32_t n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "RRSWTB01", 8) == 0 && std::fread(&n, 4, 1, f) == 1;
    for (uint32_t r = 0; ok && r < n; ++r) {
        char name[32];
        uint32_t hdr[5];
        uint64_t cnt;
        ok = std::fread(name, 1, 32, f) == 32 && std::fread(hdr, 4, 5, f) == 5 && std::fread(&cnt, 8, 1, f) == 1;
        if (!ok || cnt > (1u << 24)) { ok = false; break; }
        std::vector<double> v(cnt);
        ok = std::fread(v.data(), 8, cnt, f) == cnt;
        name[31] = 0;
        rec[name] = std::move(v);
    }
    std::fclose(f);
    return ok;
}

// GF(2) matrix of the KISS xorshift y ^= y<<13; y ^= y>>17; y ^= y<<5
uint32_t xs_step(uint32_t y) {
    y ^= y << 13;
    y ^= y >> 17;
    y ^= y << 5;
    return y;
}

// Build the table blob: absorption tables transposed to [ind][ig].
int build_tables(State& st) {
    std::map<std::string, std::vector<double>> rec;
    if (!read_tables(table_path(), rec)) return RRTMG_SW_ETABLES;
    auto has = [&](const std::string& k) { return rec.count(k) && !rec[k].empty(); };
    std::vector<double>& B = st.blob64;
    B.clear();
    auto put = [&](const std::vector<double>& v) {
        const int off = (int)B.size();
        B.insert(B.end(), v.begin(), v.end());
        return off;
    };
    auto put_T = [&](const std::vector<double>& v, int ng) {  // (nind, ng) Fortran -> [ind][ig]
        const int off = (int)B.size();
        const size_t nind = v.size() / ng;
        for (size_t ind = 0; ind < nind; ++ind)
            for (int ig = 0; ig < ng; ++ig) B.push_back(v[ind + nind * ig]);
        return off;
    };
    DevTables& T = st.tabs;
    std::memset(&T, 0, sizeof(T));
    int g0 = 0;
    for (int ib = 0; ib < 14; ++ib) {
        const std::string p = "b" + std::to_string(ib + 16) + ".";
        BandOff& b = T.b[ib];
        b.ng = kNG[ib];
        b.g0 = g0;
        b.nspa = kNSPA[ib];
        b.nspb = kNSPB[ib];
        for (int g = 0; g < b.ng; ++g) {
            T.ngb[g0 + g] = (int8_t)ib;
            T.gib[g0 + g] = (uint8_t)(g + 1);
        }
        g0 += b.ng;
        if (!has(p + "sfluxref")) return RRTMG_SW_ETABLES;
        b.absa = has(p + "ka") ? put_T(rec[p + "ka"], b.ng) : -1;
        b.absb = has(p + "kb") ? put_T(rec[p + "kb"], b.ng) : -1;
        b.selfref = has(p + "selfref") ? put_T(rec[p + "selfref"], b.ng) : -1;
        b.forref = has(p + "forref") ? put_T(rec[p + "forref"], b.ng) : -1;
        b.nfr = has(p + "forref") ? (int)(rec[p + "forref"].size() / b.ng) : 0;
        b.sfluxref = put(rec[p + "sfluxref"]);
        b.irradnce = put(rec[p + "irradnce"]);
        b.facbrght = put(rec[p + "facbrght"]);
        b.snsptdrk = put(rec[p + "snsptdrk"]);
        b.rayl = has(p + "rayl") ? put(rec[p + "rayl"]) : -1;
        b.rayla = has(p + "rayla") ? put(rec[p + "rayla"]) : -1;
        b.raylb = has(p + "raylb") ? put(rec[p + "raylb"]) : -1;
        b.abso3a = has(p + "abso3a") ? put(rec[p + "abso3a"]) : -1;
        b.abso3b = has(p + "abso3b") ? put(rec[p + "abso3b"]) : -1;
        b.absch4 = has(p + "absch4") ? put(rec[p + "absch4"]) : -1;
        b.absco2 = has(p + "absco2") ? put(rec[p + "absco2"]) : -1;
        b.absh2o = has(p + "absh2o") ? put(rec[p + "absh2o"]) : -1;
    }
    const char* names[] = {"pref", "preflog", "tref", "extliq1", "ssaliq1", "asyliq1", "extice2", "ssaice2",
                           "asyice2", "extice3", "ssaice3", "asyice3", "fdlice3", "abari", "bbari", "cbari",
                           "dbari", "ebari", "fbari", "rsrtaua", "rsrpiza", "rsrasya", "wavenum2", "mgavgcyc",
                           "sbavgcyc"};
    for (const char* nm : names)
        if (!has(nm)) return RRTMG_SW_ETABLES;
    T.pref = put(rec["pref"]);
    T.preflog = put(rec["preflog"]);
    T.tref = put(rec["tref"]);
    T.extliq1 = put(rec["extliq1"]); T.ssaliq1 = put(rec["ssaliq1"]); T.asyliq1 = put(rec["asyliq1"]);
    T.extice2 = put(rec["extice2"]); T.ssaice2 = put(rec["ssaice2"]); T.asyice2 = put(rec["asyice2"]);
    T.extice3 = put(rec["extice3"]); T.ssaice3 = put(rec["ssaice3"]); T.asyice3 = put(rec["asyice3"]);
    T.fdlice3 = put(rec["fdlice3"]);
    auto co_of = [&](const std::vector<double>& ssa) {
        std::vector<double> co(ssa.size());
        for (size_t i = 0; i < ssa.size(); ++i) co[i] = 1.0 - ssa[i];
        return co;
    };
    T.coliq1 = put(co_of(rec["ssaliq1"]));
    T.coice2 = put(co_of(rec["ssaice2"]));
    T.coice3 = put(co_of(rec["ssaice3"]));
    T.abari = put(rec["abari"]); T.bbari = put(rec["bbari"]); T.cbari = put(rec["cbari"]);
    T.dbari = put(rec["dbari"]); T.ebari = put(rec["ebari"]); T.fbari = put(rec["fbari"]);
    T.rsrtaua = put(rec["rsrtaua"]); T.rsrpiza = put(rec["rsrpiza"]); T.rsrasya = put(rec["rsrasya"]);
    T.wavenum2 = put(rec["wavenum2"]);
    std::memcpy(st.mgavgcyc, rec["mgavgcyc"].data(), sizeof(st.mgavgcyc));
    std::memcpy(st.sbavgcyc, rec["sbavgcyc"].data(), sizeof(st.sbavgcyc));
    // exp_tbl (rrtmg_sw_init.f90:115-123)
    std::vector<double> et(NTBL + 1);
    const double expeps = 1.e-20, pade = 0.278;
    T.bpade = 1.0 / pade;
    et[0] = 1.0;
    et[NTBL] = expeps;
    for (int itr = 1; itr <= NTBL - 1; ++itr) {
        const double tfn = (double)itr / (double)NTBL;
        const double tau_tbl = T.bpade * tfn / (1.0 - tfn);
        et[itr] = std::exp(-tau_tbl);
        if (et[itr] <= expeps) et[itr] = expeps;
    }
    T.exp_tbl = put(et);
    // band/region descriptors of the FP32 gas optics (rrtmg_sw_taumol.f90:275-1785)
    enum { H2O = 0, CO2 = 1, O3 = 2, CH4 = 3, O2 = 4, O2CONT = 9 };
    auto reg = [&](int band, int up, int kind, int sa, int sb, float strrat, float fac, int cont, int minor,
                   int mtab, int rtype, int rtab) {
        TmRegion& r = T.tm[band - 16][up];
        const BandOff& b = T.b[band - 16];
        r.kind = (int8_t)kind; r.sa = (int8_t)sa; r.sb = (int8_t)sb; r.cont = (int8_t)cont;
        r.minor = (int8_t)minor; r.rtype = (int8_t)rtype;
        r.nsp = (int8_t)(kind == 1 ? (up ? b.nspb : b.nspa) : 1);
        r.jo = (int8_t)(up ? 13 : 1);
        r.strrat = strrat; r.fac = fac; r.mult = up ? 4.0f : 8.0f;
        r.ktab = up ? b.absb : b.absa;
        r.mtab = mtab;
        r.rtab = rtab;
    };
    reg(16, 0, 1, H2O, CH4, 252.131f, 1.f, 1, -1, 0, 0, T.b[16 - 16].rayl);
    reg(16, 1, 2, CH4, 0, 0.f, 1.f, 0, -1, 0, 0, T.b[16 - 16].rayl);
    reg(17, 0, 1, H2O, CO2, 0.364641f, 1.f, 1, -1, 0, 0, T.b[17 - 16].rayl);
    reg(17, 1, 1, H2O, CO2, 0.364641f, 1.f, 2, -1, 0, 0, T.b[17 - 16].rayl);
    reg(18, 0, 1, H2O, CH4, 38.9589f, 1.f, 1, -1, 0, 0, T.b[18 - 16].rayl);
    reg(18, 1, 2, CH4, 0, 0.f, 1.f, 0, -1, 0, 0, T.b[18 - 16].rayl);
    reg(19, 0, 1, H2O, CO2, 5.49281f, 1.f, 1, -1, 0, 0, T.b[19 - 16].rayl);
    reg(19, 1, 2, CO2, 0, 0.f, 1.f, 0, -1, 0, 0, T.b[19 - 16].rayl);
    reg(20, 0, 2, H2O, 0, 0.f, 1.f, 1, CH4, T.b[20 - 16].absch4, 0, T.b[20 - 16].rayl);
    reg(20, 1, 2, H2O, 0, 0.f, 1.f, 2, CH4, T.b[20 - 16].absch4, 0, T.b[20 - 16].rayl);
    reg(21, 0, 1, H2O, CO2, 0.0045321f, 1.f, 1, -1, 0, 0, T.b[21 - 16].rayl);
    reg(21, 1, 1, H2O, CO2, 0.0045321f, 1.f, 2, -1, 0, 0, T.b[21 - 16].rayl);
    reg(22, 0, 1, H2O, O2, (float)(1.6 * 0.022708), 1.f, 1, O2CONT, 0, 0, T.b[22 - 16].rayl);
    reg(22, 1, 2, O2, 0, 0.f, 1.6f, 0, O2CONT, 0, 0, T.b[22 - 16].rayl);
    reg(23, 0, 2, H2O, 0, 0.f, 1.029f, 1, -1, 0, 1, T.b[23 - 16].rayl);
    reg(23, 1, 0, 0, 0, 0.f, 1.f, 0, -1, 0, 1, T.b[23 - 16].rayl);
    reg(24, 0, 1, H2O, O2, 0.124692f, 1.f, 1, O3, T.b[24 - 16].abso3a, 2, T.b[24 - 16].rayla);
    reg(24, 1, 2, O2, 0, 0.f, 1.f, 0, O3, T.b[24 - 16].abso3b, 1, T.b[24 - 16].raylb);
    reg(25, 0, 2, H2O, 0, 0.f, 1.f, 0, O3, T.b[25 - 16].abso3a, 1, T.b[25 - 16].rayl);
    reg(25, 1, 0, 0, 0, 0.f, 1.f, 0, O3, T.b[25 - 16].abso3b, 1, T.b[25 - 16].rayl);
    reg(26, 0, 0, 0, 0, 0.f, 1.f, 0, -1, 0, 1, T.b[26 - 16].rayl);
    reg(26, 1, 0, 0, 0, 0.f, 1.f, 0, -1, 0, 1, T.b[26 - 16].rayl);
    reg(27, 0, 2, O3, 0, 0.f, 1.f, 0, -1, 0, 1, T.b[27 - 16].rayl);
    reg(27, 1, 2, O3, 0, 0.f, 1.f, 0, -1, 0, 1, T.b[27 - 16].rayl);
    reg(28, 0, 1, O3, O2, 6.67029e-07f, 1.f, 0, -1, 0, 0, T.b[28 - 16].rayl);
    reg(28, 1, 1, O3, O2, 6.67029e-07f, 1.f, 0, -1, 0, 0, T.b[28 - 16].rayl);
    reg(29, 0, 2, H2O, 0, 0.f, 1.f, 1, CO2, T.b[29 - 16].absco2, 0, T.b[29 - 16].rayl);
    reg(29, 1, 2, CO2, 0, 0.f, 1.f, 0, H2O, T.b[29 - 16].absh2o, 0, T.b[29 - 16].rayl);
    T.total = (int)B.size();
    T.oneminus = 1.0 - 1.e-06;  // rrtmg_sw_rad.f90:563-565
    T.bpade_f = (float)T.bpade;
    T.oneminus_f = (float)T.oneminus;
    // xorshift jump matrices
    for (int j = 0; j < 32; ++j) T.xs_jump[0][j] = xs_step(1u << j);
    for (int k = 1; k < 32; ++k)
        for (int j = 0; j < 32; ++j) {
            uint32_t y = T.xs_jump[k - 1][j], r = 0;
            for (int b = 0; b < 32; ++b)
                if (y >> b & 1u) r ^= T.xs_jump[k - 1][b];
            T.xs_jump[k][j] = r;
        }
    // thread layout of the solve CTA: warps of whole bands, both columns
    // of a band side by side (band sizes 2*ng: 12,24,16,16,20,20,4,20,16,12,12,16,12,24)
    {
        const int seg[][3] = {  // band, first g in band, count (per column)
            {2, 0, 8}, {3, 0, 8}, {8, 0, 8}, {11, 0, 8}, {4, 0, 10}, {0, 0, 6}, {5, 0, 10}, {9, 0, 6},
            {7, 0, 10}, {10, 0, 6}, {1, 0, 12}, {6, 0, 2}, {12, 0, 2}, {13, 0, 12}, {12, 2, 4}};
        int t = 0, bg0[14], acc = 0;
        for (int ib = 0; ib < 14; ++ib) { bg0[ib] = acc; acc += kNG[ib]; }
        for (const auto& sg : seg)
            for (int cc = 0; cc < 2; ++cc)
                for (int k = 0; k < sg[2]; ++k) T.thr_cg[t++] = (uint8_t)((cc << 7) | (bg0[sg[0]] + sg[1] + k));
        if (t != CTA_THREADS) return RRTMG_SW_ETABLES;
    }
    return RRTMG_SW_OK;
}

int upload(State& st) {
    DevTables& T = st.tabs;
    const double grav = 9.8066, secdy = 8.6400e4;  // rrtmg_sw_init.f90:207-243
    T.heatfac = grav * secdy / (st.cpdair * 1.e2);   // rrtmg_sw_init.f90:258
    CK(st.d_tab64.ensure(st.blob64.size() * sizeof(double)));
    CK(cudaMemcpy(st.d_tab64.p, st.blob64.data(), st.blob64.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> b32(st.blob64.begin(), st.blob64.end());
    CK(st.d_tab32.ensure(b32.size() * sizeof(float)));
    CK(cudaMemcpy(st.d_tab32.p, b32.data(), b32.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(st.bounds.ensure(sizeof(int)));
    CK(cudaMemset(st.bounds.p, 0, sizeof(int)));
    T.bounds_err = (int*)st.bounds.p;
    CK(upload_tables_fp64(T));
    CK(upload_tables_fp32(T));
    CK(upload_tables_ad(T));
    return RRTMG_SW_OK;
}

// Bounds-check builds: after a completed solve, the table-bounds word (set
// by the kernels' ldt) turns the call's status into RRTMG_SW_EBOUNDS and is
// cleared.  Other builds return rc unchanged.
int bounds_status(State& st, int rc) {
#ifdef RRTMG_BOUNDS_CHECK
    int h = 0;
    if (cudaMemcpy(&h, st.bounds.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return RRTMG_SW_ECUDA;
    if (h) {
        cudaMemset(st.bounds.p, 0, sizeof(int));
        return RRTMG_SW_EBOUNDS;
    }
#else
    (void)st;
#endif
    return rc;
}

// earth_sun (rrtmg_sw_rad.f90:844-868)
double earth_sun(int idn) {
    const double pi = 2.0 * std::asin(1.0);
    const double gamma = 2.0 * pi * (idn - 1) / 365.0;
    return 1.000110 + .034221 * std::cos(gamma) + .001289 * std::sin(gamma) + .000719 * std::cos(2.0 * gamma) +
           .000077 * std::sin(2.0 * gamma);
}

// Per-call solar variability and Earth-Sun scaling of inatm_sw
// (rrtmg_sw_rad.f90:1245-1512): scalars of the call, not of a column.
void solar_setup(const State& st, const rrtmg_sw_args* a, SolveParams& P) {
    const double Iint = 1360.37, Fint = 0.996047, Sint = -0.511590;
    const double Foffset = 0.14959542, Soffset = 0.00066696;
    const double favg = 0.1567652, savg = 902.71260;
    const double cmin = 0.0189, cmax = 0.3750, dmin2max = 0.3561, dmax2min = 0.6439;
    const double rrsw_scon = 1.36822e+03;
    const int isolvar = a->isolvar;
    double solvar[14];
    for (int i = 0; i < 14; ++i) {
        solvar[i] = 1.0;
        P.svar_f_bnd[i] = P.svar_s_bnd[i] = P.svar_i_bnd[i] = 1.0;
    }
    P.isolvar = isolvar;
    double svar_f = 1.0, svar_s = 1.0, svar_i = 1.0;  // per-call factors of isolvar 0-2
    double scl[2] = {1.0, 1.0}, ndx[2] = {favg, savg}, scf = 0.0;
    if (isolvar == 1 && a->indsolvar && a->solcycfrac) {
        scf = *a->solcycfrac;
        const double* iv = a->indsolvar;
        if (iv[0] != 1.0 || iv[1] != 1.0) {
            if (scf >= 0.0 && scf < cmin) {
                const double w = (scf + 1.0 - cmax) / dmax2min;
                scl[0] = iv[0] + w * (1.0 - iv[0]);
                scl[1] = iv[1] + w * (1.0 - iv[1]);
            }
            if (scf >= cmin && scf <= cmax) {
                const double w = (scf - cmin) / dmin2max;
                scl[0] = 1.0 + w * (iv[0] - 1.0);
                scl[1] = 1.0 + w * (iv[1] - 1.0);
            }
            if (scf > cmax && scf <= 1.0) {
                const double w = (scf - cmax) / dmax2min;
                scl[0] = iv[0] + w * (1.0 - iv[0]);
                scl[1] = iv[1] + w * (1.0 - iv[1]);
            }
        }
    }
    if (isolvar == 2 && a->indsolvar) { ndx[0] = a->indsolvar[0]; ndx[1] = a->indsolvar[1]; }
    double adjflx = a->adjes;
    if (a->dyofyr > 0) adjflx = earth_sun(a->dyofyr);
    auto cycle = [&](double& f0, double& s0) {  // mean solar cycle lookup (:1329-1359)
        const int nf = 134;
        if (scf <= 0.0) { f0 = st.mgavgcyc[0]; s0 = st.sbavgcyc[0]; return; }
        if (scf >= 1.0) { f0 = st.mgavgcyc[nf - 1]; s0 = st.sbavgcyc[nf - 1]; return; }
        const double il = 1.0 / (nf - 2), ih = 0.5 * il;
        int sfid = 1;
        double lo = 0.0, hi = ih;
        if (scf > ih && scf < 1.0 - ih) {
            sfid = (int)std::floor((scf - ih) * (nf - 2)) + 2;
            lo = (sfid - 2) * il + ih;
            hi = lo + il;
        }
        if (scf >= 1.0 - ih) { sfid = (nf - 2) + 1; lo = 1.0 - ih; hi = 1.0; }
        const double fr = (scf - lo) / (hi - lo);
        f0 = st.mgavgcyc[sfid - 1] + fr * (st.mgavgcyc[sfid] - st.mgavgcyc[sfid - 1]);
        s0 = st.sbavgcyc[sfid - 1] + fr * (st.sbavgcyc[sfid] - st.sbavgcyc[sfid - 1]);
    };
    const double scon = a->scon;
    if (scon == 0.0) {
        if (isolvar == -1)
            for (int i = 0; i < 14; ++i) solvar[i] = a->bndsolvar ? a->bndsolvar[i] : 1.0;
        if (isolvar == 1) {
            double f0, s0;
            cycle(f0, s0);
            svar_f = scl[0] * (f0 - Foffset) / (favg - Foffset);
            svar_s = scl[1] * (s0 - Soffset) / (savg - Soffset);
        }
        if (isolvar == 2) {
            svar_f = (ndx[0] - Foffset) / (favg - Foffset);
            svar_s = (ndx[1] - Soffset) / (savg - Soffset);
        }
        if (isolvar == 3)
            for (int i = 0; i < 14; ++i) {
                solvar[i] = a->bndsolvar ? a->bndsolvar[i] : 1.0;
                P.svar_f_bnd[i] = P.svar_s_bnd[i] = P.svar_i_bnd[i] = solvar[i];
            }
    }
    if (scon > 0.0) {
        if (isolvar == -1)
            for (int i = 0; i < 14; ++i) solvar[i] = a->bndsolvar ? a->bndsolvar[i] * scon / rrsw_scon : scon / rrsw_scon;
        if (isolvar == 0) {
            const double r = scon / (Fint + Sint + Iint);
            svar_f = svar_s = svar_i = r;
        }
        if (isolvar == 1) {
            double f0, s0;
            cycle(f0, s0);
            svar_i = (scon - (scl[0] * Fint + scl[1] * Sint)) / Iint;
            svar_f = scl[0] * (f0 - Foffset) / (favg - Foffset);
            svar_s = scl[1] * (s0 - Soffset) / (savg - Soffset);
        }
        if (isolvar == 3) {
            const double c = Fint + Sint + Iint;
            for (int i = 0; i < 14; ++i) {
                solvar[i] = a->bndsolvar ? a->bndsolvar[i] * scon / c : scon / c;
                P.svar_f_bnd[i] = P.svar_s_bnd[i] = P.svar_i_bnd[i] = solvar[i];
            }
        }
    }
    // the kernel reads per-band factors: isolvar 0-2 use the same three everywhere
    if (isolvar != 3)
        for (int i = 0; i < 14; ++i) {
            P.svar_f_bnd[i] = svar_f;
            P.svar_s_bnd[i] = svar_s;
            P.svar_i_bnd[i] = svar_i;
        }
    for (int i = 0; i < 14; ++i) P.adjflux[i] = isolvar < 0 ? adjflx * solvar[i] : adjflx;
}

// A call with no columns does nothing, as the reference's column loop
// (rrtmg_sw_rad.f90:640) does; check_args reports it as kEmpty and the
// entry points return RRTMG_SW_OK.
constexpr int kEmpty = -1;

// Any nlay >= 1 is accepted here, as the reference's driver accepts it; the
// KISS subcolumn seed reads the bottom four layer pressures
// (mcica_subcol_gen_sw.f90:470-478), so make_params requires nlay >= 4 for
// the fused McICA path with irng = 0 only (RRTMG_SW_EKISSSEED), and a profile without
// layers on both sides of the 100 hPa switch is reported by the solve
// (RRTMG_SW_ELAYTROP).
int check_args(const rrtmg_sw_args* a) {
    if (a && a->ncol == 0) return kEmpty;
    if (!a || a->ncol < 0 || a->nlay < 1 || a->nlay > MAX_NLAY) return RRTMG_SW_EARGS;
    const double* req[] = {a->play, a->plev, a->tlay, a->h2ovmr, a->o3vmr, a->co2vmr, a->ch4vmr, a->o2vmr,
                           a->asdir, a->asdif, a->aldir, a->aldif, a->coszen};
    for (const double* p : req)
        if (!p) return RRTMG_SW_EARGS;
    if (!a->swuflx || !a->swdflx || !a->swhr || !a->swuflxc || !a->swdflxc || !a->swhrc) return RRTMG_SW_EARGS;
    return RRTMG_SW_OK;
}

// Fill SolveParams from args whose pointers are device pointers.
int make_params(State& st, const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, SolveParams& P, bool nomcica = false) {
    std::memset(&P, 0, sizeof(P));
    P.ncol = a->ncol;
    P.nlay = a->nlay;
    P.icld = (a->icld < 0 || a->icld > 5) ? 2 : a->icld;   // rrtmg_sw_rad.f90:589 (4/5 accepted)
    P.iaer = (a->iaer != 0 && a->iaer != 6 && a->iaer != 10) ? 0 : a->iaer;  // :597
    P.idelm = a->idelm == 0 ? 0 : 1;
    P.inflag = a->inflgsw;
    P.iceflag = a->iceflgsw;
    P.liqflag = a->liqflgsw;
    P.fused = (c && !nomcica) ? 1 : 0;
    P.nomcica = nomcica ? 1 : 0;
    P.extra = (a->dirdflux || a->difdflux || a->uvdflx || a->nidflx || a->dirdnuv || a->difdnuv || a->dirdnir ||
               a->difdnir) ? 1 : 0;
    P.npairs = (a->ncol + COLS_PER_CTA - 1) / COLS_PER_CTA;
    solar_setup(st, a, P);
    P.play = a->play; P.plev = a->plev; P.tlay = a->tlay;
    P.h2ovmr = a->h2ovmr; P.o3vmr = a->o3vmr; P.co2vmr = a->co2vmr; P.ch4vmr = a->ch4vmr; P.o2vmr = a->o2vmr;
    P.asdir = a->asdir; P.asdif = a->asdif; P.aldir = a->aldir; P.aldif = a->aldif; P.coszen = a->coszen;
    if (P.icld >= 1 && !c) {
        P.cldfmcl = a->cldfmcl; P.taucmcl = a->taucmcl; P.ssacmcl = a->ssacmcl; P.asmcmcl = a->asmcmcl;
        P.fsfcmcl = a->fsfcmcl; P.ciwpmcl = a->ciwpmcl; P.clwpmcl = a->clwpmcl;
        P.reicmcl = a->reicmcl; P.relqmcl = a->relqmcl;
        if (!P.cldfmcl || !P.taucmcl || !P.ssacmcl || !P.asmcmcl || !P.fsfcmcl || !P.ciwpmcl || !P.clwpmcl ||
            !P.reicmcl || !P.relqmcl)
            return RRTMG_SW_EARGS;
    }
    if (nomcica && P.icld >= 1) {
        // rrtmg_sw_rad.nomcica.f90:98-111 cloud arguments (cldfr, taucld .. reliq)
        P.cldfrac = c->cldfrac; P.ciwp = c->ciwp; P.clwp = c->clwp; P.rei = c->rei; P.rel = c->rel;
        P.tauc = c->tauc; P.ssac = c->ssac; P.asmc = c->asmc; P.fsfc = c->fsfc;
        if (!P.cldfrac || !P.ciwp || !P.clwp || !P.rei || !P.rel) return RRTMG_SW_EARGS;
        if (P.inflag == 0 && (!P.tauc || !P.ssac || !P.asmc || !P.fsfc)) return RRTMG_SW_EARGS;
    }
    if (c && !nomcica && P.icld >= 1) {
        P.irng = c->irng != 0 ? 1 : 0;  // mcica:455
        if (P.irng == 0 && P.nlay < 4) return RRTMG_SW_EKISSSEED;  // seeds from the bottom four layers
        P.permuteseed = c->permuteseed;
        P.cldfrac = c->cldfrac; P.ciwp = c->ciwp; P.clwp = c->clwp; P.rei = c->rei; P.rel = c->rel;
        P.tauc = c->tauc; P.ssac = c->ssac; P.asmc = c->asmc; P.fsfc = c->fsfc; P.alpha = c->alpha;
        if (!P.cldfrac || !P.ciwp || !P.clwp || !P.rei || !P.rel) return RRTMG_SW_EARGS;
        if (P.inflag == 0 && (!P.tauc || !P.ssac || !P.asmc || !P.fsfc)) return RRTMG_SW_EARGS;
        if (P.icld >= 4 && !P.alpha) return RRTMG_SW_EARGS;
    }
    if (P.iaer == 10) {
        P.tauaer = a->tauaer; P.ssaaer = a->ssaaer; P.asmaer = a->asmaer;
        if (!P.tauaer || !P.ssaaer || !P.asmaer) return RRTMG_SW_EARGS;
    }
    if (P.iaer == 6) {
        P.ecaer = a->ecaer;
        if (!P.ecaer) return RRTMG_SW_EARGS;
    }
    P.swuflx = a->swuflx; P.swdflx = a->swdflx; P.swhr = a->swhr;
    P.swuflxc = a->swuflxc; P.swdflxc = a->swdflxc; P.swhrc = a->swhrc;
    double* xo[8] = {a->dirdflux, a->difdflux, a->uvdflx, a->nidflx, a->dirdnuv, a->difdnuv, a->dirdnir, a->difdnir};
    for (int i = 0; i < 8; ++i) P.xout[i] = xo[i];
    double* bo[5] = {a->bndfu, a->bndfd, a->bndfddir, a->bndcu, a->bndcd};
    P.bands = 0;
    for (int i = 0; i < 5; ++i) {
        P.bout[i] = bo[i];
        if (bo[i]) P.bands = 1;
    }
    return RRTMG_SW_OK;
}

// Draws of a call's MT stream (mcica_subcol_gen_sw.f90 MT branch): one per
// (subcolumn, column, layer), two for icld 4/5, one per (subcolumn, column)
// for icld 3.
uint64_t mt_stream_length(int icld, int ncol, int nlay) {
    const uint64_t sc = (uint64_t)NGPT * (uint64_t)ncol;
    if (icld == 3) return sc;
    return (icld >= 4 ? 2ull : 1ull) * sc * (uint64_t)nlay;
}

// Bytes of a launch's scratch before the tiled kernel's overflow list, and
// the list's size for npairs column pairs (count word + pair indices).
size_t ovf_offset(size_t slots_bytes) { return (slots_bytes + 255) & ~(size_t)255; }
size_t ovf_bytes(int npairs) { return (size_t)(npairs + 1) * sizeof(int); }

// Queue one solve on `s` (device pointers in a/c) with the given scratch
// buffer and device error word; nothing is synchronised.  Pout / liout
// receive the parameters and launch shape (the tiled FP32 kernel's overflow
// list is read by the caller).
int enqueue_solve(State& st, const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, cudaStream_t s, bool nomcica,
                  DevBuf& scratch, int* err, int& launches, SolveParams* Pout = nullptr,
                  LaunchInfo* liout = nullptr, bool allow_tiled = true, unsigned long long* stats = nullptr) {
    SolveParams P;
    int rc = make_params(st, a, c, P, nomcica);
    if (rc) return rc;
    P.err = err;
    P.stats = stats;
    launches = 1;
    if (P.fused && P.icld >= 1 && P.irng) {
        // the call's MT stream, generated in parallel segments, read by the solve
        const uint64_t nr = mt_stream_length(P.icld, P.ncol, P.nlay);
        DevBuf& rs = st.stage["mt_stream"];
        CK(rs.ensure((nr + 2) * sizeof(uint32_t)));  // + the mask's read-ahead past the last run
        CK(launch_mt_jump((uint32_t)P.permuteseed, nr, (uint32_t*)rs.p, st.num_sms, 0, s));
        P.mt = (const uint32_t*)rs.p;
        launches += 2;
    }
    const bool fp32 = st.form == RRTMG_SW_FORM_FP32;
    LaunchInfo li = fp32 ? plan_fp32(P, st.num_sms, allow_tiled && !st.no_tiled) : plan_fp64(P, st.num_sms);
    st.last_kernel = !fp32 ? RRTMG_SW_KERNEL_FP64 : li.tiled ? RRTMG_SW_KERNEL_FP32_TILED : RRTMG_SW_KERNEL_FP32;
    st.last_tile_slots = fp32 && li.tiled ? li.tile_slots : 0;
    if (!fp32) li.slot_bytes = slot_elems(P.nlay, P.idelm, false) * sizeof(double);
    P.slot_elems = li.slot_bytes / (fp32 ? sizeof(float) : sizeof(double));
    // tiled: per-CTA areas, then the pairs' prepared blocks, then the overflow list
    const size_t off_prep = ovf_offset((size_t)li.grid * li.slot_bytes);
    const size_t off = ovf_offset(off_prep + (size_t)P.npairs * li.prep_bytes);
    CK(scratch.ensure(li.tiled ? off + ovf_bytes(P.npairs) : (size_t)li.grid * li.slot_bytes));
    P.scratch = scratch.p;
    if (li.tiled) {
        P.tprep = (char*)scratch.p + off_prep;
        P.tovfcount = (int*)((char*)scratch.p + off);
        P.tovf = P.tovfcount + 1;
        P.tovfcap = P.npairs;
        P.tile_qcap = st.tile_qcap;
        P.tile_slots = li.tile_slots;
        CK(cudaMemsetAsync(P.tovfcount, 0, sizeof(int), s));
        launches += 1;  // the preparation kernel
    }
    if (fp32) CK(launch_solve_fp32(P, (const float*)st.d_tab32.p, (const double*)st.d_tab64.p, li, s));
    else CK(launch_solve_fp64(P, (const double*)st.d_tab64.p, li, s));
    if (Pout) *Pout = P;
    if (liout) *liout = li;
    return RRTMG_SW_OK;
}

// The tiled FP32 kernel listed `count` column pairs whose FP64 cells
// exceeded its capacities (their outputs are not final): solve them again
// with the scratch-based kernel (k_solve<float>, whose FP64 redo has no such
// limit) through its column map, on the same stream.  With more pairs than
// the list holds, every pair is solved again.  `colmap` is device memory for
// 2 * count + 1 ints; `scratch(bytes)` returns device scratch of that size
// (the tiled launch must have finished: its scratch is reused).
template <typename ScratchFn>
int tiled_fallback(State& st, const SolveParams& Pt, int count, cudaStream_t s, int* colmap, ScratchFn scratch,
                   int& launches) {
    SolveParams P = Pt;
    if (count <= Pt.tovfcap) {
        std::vector<int> pairs(count);
        CK(cudaMemcpyAsync(pairs.data(), Pt.tovf, count * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        std::sort(pairs.begin(), pairs.end());
        std::vector<int> cols(2 * (size_t)count + 1);
        for (int i = 0; i < count; ++i)
            for (int c2 = 0; c2 < COLS_PER_CTA; ++c2) {
                const int k = COLS_PER_CTA * pairs[i] + c2;
                cols[COLS_PER_CTA * i + c2] = k < P.ncol ? k : P.ncol;  // ncol: empty slot
            }
        cols[2 * (size_t)count] = 2 * count;
        CK(cudaMemcpyAsync(colmap, cols.data(), cols.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        P.colmap = colmap;
        P.mapcount = colmap + 2 * (size_t)count;
        P.npairs = count;
    }
    P.tovf = nullptr;
    P.tovfcount = nullptr;
    P.tovfcap = 0;
    LaunchInfo li = plan_fp32(P, st.num_sms, false);
    void* sp = scratch((size_t)li.grid * li.slot_bytes);
    if (!sp) return RRTMG_SW_ESCRATCH;
    P.scratch = sp;
    P.slot_elems = li.slot_bytes / sizeof(float);
    CK(launch_solve_fp32(P, (const float*)st.d_tab32.p, (const double*)st.d_tab64.p, li, s));
    launches += 1;
    return RRTMG_SW_OK;
}

// Queue one solve on `s`; returns after reading back the device error word
// (and, after the tiled FP32 kernel, after solving again any column pairs it
// could not finish).
int solve_dev(State& st, const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, cudaStream_t s, bool nomcica = false,
              bool allow_tiled = true) {
    CK(st.errw.ensure(sizeof(int)));
    int* err = (int*)st.errw.p;
    CK(cudaMemsetAsync(err, 0, sizeof(int), s));
    int launches = 0;
    SolveParams P;
    LaunchInfo li;
    CK(st.statsw.ensure(4 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(st.statsw.p, 0, 4 * sizeof(unsigned long long), s));
    const int rc = enqueue_solve(st, a, c, s, nomcica, st.scratch, err, launches, &P, &li, allow_tiled,
                                 (unsigned long long*)st.statsw.p);
    if (rc) return rc;
    st.h_err[1] = 0;
    CK(cudaMemcpyAsync(st.h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (li.tiled) CK(cudaMemcpyAsync(st.h_err + 1, P.tovfcount, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (li.tiled && st.h_err[0] == 0 && st.h_err[1] > 0) {
        DevBuf& cm = st.stage["tovf_colmap"];
        CK(cm.ensure((2 * (size_t)std::min(st.h_err[1], P.tovfcap) + 1) * sizeof(int)));
        const int r2 = tiled_fallback(st, P, st.h_err[1], s, (int*)cm.p, [&](size_t b) -> void* {
            return st.scratch.ensure(b) == cudaSuccess ? st.scratch.p : nullptr;
        }, launches);
        if (r2) return r2;
        CK(cudaMemcpyAsync(st.h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    CK(cudaMemcpyAsync(st.h_stats, st.statsw.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < 4; ++i) st.last_stats[i] = (long long)st.h_stats[i];
    st.last_launches = launches;
    return bounds_status(st, *st.h_err);
}

// ---------------------------------------------------------------------------
// Page-locked host arrays in column chunks on two streams: a chunk's inputs
// go in, its solve runs and its outputs come back while the other stream's
// chunk copies, so most of the transfer time hides behind the solves.  Columns are
// independent (KISS subcolumn streams are seeded per column), so a chunk is
// the rrtmg_sw call of its column slices and the results are those of one
// call; MT streams (irng = 1) depend on ncol and keep the single-call path.
constexpr int kChunkCols = 16384;  // columns per chunk (even: whole column pairs)
// a chunk's tiled solve left column pairs for the scratch-based kernel: the
// chunked call is repeated as one call without the tiled kernel
constexpr int kRetryUntiled = -2;
constexpr int kChunkStreams = 2;

struct ChunkStreams {
    cudaStream_t s[kChunkStreams] = {nullptr, nullptr};
    DevBuf scratch[kChunkStreams], err[kChunkStreams];
    int* h_err = nullptr;  // pinned, one word per stream
    int* h_ovf = nullptr;  // pinned, the tiled kernel's overflow count of each chunk
    int ovf_cap = 0;
    int device = -1;
};

ChunkStreams& CS() {
    static ChunkStreams c;
    return c;
}

// Whether a host array is page-locked (pinned or registered): only then do
// asynchronous copies overlap the solves; pageable arrays take one staged
// copy per array instead.
bool pinned(const void* p) {
    if (!p) return true;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

bool all_pinned(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c) {
    const void* ps[] = {a->play, a->plev, a->tlay, a->h2ovmr, a->o3vmr, a->co2vmr, a->ch4vmr, a->o2vmr, a->asdir,
                        a->asdif, a->aldir, a->aldif, a->coszen, a->swuflx, a->swdflx, a->swhr, a->swuflxc,
                        a->swdflxc, a->swhrc};
    for (const void* p : ps)
        if (!pinned(p)) return false;
    if (c && (!pinned(c->cldfrac) || !pinned(c->ciwp) || !pinned(c->clwp))) return false;
    if (!c && a->icld >= 1 && !pinned(a->taucmcl)) return false;
    return true;
}

int solve_host_chunked(State& st, const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, bool nomcica) {
    ChunkStreams& cs = CS();
    if (cs.device != st.device) {
        for (int i = 0; i < kChunkStreams; ++i) {
            if (!cs.s[i]) CK(cudaStreamCreateWithFlags(&cs.s[i], cudaStreamNonBlocking));
        }
        if (!cs.h_err) CK(cudaMallocHost((void**)&cs.h_err, kChunkStreams * sizeof(int)));
        cs.device = st.device;
    }
    const size_t C = (size_t)a->ncol, L = (size_t)a->nlay, L1 = L + 1;
    const int icld = (a->icld < 0 || a->icld > 5) ? 2 : a->icld;
    const int iaer = a->iaer;
    for (int i = 0; i < kChunkStreams; ++i) {
        CK(cs.err[i].ensure(sizeof(int)));
        CK(cudaMemsetAsync(cs.err[i].p, 0, sizeof(int), cs.s[i]));
    }
    cudaError_t e = cudaSuccess;
    int launches = 0;
    const int nch = (int)((C + kChunkCols - 1) / kChunkCols);
    if (cs.ovf_cap < nch) {
        if (cs.h_ovf) cudaFreeHost(cs.h_ovf);
        cs.h_ovf = nullptr;
        cs.ovf_cap = 0;
        CK(cudaMallocHost((void**)&cs.h_ovf, nch * sizeof(int)));
        cs.ovf_cap = nch;
    }
    for (int ch = 0; ch < nch; ++ch) cs.h_ovf[ch] = 0;
    CK(st.statsw.ensure(4 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(st.statsw.p, 0, 4 * sizeof(unsigned long long), cs.s[0]));
    CK(cudaStreamSynchronize(cs.s[0]));  // zeroed before either stream's first solve
    for (int ch = 0; ch < nch && e == cudaSuccess; ++ch) {
        const int si = ch % kChunkStreams;
        cudaStream_t s = cs.s[si];
        const size_t c0 = (size_t)ch * kChunkCols, w = std::min((size_t)kChunkCols, C - c0);
        const std::string pre = "chunk" + std::to_string(si) + ":";
        // an array with `inner` contiguous elements per column and `outer`
        // column planes: columns [c0, c0 + w) as a compact (inner, w, outer) slice
        auto buf = [&](const char* name, size_t n) -> double* {
            DevBuf& b = st.stage[pre + name];
            if (e == cudaSuccess) e = b.ensure(n * sizeof(double));
            return e == cudaSuccess ? (double*)b.p : nullptr;
        };
        auto in = [&](const char* name, const double* h, size_t inner, size_t outer) -> const double* {
            if (!h) return nullptr;
            double* d = buf(name, inner * w * outer);
            if (e == cudaSuccess)
                e = cudaMemcpy2DAsync(d, inner * w * sizeof(double), h + inner * c0, inner * C * sizeof(double),
                                      inner * w * sizeof(double), outer, cudaMemcpyHostToDevice, s);
            return d;
        };
        auto out = [&](const char* name, double* h, size_t n) -> double* { return h ? buf(name, n) : nullptr; };
        auto back = [&](double* h, const double* d, size_t outer) {
            if (h && d && e == cudaSuccess)
                e = cudaMemcpy2DAsync(h + c0, C * sizeof(double), d, w * sizeof(double), w * sizeof(double), outer,
                                      cudaMemcpyDeviceToHost, s);
        };
        rrtmg_sw_args d = *a;
        d.ncol = (int32_t)w;
        d.play = in("play", a->play, 1, L); d.plev = in("plev", a->plev, 1, L1); d.tlay = in("tlay", a->tlay, 1, L);
        d.tlev = nullptr; d.tsfc = nullptr; d.n2ovmr = nullptr;  // dead inputs in the SW solve
        d.h2ovmr = in("h2o", a->h2ovmr, 1, L); d.o3vmr = in("o3", a->o3vmr, 1, L);
        d.co2vmr = in("co2", a->co2vmr, 1, L); d.ch4vmr = in("ch4", a->ch4vmr, 1, L);
        d.o2vmr = in("o2", a->o2vmr, 1, L);
        d.asdir = in("asdir", a->asdir, 1, 1); d.asdif = in("asdif", a->asdif, 1, 1);
        d.aldir = in("aldir", a->aldir, 1, 1); d.aldif = in("aldif", a->aldif, 1, 1);
        d.coszen = in("coszen", a->coszen, 1, 1);
        if (icld >= 1 && !c) {
            d.cldfmcl = in("cldfmcl", a->cldfmcl, NGPT, L); d.taucmcl = in("taucmcl", a->taucmcl, NGPT, L);
            d.ssacmcl = in("ssacmcl", a->ssacmcl, NGPT, L); d.asmcmcl = in("asmcmcl", a->asmcmcl, NGPT, L);
            d.fsfcmcl = in("fsfcmcl", a->fsfcmcl, NGPT, L); d.ciwpmcl = in("ciwpmcl", a->ciwpmcl, NGPT, L);
            d.clwpmcl = in("clwpmcl", a->clwpmcl, NGPT, L);
            d.reicmcl = in("reicmcl", a->reicmcl, 1, L); d.relqmcl = in("relqmcl", a->relqmcl, 1, L);
        }
        rrtmg_sw_clouds dc{};
        if (c) {
            dc = *c;
            dc.cldfrac = in("cldfrac", c->cldfrac, 1, L); dc.ciwp = in("ciwp", c->ciwp, 1, L);
            dc.clwp = in("clwp", c->clwp, 1, L); dc.rei = in("rei", c->rei, 1, L); dc.rel = in("rel", c->rel, 1, L);
            dc.tauc = in("tauc", c->tauc, NBND, L); dc.ssac = in("ssac", c->ssac, NBND, L);
            dc.asmc = in("asmc", c->asmc, NBND, L); dc.fsfc = in("fsfc", c->fsfc, NBND, L);
            dc.alpha = in("alpha", c->alpha, 1, L);
        }
        if (iaer == 10) {
            d.tauaer = in("tauaer", a->tauaer, 1, NBND * L); d.ssaaer = in("ssaaer", a->ssaaer, 1, NBND * L);
            d.asmaer = in("asmaer", a->asmaer, 1, NBND * L);
        }
        if (iaer == 6) d.ecaer = in("ecaer", a->ecaer, 1, 6 * L);
        d.swuflx = out("swuflx", a->swuflx, w * L1); d.swdflx = out("swdflx", a->swdflx, w * L1);
        d.swuflxc = out("swuflxc", a->swuflxc, w * L1); d.swdflxc = out("swdflxc", a->swdflxc, w * L1);
        d.swhr = out("swhr", a->swhr, w * L); d.swhrc = out("swhrc", a->swhrc, w * L);
        const char* xn[8] = {"x0", "x1", "x2", "x3", "x4", "x5", "x6", "x7"};
        double* xh[8] = {a->dirdflux, a->difdflux, a->uvdflx, a->nidflx, a->dirdnuv, a->difdnuv, a->dirdnir,
                         a->difdnir};
        double* xd[8];
        for (int i = 0; i < 8; ++i) xd[i] = out(xn[i], xh[i], w * L1);
        d.dirdflux = xd[0]; d.difdflux = xd[1]; d.uvdflx = xd[2]; d.nidflx = xd[3];
        d.dirdnuv = xd[4]; d.difdnuv = xd[5]; d.dirdnir = xd[6]; d.difdnir = xd[7];
        const char* bn[5] = {"b0", "b1", "b2", "b3", "b4"};
        double* bh[5] = {a->bndfu, a->bndfd, a->bndfddir, a->bndcu, a->bndcd};
        double* bd[5];
        for (int i = 0; i < 5; ++i) bd[i] = out(bn[i], bh[i], w * L1 * NBND);
        d.bndfu = bd[0]; d.bndfd = bd[1]; d.bndfddir = bd[2]; d.bndcu = bd[3]; d.bndcd = bd[4];
        if (e != cudaSuccess) break;
        int nl = 0;
        SolveParams Pc;
        LaunchInfo lic;
        const int rc = enqueue_solve(st, &d, c ? &dc : nullptr, s, nomcica, cs.scratch[si], (int*)cs.err[si].p, nl,
                                     &Pc, &lic, true, (unsigned long long*)st.statsw.p);
        if (rc) {
            for (int i = 0; i < kChunkStreams; ++i) cudaStreamSynchronize(cs.s[i]);
            return rc;
        }
        // the chunk's overflow count, read before the next chunk on this stream reuses the scratch
        if (lic.tiled) e = cudaMemcpyAsync(cs.h_ovf + ch, Pc.tovfcount, sizeof(int), cudaMemcpyDeviceToHost, s);
        launches += nl;
        back(a->swuflx, d.swuflx, L1); back(a->swdflx, d.swdflx, L1);
        back(a->swuflxc, d.swuflxc, L1); back(a->swdflxc, d.swdflxc, L1);
        back(a->swhr, d.swhr, L); back(a->swhrc, d.swhrc, L);
        for (int i = 0; i < 8; ++i) back(xh[i], xd[i], L1);
        for (int i = 0; i < 5; ++i) back(bh[i], bd[i], L1 * NBND);
    }
    for (int i = 0; i < kChunkStreams; ++i) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(cs.h_err + i, cs.err[i].p, sizeof(int), cudaMemcpyDeviceToHost, cs.s[i]);
    }
    for (int i = 0; i < kChunkStreams; ++i) {
        const cudaError_t e2 = cudaStreamSynchronize(cs.s[i]);
        if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) return cuda_fail(e);
    CK(cudaMemcpyAsync(st.h_stats, st.statsw.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, cs.s[0]));
    CK(cudaStreamSynchronize(cs.s[0]));
    for (int i = 0; i < 4; ++i) st.last_stats[i] = (long long)st.h_stats[i];
    st.last_launches = launches;
    for (int i = 0; i < kChunkStreams; ++i)
        if (cs.h_err[i]) return cs.h_err[i];
    for (int ch = 0; ch < nch; ++ch)
        if (cs.h_ovf[ch] > 0) return kRetryUntiled;  // rare: the caller solves the call again in one piece
    return bounds_status(st, RRTMG_SW_OK);
}

// Host-array path: stage every array in a named device buffer.
struct Stager {
    State& st;
    cudaStream_t s;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T* in(const char* name, const T* h, size_t n) {
        if (!h || err != cudaSuccess) return nullptr;
        DevBuf& b = st.stage[name];
        if ((err = b.ensure(n * sizeof(T))) != cudaSuccess) return nullptr;
        err = cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s);
        return (T*)b.p;
    }
    double* out(const char* name, double* h, size_t n) {
        if (!h || err != cudaSuccess) return nullptr;
        DevBuf& b = st.stage[name];
        if ((err = b.ensure(n * sizeof(double))) != cudaSuccess) return nullptr;
        return (double*)b.p;
    }
    void back(double* h, const double* d, size_t n) {
        if (h && d && err == cudaSuccess) err = cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, s);
    }
};

int solve_host(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, bool nomcica = false) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    int rc = ready(st);
    if (rc) return rc;
    rc = check_args(a);
    if (rc) return rc == kEmpty ? RRTMG_SW_OK : rc;
    const bool mt = c && !nomcica && a->icld >= 1 && c->irng != 0;
    bool allow_tiled = true;
    if (!mt && a->ncol >= 2 * kChunkCols && all_pinned(a, c)) {
        rc = solve_host_chunked(st, a, c, nomcica);
        if (rc != kRetryUntiled) return rc;
        allow_tiled = false;
    }
    const size_t C = a->ncol, L = a->nlay, CL = C * L, CL1 = C * (L + 1), G = (size_t)NGPT * CL;
    cudaStream_t s = st.host_stream;
    Stager sg{st, s};
    rrtmg_sw_args d = *a;
    d.play = sg.in("play", a->play, CL); d.plev = sg.in("plev", a->plev, CL1); d.tlay = sg.in("tlay", a->tlay, CL);
    d.tlev = nullptr; d.tsfc = nullptr; d.n2ovmr = nullptr;  // dead inputs in the SW solve
    d.h2ovmr = sg.in("h2o", a->h2ovmr, CL); d.o3vmr = sg.in("o3", a->o3vmr, CL); d.co2vmr = sg.in("co2", a->co2vmr, CL);
    d.ch4vmr = sg.in("ch4", a->ch4vmr, CL); d.o2vmr = sg.in("o2", a->o2vmr, CL);
    d.asdir = sg.in("asdir", a->asdir, C); d.asdif = sg.in("asdif", a->asdif, C);
    d.aldir = sg.in("aldir", a->aldir, C); d.aldif = sg.in("aldif", a->aldif, C);
    d.coszen = sg.in("coszen", a->coszen, C);
    const int icld = (a->icld < 0 || a->icld > 5) ? 2 : a->icld;
    if (icld >= 1 && !c) {
        d.cldfmcl = sg.in("cldfmcl", a->cldfmcl, G); d.taucmcl = sg.in("taucmcl", a->taucmcl, G);
        d.ssacmcl = sg.in("ssacmcl", a->ssacmcl, G); d.asmcmcl = sg.in("asmcmcl", a->asmcmcl, G);
        d.fsfcmcl = sg.in("fsfcmcl", a->fsfcmcl, G); d.ciwpmcl = sg.in("ciwpmcl", a->ciwpmcl, G);
        d.clwpmcl = sg.in("clwpmcl", a->clwpmcl, G);
        d.reicmcl = sg.in("reicmcl", a->reicmcl, CL); d.relqmcl = sg.in("relqmcl", a->relqmcl, CL);
    }
    rrtmg_sw_clouds dc{};
    if (c) {
        dc = *c;
        dc.cldfrac = sg.in("cldfrac", c->cldfrac, CL); dc.ciwp = sg.in("ciwp", c->ciwp, CL);
        dc.clwp = sg.in("clwp", c->clwp, CL); dc.rei = sg.in("rei", c->rei, CL); dc.rel = sg.in("rel", c->rel, CL);
        dc.tauc = sg.in("tauc", c->tauc, 14 * CL); dc.ssac = sg.in("ssac", c->ssac, 14 * CL);
        dc.asmc = sg.in("asmc", c->asmc, 14 * CL); dc.fsfc = sg.in("fsfc", c->fsfc, 14 * CL);
        dc.alpha = sg.in("alpha", c->alpha, CL);
    }
    const int iaer = a->iaer;
    if (iaer == 10) {
        d.tauaer = sg.in("tauaer", a->tauaer, 14 * CL); d.ssaaer = sg.in("ssaaer", a->ssaaer, 14 * CL);
        d.asmaer = sg.in("asmaer", a->asmaer, 14 * CL);
    }
    if (iaer == 6) d.ecaer = sg.in("ecaer", a->ecaer, 6 * CL);
    d.swuflx = sg.out("swuflx", a->swuflx, CL1); d.swdflx = sg.out("swdflx", a->swdflx, CL1);
    d.swuflxc = sg.out("swuflxc", a->swuflxc, CL1); d.swdflxc = sg.out("swdflxc", a->swdflxc, CL1);
    d.swhr = sg.out("swhr", a->swhr, CL); d.swhrc = sg.out("swhrc", a->swhrc, CL);
    const char* xn[8] = {"x0", "x1", "x2", "x3", "x4", "x5", "x6", "x7"};
    double* xh[8] = {a->dirdflux, a->difdflux, a->uvdflx, a->nidflx, a->dirdnuv, a->difdnuv, a->dirdnir, a->difdnir};
    double* xd[8];
    for (int i = 0; i < 8; ++i) xd[i] = sg.out(xn[i], xh[i], CL1);
    d.dirdflux = xd[0]; d.difdflux = xd[1]; d.uvdflx = xd[2]; d.nidflx = xd[3];
    d.dirdnuv = xd[4]; d.difdnuv = xd[5]; d.dirdnir = xd[6]; d.difdnir = xd[7];
    const char* bn[5] = {"b0", "b1", "b2", "b3", "b4"};
    double* bh[5] = {a->bndfu, a->bndfd, a->bndfddir, a->bndcu, a->bndcd};
    double* bd[5];
    for (int i = 0; i < 5; ++i) bd[i] = sg.out(bn[i], bh[i], 14 * CL1);
    d.bndfu = bd[0]; d.bndfd = bd[1]; d.bndfddir = bd[2]; d.bndcu = bd[3]; d.bndcd = bd[4];
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    rc = solve_dev(st, &d, c ? &dc : nullptr, s, nomcica, allow_tiled);
    if (rc) return rc;
    sg.back(a->swuflx, d.swuflx, CL1); sg.back(a->swdflx, d.swdflx, CL1);
    sg.back(a->swuflxc, d.swuflxc, CL1); sg.back(a->swdflxc, d.swdflxc, CL1);
    sg.back(a->swhr, d.swhr, CL); sg.back(a->swhrc, d.swhrc, CL);
    for (int i = 0; i < 8; ++i) sg.back(xh[i], xd[i], CL1);
    for (int i = 0; i < 5; ++i) sg.back(bh[i], bd[i], 14 * CL1);
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    CK(cudaStreamSynchronize(s));
    return RRTMG_SW_OK;
}

// ---------------------------------------------------------------------------
// Fixed scratch for rrtmg_sw_static_dev_c.  For callers that may not allocate
// device memory once they run (a model whose pool owns the GPU, a time step
// that forbids allocation): the per-CTA pass-1 -> pass-2 scratch lives in
// this module-scope area instead of the cudaMalloc'd workspace.  Its contents
// never need clearing (every slot value is written before it is read); the
// error word is cleared on the stream by each call.  One area per device, so
// two solves on it at once would race; calls are serialised by State::mu and
// each call waits for its kernel.  The area belongs to this library's CUDA
// module: with lazy module loading (the CUDA 12+ default) a device reserves
// it when the module is first used there; with CUDA_MODULE_LOADING=EAGER every
// device a process creates a context on reserves it at context creation,
// whether or not the entry point is ever called.
constexpr size_t kStaticScratchBytes = size_t(256) << 20;
constexpr int kMaxDevices = 64;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
static __device__ __align__(256) int g_static_err;

struct StaticArea {
    void* scratch = nullptr;
    int* err = nullptr;
};
StaticArea g_static_area[kMaxDevices];  // filled on the first call per device, under State::mu

// Address of the area on the current device (looked up once per device; the
// lookup also loads this module on that device).
cudaError_t static_area(int dev, StaticArea& out) {
    StaticArea& a = g_static_area[dev];
    if (!a.scratch) {
        void* p = nullptr;
        void* e = nullptr;
        cudaError_t r = cudaGetSymbolAddress(&p, g_static_scratch);
        if (r != cudaSuccess) return r;
        r = cudaGetSymbolAddress(&e, g_static_err);
        if (r != cudaSuccess) return r;
        a.scratch = p;
        a.err = (int*)e;
    }
    out = a;
    return cudaSuccess;
}

// The last kStaticTail bytes of the static area hold the tiled FP32
// kernel's overflow list (a count and up to kStaticOvfCap column pairs) and
// the column map of their second solve; slots come from the rest.
constexpr int kStaticOvfCap = 4096;
constexpr size_t kStaticTail = (((size_t)(1 + kStaticOvfCap) + (2 * (size_t)kStaticOvfCap + 1)) * sizeof(int) +
                                255) & ~(size_t)255;

int solve_static(State& st, const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, cudaStream_t s) {
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev != st.device) return RRTMG_SW_ENOTINIT;  // tables live on the device rrtmg_sw_ini_c used
    if (dev < 0 || dev >= kMaxDevices) return RRTMG_SW_EARGS;
    SolveParams P;
    int rc = make_params(st, a, c, P);
    if (rc) return rc;
    if (P.irng) return RRTMG_SW_EIRNG;  // the MT stream needs a device buffer
    const bool fp32 = st.form == RRTMG_SW_FORM_FP32;
    const size_t avail = kStaticScratchBytes - kStaticTail;
    LaunchInfo li = fp32 ? plan_fp32(P, st.num_sms, !st.no_tiled) : plan_fp64(P, st.num_sms);
    // the tiled kernel's prepared blocks (one per pair) must fit beside its
    // per-CTA areas; larger calls take the scratch-based kernel
    const size_t off_prep = (((size_t)li.grid * li.slot_bytes) + 255) & ~(size_t)255;
    if (li.tiled && off_prep + (size_t)P.npairs * li.prep_bytes > avail) li = plan_fp32(P, st.num_sms, false);
    st.last_kernel = !fp32 ? RRTMG_SW_KERNEL_FP64 : li.tiled ? RRTMG_SW_KERNEL_FP32_TILED : RRTMG_SW_KERNEL_FP32;
    st.last_tile_slots = fp32 && li.tiled ? li.tile_slots : 0;
    if (!fp32) li.slot_bytes = slot_elems(P.nlay, P.idelm, false) * sizeof(double);
    const size_t slots = avail / li.slot_bytes;
    // one slot per SM, or per column pair when the call has fewer pairs
    const size_t need = (size_t)std::min(li.grid, st.num_sms);
    if (slots < need) return RRTMG_SW_ESCRATCH;
    if ((size_t)li.grid > slots) li.grid = (int)slots;
    P.slot_elems = li.slot_bytes / (fp32 ? sizeof(float) : sizeof(double));
    StaticArea area;
    CK(static_area(dev, area));
    P.scratch = area.scratch;
    P.err = area.err;
    int* tail = (int*)((char*)area.scratch + avail);
    if (li.tiled) {
        P.tprep = (char*)area.scratch + off_prep;
        P.tovfcount = tail;
        P.tovf = tail + 1;
        P.tovfcap = std::min(P.npairs, kStaticOvfCap);
        P.tile_qcap = st.tile_qcap;
        P.tile_slots = li.tile_slots;
        CK(cudaMemsetAsync(P.tovfcount, 0, sizeof(int), s));
    }
    CK(cudaMemsetAsync(P.err, 0, sizeof(int), s));
    if (fp32) CK(launch_solve_fp32(P, (const float*)st.d_tab32.p, (const double*)st.d_tab64.p, li, s));
    else CK(launch_solve_fp64(P, (const double*)st.d_tab64.p, li, s));
    int launches = li.tiled ? 2 : 1;
    int h[2] = {0, 0};  // pageable: the copies complete before the calls return
    CK(cudaMemcpyAsync(&h[0], P.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (li.tiled) CK(cudaMemcpyAsync(&h[1], P.tovfcount, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (li.tiled && h[0] == 0 && h[1] > 0) {
        // column pairs the tiled kernel left: the scratch-based kernel, in the
        // same area (its column map after the overflow list)
        const int r2 = tiled_fallback(st, P, h[1], s, tail + 1 + kStaticOvfCap,
                                      [&](size_t b) -> void* { return b <= avail ? area.scratch : nullptr; },
                                      launches);
        if (r2) return r2;
        CK(cudaMemcpyAsync(&h[0], P.err, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    st.last_launches = launches;
    return bounds_status(st, h[0]);
}

// ---------------------------------------------------------------------------
// Tangent-linear / adjoint with host arrays (see solve_ad.cu).
int solve_ad_host(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, const rrtmg_sw_ad_args* ad, bool tl) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    const int rr = ready(st);
    if (rr) return rr;
    if (a && ad && a->ncol == 0) return RRTMG_SW_OK;
    if (!a || !ad || a->ncol < 0 || a->nlay < 1 || a->nlay > MAX_NLAY) return RRTMG_SW_EARGS;
    const double* req[] = {a->play, a->plev, a->tlay, a->h2ovmr, a->o3vmr, a->co2vmr, a->ch4vmr, a->o2vmr,
                           a->asdir, a->asdif, a->aldir, a->aldif, a->coszen};
    for (const double* p : req)
        if (!p) return RRTMG_SW_EARGS;
    const int icld = (a->icld < 0 || a->icld > 5) ? 2 : a->icld;
    if (icld >= 1 && !c) return RRTMG_SW_EARGS;
    const size_t C = a->ncol, L = a->nlay, CL = C * L, CL1 = C * (L + 1);
    cudaStream_t s = st.host_stream;
    Stager sg{st, s};
    rrtmg_sw_args d = *a;
    d.play = sg.in("play", a->play, CL); d.plev = sg.in("plev", a->plev, CL1); d.tlay = sg.in("tlay", a->tlay, CL);
    d.h2ovmr = sg.in("h2o", a->h2ovmr, CL); d.o3vmr = sg.in("o3", a->o3vmr, CL); d.co2vmr = sg.in("co2", a->co2vmr, CL);
    d.ch4vmr = sg.in("ch4", a->ch4vmr, CL); d.o2vmr = sg.in("o2", a->o2vmr, CL);
    d.asdir = sg.in("asdir", a->asdir, C); d.asdif = sg.in("asdif", a->asdif, C);
    d.aldir = sg.in("aldir", a->aldir, C); d.aldif = sg.in("aldif", a->aldif, C);
    d.coszen = sg.in("coszen", a->coszen, C);
    d.tlev = nullptr; d.tsfc = nullptr; d.n2ovmr = nullptr;
    if (a->iaer == 10) {
        d.tauaer = sg.in("tauaer", a->tauaer, 14 * CL); d.ssaaer = sg.in("ssaaer", a->ssaaer, 14 * CL);
        d.asmaer = sg.in("asmaer", a->asmaer, 14 * CL);
    }
    if (a->iaer == 6) d.ecaer = sg.in("ecaer", a->ecaer, 6 * CL);
    rrtmg_sw_clouds dc{};
    if (c && icld >= 1) {
        dc = *c;
        dc.cldfrac = sg.in("cldfrac", c->cldfrac, CL); dc.ciwp = sg.in("ciwp", c->ciwp, CL);
        dc.clwp = sg.in("clwp", c->clwp, CL); dc.rei = sg.in("rei", c->rei, CL); dc.rel = sg.in("rel", c->rel, CL);
        dc.tauc = sg.in("tauc", c->tauc, 14 * CL); dc.ssac = sg.in("ssac", c->ssac, 14 * CL);
        dc.asmc = sg.in("asmc", c->asmc, 14 * CL); dc.fsfc = sg.in("fsfc", c->fsfc, 14 * CL);
        dc.alpha = sg.in("alpha", c->alpha, CL);
    }
    // the flux outputs are not written; make_params only records them
    AdParams A{};
    A.w_toa = ad->w_toa_up; A.w_net = ad->w_sfc_net; A.w_hr = ad->w_hr_sum;
    A.store = ad->store > 0 ? 1 : 0;  // store < 0: chosen below from free device memory
    A.tl = tl ? 1 : 0;
    A.J = sg.out("adJ", ad->J, C);
    A.dJ = tl ? sg.out("addJ", ad->dJ, C) : nullptr;
    double* gh[5] = {ad->tlay, ad->h2ovmr, ad->o3vmr, ad->clwp, ad->ciwp};
    double* ah[4] = {ad->asdir, ad->asdif, ad->aldir, ad->aldif};
    const char* gn[5] = {"adg0", "adg1", "adg2", "adg3", "adg4"};
    const char* an[4] = {"ada0", "ada1", "ada2", "ada3"};
    double* gd[5];
    double* ad4[4];
    for (int i = 0; i < 5; ++i) {
        if (tl) { A.dir[i] = sg.in(gn[i], (const double*)gh[i], CL); gd[i] = nullptr; }
        else { gd[i] = sg.out(gn[i], gh[i], CL); A.g[i] = gd[i]; }
    }
    for (int i = 0; i < 4; ++i) {
        if (tl) { A.dira[i] = sg.in(an[i], (const double*)ah[i], C); ad4[i] = nullptr; }
        else { ad4[i] = sg.out(an[i], ah[i], C); A.ga[i] = ad4[i]; }
    }
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    SolveParams P;
    int rc = make_params(st, &d, (c && icld >= 1) ? &dc : nullptr, P);
    if (rc) return rc;
    if (P.irng) return RRTMG_SW_EIRNG;
    CK(st.errw.ensure(sizeof(int)));
    P.err = (int*)st.errw.p;
    const int grid = adjoint_grid(P, st.num_sms);
    if (ad->store < 0) {
        // stored Jacobians when their scratch fits in half the free memory
        // (beyond what is already allocated), else recomputed
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        const size_t need = (size_t)grid * adjoint_slot_elems(P.nlay, 1) * sizeof(double);
        A.store = need <= st.scratch.bytes + fr / 2 ? 1 : 0;
    }
    st.last_ad_store = A.store;
    P.slot_elems = adjoint_slot_elems(P.nlay, A.store);
    CK(st.scratch.ensure((size_t)grid * P.slot_elems * sizeof(double)));
    P.scratch = st.scratch.p;
    CK(cudaMemsetAsync(P.err, 0, sizeof(int), s));
    CK(launch_adjoint(P, A, (const double*)st.d_tab64.p, st.num_sms, nullptr, s));
    st.last_launches = 1;
    sg.back(ad->J, A.J, C);
    if (tl) sg.back(ad->dJ, A.dJ, C);
    for (int i = 0; i < 5 && !tl; ++i) sg.back(gh[i], gd[i], CL);
    for (int i = 0; i < 4 && !tl; ++i) sg.back(ah[i], ad4[i], C);
    CK(cudaMemcpyAsync(st.h_err, P.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    CK(cudaStreamSynchronize(s));
    return bounds_status(st, *st.h_err);
}

// ---------------------------------------------------------------------------
// Batch plans: many instances in one persistent launch (k_compact + k_solve_batch),
// captured once in a CUDA graph and replayed.
struct BatchPlan {
    int n = 0, form = 0, grid = 0, desc = 0, device = 0;
    int tile = COLS_PER_CTA;  // columns per CTA (x 112 g-points)
    size_t smem = 0;
    DevBuf params, maps, offs, counts, scratch, errw;
    int* h_err = nullptr;  // pinned
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<float> tune_ms;  // per candidate: (tile, order, blocks per SM) in trial order
    std::vector<int> tune_cfg;   // per candidate: tile << 16 | deepest first << 8 | blocks per SM
};

// Kernel launch of a plan with tile bp.tile, shared memory bp.smem.
cudaError_t batch_launch(State& st, BatchPlan& bp, int grid, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bp.errw.p, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    e = launch_compact((const SolveParams*)bp.params.p, bp.n, (int*)bp.maps.p, (const long long*)bp.offs.p,
                       (int*)bp.counts.p, s);
    if (e != cudaSuccess) return e;
    if (bp.form == RRTMG_SW_FORM_FP32)
        return launch_batch_fp32((const SolveParams*)bp.params.p, bp.n, (const int*)bp.counts.p,
                                 (const float*)st.d_tab32.p, (const double*)st.d_tab64.p, grid, bp.smem, bp.tile,
                                 s);
    return launch_batch_fp64((const SolveParams*)bp.params.p, bp.n, (const int*)bp.counts.p,
                             (const double*)st.d_tab64.p, grid, bp.smem, bp.tile, s);
}

// Upload the instances' parameters in the given order (sunlit lists and
// counts follow the order).
cudaError_t batch_upload(BatchPlan& bp, std::vector<SolveParams> P, const std::vector<int>& order, cudaStream_t s) {
    std::vector<SolveParams> Q(bp.n);
    std::vector<long long> off(bp.n);
    long long o = 0;
    for (int k = 0; k < bp.n; ++k) {
        Q[k] = P[order[k]];
        off[k] = o;
        Q[k].colmap = (const int*)bp.maps.p + o;
        Q[k].mapcount = (const int*)bp.counts.p + k;
        o += Q[k].ncol;
    }
    cudaError_t e = cudaMemcpyAsync(bp.params.p, Q.data(), sizeof(SolveParams) * bp.n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(bp.offs.p, off.data(), sizeof(long long) * bp.n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

void batch_release(BatchPlan* bp) {
    if (!bp) return;
    if (bp->exec) cudaGraphExecDestroy(bp->exec);
    if (bp->graph) cudaGraphDestroy(bp->graph);
    bp->params.release(); bp->maps.release(); bp->offs.release(); bp->counts.release();
    bp->scratch.release(); bp->errw.release();
    if (bp->h_err) cudaFreeHost(bp->h_err);
    delete bp;
}

int batch_plan(State& st, const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, int n, cudaStream_t s, BatchPlan** out) {
    if (n < 1 || n > MAX_BATCH) return RRTMG_SW_EARGS;
    BatchPlan* bp = new BatchPlan();
    bp->n = n;
    bp->form = st.form;
    bp->device = st.device;
    const bool fp32 = st.form == RRTMG_SW_FORM_FP32;
    std::vector<SolveParams> P(n);
    // tile candidates: 2 or 4 columns x 112 g-points per CTA; shared memory
    // and scratch slots sized for the deepest instance
    constexpr int NTILE = 2;
    const int tiles[NTILE] = {2, 4};
    size_t slot[NTILE] = {0, 0}, smem[NTILE] = {0, 0};
    int per_sm[NTILE] = {0, 0};
    long long cols = 0;
    for (int i = 0; i < n; ++i) {
        int rc = check_args(a + i);
        if (rc == kEmpty) rc = RRTMG_SW_EARGS;  // a batch instance needs columns
        if (!rc) rc = make_params(st, a + i, (c && a[i].icld >= 1) ? c + i : nullptr, P[i]);
        if (!rc && P[i].irng) rc = RRTMG_SW_EIRNG;
        if (rc) { batch_release(bp); return rc; }
        for (int k = 0; k < NTILE; ++k) {
            slot[k] = std::max(slot[k], slot_elems(P[i].nlay, P[i].idelm, fp32, tiles[k]));
            smem[k] = std::max(smem[k], fp32 ? solve_smem_fp32(P[i], tiles[k]) : solve_smem_fp64(P[i], tiles[k]));
        }
        cols += P[i].ncol;
    }
    const size_t esz = fp32 ? sizeof(float) : sizeof(double);
    size_t scratch_bytes = 0;
    for (int k = 0; k < NTILE; ++k) {
        per_sm[k] = fp32 ? batch_blocks_per_sm_fp32(smem[k], tiles[k]) : batch_blocks_per_sm_fp64(smem[k], tiles[k]);
        if (per_sm[k] > 0) scratch_bytes = std::max(scratch_bytes, (size_t)st.num_sms * per_sm[k] * slot[k] * esz);
    }
    const bool tile_ok = st.batch_tile == 0 || st.batch_tile == 2 || (st.batch_tile == 4 && per_sm[1] >= 1);
    if (per_sm[0] < 1 || !tile_ok) { batch_release(bp); return RRTMG_SW_EARGS; }
    cudaError_t e = cudaSuccess;
    if ((e = bp->params.ensure(sizeof(SolveParams) * n)) != cudaSuccess ||
        (e = bp->maps.ensure(sizeof(int) * (size_t)(cols > 0 ? cols : 1))) != cudaSuccess ||
        (e = bp->offs.ensure(sizeof(long long) * n)) != cudaSuccess ||
        (e = bp->counts.ensure(sizeof(int) * n)) != cudaSuccess ||
        (e = bp->scratch.ensure(scratch_bytes)) != cudaSuccess ||
        (e = bp->errw.ensure(sizeof(int))) != cudaSuccess ||
        (e = cudaMallocHost((void**)&bp->h_err, sizeof(int))) != cudaSuccess) {
        batch_release(bp);
        return cuda_fail(e);
    }
    for (int i = 0; i < n; ++i) {
        P[i].scratch = bp->scratch.p;
        P[i].err = (int*)bp->errw.p;
    }
    // autotuner: tile (columns x g-points per CTA) x instance order (as
    // given / deepest first) x resident CTAs per SM, one timed run each
    std::vector<int> given(n), desc(n);
    for (int i = 0; i < n; ++i) given[i] = desc[i] = i;
    std::stable_sort(desc.begin(), desc.end(), [&](int x, int y) { return P[x].nlay > P[y].nlay; });
    auto set_tile = [&](int k) {
        bp->tile = tiles[k];
        bp->smem = smem[k];
        for (int i = 0; i < n; ++i) P[i].slot_elems = slot[k];
    };
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int best_k = 1, best_desc = 0, best_t = 0;
    for (int t = 0; t < NTILE && e == cudaSuccess; ++t) {
        if (per_sm[t] < 1) continue;  // the tile's shared memory does not fit
        if (st.batch_tile && st.batch_tile != tiles[t]) continue;
        set_tile(t);
        for (int od = 0; od < 2 && e == cudaSuccess; ++od) {
            if ((e = batch_upload(*bp, P, od ? desc : given, s)) != cudaSuccess) break;
            for (int k = 1; k <= per_sm[t] && e == cudaSuccess; ++k) {
                const int grid = st.num_sms * k;
                if ((e = batch_launch(st, *bp, grid, s)) != cudaSuccess) break;  // warm-up
                cudaEventRecord(e0, s);
                if ((e = batch_launch(st, *bp, grid, s)) != cudaSuccess) break;
                cudaEventRecord(e1, s);
                if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                bp->tune_ms.push_back(ms);
                bp->tune_cfg.push_back(tiles[t] << 16 | od << 8 | k);
                if (ms < best) { best = ms; best_k = k; best_desc = od; best_t = t; }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    set_tile(best_t);
    if (e == cudaSuccess) e = batch_upload(*bp, P, best_desc ? desc : given, s);
    bp->grid = st.num_sms * best_k;
    bp->desc = best_desc;
    // capture compaction + solve into a graph on a private stream
    cudaStream_t cs = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t le = batch_launch(st, *bp, bp->grid, cs);
        e = cudaStreamEndCapture(cs, &bp->graph);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&bp->exec, bp->graph, 0);
    if (cs) cudaStreamDestroy(cs);
    if (e != cudaSuccess) { batch_release(bp); return cuda_fail(e); }
    *out = bp;
    return RRTMG_SW_OK;
}

}  // namespace

extern "C" {

int rrtmg_sw_ini_c(double cpdair) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    st.cpdair = cpdair;
    if (!st.init) {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        st.device = dev;
        CK(cudaDeviceGetAttribute(&st.num_sms, cudaDevAttrMultiProcessorCount, dev));
        const int rc = build_tables(st);
        if (rc) return rc;
        CK(cudaMallocHost((void**)&st.h_err, 2 * sizeof(int)));
        CK(cudaMallocHost((void**)&st.h_stats, 4 * sizeof(unsigned long long)));
        CK(cudaStreamCreateWithFlags(&st.host_stream, cudaStreamNonBlocking));
    }
    {
        const char* t = std::getenv("RRTMG_SW_TILED");
        st.no_tiled = t && std::strcmp(t, "0") == 0;
        const char* q = std::getenv("RRTMG_SW_TILE_QCAP");
        st.tile_qcap = q ? std::atoi(q) : 0;
        const char* bt = std::getenv("RRTMG_SW_BATCH_TILE");
        st.batch_tile = bt ? std::atoi(bt) : 0;
    }
    const int rc = upload(st);
    if (rc) return rc;
    st.init = true;
    return RRTMG_SW_OK;
}

int rrtmg_sw_c(const rrtmg_sw_args* a) { return solve_host(a, nullptr); }

int rrtmg_sw_mcica_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c) {
    if (!c) return RRTMG_SW_EARGS;
    return solve_host(a, c);
}

int rrtmg_sw_dev_c(const rrtmg_sw_args* a, void* stream) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    const int rc = check_args(a);
    if (rc) return rc == kEmpty ? RRTMG_SW_OK : rc;
    return solve_dev(st, a, nullptr, (cudaStream_t)stream);
}

int rrtmg_sw_nomcica_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c) {
    if (!c) return RRTMG_SW_EARGS;
    return solve_host(a, c, true);
}

int rrtmg_sw_nomcica_dev_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, void* stream) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (!c) return RRTMG_SW_EARGS;
    const int rc = check_args(a);
    if (rc) return rc == kEmpty ? RRTMG_SW_OK : rc;
    return solve_dev(st, a, c, (cudaStream_t)stream, true);
}

int rrtmg_sw_mcica_dev_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, void* stream) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (!c) return RRTMG_SW_EARGS;
    const int rc = check_args(a);
    if (rc) return rc == kEmpty ? RRTMG_SW_OK : rc;
    return solve_dev(st, a, c, (cudaStream_t)stream);
}

int rrtmg_sw_static_dev_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, void* stream) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    const int rc = check_args(a);
    if (rc) return rc == kEmpty ? RRTMG_SW_OK : rc;
    return solve_static(st, a, c, (cudaStream_t)stream);
}

int mcica_subcol_sw_c(int32_t ncol, int32_t nlay, int32_t icld, int32_t permuteseed, int32_t irng,
                      const double* play, const double* cldfrac, const double* ciwp, const double* clwp,
                      const double* rei, const double* rel, const double* tauc, const double* ssac,
                      const double* asmc, const double* fsfc, const double* alpha, double* cldfmcl,
                      double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl, double* taucmcl,
                      double* ssacmcl, double* asmcmcl, double* fsfcmcl) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (icld == 0) return RRTMG_SW_OK;                 // mcica:261
    if (icld < 0 || icld > 5) return RRTMG_SW_EICLD;    // mcica:262-264
    if (ncol == 0) return RRTMG_SW_OK;
    if (ncol < 0 || nlay < 1 || !play || !cldfrac || !ciwp || !clwp || !rei || !rel) return RRTMG_SW_EARGS;
    if (irng == 0 && nlay < 4) return RRTMG_SW_EKISSSEED;  // KISS seeds from the bottom four layers (mcica:470-478)
    if (icld >= 4 && !alpha) return RRTMG_SW_EARGS;
    if (irng != 0) irng = 1;                            // mcica:455
    const size_t C = ncol, L = nlay, CL = C * L, G = (size_t)NGPT * CL;
    cudaStream_t s = st.host_stream;
    Stager sg{st, s};
    const double* d_play = sg.in("m_play", play, CL);
    const double* d_cf = sg.in("m_cf", cldfrac, CL);
    const double* d_ciwp = sg.in("m_ciwp", ciwp, CL);
    const double* d_clwp = sg.in("m_clwp", clwp, CL);
    const double* d_tauc = sg.in("m_tauc", tauc, 14 * CL);
    const double* d_ssac = sg.in("m_ssac", ssac, 14 * CL);
    const double* d_asmc = sg.in("m_asmc", asmc, 14 * CL);
    const double* d_fsfc = sg.in("m_fsfc", fsfc, 14 * CL);
    const double* d_alpha = sg.in("m_alpha", alpha, CL);
    double* o[7];
    double* h[7] = {cldfmcl, ciwpmcl, clwpmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl};
    const char* on[7] = {"mo0", "mo1", "mo2", "mo3", "mo4", "mo5", "mo6"};
    for (int i = 0; i < 7; ++i) {
        if (!h[i]) return RRTMG_SW_EARGS;
        o[i] = sg.out(on[i], h[i], G);
    }
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    if (!d_tauc || !d_ssac || !d_asmc || !d_fsfc) d_tauc = d_ssac = d_asmc = d_fsfc = nullptr;
    CK(st.errw.ensure(sizeof(int)));
    CK(cudaMemsetAsync(st.errw.p, 0, sizeof(int), s));
    if (irng == 0) {
        CK(launch_mcica_kiss(ncol, nlay, icld, permuteseed, d_play, d_cf, d_ciwp, d_clwp, d_tauc, d_ssac, d_asmc,
                             d_fsfc, d_alpha, o[0], o[1], o[2], o[3], o[4], o[5], o[6], (int*)st.errw.p, s));
        st.last_launches = 1;
    } else {
        const uint64_t nr = mt_stream_length(icld, ncol, nlay);
        DevBuf& rs = st.stage["mt_stream"];
        CK(rs.ensure((nr + 2) * sizeof(uint32_t)));  // + the mask's read-ahead past the last run
        CK(launch_mt_jump((uint32_t)permuteseed, nr, (uint32_t*)rs.p, st.num_sms, 0, s));
        CK(launch_mcica_stream(ncol, nlay, icld, (const uint32_t*)rs.p, d_cf, d_ciwp, d_clwp, d_tauc, d_ssac, d_asmc,
                               d_fsfc, d_alpha, o[0], o[1], o[2], o[3], o[4], o[5], o[6], s));
        st.last_launches = 3;
    }
    CK(cudaMemcpyAsync(st.h_err, st.errw.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    for (int i = 0; i < 7; ++i) sg.back(h[i], o[i], G);
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    CK(cudaStreamSynchronize(s));
    if (*st.h_err) return *st.h_err;
    // reicmcl/relqmcl are plain copies (mcica:268-269)
    if (reicmcl) std::memcpy(reicmcl, rei, CL * sizeof(double));
    if (relqmcl) std::memcpy(relqmcl, rel, CL * sizeof(double));
    return RRTMG_SW_OK;
}

int rrtmg_sw_setcoef_c(const rrtmg_sw_args* a, int32_t* jp, int32_t* jt, int32_t* jt1, int32_t* indself,
                       int32_t* indfor, int32_t* laytrop) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (a && a->ncol == 0) return RRTMG_SW_OK;
    if (!a || a->ncol < 0 || a->nlay < 1 || a->nlay > MAX_NLAY || !jp || !jt || !jt1 || !indself || !indfor ||
        !laytrop)
        return RRTMG_SW_EARGS;
    const double* req[] = {a->play, a->plev, a->tlay, a->h2ovmr, a->o3vmr, a->co2vmr, a->ch4vmr, a->o2vmr};
    for (const double* p : req)
        if (!p) return RRTMG_SW_EARGS;
    const size_t C = a->ncol, L = a->nlay, CL = C * L;
    cudaStream_t s = st.host_stream;
    Stager sg{st, s};
    SolveParams P;
    std::memset(&P, 0, sizeof(P));
    P.ncol = a->ncol;
    P.nlay = a->nlay;
    P.play = sg.in("play", a->play, CL); P.plev = sg.in("plev", a->plev, C * (L + 1));
    P.tlay = sg.in("tlay", a->tlay, CL); P.h2ovmr = sg.in("h2o", a->h2ovmr, CL);
    P.o3vmr = sg.in("o3", a->o3vmr, CL); P.co2vmr = sg.in("co2", a->co2vmr, CL);
    P.ch4vmr = sg.in("ch4", a->ch4vmr, CL); P.o2vmr = sg.in("o2", a->o2vmr, CL);
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    DevBuf& cf = st.stage["sc_cf"];
    DevBuf& pk = st.stage["sc_pk"];
    DevBuf& pdp = st.stage["sc_pdp"];
    CK(cf.ensure(CL * NFR * sizeof(double)));
    CK(pk.ensure(CL * sizeof(int)));
    CK(pdp.ensure(CL * sizeof(double)));
    if (st.form == RRTMG_SW_FORM_FP32)
        CK(launch_setcoef_f32(P, (const float*)st.d_tab32.p, (const double*)st.d_tab64.p, (float*)cf.p, (int*)pk.p,
                              (double*)pdp.p, s));
    else
        CK(launch_setcoef(P, (const double*)st.d_tab64.p, (double*)cf.p, (int*)pk.p, (double*)pdp.p, s));
    st.last_launches = 1;
    std::vector<int> h(CL);
    CK(cudaMemcpyAsync(h.data(), pk.p, CL * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (size_t c = 0; c < C; ++c) {
        int lt = 0;
        for (size_t l = 0; l < L; ++l) {
            const int w = h[c * L + l];
            const size_t o = c + C * l;  // (ncol, nlay), column-major
            jp[o] = w & 0xff;
            jt[o] = (w >> 8) & 0xf;
            jt1[o] = (w >> 12) & 0xf;
            indself[o] = (w >> 16) & 0xff;
            indfor[o] = (w >> 24) & 0xf;
            lt += (w >> 30) & 1;
        }
        laytrop[c] = lt;
    }
    return RRTMG_SW_OK;
}

int rrtmg_sw_mt_window_c(int32_t seed, uint64_t offset, uint32_t* window) {
    if (!window) return RRTMG_SW_EARGS;
    return mt_window_host((uint32_t)seed, offset, window) == 0 ? RRTMG_SW_OK : RRTMG_SW_EARGS;
}

int rrtmg_sw_mt_stream_dev_c(int32_t seed, uint64_t n, uint32_t* out, int32_t log_seg, void* stream) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (!out || log_seg > 40) return RRTMG_SW_EARGS;
    CK(launch_mt_jump((uint32_t)seed, n, out, st.num_sms, log_seg, (cudaStream_t)stream));
    st.last_launches = n ? 2 : 0;
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return RRTMG_SW_OK;
}

int get_alpha_c(int32_t ncol, int32_t nlay, int32_t icld, int32_t idcor, double decorr_con, const double* dz,
                const double* lat, int32_t juldat, const double* cldfrac, double* alpha) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (ncol == 0) return RRTMG_SW_OK;
    if (ncol < 0 || nlay < 1 || !dz || !lat || !cldfrac || !alpha) return RRTMG_SW_EARGS;
    const size_t CL = (size_t)ncol * nlay;
    cudaStream_t s = st.host_stream;
    Stager sg{st, s};
    const double* d_dz = sg.in("a_dz", dz, CL);
    const double* d_lat = sg.in("a_lat", lat, (size_t)ncol);
    const double* d_cf = sg.in("a_cf", cldfrac, CL);
    double* d_al = sg.in("a_alpha", alpha, CL);  // alpha(:,:) keeps input values where not set
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    CK(launch_get_alpha(ncol, nlay, icld, idcor, decorr_con, d_dz, d_lat, juldat, d_cf, d_al, s));
    st.last_launches = 1;
    sg.back(alpha, d_al, CL);
    if (sg.err != cudaSuccess) return cuda_fail(sg.err);
    CK(cudaStreamSynchronize(s));
    return RRTMG_SW_OK;
}

// The form is read by each solve while it holds the library mutex, so a
// switch waits for a call in progress and never changes it half way.
int rrtmg_sw_set_form_c(int32_t form) {
    if (form != RRTMG_SW_FORM_FP64 && form != RRTMG_SW_FORM_FP32) return RRTMG_SW_EARGS;
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    st.form = form;
    return RRTMG_SW_OK;
}

int rrtmg_sw_get_form_c(void) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    return st.form;
}

int rrtmg_sw_last_launch_count_c(void) { return S().last_launches; }
int rrtmg_sw_last_kernel_c(void) { return S().last_kernel; }
int rrtmg_sw_last_tile_slots_c(void) { return S().last_tile_slots; }
int rrtmg_sw_last_fp32_stats_c(int64_t* stats) {
    if (!stats) return RRTMG_SW_EARGS;
    for (int i = 0; i < 4; ++i) stats[i] = S().last_stats[i];
    return RRTMG_SW_OK;
}

int rrtmg_sw_last_ad_store_c(void) { return S().last_ad_store; }

const char* rrtmg_sw_errstr_c(int32_t code) {
    switch (code) {
    case RRTMG_SW_OK: return "OK";
    case RRTMG_SW_ENOTINIT: return "RRTMG_SW_INI NOT CALLED";
    case RRTMG_SW_ETABLES: return "COEFFICIENT TABLE FILE MISSING OR CORRUPT";
    case RRTMG_SW_EARGS: return "INVALID ARGUMENTS";
    case RRTMG_SW_ECUDA: return "CUDA ERROR";
    case RRTMG_SW_ESCRATCH: return "REQUEST EXCEEDS THE 256 MIB STATIC SCRATCH (ONE SLOT PER SM OR COLUMN PAIR)";
    case RRTMG_SW_EINFLAG1: return "INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA";
    case RRTMG_SW_EICERAD: return "ICE RADIUS OUT OF BOUNDS";
    case RRTMG_SW_EICEDGE: return "ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS";
    case RRTMG_SW_EICEPROP: return "ICE OPTICAL PROPERTY OUT OF PHYSICAL LIMITS";
    case RRTMG_SW_ELIQRAD: return "LIQUID EFFECTIVE RADIUS OUT OF BOUNDS";
    case RRTMG_SW_ELIQPROP: return "LIQUID OPTICAL PROPERTY OUT OF PHYSICAL LIMITS";
    case RRTMG_SW_EICLD: return "MCICA_SUBCOL: INVALID ICLD";
    case RRTMG_SW_EKISSSEED: return "MCICA_SUBCOL: KISSVEC SEED GENERATOR REQUIRES PMID FROM BOTTOM FOUR LAYERS.";
    case RRTMG_SW_ELAYTROP: return "PROFILE MUST HAVE LAYERS ON BOTH SIDES OF THE 100 HPA SWITCH";
    case RRTMG_SW_EIRNG: return "IRNG = 1 (MT19937) NOT AVAILABLE ON THIS ENTRY POINT";
    case RRTMG_SW_EPARTIAL: return "PARTIAL CLOUD NOT ALLOWED";
    case RRTMG_SW_EBOUNDS: return "TABLE INDEX OUT OF RANGE (BOUNDS-CHECK BUILD)";
    case RRTMG_SW_ETIMEOUT: return "WAIT BETWEEN THE WARPS OF THE TILED SOLVE TIMED OUT";
    default: return "UNKNOWN ERROR";
    }
}

const char* rrtmg_sw_last_cuda_error_c(void) { return S().last_cuda.c_str(); }

int rrtmg_sw_ad_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, const rrtmg_sw_ad_args* ad) {
    return solve_ad_host(a, c, ad, false);
}

int rrtmg_sw_tl_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, const rrtmg_sw_ad_args* ad) {
    return solve_ad_host(a, c, ad, true);
}

int rrtmg_sw_batch_plan_c(const rrtmg_sw_args* a, const rrtmg_sw_clouds* c, int32_t n, void* stream, void** plan) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    if (const int r0 = ready(st)) return r0;
    if (!a || !plan) return RRTMG_SW_EARGS;
    BatchPlan* bp = nullptr;
    const int rc = batch_plan(st, a, c, n, (cudaStream_t)stream, &bp);
    *plan = bp;
    return rc;
}

int rrtmg_sw_batch_run_c(void* plan, void* stream) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    BatchPlan* bp = (BatchPlan*)plan;
    if (!st.init) return RRTMG_SW_ENOTINIT;
    if (!bp) return RRTMG_SW_EARGS;
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev != bp->device) return RRTMG_SW_ENOTINIT;  // the plan's graph and buffers live on its device
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaGraphLaunch(bp->exec, s));
    st.last_launches = 2;
    CK(cudaMemcpyAsync(bp->h_err, bp->errw.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return bounds_status(st, *bp->h_err);
}

int rrtmg_sw_batch_info_c(void* plan, int32_t* grid, int32_t* deepest_first, float* trial_ms, int32_t* ntrials) {
    BatchPlan* bp = (BatchPlan*)plan;
    if (!bp) return RRTMG_SW_EARGS;
    if (grid) *grid = bp->grid;
    if (deepest_first) *deepest_first = bp->desc;
    if (ntrials) {
        const int cap = *ntrials;
        *ntrials = (int)bp->tune_ms.size();
        for (int i = 0; trial_ms && i < cap && i < (int)bp->tune_ms.size(); ++i) trial_ms[i] = bp->tune_ms[i];
    }
    return RRTMG_SW_OK;
}

int rrtmg_sw_batch_tile_c(void* plan, int32_t* cols, int32_t* gpoints, int32_t* trial_cfg, int32_t* ntrials) {
    BatchPlan* bp = (BatchPlan*)plan;
    if (!bp) return RRTMG_SW_EARGS;
    if (cols) *cols = bp->tile;
    if (gpoints) *gpoints = NGPT;
    if (ntrials) {
        const int cap = *ntrials;
        *ntrials = (int)bp->tune_cfg.size();
        for (int i = 0; trial_cfg && i < cap && i < (int)bp->tune_cfg.size(); ++i) trial_cfg[i] = bp->tune_cfg[i];
    }
    return RRTMG_SW_OK;
}

int rrtmg_sw_batch_free_c(void* plan) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    batch_release((BatchPlan*)plan);
    return RRTMG_SW_OK;
}

int rrtmg_sw_finalize_c(void) {
    State& st = S();
    std::lock_guard<std::mutex> lk(st.mu);
    st.d_tab64.release();
    st.d_tab32.release();
    st.scratch.release();
    st.errw.release();
    st.statsw.release();
    st.bounds.release();
    for (auto& kv : st.stage) kv.second.release();
    st.stage.clear();
    if (st.h_err) cudaFreeHost(st.h_err);
    st.h_err = nullptr;
    if (st.h_stats) cudaFreeHost(st.h_stats);
    st.h_stats = nullptr;
    if (st.host_stream) cudaStreamDestroy(st.host_stream);
    st.host_stream = nullptr;
    // a later rrtmg_sw_ini_c (after a cudaDeviceReset, say) looks the static
    // area's address up again
    for (StaticArea& sa : g_static_area) sa = StaticArea{};
    ChunkStreams& cs = CS();
    for (int i = 0; i < kChunkStreams; ++i) {
        cs.scratch[i].release();
        cs.err[i].release();
        if (cs.s[i]) cudaStreamDestroy(cs.s[i]);
        cs.s[i] = nullptr;
    }
    if (cs.h_err) cudaFreeHost(cs.h_err);
    cs.h_err = nullptr;
    if (cs.h_ovf) cudaFreeHost(cs.h_ovf);
    cs.h_ovf = nullptr;
    cs.ovf_cap = 0;
    cs.device = -1;
    mt_release_device_tables();
    st.init = false;
    return RRTMG_SW_OK;
}

}  // extern "C"
