// kernel.cuh -- the fused solve kernel (see solve.cuh for the pieces).
#pragma once

#include "solve.cuh"

namespace rrsw {

// levels buffered per reduction round of the g-point sums
constexpr int KLEV = 4;
// FP32 form: cells to redo in FP64 queued per column group (one int each:
// thread << 20 | g-point << 12 | layer << 1 | cloudy); cells past the queue
// are marked in the scratch and redone by their own thread
constexpr int REDO_QUEUE = 1024;
// columns per CTA of the batch kernel's tiles (the single-call kernels take
// COLS_PER_CTA); sMisc holds their laytrop words, then the queue length
constexpr int MAX_TILE_COLS = 4;
constexpr int MISC_QN = MAX_TILE_COLS;
constexpr int KLEV_F32 = 1;
// (FP64 tiles of 4 columns buffer 2 levels: their shared memory then fits
// the 137-layer case at one CTA per SM; the sums do not depend on it)
__host__ __device__ constexpr int klev_of(size_t rsz, int nc = COLS_PER_CTA) {
    return rsz == 4 ? KLEV_F32 : (nc > 2 ? KLEV / 2 : KLEV);
}
constexpr int NQ_MAX = 16;
// g-point sums per level: fu, fd, cu, cd, fddir, cddir; the FP32 form adds
// the absorption of the layer below the level (total, clear) for its
// heating rates; with the extra outputs, + uvfd, uvcd, uvfddir, uvcddir,
// nifd, nicd, nifddir, nicddir.
template <typename R>
__host__ __device__ constexpr int num_abs() { return sizeof(R) == 4 ? 2 : 0; }
template <typename R>
__host__ __device__ inline int num_q(bool extra) { return 6 + num_abs<R>() + (extra ? 8 : 0); }

// scratch fields per level (pass 1 -> pass 2)
enum { S_REFC, S_REFDC, S_TRAC, S_TRADC, S_DBTC, S_RUPC, S_RUPDC,
       S_REF, S_REFD, S_TRA, S_TRAD, S_DBT, S_RUP, S_RUPD, S_DBTCN, S_DBTN, NS_MAX };

__device__ inline double DM(double a, double b) { return __dmul_rn(a, b); }
__device__ inline double DA(double a, double b) { return __dadd_rn(a, b); }
__device__ inline double DS(double a, double b) { return __dsub_rn(a, b); }

// inatm_sw (rrtmg_sw_rad.f90:1527-1586) and setcoef_sw
// (rrtmg_sw_setcoef.f90:158-301) for one (column, layer), in FP64 with
// explicit roundings so both arithmetic forms see identical indices.  The
// results go to index `at` of the [NFR][L] / [L] arrays (default lay - 1).
template <typename R>
__device__ inline void prep_layer(const SolveParams& P, int col, int lay, R* cf, int* pk, double* pdp,
                                  int L, const double* __restrict__ tab64, double* cf64 = nullptr, int at = -1) {
    const int li = lay - 1;
    const int i = at >= 0 ? at : li;
    if (col >= P.ncol) {
        for (int f = 0; f < NFR; ++f) cf[f * L + i] = R(0);
        if (cf64)
            for (int f = 0; f < NFR; ++f) cf64[f * L + i] = 0.0;
        pk[i] = 1 | (1 << 8) | (1 << 12) | (1 << 16) | (1 << 24);
        pdp[i] = 1.0;
        return;
    }
    const size_t n = (size_t)P.ncol;
    const size_t k = (size_t)col + n * (size_t)li;
    const double p = P.play[k], t = P.tlay[k];
    const double pzb = P.plev[k], pzt = P.plev[k + n];
    const double h2o = P.h2ovmr[k];
    const double amd = 28.9660, amw = 18.0160, avogad = 6.02214199e+23, grav = 9.8066;
    const double amm = DA(DM(DS(1.0, h2o), amd), DM(h2o, amw));
    const double coldry = DM(DM(DS(pzb, pzt), 1.e3), avogad) / DM(DM(DM(1.e2, grav), amm), DA(1.0, h2o));
    const double w0 = DM(coldry, h2o), w1 = DM(coldry, P.co2vmr[k]), w2 = DM(coldry, P.o3vmr[k]);
    const double w5 = DM(coldry, P.ch4vmr[k]), w6 = DM(coldry, P.o2vmr[k]);
    pdp[i] = DS(pzb, pzt);
    const double stpfac = 296.0 / 1013.0;
    const double plog = log(p);
    int jp = (int)DS(36.0, DM(5.0, DA(plog, 0.04)));
    jp = jp < 1 ? 1 : (jp > 58 ? 58 : jp);
    const double fp = DM(5.0, DS(ldt(tab64, cT.preflog + jp - 1), plog));
    const double tr0 = ldt(tab64, cT.tref + jp - 1), tr1 = ldt(tab64, cT.tref + jp);
    int jt = (int)DA(3.0, DS(t, tr0) / 15.0);
    jt = jt < 1 ? 1 : (jt > 4 ? 4 : jt);
    const double ft = DS(DS(t, tr0) / 15.0, (double)(jt - 3));
    int jt1 = (int)DA(3.0, DS(t, tr1) / 15.0);
    jt1 = jt1 < 1 ? 1 : (jt1 > 4 ? 4 : jt1);
    const double ft1 = DS(DS(t, tr1) / 15.0, (double)(jt1 - 3));
    const double water = w0 / coldry;
    const double scalefac = DM(p, stpfac) / t;
    double forfac, forfrac, selffac, selffrac;
    int indfor, indself, low;
    if (plog > 4.56) {
        low = 1;
        forfac = scalefac / DA(1.0, water);
        double factor = DS(332.0, t) / 36.0;
        indfor = (int)factor;
        indfor = indfor < 1 ? 1 : (indfor > 2 ? 2 : indfor);
        forfrac = DS(factor, (double)indfor);
        selffac = DM(water, forfac);
        factor = DS(t, 188.0) / 7.2;
        indself = (int)factor - 7;
        indself = indself < 1 ? 1 : (indself > 9 ? 9 : indself);
        selffrac = DS(factor, (double)(indself + 7));
    } else {
        low = 0;
        forfac = scalefac / DA(1.0, water);
        const double factor = DS(t, 188.0) / 36.0;
        indfor = 3;
        forfrac = DS(factor, 1.0);
        selffac = 0.0;
        selffrac = 0.0;
        indself = 0;
    }
    const double colh2o = DM(1.e-20, w0);
    double colco2 = DM(1.e-20, w1), colo3 = DM(1.e-20, w2), colch4 = DM(1.e-20, w5), colo2 = DM(1.e-20, w6);
    const double colmol = DA(DM(1.e-20, coldry), colh2o);
    if (colco2 == 0.0) colco2 = DM(1.e-32, coldry);
    if (colch4 == 0.0) colch4 = DM(1.e-32, coldry);
    if (colo2 == 0.0) colo2 = DM(1.e-32, coldry);
    const double compfp = DS(1.0, fp);
    if (cf64) {
        // FP32 form: the FP64 coefficients too, for cells redone in FP64
        cf64[F_FAC10 * L + i] = DM(compfp, ft);
        cf64[F_FAC00 * L + i] = DM(compfp, DS(1.0, ft));
        cf64[F_FAC11 * L + i] = DM(fp, ft1);
        cf64[F_FAC01 * L + i] = DM(fp, DS(1.0, ft1));
        cf64[F_H2O * L + i] = colh2o;
        cf64[F_CO2 * L + i] = colco2;
        cf64[F_O3 * L + i] = colo3;
        cf64[F_CH4 * L + i] = colch4;
        cf64[F_O2 * L + i] = colo2;
        cf64[F_MOL * L + i] = colmol;
        cf64[F_SELFFAC * L + i] = selffac;
        cf64[F_SELFFRAC * L + i] = selffrac;
        cf64[F_FORFAC * L + i] = forfac;
        cf64[F_FORFRAC * L + i] = forfrac;
        cf64[F_PDP * L + i] = pdp[i];
    }
    cf[F_FAC10 * L + i] = (R)DM(compfp, ft);
    cf[F_FAC00 * L + i] = (R)DM(compfp, DS(1.0, ft));
    cf[F_FAC11 * L + i] = (R)DM(fp, ft1);
    cf[F_FAC01 * L + i] = (R)DM(fp, DS(1.0, ft1));
    cf[F_H2O * L + i] = (R)colh2o;
    cf[F_CO2 * L + i] = (R)colco2;
    cf[F_O3 * L + i] = (R)colo3;
    cf[F_CH4 * L + i] = (R)colch4;
    cf[F_O2 * L + i] = (R)colo2;
    cf[F_MOL * L + i] = (R)colmol;
    cf[F_SELFFAC * L + i] = (R)selffac;
    cf[F_SELFFRAC * L + i] = (R)selffrac;
    cf[F_FORFAC * L + i] = (R)forfac;
    cf[F_FORFRAC * L + i] = (R)forfrac;
    cf[F_PDP * L + i] = (R)pdp[i];
    pk[i] = jp | (jt << 8) | (jt1 << 12) | (indself << 16) | (indfor << 24) | (low << 30);
}

// FP32 form: inatm_sw + setcoef_sw for one (column, layer) in FP32, with the
// FP64 form's table indices.  Every index (jp, jt, jt1, indself, indfor,
// the laytrop test) is the integer part of an expression, or a comparison;
// where the FP32 value lies within IDX_EPS of the integer or of the
// threshold (its own error is below 2e-5), the expression is evaluated again
// in FP64 exactly as prep_layer does.  The pressure thickness stays FP64
// (the top layers are thin differences of level pressures).
constexpr float IDX_EPS = 1.0e-4f;

__device__ inline bool near_int(float x) { return fabsf(x - rintf(x)) < IDX_EPS; }

__device__ inline void prep_layer_f32(const SolveParams& P, int col, int lay, float* cf, int* pk, double* pdp,
                                      int L, const float* __restrict__ tab, const double* __restrict__ tab64) {
    // explicit roundings (no FMA contraction), so every kernel that inlines
    // this gets the same coefficients bit for bit
    auto M = [](float a, float b) { return __fmul_rn(a, b); };
    auto A = [](float a, float b) { return __fadd_rn(a, b); };
    auto S = [](float a, float b) { return __fsub_rn(a, b); };
    auto D = [](float a, float b) { return __fdiv_rn(a, b); };
    const int i = lay - 1;
    if (col >= P.ncol) {
        for (int f = 0; f < NFR; ++f) cf[f * L + i] = 0.0f;
        pk[i] = 1 | (1 << 8) | (1 << 12) | (1 << 16) | (1 << 24);
        pdp[i] = 1.0;
        return;
    }
    const size_t n = (size_t)P.ncol;
    const size_t k = (size_t)col + n * (size_t)i;
    const double pd = P.play[k], td = P.tlay[k];
    const double dp = DS(P.plev[k], P.plev[k + n]);
    pdp[i] = dp;
    const float p = (float)pd, t = (float)td, h2o = (float)P.h2ovmr[k];
    const float amd = 28.9660f, amw = 18.0160f;
    // 1e3 * avogad / (1e2 * grav)
    const float cfac = (float)(1.e3 * 6.02214199e+23 / (1.e2 * 9.8066));
    const float amm = A(M(S(1.0f, h2o), amd), M(h2o, amw));
    const float coldry = D(M((float)dp, cfac), M(amm, A(1.0f, h2o)));
    const float w0 = M(coldry, h2o), w1 = M(coldry, (float)P.co2vmr[k]), w2 = M(coldry, (float)P.o3vmr[k]);
    const float w5 = M(coldry, (float)P.ch4vmr[k]), w6 = M(coldry, (float)P.o2vmr[k]);
    const float plog = logf(p);
    const float xjp = S(36.0f, M(5.0f, A(plog, 0.04f)));
    int jp = near_int(xjp) ? (int)DS(36.0, DM(5.0, DA(log(pd), 0.04))) : (int)xjp;
    jp = jp < 1 ? 1 : (jp > 58 ? 58 : jp);
    const float fp = M(5.0f, S(ldt(tab, cT.preflog + jp - 1), plog));
    const float tr0 = ldt(tab, cT.tref + jp - 1), tr1 = ldt(tab, cT.tref + jp);
    const double tr0d = ldt(tab64, cT.tref + jp - 1), tr1d = ldt(tab64, cT.tref + jp);
    const float q0 = D(S(t, tr0), 15.0f), q1 = D(S(t, tr1), 15.0f);
    const float xjt = A(3.0f, q0), xjt1 = A(3.0f, q1);
    int jt = near_int(xjt) ? (int)DA(3.0, DS(td, tr0d) / 15.0) : (int)xjt;
    jt = jt < 1 ? 1 : (jt > 4 ? 4 : jt);
    int jt1 = near_int(xjt1) ? (int)DA(3.0, DS(td, tr1d) / 15.0) : (int)xjt1;
    jt1 = jt1 < 1 ? 1 : (jt1 > 4 ? 4 : jt1);
    const float ft = S(q0, (float)(jt - 3));
    const float ft1 = S(q1, (float)(jt1 - 3));
    const float water = h2o;  // w0 / coldry
    const float scalefac = D(M(p, 296.0f / 1013.0f), t);
    const bool low = fabsf(plog - 4.56f) < IDX_EPS ? log(pd) > 4.56 : plog > 4.56f;
    float forfac, forfrac, selffac, selffrac;
    int indfor, indself;
    forfac = D(scalefac, A(1.0f, water));
    if (low) {
        const float f1 = D(S(332.0f, t), 36.0f);
        indfor = near_int(f1) ? (int)(DS(332.0, td) / 36.0) : (int)f1;
        indfor = indfor < 1 ? 1 : (indfor > 2 ? 2 : indfor);
        forfrac = S(f1, (float)indfor);
        selffac = M(water, forfac);
        const float f2 = D(S(t, 188.0f), 7.2f);
        indself = (near_int(f2) ? (int)(DS(td, 188.0) / 7.2) : (int)f2) - 7;
        indself = indself < 1 ? 1 : (indself > 9 ? 9 : indself);
        selffrac = S(f2, (float)(indself + 7));
    } else {
        indfor = 3;
        forfrac = S(D(S(t, 188.0f), 36.0f), 1.0f);
        selffac = 0.0f;
        selffrac = 0.0f;
        indself = 0;
    }
    const float colh2o = M(1.e-20f, w0);
    float colco2 = M(1.e-20f, w1), colo3 = M(1.e-20f, w2), colch4 = M(1.e-20f, w5), colo2 = M(1.e-20f, w6);
    const float colmol = A(M(1.e-20f, coldry), colh2o);
    if (colco2 == 0.0f) colco2 = M(1.e-32f, coldry);
    if (colch4 == 0.0f) colch4 = M(1.e-32f, coldry);
    if (colo2 == 0.0f) colo2 = M(1.e-32f, coldry);
    const float compfp = S(1.0f, fp);
    cf[F_FAC10 * L + i] = M(compfp, ft);
    cf[F_FAC00 * L + i] = M(compfp, S(1.0f, ft));
    cf[F_FAC11 * L + i] = M(fp, ft1);
    cf[F_FAC01 * L + i] = M(fp, S(1.0f, ft1));
    cf[F_H2O * L + i] = colh2o;
    cf[F_CO2 * L + i] = colco2;
    cf[F_O3 * L + i] = colo3;
    cf[F_CH4 * L + i] = colch4;
    cf[F_O2 * L + i] = colo2;
    cf[F_MOL * L + i] = colmol;
    cf[F_SELFFAC * L + i] = selffac;
    cf[F_SELFFRAC * L + i] = selffrac;
    cf[F_FORFAC * L + i] = forfac;
    cf[F_FORFRAC * L + i] = forfrac;
    cf[F_PDP * L + i] = (float)dp;
    pk[i] = jp | (jt << 8) | (jt1 << 12) | (indself << 16) | (indfor << 24) | ((low ? 1 : 0) << 30);
}

// Aerosol optical properties of band ib at (column, layer): iaer = 10 reads
// them, iaer = 6 combines the six ECMWF types (rrtmg_sw_rad.f90:719-765).
__device__ inline void aerosol(const SolveParams& P, int col, int lay, int ib, const double* __restrict__ tab64,
                               double& ta, double& oa, double& ga) {
    const size_t n = (size_t)P.ncol, nl = (size_t)P.nlay;
    if (P.iaer == 10) {
        const size_t k = (size_t)col + n * ((size_t)(lay - 1) + nl * (size_t)ib);
        ta = P.tauaer[k];
        oa = P.ssaaer[k];
        ga = P.asmaer[k];
    } else if (P.iaer == 6) {
        double t = 0.0, a = 0.0, o = 0.0;
        for (int ia = 0; ia < 6; ++ia) {
            const double ec = P.ecaer[(size_t)col + n * ((size_t)(lay - 1) + nl * (size_t)ia)];
            const double rt = ldt(tab64, cT.rsrtaua + ib + 14 * ia), rp = ldt(tab64, cT.rsrpiza + ib + 14 * ia),
                         ra = ldt(tab64, cT.rsrasya + ib + 14 * ia);
            t = DA(t, DM(rt, ec));
            o = DA(o, DM(DM(rt, ec), rp));
            a = DA(a, DM(DM(DM(rt, ec), rp), ra));
        }
        if (t == 0.0) { t = 0.0; a = 0.0; o = 1.0; }
        else {
            if (o != 0.0) a = a / o;
            if (t != 0.0) o = o / t;
        }
        ta = t; oa = o; ga = a;
    } else {
        ta = 0.0; oa = 1.0; ga = 0.0;
    }
}

// FP32 form: 1 - zwo of reftra:183-186 from the co-albedo (zwo = zw / (1 -
// zco q^2), q = zg / (1 - zg); 1 where the reference leaves zwo = 0), and
// in `edge` whether that estimate is too close to the 5e-7 switch to trust
// its branch.  The window is an error bound from the FP32 optics: 2e-6
// relative on the co-albedo and on the asymmetry.  Near zg = 0.5, where q
// reaches 1, 1 - zwo falls steeply with zg and the window widens
// accordingly.  With den >= 1/4 and zg <= 0.9 the window is below
// 0.0544 |zco| + 1e-13, so cells farther than 0.0631 |zco| + 1e-12 from the
// switch skip its evaluation.
__device__ inline float conservative_test(float zw, float zco, float zg, bool& edge) {
    edge = false;
    if (zg == 1.0f) return zw > 0.0f ? zco : 1.0f;
    if (!(zw > 0.0f)) return 1.0f;
    const float q = zg / (1.0f - zg);
    const float q2 = q * q;
    const float den = 1.0f - zco * q2;
    if (den == 0.0f) {
        edge = true;
        return 1.0f;
    }
    const float rden = 1.0f / den;
    const float r = zco * (1.0f - q2) * rden;
    const float dist = fabsf(r - 5.0e-7f);
    if (den >= 0.25f && zg <= 0.9f && dist > 0.0631f * fabsf(zco) + 1.0e-12f) return r;
    const float rd2 = rden * rden, opq = 1.0f + q;  // 1 + q = 1 / (1 - zg)
    const float d_dg = 2.0f * zco * q * (1.0f - zco) * rd2 * opq * opq;
    const float d_dco = fabsf(1.0f - q2) * rd2;
    const float tol = d_dg * (2.0e-6f * fabsf(zg) + 1.0e-9f) + d_dco * 2.0e-6f * zco + 1.0e-13f;
    edge = dist <= tol;
    return r;
}

// Optical inputs of one (g-point, layer) cell: gas and Rayleigh depths,
// aerosol (depth, single-scattering albedo, asymmetry, co-albedo) and the
// subcolumn's cloud after cldprmc (delta-scaled depth, albedo, asymmetry,
// co-albedo; unscaled depth taor).
template <typename R>
struct CellIn {
    R taug, taur;
    R rta, roa, rga, rcoa;
    bool cloudy;
    R cldf, tc, oc, gc, coc, taor;
};

// What pass 2 needs of a cell: clear and total layer reflectance and
// transmittance, the delta-scaled direct-beam transmittances and, for
// idelm = 0, the unscaled ones.  risky (FP32 form): a discrete choice of
// the cell -- a lookup-table entry, the conservative switch, the resonance
// k mu0 = 1 -- is too close to call in FP32.
template <typename R>
struct CellOpt {
    RT<R> rc, rt;
    R zdbtc, zdbt, dbtcn, dbtn;
    bool risky;
};

// Aerosol of band ib at (column, layer) when not staged (spcvmc:442-445 inputs).
template <typename R>
__device__ inline void aerosol_in(const SolveParams& P, int col, int lay, int ib, const double* __restrict__ tab64,
                                  CellIn<R>& ci) {
    if (P.iaer == 0) {
        ci.rta = R(0); ci.roa = R(1); ci.rga = R(0); ci.rcoa = R(0);
        return;
    }
    double ta, oa, ga;
    aerosol(P, col, lay, ib, tab64, ta, oa, ga);
    ci.rta = (R)ta; ci.roa = (R)oa; ci.rga = (R)ga; ci.rcoa = (R)DS(1.0, oa);
}

// Cloud of subcolumn g at (column, layer), then cldprmc_sw.  Fused McICA:
// `cloudy` is the mask, the physical inputs come from `cld` (the CTA's
// staged copy) or, with cld == nullptr, from the FP64 arrays; unfused: the
// subcolumn arrays (cldfmcl ...) decide and supply the cloud.
template <typename R>
__device__ inline void cloud_in(const SolveParams& P, int col, int g, int lay, int ib, bool fused, bool cloudy,
                                const R* cld, CellIn<R>& ci, const R* __restrict__ tab) {
    const size_t n = (size_t)P.ncol;
    const int L = P.nlay;
    R cldf = R(0), tc = R(0), oc = R(1), gc = R(0), fsfc = R(0), ciwp = R(0), clwp = R(0), rei = R(0), rel = R(0);
    if (P.icld >= 1 && P.nomcica) {
        // cldprop_sw (rrtmg_sw_cldprop.f90:140-370) for band ib, mixed by the
        // layer's cloud fraction in spcvrt_sw (rrtmg_sw_spcvrt.f90:429,453-454)
        const size_t kl = (size_t)col + n * (size_t)(lay - 1);
        const double cf = P.cldfrac[kl];
        ciwp = cld ? cld[0 * L + lay - 1] : (R)P.ciwp[kl];
        clwp = cld ? cld[1 * L + lay - 1] : (R)P.clwp[kl];
        rei = cld ? cld[2 * L + lay - 1] : (R)P.rei[kl];
        rel = cld ? cld[3 * L + lay - 1] : (R)P.rel[kl];
        R tin = R(0), tauctot = R(0);
        if (P.tauc) {
            const size_t kb = (size_t)ib + 14 * kl;
            tin = (R)P.tauc[kb];
            oc = (R)P.ssac[kb];
            gc = (R)P.asmc[kb];
            fsfc = (R)P.fsfc[kb];
            for (int b = 0; b < NBND; ++b) tauctot += (R)P.tauc[(size_t)b + 14 * kl];
        }
        cldf = (R)cf;
        const bool on = cf >= 1.e-20 && ((double)ciwp + (double)clwp >= 1.e-20 || (double)tauctot >= 1.e-20) &&
                        (P.inflag == 0 || P.inflag == 2);
        R taor = tin, coc = R(0);
        if (on) {
            tc = tin;
            cldprmc_g<R>(ib, P.inflag, P.iceflag, P.liqflag, cldf, ciwp, clwp, rei, rel, fsfc, tc, oc, gc, taor, coc,
                         tab, P.err, tauctot);
        } else {
            tc = R(0); oc = R(1); gc = R(0);
        }
        ci.cloudy = cf != 0.0;
        ci.cldf = cldf; ci.tc = tc; ci.oc = oc; ci.gc = gc; ci.coc = coc; ci.taor = taor;
        return;
    }
    if (P.icld >= 1) {
        const size_t kl = (size_t)col + n * (size_t)(lay - 1);
        if (fused) {
            if (cloudy) {
                cldf = R(1);
                ciwp = cld ? cld[0 * L + lay - 1] : (R)P.ciwp[kl];
                clwp = cld ? cld[1 * L + lay - 1] : (R)P.clwp[kl];
                if (P.tauc) {
                    const size_t kb = (size_t)ib + 14 * kl;
                    tc = (R)P.tauc[kb];
                    oc = (R)P.ssac[kb];
                    gc = (R)P.asmc[kb];
                    fsfc = (R)P.fsfc[kb];
                }
            }
            rei = cld ? cld[2 * L + lay - 1] : (R)P.rei[kl];
            rel = cld ? cld[3 * L + lay - 1] : (R)P.rel[kl];
        } else {
            const size_t kg = (size_t)g + NGPT * kl;
            const double cf = P.cldfmcl[kg];
            cloudy = cf != 0.0;
            cldf = (R)cf;
            tc = (R)P.taucmcl[kg];
            oc = (R)P.ssacmcl[kg];
            gc = (R)P.asmcmcl[kg];
            fsfc = (R)P.fsfcmcl[kg];
            ciwp = (R)P.ciwpmcl[kg];
            clwp = (R)P.clwpmcl[kg];
            rei = (R)P.reicmcl[kl];
            rel = (R)P.relqmcl[kl];
        }
    }
    R taor = tc, coc = R(1) - oc;
    if (P.icld >= 1 && cloudy)
        cldprmc_g<R>(ib, P.inflag, P.iceflag, P.liqflag, cldf, ciwp, clwp, rei, rel, fsfc, tc, oc, gc, taor, coc, tab,
                     P.err);
    ci.cloudy = P.icld >= 1 && cloudy;
    ci.cldf = cldf; ci.tc = tc; ci.oc = oc; ci.gc = gc; ci.coc = coc; ci.taor = taor;
}

// FP32 form: a direct-beam lookup exp(-x) (rrtmg_sw_spcvmc.f90:558-585) is
// risky when it sits so close to the edge between two table entries that
// the FP64 form may take the other one, and the step would move this
// layer's heating rate by more than BEAM_HR_TOL K/day (hrs = incident flux
// * heatfac / dp) or the g-point's direct flux below the layer by more than
// BEAM_F_TOL W/m2 (zinc = the g-point's incident flux): in thick, hazy
// layers near the surface a step moves the surface flux far more than the
// layer's heating rate, and steps of many layers add up there.  The window
// assumes BEAM_EPS relative uncertainty in the FP32 optical depth.
constexpr float BEAM_EPS = 5.0e-7f;
constexpr float BEAM_HR_TOL = 2.0e-3f;
constexpr float BEAM_F_TOL = 1.0e-3f;
// The direct-beam lookup of tbl_exp (x > od_lo: u = x / (bpade + x), entry
// int(1e4 u + 0.5)) together with beam_risky's test, sharing its division:
// the window 1e4 b x / (b + x)^2 * BEAM_EPS is 1e4 u (1 - u) * BEAM_EPS, and
// one entry's step in exp(-x) is e (b + x)^2 / (1e4 b).
__device__ inline float tbl_exp_beam(float x, const float* __restrict__ tab, float hrs, float zinc, bool& risky) {
    if (x <= 0.06f) return 1.0f - x + 0.5f * x * x;
    const float u = x / (cT.bpade_f + x);
    const float t = 10000.0f * u + 0.5f;
    const int itind = (int)t;
    const float e = ldt(tab, cT.exp_tbl + itind);
    const float fr = t - (float)itind;
    if (fminf(fr, 1.0f - fr) < 10000.0f * u * (1.0f - u) * BEAM_EPS) {
        const float bx = cT.bpade_f + x;
        const float de = e * bx * bx / (cT.bpade_f * 10000.0f);
        if (hrs * de > BEAM_HR_TOL || zinc * de > BEAM_F_TOL) risky = true;
    }
    return e;
}

// Layer optics of one cell (rrtmg_sw_spcvmc.f90:442-585): clear optics
// with aerosol, delta-M scaling, reftra for clear and (if cloudy) total sky,
// cloud-fraction mixing and the direct beams.  Shared by both forms; the
// FP32 form also carries the co-albedo and flags risky cells.
template <typename R>
__device__ inline CellOpt<R> cell_optics(const CellIn<R>& ci, int idelm, R prmu0, const R* __restrict__ tab,
                                         const double* __restrict__ tab64, float hrs, float zinc = 0.0f) {
    CellOpt<R> o;
    o.risky = false;
    o.dbtcn = o.dbtn = R(0);
    R ztauc = ci.taur + ci.taug + ci.rta;
    R zomcc = ci.taur * R(1) + ci.rta * ci.roa;
    R zgcc = ci.rga * ci.roa * ci.rta / zomcc;
    R zcoc = R(0);
    if constexpr (sizeof(R) == 4) zcoc = (ci.taug + ci.rta * ci.rcoa) / ztauc;  // co-albedo
    zomcc = zomcc / ztauc;
    const R zclear = R(1) - ci.cldf, zcloud = ci.cldf;
    if (idelm == 0) {
        const R zdbtmc = tbl_exp<R>(ztauc / prmu0, tab);
        const R tauorig = ztauc + ci.taor;
        const R zdbtmo = tbl_exp<R>(tauorig / prmu0, tab);
        o.dbtcn = zdbtmc;
        o.dbtn = zclear * zdbtmc + zcloud * zdbtmo;
    }
    // delta scaling, clear (spcvmc:492-496)
    const R zf = zgcc * zgcc;
    const R zwf = zomcc * zf;
    ztauc = (R(1) - zwf) * ztauc;
    zomcc = (zomcc - zwf) / (R(1) - zwf);
    zgcc = (zgcc - zf) / (R(1) - zf);
    if constexpr (sizeof(R) == 4) zcoc = zcoc / (R(1) - zwf);
    o.rc = reftra_g<R>(ztauc, zomcc, zcoc, zgcc, prmu0, tab, tab64);
    const R xc = ztauc / prmu0;
    if constexpr (sizeof(R) == 4) {
        bool br = false;
        o.zdbtc = tbl_exp_beam(xc, tab, hrs, zinc, br);
        o.risky = o.rc.risky || br;
    } else {
        o.zdbtc = tbl_exp<R>(xc, tab);
    }
    o.rt = o.rc;
    o.zdbt = o.zdbtc;
    if (ci.cloudy) {
        // total sky: clear + delta-scaled cloud (spcvmc:500-505); reftra
        // only where cldf > repclc (:427); mixed by cloud fraction (:546-549)
        const R ztauo = ztauc + ci.tc;
        R zomco = ztauc * zomcc + ci.tc * ci.oc;
        const R zgco = (ci.tc * ci.oc * ci.gc + ztauc * zomcc * zgcc) / zomco;
        R zcoo = R(0);
        if constexpr (sizeof(R) == 4) zcoo = (ztauc * zcoc + ci.tc * ci.coc) / ztauo;
        zomco = zomco / ztauo;
        RT<R> ro;
        if (ci.cldf > R(1.e-12)) {
            if constexpr (sizeof(R) == 4) ro = reftra_f32_cloudy(ztauo, zomco, zcoo, zgco, prmu0, tab, tab64);
            else ro = reftra_g<R>(ztauo, zomco, zcoo, zgco, prmu0, tab, tab64, 1);
        } else {
            ro.ref = R(0); ro.tra = R(1); ro.refd = R(0); ro.trad = R(1);
            ro.adir = R(0); ro.adif = R(0); ro.risky = false;
        }
        o.rt.ref = zclear * o.rc.ref + zcloud * ro.ref;
        o.rt.refd = zclear * o.rc.refd + zcloud * ro.refd;
        o.rt.tra = zclear * o.rc.tra + zcloud * ro.tra;
        o.rt.trad = zclear * o.rc.trad + zcloud * ro.trad;
        const R xo = ztauo / prmu0;
        R zdbtmo;
        bool bro = false;
        if constexpr (sizeof(R) == 4) zdbtmo = tbl_exp_beam(xo, tab, hrs, zinc, bro);
        else zdbtmo = tbl_exp<R>(xo, tab);
        o.zdbt = zclear * o.zdbtc + zcloud * zdbtmo;
        if constexpr (sizeof(R) == 4) {
            o.rt.adir = zclear * o.rc.adir + zcloud * ro.adir;
            o.rt.adif = zclear * o.rc.adif + zcloud * ro.adif;
            o.risky = o.risky || ro.risky || bro;
        }
    }
    return o;
}

// FP32 form: one cell exactly as the FP64 form computes it -- gas optics
// from the FP64 layer coefficients, aerosol and cloud from the FP64 inputs
// -- returned in FP32 with its absorptances.  Used for the rare risky cells.
static __device__ __noinline__ CellOpt<float> cell_optics_fp64(const SolveParams& P, const Coef<double>& C64, int col,
                                                               int g, int lay, int ib, int igb, bool fused,
                                                               bool cloudy, double cossza,
                                                               const double* __restrict__ tab64, int clay = -1) {
    // clay: the layer's index in C64 (C64 may hold this layer alone)
    CellIn<double> ci;
    taumol_g<double>(ib, igb, clay >= 1 ? clay : lay, C64, tab64, ci.taug, ci.taur);
    aerosol_in(P, col, lay, ib, tab64, ci);
    cloud_in<double>(P, col, g, lay, ib, fused, cloudy, nullptr, ci, tab64);
    const CellOpt<double> d = cell_optics<double>(ci, P.idelm, cossza, tab64, tab64, 0.0f);
    CellOpt<float> o;
    auto cvt = [](const RT<double>& r) {
        RT<float> f;
        f.ref = (float)r.ref; f.refd = (float)r.refd; f.tra = (float)r.tra; f.trad = (float)r.trad;
        f.adir = (float)(1.0 - r.ref - r.tra);
        f.adif = (float)(1.0 - r.refd - r.trad);
        f.risky = false;
        return f;
    };
    o.rc = cvt(d.rc);
    o.rt = cvt(d.rt);
    o.zdbtc = (float)d.zdbtc;
    o.zdbt = (float)d.zdbt;
    o.dbtcn = (float)d.dbtcn;
    o.dbtn = (float)d.dbtn;
    o.risky = false;
    return o;
}

// A redone cell into its thread's scratch column sv0 (stride nt, the CTA's
// threads, per field, NS fields per level; the transmittance slots hold
// absorptances).
__device__ inline void store_cell(float* sv0, int nt, int NS, int L, int lay, const CellOpt<float>& co, int idelm) {
    float* sv = sv0 + (size_t)(L - lay) * NS * nt;
    sv[S_REFC * nt] = co.rc.ref;
    sv[S_REFDC * nt] = co.rc.refd;
    sv[S_TRAC * nt] = co.rc.adir;
    sv[S_TRADC * nt] = co.rc.adif;
    sv[S_DBTC * nt] = co.zdbtc;
    sv[S_REF * nt] = co.rt.ref;
    sv[S_REFD * nt] = co.rt.refd;
    sv[S_TRA * nt] = co.rt.adir;
    sv[S_TRAD * nt] = co.rt.adif;
    sv[S_DBT * nt] = co.zdbt;
    if (idelm == 0) {
        sv[S_DBTCN * nt] = co.dbtcn;
        sv[S_DBTN * nt] = co.dbtn;
    }
}

// Whether a cell redone in FP64 differs from the FP32 values in its
// scratch column by more than 1e-6 relative in any field (an FP32 choice
// that went the other way moves a field by ~5e-5 or more; FP32 rounding of
// the rest stays far below).
__device__ inline bool cell_changed(const float* sv0, int nt, int NS, int L, int lay, const CellOpt<float>& co) {
    const float* sv = sv0 + (size_t)(L - lay) * NS * nt;
    const float nv[10] = {co.rc.ref, co.rc.refd, co.rc.adir, co.rc.adif, co.zdbtc,
                          co.rt.ref, co.rt.refd, co.rt.adir, co.rt.adif, co.zdbt};
    const int fld[10] = {S_REFC, S_REFDC, S_TRAC, S_TRADC, S_DBTC, S_REF, S_REFD, S_TRA, S_TRAD, S_DBT};
    bool ch = false;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const float o = sv[fld[i] * nt];
        if (!(fabsf(nv[i] - o) <= 1.0e-6f * fabsf(nv[i]))) ch = true;
    }
    return ch;
}

// FP32 form: the FP64 form's coefficients of one layer of one column (setcoef
// again, in FP64), as a Coef whose only layer is layer 1; cell_optics_fp64
// takes it with clay = 1.  The FP32 form keeps no FP64 copy of its
// coefficients: the few cells it redoes per column pair recompute theirs.
struct Coef64At {
    double cf[NFR];
    int pk;
};
__device__ inline Coef<double> coef64_at(const SolveParams& P, int col, int lay, int laytrop,
                                         const double* __restrict__ tab64, Coef64At& b) {
    double pdpv;
    prep_layer<double>(P, col, lay, b.cf, &b.pk, &pdpv, 1, tab64, nullptr, 0);
    return Coef<double>{b.cf, &b.pk, 1, lay <= laytrop ? 1 : 0};
}

// FP32 form: the upward adding recurrence (vrtqdr:122-140) of one (column,
// g-point) again from layer `from` to the top, over cells already redone in
// FP64 by the CTA's queue, redoing in FP64 any cell still marked in the
// scratch (one the queue could not hold).
static __device__ __noinline__ void redo_cells_fp64(const SolveParams& P, int laytrop, float* sv0, int nt, int NS,
                                                    int col, int g, int ib, int igb, bool fused, double cossza,
                                                    const double* __restrict__ tab64, float albp, float albd,
                                                    int from) {
    const int L = P.nlay;
    auto at = [&](int lay, int fld) -> float& { return sv0[((size_t)(L - lay) * NS + fld) * nt]; };
    float rupc_b = albp, rupdc_b = albd, rup_b = albp, rupd_b = albd;
    if (from > 1) {
        rupc_b = at(from - 1, S_RUPC);
        rupdc_b = at(from - 1, S_RUPDC);
        rup_b = at(from - 1, S_RUP);
        rupd_b = at(from - 1, S_RUPD);
    }
    for (int lay = from; lay <= L; ++lay) {
        if (lay < L) {  // the next layer's cell fields into L1 while this one is swept
#pragma unroll
            for (int f = 0; f < S_DBTCN; ++f) asm volatile("prefetch.global.L1 [%0];" ::"l"(&at(lay + 1, f)));
        }
        const float mark = at(lay, S_DBTC);
        if (mark < 0.0f) {
            Coef64At b;
            const Coef<double> C64 = coef64_at(P, col, lay, laytrop, tab64, b);
            const CellOpt<float> co =
                cell_optics_fp64(P, C64, col, g, lay, ib, igb, fused, mark < -1.5f, cossza, tab64, 1);
            store_cell(sv0, nt, NS, L, lay, co, P.idelm);
        }
        {
            const float ref = at(lay, S_REFC), refd = at(lay, S_REFDC), dbt = at(lay, S_DBTC);
            const float tra = 1.0f - ref - at(lay, S_TRAC), trad = 1.0f - refd - at(lay, S_TRADC);
            const float zr = 1.0f / (1.0f - rupdc_b * refd);
            const float rupc = ref + (trad * ((tra - dbt) * rupdc_b + dbt * rupc_b)) * zr;
            rupdc_b = refd + trad * trad * rupdc_b * zr;
            rupc_b = rupc;
            at(lay, S_RUPC) = rupc_b;
            at(lay, S_RUPDC) = rupdc_b;
        }
        {
            const float ref = at(lay, S_REF), refd = at(lay, S_REFD), dbt = at(lay, S_DBT);
            const float tra = 1.0f - ref - at(lay, S_TRA), trad = 1.0f - refd - at(lay, S_TRAD);
            const float zr = 1.0f / (1.0f - rupd_b * refd);
            const float rup = ref + (trad * ((tra - dbt) * rupd_b + dbt * rup_b)) * zr;
            rupd_b = refd + trad * trad * rupd_b * zr;
            rup_b = rup;
            at(lay, S_RUP) = rup_b;
            at(lay, S_RUPD) = rupd_b;
        }
    }
}

template <typename R>
__device__ inline void warp_sum4(R& v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
}

// Shared-memory carve-up of one CTA of nc columns (x 112 g-points); the
// host sizes the launch with the same function.
struct Smem {
    size_t tm, rq, pdp, coef, hrf, pk, misc, kc, ka, omcf, cld, seed, aer, xs, red, flux, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline Smem smem_layout(int L, int nq, bool fused, bool aer_stage, size_t rsz,
                                            int nc = COLS_PER_CTA) {
    const int nt = nc * NGPT;
    Smem m;
    size_t o = 0;
    m.tm = o;
    // FP32 form: taumol descriptors first, at a fixed offset (the batch
    // kernel fills them once and re-lays the rest out per instance)
    if (rsz == sizeof(float)) o = align16(o + NBND * 2 * sizeof(TmSmem));
    // FP32 form: queue of the cells to redo in FP64
    m.rq = o;
    if (rsz == sizeof(float)) o = align16(o + (REDO_QUEUE + nt) * sizeof(int));
    m.pdp = o;  o = align16(o + nc * L * sizeof(double));
    m.coef = o; o = align16(o + nc * NFR * L * rsz);
    m.hrf = o;
    if (rsz == sizeof(float)) {
        // FP32 form: heatfac / dp per layer
        m.hrf = o; o = align16(o + nc * L * sizeof(float));
    }
    m.pk = o;   o = align16(o + nc * L * sizeof(int));
    m.misc = o; o = align16(o + 8 * sizeof(int));  // laytrop per column [0, nc), redo queue length [MISC_QN]
    m.kc = m.ka = m.omcf = m.cld = m.seed = m.xs = m.aer = o;
    if (fused) {
        m.kc = o;   o = align16(o + nc * L * sizeof(long long));
        m.ka = o;   o = align16(o + nc * L * sizeof(long long));
        m.omcf = o; o = align16(o + nc * L * sizeof(double));
        m.cld = o;  o = align16(o + nc * 4 * L * rsz);
        m.seed = o; o = align16(o + nc * 4 * sizeof(uint32_t));
        m.xs = o;   o = align16(o + NGPT * 32 * sizeof(uint32_t));
    }
    if (aer_stage) {
        m.aer = o;  o = align16(o + nc * 3 * NBND * L * rsz);
    }
    m.red = o;  o = align16(o + klev_of(rsz, nc) * nq * nt * rsz);
    m.flux = o; o = align16(o + nc * nq * (L + 1) * rsz);
    m.total = o;
    return m;
}

// Whether the CTA stages per-layer cloud inputs (fused McICA or the
// non-McICA path); the host sizes shared memory with the same test.
__host__ __device__ inline bool stages_clouds(const SolveParams& P) { return (P.fused || P.nomcica) && P.icld >= 1; }

template <typename R>
__host__ __device__ inline bool stage_aerosol(int iaer) {
    // the FP32 form converts the FP64 aerosol inputs once per (column, layer, band)
    return sizeof(R) == 4 && iaer != 0;
}

// Shared-memory views of one CTA of nc columns for the parameters P.
template <typename R>
struct CtaView {
    const TmSmem* sTm;  // [14][2] FP32 form: taumol descriptors
    int* sRq;           // [REDO_QUEUE] FP32 form: cells to redo in FP64, then [nc*112] replay start per thread
    double* sPdp;       // [nc][L]
    R* sCoef;           // [nc][NFR][L]
    float* sHrf;        // [nc][L] FP32 form: heatfac / dp
    int* sPk;           // [nc][L]
    int* sMisc;         // laytrop [nc], redo queue length [MISC_QN]
    long long* sKc;     // [nc][L] McICA threshold of 1 - cldf
    long long* sKa;     // [nc][L] McICA threshold of alpha
    double* sOmcf;      // [nc][L] 1 - cldf (icld 2)
    R* sCld;            // [nc][4][L] ciwp, clwp, rei, rel
    uint32_t* sSeed;    // [nc][4]
    uint32_t* sXs;      // [112][32] columns of M^n
    R* sAer;            // [nc][3][14][L] tau, ssa, asym
    R* sRed;            // [KLEV][NQ][nc*112]
    R* sFlux;           // [nc][NQ][L+1]
};

template <typename R>
__device__ inline CtaView<R> cta_view(unsigned char* smem_raw, const SolveParams& P, int nc = COLS_PER_CTA) {
    const Smem M =
        smem_layout(P.nlay, num_q<R>(P.extra != 0), stages_clouds(P), stage_aerosol<R>(P.iaer), sizeof(R), nc);
    CtaView<R> v;
    v.sTm = (const TmSmem*)(smem_raw + M.tm);
    v.sRq = (int*)(smem_raw + M.rq);
    v.sPdp = (double*)(smem_raw + M.pdp);
    v.sCoef = (R*)(smem_raw + M.coef);
    v.sHrf = (float*)(smem_raw + M.hrf);
    v.sPk = (int*)(smem_raw + M.pk);
    v.sMisc = (int*)(smem_raw + M.misc);
    v.sKc = (long long*)(smem_raw + M.kc);
    v.sKa = (long long*)(smem_raw + M.ka);
    v.sOmcf = (double*)(smem_raw + M.omcf);
    v.sCld = (R*)(smem_raw + M.cld);
    v.sSeed = (uint32_t*)(smem_raw + M.seed);
    v.sXs = (uint32_t*)(smem_raw + M.xs);
    v.sAer = (R*)(smem_raw + M.aer);
    v.sRed = (R*)(smem_raw + M.red);
    v.sFlux = (R*)(smem_raw + M.flux);
    return v;
}

// FP32 form: the taumol descriptors of every band and region into shared
// memory (offset 0 of the dynamic area); read after the next barrier.
template <typename R>
__device__ inline void fill_tm(unsigned char* smem_raw) {
    if constexpr (sizeof(R) == 4) {
        TmSmem* d = (TmSmem*)smem_raw;
        for (int i = threadIdx.x; i < NBND * 2; i += blockDim.x) {
            TmSmem t;
            t.r = cT.tm[i / 2][i % 2];
            t.selfref = cT.b[i / 2].selfref;
            t.forref = cT.b[i / 2].forref;
            t.ng = cT.b[i / 2].ng;
            t.pad = 0;
            d[i] = t;
        }
    }
}

// McICA stream jump of subcolumn g (this thread's) for parameters P; the
// xorshift parts go to sXs (one column of M^n per g-point, filled by the
// CTA's first 112 threads).
__device__ inline KissJump kiss_setup(const SolveParams& P, uint32_t* sXs, int g) {
    KissJump J{1u, 0u, 1u, 1u};
    if (P.fused && P.icld >= 1) {
        J = kiss_jump_consts(kiss_offset(P.icld, g, P.nlay, P.permuteseed));
        if (threadIdx.x < NGPT)
            xorshift_power(kiss_offset(P.icld, threadIdx.x, P.nlay, P.permuteseed), sXs + threadIdx.x * 32);
    }
    return J;
}

// Column slot and g-point of solve-CTA thread t.  The FP64 forms (taumol_g
// runs a different FP64 code path per band) use warps of whole bands from
// two columns (cT.thr_cg over each 224 threads, columns 2k and 2k+1:
// 2200 -> 1750 ms at 262 144 x 60); the FP32 form (one descriptor-driven
// taumol path, but cloudy layers that differ by column) is faster with 32
// consecutive g-points of one column per warp.
template <typename R>
__device__ inline int thread_col(int t) {
    if constexpr (sizeof(R) == 4) return t / NGPT;
    else return 2 * (t / (2 * NGPT)) + (cT.thr_cg[t % (2 * NGPT)] >> 7);
}
template <typename R>
__device__ inline int thread_g(int t) {
    if constexpr (sizeof(R) == 4) return t % NGPT;
    else return cT.thr_cg[t % (2 * NGPT)] & 127;
}

// Column of slot c2 of column group `pair` (nc columns): consecutive
// columns, or through the sunlit-column list of a batch (P.colmap, nmapped
// entries); ncol marks an empty slot.
__device__ inline int pair_col(const SolveParams& P, int pair, int c2, int nmapped, int nc = COLS_PER_CTA) {
    const int k = nc * pair + c2;
    if (!P.colmap) return k;
    return k < nmapped ? P.colmap[k] : P.ncol;
}

// One group of NC columns (a column pair in the single-call kernels): prep,
// pass 1, pass 2 and outputs, NC x 112 threads.
template <typename R, bool MT = false, int NC = COLS_PER_CTA>
__device__ __forceinline__ void solve_pair(const SolveParams& P, int pair, const CtaView<R>& V, const KissJump& J,
                                           R* scr, const R* __restrict__ tab, const double* __restrict__ tab64) {
    const int L = P.nlay;
    const int NQ = num_q<R>(P.extra != 0);
    constexpr int QX = 6 + num_abs<R>();  // first extra-output sum
    const bool fused = P.fused && P.icld >= 1;
    const bool nomc = P.nomcica && P.icld >= 1;
    const bool aer_stage = stage_aerosol<R>(P.iaer);
    double* sPdp = V.sPdp;
    R* sCoef = V.sCoef;
    float* sHrf = V.sHrf;
    int* sPk = V.sPk;
    int* sMisc = V.sMisc;
    long long* sKc = V.sKc;
    long long* sKa = V.sKa;
    double* sOmcf = V.sOmcf;
    R* sCld = V.sCld;
    uint32_t* sSeed = V.sSeed;
    uint32_t* sXs = V.sXs;
    R* sAer = V.sAer;
    R* sRed = V.sRed;
    R* sFlux = V.sFlux;
    constexpr int NT = NC * NGPT;
    static_assert(NC % 2 == 0 && NC <= MAX_TILE_COLS, "column pairs (the FP64 thread map), up to MAX_TILE_COLS");
    const int tid = threadIdx.x;
    const int cc = thread_col<R>(tid), g = thread_g<R>(tid);
    const int ib = cT.ngb[g], igb = cT.gib[g];
    const bool uv = ib >= 9 && ib <= 12;  // bands 25-28 (spcvmc:629)
    const int NS = P.idelm == 0 ? NS_MAX : S_DBTCN;
    const size_t n = (size_t)P.ncol;
    const int nmapped = P.colmap ? *P.mapcount : 0;
    (void)nomc;
    __syncthreads();
    // ---------------- prep: one (column, layer) per item; FP64 in the FP64
    // form, FP32 with the FP64 form's indices in the FP32 form
    for (int it = tid; it < NC * L; it += NT) {
        const int c2 = it / L, lay = it % L + 1;
        const int pcol = pair_col(P, pair, c2, nmapped, NC);
        constexpr bool f32 = sizeof(R) == 4;
        if constexpr (f32)
            prep_layer_f32(P, pcol, lay, sCoef + c2 * NFR * L, sPk + c2 * L, sPdp + c2 * L, L, tab, tab64);
        else
            prep_layer<R>(P, pcol, lay, sCoef + c2 * NFR * L, sPk + c2 * L, sPdp + c2 * L, L, tab64);
        if (f32) sHrf[c2 * L + lay - 1] = (float)(cT.heatfac / sPdp[c2 * L + lay - 1]);
        const bool real = pcol < P.ncol;
        const size_t kl = (size_t)pcol + n * (size_t)(lay - 1);
        if (fused) {
            double cf = real ? P.cldfrac[kl] : 0.0;
            if (cf < 1.0e-20) cf = 0.0;
            const double omcf = DS(1.0, cf);
            sOmcf[c2 * L + lay - 1] = omcf;
            if constexpr (MT) {
                sKc[c2 * L + lay - 1] = mt_threshold(omcf);
                sKa[c2 * L + lay - 1] = (P.icld >= 4 && real) ? mt_threshold(P.alpha[kl]) : 0ll;
            } else {
                sKc[c2 * L + lay - 1] = kiss_threshold(omcf);
                sKa[c2 * L + lay - 1] = (P.icld >= 4 && real) ? kiss_threshold(P.alpha[kl]) : 0ll;
            }
            R* cd = sCld + c2 * 4 * L;
            cd[0 * L + lay - 1] = real ? (R)P.ciwp[kl] : R(0);
            cd[1 * L + lay - 1] = real ? (R)P.clwp[kl] : R(0);
            cd[2 * L + lay - 1] = real ? (R)P.rei[kl] : R(0);
            cd[3 * L + lay - 1] = real ? (R)P.rel[kl] : R(0);
            if (lay == 1) {
                uint32_t* sd = sSeed + c2 * 4;
                if (real && !MT) {
                    const double p1 = DM(P.play[pcol], 1.e2), p2 = DM(P.play[pcol + n], 1.e2);
                    if (p1 < p2) set_error(P.err, E_KISSSEED);
                    sd[0] = kiss_seed(p1);
                    sd[1] = kiss_seed(p2);
                    sd[2] = kiss_seed(DM(P.play[pcol + 2 * n], 1.e2));
                    sd[3] = kiss_seed(DM(P.play[pcol + 3 * n], 1.e2));
                } else {
                    sd[0] = sd[1] = sd[2] = sd[3] = 1u;
                }
            }
        }
        if (nomc) {
            // spcvrt_sw takes clear or overcast layers only (rrtmg_sw_rad.nomcica.f90:617-621)
            const double cf = real ? P.cldfrac[kl] : 0.0;
            if (cf > 1.e-6 && cf < 1.0 - 1.e-6) set_error(P.err, E_PARTIAL);
            R* cd = sCld + c2 * 4 * L;
            cd[0 * L + lay - 1] = real ? (R)P.ciwp[kl] : R(0);
            cd[1 * L + lay - 1] = real ? (R)P.clwp[kl] : R(0);
            cd[2 * L + lay - 1] = real ? (R)P.rei[kl] : R(0);
            cd[3 * L + lay - 1] = real ? (R)P.rel[kl] : R(0);
        }
        if (aer_stage) {
            for (int b = 0; b < NBND; ++b) {
                double ta = 0.0, oa = 1.0, ga = 0.0;
                if (real) aerosol(P, pcol, lay, b, tab64, ta, oa, ga);
                R* ad = sAer + c2 * 3 * NBND * L;
                ad[(0 * NBND + b) * L + lay - 1] = (R)ta;
                ad[(1 * NBND + b) * L + lay - 1] = (R)DS(1.0, oa);  // co-albedo, formed in FP64
                ad[(2 * NBND + b) * L + lay - 1] = (R)ga;
            }
        }
    }
    __syncthreads();
    if (g == 0) {
        int lt = 0;
        for (int i = 0; i < L; ++i) lt += (sPk[cc * L + i] >> 30) & 1;
        sMisc[cc] = lt;
        if (cc == 0) sMisc[MISC_QN] = 0;  // FP32 form: redo queue length
    }
    __syncthreads();
    const int col = pair_col(P, pair, cc, nmapped, NC);
    const Coef<R> C{sCoef + cc * NFR * L, sPk + cc * L, L, sMisc[cc]};
    bool active = col < P.ncol;
    if (active && (C.laytrop < 1 || C.laytrop >= L)) {
        set_error(P.err, E_LAYTROP);
        active = false;
    }

    // ---------------- per (column, g-point) setup
    R zinc = R(0), albp = R(0), albd = R(0);
    double cossza = 1.0;
    McicaMask<MT> mc;
    if (active) {
        cossza = P.coszen[col];
        if (cossza < 1.e-10) cossza = 1.e-10;
        const bool nir = ib <= 8 || ib == 13;
        albp = (R)(nir ? P.aldir[col] : P.asdir[col]);
        albd = (R)(nir ? P.aldif[col] : P.asdif[col]);
        // zincflx = adjflux * ssi * prmu0 (spcvmc:349-356)
        R src;
        if constexpr (sizeof(R) == 4) src = solar_source_generic(ib, igb, C, P, tab, V.sTm);
        else src = solar_source<R>(ib, igb, C, P, tab);
        zinc = R(P.adjflux[ib]) * src * (R)cossza;
        if (fused)
            mc.start(kiss_start(sSeed + cc * 4, J, sXs + g * 32), P.icld,
                     MT ? P.mt + mt_offset(P.icld, g, col, P.ncol, L) : nullptr);
    }
    const R prmu0 = (R)cossza;
    const R* cld = sCld + cc * 4 * L;
    const R* aer = sAer + cc * 3 * NBND * L;

    // ---------------- pass 1: bottom -> top
    R rupc_b = albp, rupdc_b = albd, rup_b = albp, rupd_b = albd;
    int redo_from = L + 1;  // FP32 form: lowest layer to redo in FP64
    for (int lay = 1; lay <= L; ++lay) {
        const int jk = L + 1 - lay;
        R* sv = scr + (size_t)(jk - 1) * NS * NT + tid;
        if (!active) continue;
        R taug, taur;
        if constexpr (sizeof(R) == 4) {
            int js;
            float fs;
            taumol_generic(ib, igb, lay, C, tab, V.sTm, taug, taur, js, fs);
        } else {
            taumol_g<R>(ib, igb, lay, C, tab, taug, taur);
        }
        CellIn<R> ci;
        ci.taug = taug;
        ci.taur = taur;
        if (aer_stage) {
            ci.rta = aer[(0 * NBND + ib) * L + lay - 1];
            ci.rcoa = aer[(1 * NBND + ib) * L + lay - 1];
            ci.roa = R(1) - ci.rcoa;
            ci.rga = aer[(2 * NBND + ib) * L + lay - 1];
        } else {
            aerosol_in(P, col, lay, ib, tab64, ci);
        }
        // cloud of this subcolumn (McICA) at this layer
        bool cloudy = false;
        if (P.icld >= 1 && fused)
            cloudy = mc.step(lay, sKc[cc * L + lay - 1], sKa[cc * L + lay - 1], sOmcf[cc * L + lay - 1]);
        cloud_in<R>(P, col, g, lay, ib, fused, cloudy, cld, ci, tab);
        const R hrs = zinc * sHrf[cc * L + lay - 1];
        const CellOpt<R> co = cell_optics<R>(ci, P.idelm, prmu0, tab, tab64, hrs, (float)zinc);
        // FP32 form: a table entry, the conservative switch or the
        // resonance of this cell is too close to call in FP32; it is
        // queued and redone after this pass as the FP64 form does (a cell
        // past the queue's end is marked in the scratch instead, S_DBTC < 0,
        // -2 if cloudy, and redone by its own thread)
        int redo = 0;
        if constexpr (sizeof(R) == 4) {
            if (co.risky) {
                const int qi = atomicAdd(sMisc + MISC_QN, 1);
                if (qi < REDO_QUEUE) {
                    V.sRq[qi] = (tid << 20) | (g << 12) | (lay << 1) | (ci.cloudy ? 1 : 0);
                } else {
                    redo = ci.cloudy ? 2 : 1;
                    if (lay < redo_from) redo_from = lay;
                }
            }
        }
        const RT<R>& rc = co.rc;
        const RT<R>& rt = co.rt;
        const R zdbtc = co.zdbtc, zdbt = co.zdbt;
        if (P.idelm == 0) {
            sv[S_DBTCN * NT] = co.dbtcn;
            sv[S_DBTN * NT] = co.dbtn;
        }
        // upward adding recurrence (vrtqdr:122-140)
        {
            const R zr = R(1) / (R(1) - rupdc_b * rc.refd);
            const R rupc = rc.ref + (rc.trad * ((rc.tra - zdbtc) * rupdc_b + zdbtc * rupc_b)) * zr;
            const R rupdc = rc.refd + rc.trad * rc.trad * rupdc_b * zr;
            rupc_b = rupc;
            rupdc_b = rupdc;
        }
        {
            const R zr = R(1) / (R(1) - rupd_b * rt.refd);
            const R rup = rt.ref + (rt.trad * ((rt.tra - zdbt) * rupd_b + zdbt * rup_b)) * zr;
            const R rupd = rt.refd + rt.trad * rt.trad * rupd_b * zr;
            rup_b = rup;
            rupd_b = rupd;
        }
        // the FP32 form keeps the absorptances in the transmittance slots
        // and rebuilds ptra = 1 - pref - adir, ptrad = 1 - prefd - adif
        constexpr bool keep_abs = sizeof(R) == 4;
        sv[S_REFC * NT] = rc.ref;
        sv[S_REFDC * NT] = rc.refd;
        sv[S_TRAC * NT] = keep_abs ? rc.adir : rc.tra;
        sv[S_TRADC * NT] = keep_abs ? rc.adif : rc.trad;
        sv[S_DBTC * NT] = redo ? -(R)redo : zdbtc;
        sv[S_RUPC * NT] = rupc_b;
        sv[S_RUPDC * NT] = rupdc_b;
        sv[S_REF * NT] = rt.ref;
        sv[S_REFD * NT] = rt.refd;
        sv[S_TRA * NT] = keep_abs ? rt.adir : rt.tra;
        sv[S_TRAD * NT] = keep_abs ? rt.adif : rt.trad;
        sv[S_DBT * NT] = zdbt;
        sv[S_RUP * NT] = rup_b;
        sv[S_RUPD * NT] = rupd_b;
    }

    if constexpr (sizeof(R) == 4) {
        // the queued cells, one per thread across the CTA, so the FP64 work
        // of a warp is dense; a redone cell that differs from its FP32 values
        // replaces them, and its thread goes over its up-sweep again from
        // there (so does a thread with a cell the queue could not hold)
        int* sRf = V.sRq + REDO_QUEUE;
        sRf[tid] = L + 1;
        __syncthreads();
        const int nq = min(sMisc[MISC_QN], REDO_QUEUE);
        if (tid == 0 && P.stats) {
            atomicAdd(P.stats, (unsigned long long)sMisc[MISC_QN]);
            if (sMisc[MISC_QN] > REDO_QUEUE) atomicAdd(P.stats + 1, (unsigned long long)(sMisc[MISC_QN] - REDO_QUEUE));
        }
        for (int i = tid; i < nq; i += NT) {
            const int e = V.sRq[i];
            const int t = e >> 20, c2 = thread_col<float>(t), gg = (e >> 12) & 127, lay = (e >> 1) & 2047;
            const int pcol = pair_col(P, pair, c2, nmapped, NC);
            Coef64At b;
            const Coef<double> Cq = coef64_at(P, pcol, lay, sMisc[c2], tab64, b);
            double cz = P.coszen[pcol];
            if (cz < 1.e-10) cz = 1.e-10;
            const CellOpt<float> co = cell_optics_fp64(P, Cq, pcol, gg, lay, cT.ngb[gg], cT.gib[gg], fused, e & 1, cz,
                                                       tab64, 1);
            if (cell_changed(scr + t, NT, NS, L, lay, co)) {
                store_cell(scr + t, NT, NS, L, lay, co, P.idelm);
                atomicMin(sRf + t, lay);
            }
        }
        __syncthreads();
        const int from = min(redo_from, sRf[tid]);
        if (active && from <= L)
            redo_cells_fp64(P, C.laytrop, scr + tid, NT, NS, col, g, ib, igb, fused, cossza, tab64, albp, albd, from);
    }

    // ---------------- pass 2: top -> bottom, level fluxes and g sums
    R tdbtc = R(1), tdnc = R(1), rdndc = R(0);
    R tdbt = R(1), tdn = R(1), rdnd = R(0);
    R tdbtcn = R(1), tdbtn = R(1);
    // FP32 form: absorption of the layer above the current level, less
    // the part that its lower face's upward flux still has to add
    R absc = R(0), abst = R(0), adifc_up = R(0), adift_up = R(0);
    for (int jk = 1; jk <= L + 1; ++jk) {
        R q[NQ_MAX];
#pragma unroll
        for (int i = 0; i < NQ_MAX; ++i) q[i] = R(0);
        R refc = R(0), refdc = R(0), trac = R(0), tradc = R(0), dbtc = R(0), rupc, rupdc;
        R ref = R(0), refd = R(0), tra = R(0), trad = R(0), dbt = R(0), rup, rupd, dbtcn = R(0), dbtn = R(0);
        R adirc = R(0), adifc = R(0), adirt = R(0), adift = R(0);
        if (jk <= L) {
            const R* sv = scr + (size_t)(jk - 1) * NS * NT + tid;
            refc = sv[S_REFC * NT]; refdc = sv[S_REFDC * NT];
            trac = sv[S_TRAC * NT]; tradc = sv[S_TRADC * NT];
            dbtc = sv[S_DBTC * NT];
            rupc = sv[S_RUPC * NT]; rupdc = sv[S_RUPDC * NT];
            ref = sv[S_REF * NT]; refd = sv[S_REFD * NT];
            tra = sv[S_TRA * NT]; trad = sv[S_TRAD * NT];
            dbt = sv[S_DBT * NT];
            if constexpr (sizeof(R) == 4) {
                adirc = trac; adifc = tradc; adirt = tra; adift = trad;
                trac = R(1) - refc - adirc;
                tradc = R(1) - refdc - adifc;
                tra = R(1) - ref - adirt;
                trad = R(1) - refd - adift;
            }
            rup = sv[S_RUP * NT]; rupd = sv[S_RUPD * NT];
            if (P.idelm == 0) { dbtcn = sv[S_DBTCN * NT]; dbtn = sv[S_DBTN * NT]; }
            if constexpr (sizeof(R) == 4) {
                // the next level's fields into L1 while this level computes and
                // reduces (the level barriers keep its loads from moving up)
                if (jk < L) {
                    const R* nx = sv + (size_t)NS * NT;
#pragma unroll
                    for (int f = 0; f < S_DBTCN; ++f) asm volatile("prefetch.global.L1 [%0];" ::"l"(nx + f * NT));
                }
            }
        } else {
            rupc = albp; rupdc = albd; rup = albp; rupd = albd;
        }
        if (active) {
            // level fluxes (vrtqdr:163-169)
            const R zrc = R(1) / (R(1) - rdndc * rupdc);
            const R cu = (tdbtc * rupc + (tdnc - tdbtc) * rupdc) * zrc;
            const R cdif = (tdnc - tdbtc + tdbtc * rupc * rdndc) * zrc;
            const R cd = tdbtc + cdif;
            const R zrt = R(1) / (R(1) - rdnd * rupd);
            const R fu = (tdbt * rup + (tdn - tdbt) * rupd) * zrt;
            const R fdif = (tdn - tdbt + tdbt * rup * rdnd) * zrt;
            const R fd = tdbt + fdif;
            if constexpr (sizeof(R) == 4) {
                // layer jk-1 absorbs what enters it: the direct and diffuse
                // beams at its top (kept from the previous level) and the
                // upward flux at its bottom face, this level
                q[6] = zinc * (abst + fu * adift_up);
                q[7] = zinc * (absc + cu * adifc_up);
                abst = tdbt * adirt + fdif * adift;
                absc = tdbtc * adirc + cdif * adifc;
                adift_up = adift;
                adifc_up = adifc;
            }
            const R dirf = P.idelm == 0 ? tdbtn : tdbt;
            const R dirc = P.idelm == 0 ? tdbtcn : tdbtc;
            q[0] = zinc * fu;
            q[1] = zinc * fd;
            q[2] = zinc * cu;
            q[3] = zinc * cd;
            q[4] = zinc * dirf;
            q[5] = zinc * dirc;
            if (P.extra) {
                if (uv) { q[QX] = q[1]; q[QX + 1] = q[3]; q[QX + 2] = q[4]; q[QX + 3] = q[5]; }
                else { q[QX + 4] = q[1]; q[QX + 5] = q[3]; q[QX + 6] = q[4]; q[QX + 7] = q[5]; }
            }
            if (jk <= L) {
                // downward recurrences (vrtqdr:144-159) and direct beam (spcvmc:575-585)
                const R zr1 = R(1) / (R(1) - refdc * rdndc);
                const R tdnc_n = tdbtc * trac + (tradc * ((tdnc - tdbtc) + tdbtc * refc * rdndc)) * zr1;
                rdndc = refdc + tradc * tradc * rdndc * zr1;
                tdnc = tdnc_n;
                const R zr2 = R(1) / (R(1) - refd * rdnd);
                const R tdn_n = tdbt * tra + (trad * ((tdn - tdbt) + tdbt * ref * rdnd)) * zr2;
                rdnd = refd + trad * trad * rdnd * zr2;
                tdn = tdn_n;
                tdbtc = dbtc * tdbtc;
                tdbt = dbt * tdbt;
                tdbtcn = dbtcn * tdbtcn;
                tdbtn = dbtn * tdbtn;
            }
        }
        constexpr int KL = klev_of(sizeof(R), NC);
        const int slot = (jk - 1) % KL;
#pragma unroll
        for (int i = 0; i < NQ_MAX; ++i)
            if (i < NQ) sRed[(slot * NQ + i) * NT + cc * NGPT + g] = q[i];
        if (slot == KL - 1 || jk == L + 1) {
            __syncthreads();
            const int nlev = slot + 1;
            const int items = NC * NQ * nlev;
            for (int base = 0; base < items * 4; base += NT) {
                const int t = base + tid;
                const int item = t >> 2, part = t & 3;
                R v = R(0);
                int c2 = 0, qi = 0, s = 0;
                if (item < items) {
                    c2 = item / (NQ * nlev);
                    qi = (item / nlev) % NQ;
                    s = item % nlev;
                    const R* src = sRed + (s * NQ + qi) * NT + c2 * NGPT + part * 28;
                    for (int j = 0; j < 28; ++j) v += src[j];
                }
                warp_sum4(v);
                if (item < items && part == 0) {
                    const int jl = jk - slot + s;  // level (1 = top)
                    sFlux[(c2 * NQ + qi) * (L + 1) + (L + 1 - jl)] = v;
                }
            }
            if (P.bands) {
                // per-band sums of fu, fd, fddir, cu, cd (spcvmc:619-630 per band)
                const int bitems = NC * NBND * 5 * nlev;
                for (int t = tid; t < bitems; t += NT) {
                    const int s = t % nlev, qs = (t / nlev) % 5, b = (t / (nlev * 5)) % NBND;
                    const int c2 = t / (nlev * 5 * NBND);
                    const int qi = qs == 0 ? 0 : qs == 1 ? 1 : qs == 2 ? 4 : qs == 3 ? 2 : 3;
                    const R* src = sRed + (s * NQ + qi) * NT + c2 * NGPT + cT.b[b].g0;
                    R v = R(0);
                    for (int j = 0; j < cT.b[b].ng; ++j) v += src[j];
                    const int ocol = pair_col(P, pair, c2, nmapped, NC);
                    const int l = L + 1 - (jk - slot + s);  // level index, 0 = surface
                    if (ocol < P.ncol && P.bout[qs])
                        P.bout[qs][(size_t)ocol + n * ((size_t)l + (size_t)(L + 1) * b)] = (double)v;
                }
            }
            __syncthreads();
        }
    }

    // ---------------- outputs (level 0 = surface)
    for (int it = tid; it < NC * (L + 1); it += NT) {
        const int c2 = it / (L + 1), l = it % (L + 1);
        const int ocol = pair_col(P, pair, c2, nmapped, NC);
        if (ocol >= P.ncol) continue;
        const R* F = sFlux + c2 * NQ * (L + 1);
        const size_t o = (size_t)ocol + n * (size_t)l;
        const double fu = (double)F[0 * (L + 1) + l], fd = (double)F[1 * (L + 1) + l];
        const double cu = (double)F[2 * (L + 1) + l], cd = (double)F[3 * (L + 1) + l];
        P.swuflx[o] = fu;
        P.swdflx[o] = fd;
        P.swuflxc[o] = cu;
        P.swdflxc[o] = cd;
        if (l < L) {
            const double* pdp = sPdp + c2 * L;
            double hr = 0.0, hrc = 0.0;
            if (l < L - 1) {
                const double zdpgcp = cT.heatfac / pdp[l];
                if constexpr (sizeof(R) == 4) {
                    // summed layer absorption (= net-flux divergence)
                    hr = (double)F[6 * (L + 1) + l] * zdpgcp;
                    hrc = (double)F[7 * (L + 1) + l] * zdpgcp;
                } else {
                    const double fu1 = (double)F[0 * (L + 1) + l + 1], fd1 = (double)F[1 * (L + 1) + l + 1];
                    const double cu1 = (double)F[2 * (L + 1) + l + 1], cd1 = (double)F[3 * (L + 1) + l + 1];
                    hrc = DM(DS(DS(cd1, cu1), DS(cd, cu)), zdpgcp);
                    hr = DM(DS(DS(fd1, fu1), DS(fd, fu)), zdpgcp);
                }
            }
            P.swhr[o] = hr;
            P.swhrc[o] = hrc;
        }
        if (P.extra) {
            const double fddir = (double)F[4 * (L + 1) + l];
            const double uvfd = (double)F[(QX + 0) * (L + 1) + l], uvfddir = (double)F[(QX + 2) * (L + 1) + l];
            const double nifd = (double)F[(QX + 4) * (L + 1) + l], nifddir = (double)F[(QX + 6) * (L + 1) + l];
            const double vals[8] = {fddir, DS(fd, fddir), uvfd, nifd, uvfddir, DS(uvfd, uvfddir), nifddir,
                                    DS(nifd, nifddir)};
            for (int x = 0; x < 8; ++x)
                if (P.xout[x]) P.xout[x][o] = vals[x];
        }
    }

}

// FP32 form: 4 resident CTAs per SM (72 registers, ~41 KB shared memory each
// at 60 layers, level sums reduced level by level) hide more latency than 3
// CTAs with 80 registers and 4-level reductions (147 -> 128 ms at
// 262 144 x 60) or 2 with 128 registers.
// MT: fused McICA from the call's MT19937 stream (P.mt) instead of KISS.
template <typename R, bool MT>
__global__ void __launch_bounds__(CTA_THREADS, sizeof(R) == 4 ? 4 : 2)
k_solve(const SolveParams P, const R* __restrict__ tab, const double* __restrict__ tab64) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    fill_tm<R>(smem_raw);
    const CtaView<R> V = cta_view<R>(smem_raw, P);
    const KissJump J = kiss_setup(P, V.sXs, thread_g<R>(threadIdx.x));  // once per launch
    R* scr = (R*)P.scratch + (size_t)blockIdx.x * P.slot_elems;
    for (int pair = blockIdx.x; pair < P.npairs; pair += gridDim.x)
        solve_pair<R, MT>(P, pair, V, J, scr, tab, tab64);
}

// ------------------------------------------------------------------ batch
// Many independent instances (ncol and nlay differ) in one persistent
// launch.  Each instance's sunlit columns were listed by k_compact; the work
// items are the NC-column groups of those lists, instance after instance,
// and a CTA (NC x 112 threads) takes every gridDim.x-th item.  The
// parameters of the instance at hand are copied to shared memory when the
// CTA moves to a new instance.  NC (2 or 4) is the tile the batch planner
// picks by timing.

template <typename R, int NC>
__global__ void __launch_bounds__(NC * NGPT, 4 / NC)
k_solve_batch(const SolveParams* __restrict__ Pb, int ninst, const int* __restrict__ counts,
              const R* __restrict__ tab, const double* __restrict__ tab64) {
    constexpr int NT = NC * NGPT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_pref[MAX_BATCH + 1];
    __shared__ __align__(16) SolveParams sP;
    fill_tm<R>(smem_raw);
    if (threadIdx.x == 0) {
        s_pref[0] = 0;
        for (int i = 0; i < ninst; ++i) s_pref[i + 1] = s_pref[i] + (counts[i] + NC - 1) / NC;
    }
    __syncthreads();
    const int total = s_pref[ninst];
    int cur = -1;
    CtaView<R> V{};
    KissJump J{1u, 0u, 1u, 1u};
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        int lo = 0, hi = ninst;
        while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if (s_pref[mid] <= item) lo = mid;
            else hi = mid;
        }
        if (lo != cur) {
            __syncthreads();  // the previous instance's shared data is no longer read
            {
                const int* src = (const int*)(Pb + lo);
                int* dst = (int*)&sP;
                for (int w = threadIdx.x; w < (int)(sizeof(SolveParams) / sizeof(int)); w += NT) dst[w] = src[w];
            }
            __syncthreads();
            V = cta_view<R>(smem_raw, sP, NC);
            J = kiss_setup(sP, V.sXs, thread_g<R>(threadIdx.x));
            cur = lo;
        }
        R* scr = (R*)sP.scratch + (size_t)blockIdx.x * sP.slot_elems;
        solve_pair<R, false, NC>(sP, item - s_pref[lo], V, J, scr, tab, tab64);
    }
}

// Sunlit-column compaction of one instance per CTA: the columns with
// coszen > 0, in order, go to map[0 .. count); the outputs of the others
// (night columns, which the reference solves with mu0 clamped to 1e-10 and
// which come out at 1e-10 of a daytime flux) are set to zero.
static __global__ void __launch_bounds__(1024)
k_compact(const SolveParams* __restrict__ Pb, int* __restrict__ map_all, const long long* __restrict__ map_off,
          int* __restrict__ counts) {
    __shared__ int s_warp[32];
    __shared__ int s_base;
    const SolveParams& P = Pb[blockIdx.x];
    int* map = map_all + map_off[blockIdx.x];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    const size_t n = (size_t)P.ncol, L = (size_t)P.nlay;
    for (int c0 = 0; c0 < P.ncol; c0 += 1024) {
        const int c = c0 + threadIdx.x;
        const bool inb = c < P.ncol;
        const bool sun = inb && P.coszen[c] > 0.0;
        const unsigned m = __ballot_sync(0xffffffffu, sun);
        if (lane == 0) s_warp[wid] = __popc(m);
        __syncthreads();
        int before = 0, tot = 0;
        for (int w = 0; w < 32; ++w) {
            if (w < wid) before += s_warp[w];
            tot += s_warp[w];
        }
        const int rank = s_base + before + __popc(m & ((1u << lane) - 1u));
        if (sun) map[rank] = c;
        if (inb && !sun) {
            for (size_t l = 0; l <= L; ++l) {
                const size_t o = (size_t)c + n * l;
                P.swuflx[o] = 0.0; P.swdflx[o] = 0.0; P.swuflxc[o] = 0.0; P.swdflxc[o] = 0.0;
                for (int x = 0; x < 8; ++x)
                    if (P.xout[x]) P.xout[x][o] = 0.0;
                for (int q = 0; q < 5; ++q)
                    if (P.bout[q])
                        for (int b = 0; b < NBND; ++b) P.bout[q][o + n * (L + 1) * (size_t)b] = 0.0;
                if (l < L) { P.swhr[o] = 0.0; P.swhrc[o] = 0.0; }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[blockIdx.x] = s_base;
}

}  // namespace rrsw
