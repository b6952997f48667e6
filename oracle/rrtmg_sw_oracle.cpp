// rrtmg_sw_oracle.cpp -- FP64 CPU restatement of the RRTMG_SW shortwave
// column solve.  TEST INFRASTRUCTURE ONLY: the oracle for the GPU library,
// never part of the product path (see rrtmg_sw_oracle.h).
//
// Each routine follows the reference Fortran line by line; the cited
// file:line ranges are relative to the RRTMG_SW source tree.  Compile with
// -ffp-contract=off: every multiply and add is rounded separately, as the
// reference's expressions are written, evaluated left to right.
#include "rrtmg_sw_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int NBND = 14;
constexpr int NGPT = 112;
constexpr int NTBL = 10000;

// ---------------------------------------------------------------- tables
struct BandTab {
    int nspa = 1, nspb = 1, ng = 0, g0 = 0;  // g0: 0-based first global g-point
    int nfr = 3;                             // forref first dimension
    std::vector<double> absa, absb, selfref, forref, sfluxref, irradnce, facbrght, snsptdrk;
    std::vector<double> rayl, rayla, raylb, abso3a, abso3b, absch4, absco2, absh2o;
};

struct Tables {
    bool ok = false;
    BandTab b[30];
    double pref[59], preflog[59], tref[59];
    std::vector<double> extliq1, ssaliq1, asyliq1, extice2, ssaice2, asyice2;
    std::vector<double> extice3, ssaice3, asyice3, fdlice3;
    double abari[5], bbari[5], cbari[5], dbari[5], ebari[5], fbari[5];
    double rsrtaua[NBND * 6], rsrpiza[NBND * 6], rsrasya[NBND * 6];
    double wavenum1[NBND], wavenum2[NBND];
    int ngb[NGPT];
    double exp_tbl[NTBL + 1];
    double mgavgcyc[134], sbavgcyc[134];
    double bpade, heatfac, oneminus, pi;
};

Tables T;

const int kNG[14] = {6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12};
// nspa/nspb: rrtmg_sw_init.f90:194-195
const int kNSPA[14] = {9, 9, 9, 9, 1, 9, 9, 1, 9, 1, 0, 1, 9, 1};
const int kNSPB[14] = {1, 5, 1, 1, 1, 5, 1, 0, 1, 0, 0, 1, 5, 1};

// Fortran 1-based accessors
inline double A(const std::vector<double>& v, int n1, int i, int j) { return v[(i - 1) + n1 * (j - 1)]; }

// ---------------------------------------------------------------- setcoef
struct Coef {
    int nlay = 0, laytrop = 0;
    std::vector<int> jp, jt, jt1, indself, indfor;
    std::vector<double> colh2o, colco2, colo3, colch4, colo2, colmol;
    std::vector<double> fac00, fac01, fac10, fac11, selffac, selffrac, forfac, forfrac;
    void alloc(int n) {
        nlay = n;
        for (auto* v : {&jp, &jt, &jt1, &indself, &indfor}) v->assign(n + 2, 0);
        for (auto* v : {&colh2o, &colco2, &colo3, &colch4, &colo2, &colmol, &fac00, &fac01, &fac10,
                        &fac11, &selffac, &selffrac, &forfac, &forfrac})
            v->assign(n + 2, 0.0);
    }
};

// setcoef_sw (rrtmg_sw_setcoef.f90:49-305).  wkl is (7,nlay) column
// amounts; dead outputs (co2mult, coln2o, layswtch, laylow, indbound,
// tbndfrac, indlev0, t0frac) are not computed.
void setcoef(int nlay, const double* pavel, const double* tavel, const double* coldry,
             const double* wkl, Coef& c) {
    c.alloc(nlay);
    const double stpfac = 296.0 / 1013.0;
    c.laytrop = 0;
    for (int lay = 1; lay <= nlay; ++lay) {
        const double p = pavel[lay - 1], t = tavel[lay - 1], cd = coldry[lay - 1];
        const double* w = wkl + 7 * (lay - 1);
        const double plog = std::log(p);
        int jp = (int)(36.0 - 5.0 * (plog + 0.04));
        if (jp < 1) jp = 1; else if (jp > 58) jp = 58;
        c.jp[lay] = jp;
        const int jp1 = jp + 1;
        const double fp = 5.0 * (T.preflog[jp - 1] - plog);
        int jt = (int)(3.0 + (t - T.tref[jp - 1]) / 15.0);
        if (jt < 1) jt = 1; else if (jt > 4) jt = 4;
        c.jt[lay] = jt;
        const double ft = ((t - T.tref[jp - 1]) / 15.0) - (double)(jt - 3);
        int jt1 = (int)(3.0 + (t - T.tref[jp1 - 1]) / 15.0);
        if (jt1 < 1) jt1 = 1; else if (jt1 > 4) jt1 = 4;
        c.jt1[lay] = jt1;
        const double ft1 = ((t - T.tref[jp1 - 1]) / 15.0) - (double)(jt1 - 3);
        const double water = w[0] / cd;
        const double scalefac = p * stpfac / t;
        if (plog > 4.56) {
            c.laytrop = c.laytrop + 1;
            c.forfac[lay] = scalefac / (1.0 + water);
            double factor = (332.0 - t) / 36.0;
            int indf = (int)factor;
            if (indf < 1) indf = 1;
            if (indf > 2) indf = 2;
            c.indfor[lay] = indf;
            c.forfrac[lay] = factor - (double)indf;
            c.selffac[lay] = water * c.forfac[lay];
            factor = (t - 188.0) / 7.2;
            int inds = (int)factor - 7;
            if (inds < 1) inds = 1;
            if (inds > 9) inds = 9;
            c.indself[lay] = inds;
            c.selffrac[lay] = factor - (double)(inds + 7);
        } else {
            c.forfac[lay] = scalefac / (1.0 + water);
            const double factor = (t - 188.0) / 36.0;
            c.indfor[lay] = 3;
            c.forfrac[lay] = factor - 1.0;
            c.selffac[lay] = 0.0;
            c.selffrac[lay] = 0.0;
            c.indself[lay] = 0;
        }
        c.colh2o[lay] = 1.e-20 * w[0];
        c.colco2[lay] = 1.e-20 * w[1];
        c.colo3[lay] = 1.e-20 * w[2];
        c.colch4[lay] = 1.e-20 * w[5];
        c.colo2[lay] = 1.e-20 * w[6];
        c.colmol[lay] = 1.e-20 * cd + c.colh2o[lay];
        if (c.colco2[lay] == 0.0) c.colco2[lay] = 1.e-32 * cd;
        if (c.colch4[lay] == 0.0) c.colch4[lay] = 1.e-32 * cd;
        if (c.colo2[lay] == 0.0) c.colo2[lay] = 1.e-32 * cd;
        const double compfp = 1.0 - fp;
        c.fac10[lay] = compfp * ft;
        c.fac00[lay] = compfp * (1.0 - ft);
        c.fac11[lay] = fp * ft1;
        c.fac01[lay] = fp * (1.0 - ft1);
    }
}

// ---------------------------------------------------------------- taumol
struct Solar {
    int isolvar = 0;
    double svar_f = 1, svar_s = 1, svar_i = 1;
    double svar_f_bnd[NBND], svar_s_bnd[NBND], svar_i_bnd[NBND];  // index band-16
};

struct Gas {
    int nlay = 0;
    std::vector<double> taug, taur;  // (lay 1..nlay, g 1..112) -> [(lay-1) + nlay*(g-1)]
    double ssi[NGPT], sfluxzen[NGPT];
    double& tg(int lay, int ig) { return taug[(lay - 1) + nlay * (ig - 1)]; }
    double& tr(int lay, int ig) { return taur[(lay - 1) + nlay * (ig - 1)]; }
};

// The species-ratio interpolation shared by the "speccomb" bands
// (e.g. rrtmg_sw_taumol.f90:309-324).
struct Spec {
    double speccomb, fs, fac000, fac001, fac010, fac011, fac100, fac101, fac110, fac111;
    int js;
};
inline Spec spec(double cola, double colb_scaled, double mult, double f00, double f01, double f10, double f11) {
    Spec s;
    s.speccomb = cola + colb_scaled;
    double specparm = cola / s.speccomb;
    if (specparm >= T.oneminus) specparm = T.oneminus;
    const double specmult = mult * (specparm);
    s.js = 1 + (int)specmult;
    s.fs = std::fmod(specmult, 1.0);
    s.fac000 = (1.0 - s.fs) * f00;
    s.fac010 = (1.0 - s.fs) * f10;
    s.fac100 = s.fs * f00;
    s.fac110 = s.fs * f10;
    s.fac001 = (1.0 - s.fs) * f01;
    s.fac011 = (1.0 - s.fs) * f11;
    s.fac101 = s.fs * f01;
    s.fac111 = s.fs * f11;
    return s;
}

// 8-point k interpolation with row strides (1, d1, d1+1): absa uses d1=9
// (taumol.f90:331-338), the 5-wide upper tables d1=5 (:443-450).
inline double k8(const Spec& s, const std::vector<double>& k, int n1, int ind0, int ind1, int ig, int d1) {
    return (s.fac000 * A(k, n1, ind0, ig) + s.fac100 * A(k, n1, ind0 + 1, ig) +
            s.fac010 * A(k, n1, ind0 + d1, ig) + s.fac110 * A(k, n1, ind0 + d1 + 1, ig) +
            s.fac001 * A(k, n1, ind1, ig) + s.fac101 * A(k, n1, ind1 + 1, ig) +
            s.fac011 * A(k, n1, ind1 + d1, ig) + s.fac111 * A(k, n1, ind1 + d1 + 1, ig));
}
inline double k4(const Coef& c, int lay, const std::vector<double>& k, int n1, int ind0, int ind1, int ig) {
    return c.fac00[lay] * A(k, n1, ind0, ig) + c.fac10[lay] * A(k, n1, ind0 + 1, ig) +
           c.fac01[lay] * A(k, n1, ind1, ig) + c.fac11[lay] * A(k, n1, ind1 + 1, ig);
}
// self-continuum and foreign-continuum terms (taumol.f90:340-346)
inline double selfterm(const Coef& c, int lay, const BandTab& B, int ig) {
    const int inds = c.indself[lay];
    return c.selffac[lay] * (A(B.selfref, 10, inds, ig) + c.selffrac[lay] *
                             (A(B.selfref, 10, inds + 1, ig) - A(B.selfref, 10, inds, ig)));
}
inline double forterm(const Coef& c, int lay, const BandTab& B, int ig) {
    const int indf = c.indfor[lay];
    return c.forfac[lay] * (A(B.forref, B.nfr, indf, ig) + c.forfrac[lay] *
                            (A(B.forref, B.nfr, indf + 1, ig) - A(B.forref, B.nfr, indf, ig)));
}
// the bracket colh2o * (self + foreign) of most lower-atmosphere loops
inline double selffor(const Coef& c, int lay, const BandTab& B, int ig) {
    return selfterm(c, lay, B, ig) + forterm(c, lay, B, ig);
}
inline double forpart(const Coef& c, int lay, const BandTab& B, int ig) {
    const int indf = c.indfor[lay];
    return (A(B.forref, B.nfr, indf, ig) + c.forfrac[lay] *
            (A(B.forref, B.nfr, indf + 1, ig) - A(B.forref, B.nfr, indf, ig)));
}
inline double interp_js(const std::vector<double>& v, int ng, int ig, int js, double fs) {
    return A(v, ng, ig, js) + fs * (A(v, ng, ig, js + 1) - A(v, ng, ig, js));
}

// Solar source at the reference layer for one g-point: the sfluxzen/ssi
// statements of every taumolNN (e.g. taumol.f90:364-378, 495-517).  When
// `interp` the source tables are interpolated in the species index js.
void set_source(Gas& G, const Solar& S, const BandTab& B, int ig, bool interp, int js, double fs,
                double scale) {
    const int gg = B.g0 + ig - 1;
    const int ib = B.g0 >= 0 ? T.ngb[gg] - 16 : 0;
    double sf, fb, sd, ir;
    if (interp) {
        sf = interp_js(B.sfluxref, B.ng, ig, js, fs);
        fb = interp_js(B.facbrght, B.ng, ig, js, fs);
        sd = interp_js(B.snsptdrk, B.ng, ig, js, fs);
        ir = interp_js(B.irradnce, B.ng, ig, js, fs);
    } else {
        sf = B.sfluxref[ig - 1];
        fb = B.facbrght[ig - 1];
        sd = B.snsptdrk[ig - 1];
        ir = B.irradnce[ig - 1];
    }
    G.sfluxzen[gg] = scale == 1.0 ? sf : scale * sf;
    if (S.isolvar >= 0 && S.isolvar <= 2)
        G.ssi[gg] = S.svar_f * fb + S.svar_s * sd + S.svar_i * ir;
    if (S.isolvar == 3)
        G.ssi[gg] = S.svar_f_bnd[ib] * fb + S.svar_s_bnd[ib] * sd + S.svar_i_bnd[ib] * ir;
}

// jp(lay+1) at lay == nlay lies outside the reference's initialised
// range (rrtmg_sw_rad.f90:438 declares jp(nlay+1)); treat it as "no switch".
inline int jp_next(const Coef& c, int lay) { return lay + 1 <= c.nlay ? c.jp[lay + 1] : -1000; }

// taumol_sw (rrtmg_sw_taumol.f90:50-268) and taumol16..taumol29 (:275-1785).
void taumol(const Coef& c, const Solar& S, Gas& G) {
    const int nlay = c.nlay, laytrop = c.laytrop;
    G.nlay = nlay;
    G.taug.assign((size_t)nlay * NGPT, 0.0);
    G.taur.assign((size_t)nlay * NGPT, 0.0);
    for (int i = 0; i < NGPT; ++i) { G.ssi[i] = 0.0; G.sfluxzen[i] = 0.0; }
    const double oneminus = T.oneminus;
    (void)oneminus;

    // ---- band 16 (:275-383)
    {
        const BandTab& B = T.b[16]; const int g0 = B.g0; const int layreffr = 18;
        const double strrat1 = 252.131;
        for (int lay = 1; lay <= laytrop; ++lay) {
            Spec s = spec(c.colh2o[lay], strrat1 * c.colch4[lay], 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9) + c.colh2o[lay] * selffor(c, lay, B, ig);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        int laysolfr = nlay;
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = c.colch4[lay] * k4(c, lay, B.absb, 235, ind0, ind1, ig);
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 17
    {
        const BandTab& B = T.b[17]; const int g0 = B.g0; const int layreffr = 30;
        const double strrat = 0.364641;
        for (int lay = 1; lay <= laytrop; ++lay) {
            Spec s = spec(c.colh2o[lay], strrat * c.colco2[lay], 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9) + c.colh2o[lay] * selffor(c, lay, B, ig);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        int laysolfr = nlay;
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
            Spec s = spec(c.colh2o[lay], strrat * c.colco2[lay], 4.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + s.js;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absb, 1175, ind0, ind1, ig, 5) +
                                     c.colh2o[lay] * c.forfac[lay] * forpart(c, lay, B, ig);
                if (lay == laysolfr) set_source(G, S, B, ig, true, s.js, s.fs, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // bands 18 (:528-643) and 19 (:646-761): speccomb lower, 4-point upper
    for (int band : {18, 19}) {
        const BandTab& B = T.b[band]; const int g0 = B.g0;
        const double strrat = band == 18 ? 38.9589 : 5.49281;
        const int layreffr = band == 18 ? 6 : 3;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            const double colb = band == 18 ? c.colch4[lay] : c.colco2[lay];
            Spec s = spec(c.colh2o[lay], strrat * colb, 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9) + c.colh2o[lay] * selffor(c, lay, B, ig);
                if (lay == laysolfr) set_source(G, S, B, ig, true, s.js, s.fs, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            const double colb = band == 18 ? c.colch4[lay] : c.colco2[lay];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = colb * k4(c, lay, B.absb, 235, ind0, ind1, ig);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 20 (:764-859)
    {
        const BandTab& B = T.b[20]; const int g0 = B.g0; const int layreffr = 3;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + 1;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = c.colh2o[lay] * ((k4(c, lay, B.absa, 65, ind0, ind1, ig)) + selfterm(c, lay, B, ig) + forterm(c, lay, B, ig)) +
                                     c.colch4[lay] * B.absch4[ig - 1];
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                // (:846-853) the foreign term sits inside the same bracket
                G.tg(lay, g0 + ig) = c.colh2o[lay] * (k4(c, lay, B.absb, 235, ind0, ind1, ig) + c.forfac[lay] * forpart(c, lay, B, ig)) +
                                     c.colch4[lay] * B.absch4[ig - 1];
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 21 (:862-1000)
    {
        const BandTab& B = T.b[21]; const int g0 = B.g0; const int layreffr = 8;
        const double strrat = 0.0045321;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            Spec s = spec(c.colh2o[lay], strrat * c.colco2[lay], 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9) + c.colh2o[lay] * selffor(c, lay, B, ig);
                if (lay == laysolfr) set_source(G, S, B, ig, true, s.js, s.fs, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            Spec s = spec(c.colh2o[lay], strrat * c.colco2[lay], 4.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + s.js;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absb, 1175, ind0, ind1, ig, 5) +
                                     c.colh2o[lay] * c.forfac[lay] * forpart(c, lay, B, ig);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 22 (:1003-1128)
    {
        const BandTab& B = T.b[22]; const int g0 = B.g0; const int layreffr = 2;
        const double o2adj = 1.6, strrat = 0.022708;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            const double o2cont = 4.35e-4 * c.colo2[lay] / (350.0 * 2.0);
            Spec s = spec(c.colh2o[lay], o2adj * strrat * c.colo2[lay], 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9) + c.colh2o[lay] * selffor(c, lay, B, ig) + o2cont;
                if (lay == laysolfr) set_source(G, S, B, ig, true, s.js, s.fs, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            const double o2cont = 4.35e-4 * c.colo2[lay] / (350.0 * 2.0);
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = c.colo2[lay] * o2adj * k4(c, lay, B.absb, 235, ind0, ind1, ig) + o2cont;
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 23 (:1131-1214)
    {
        const BandTab& B = T.b[23]; const int g0 = B.g0; const int layreffr = 6;
        const double givfac = 1.029;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + 1;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + 1;
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * B.rayl[ig - 1];
                G.tg(lay, g0 + ig) = c.colh2o[lay] * (givfac * k4(c, lay, B.absa, 65, ind0, ind1, ig) + selfterm(c, lay, B, ig) + forterm(c, lay, B, ig));
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay)
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = 0.0;
                G.tr(lay, g0 + ig) = c.colmol[lay] * B.rayl[ig - 1];
            }
    }
    // band 24 (:1217-1335)
    {
        const BandTab& B = T.b[24]; const int g0 = B.g0; const int layreffr = 1;
        const double strrat = 0.124692;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            Spec s = spec(c.colh2o[lay], strrat * c.colo2[lay], 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * (A(B.rayla, B.ng, ig, s.js) + s.fs * (A(B.rayla, B.ng, ig, s.js + 1) - A(B.rayla, B.ng, ig, s.js)));
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9) + c.colo3[lay] * B.abso3a[ig - 1] +
                                     c.colh2o[lay] * selffor(c, lay, B, ig);
                if (lay == laysolfr) set_source(G, S, B, ig, true, s.js, s.fs, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * B.raylb[ig - 1];
                G.tg(lay, g0 + ig) = c.colo2[lay] * k4(c, lay, B.absb, 235, ind0, ind1, ig) + c.colo3[lay] * B.abso3b[ig - 1];
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 25 (:1338-1411)
    {
        const BandTab& B = T.b[25]; const int g0 = B.g0; const int layreffr = 2;
        int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay) {
            if (c.jp[lay] < layreffr && jp_next(c, lay) >= layreffr) laysolfr = std::min(lay + 1, laytrop);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + 1;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + 1;
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * B.rayl[ig - 1];
                G.tg(lay, g0 + ig) = c.colh2o[lay] * k4(c, lay, B.absa, 65, ind0, ind1, ig) + c.colo3[lay] * B.abso3a[ig - 1];
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        for (int lay = laytrop + 1; lay <= nlay; ++lay)
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * B.rayl[ig - 1];
                G.tg(lay, g0 + ig) = c.colo3[lay] * B.abso3b[ig - 1];
                G.tr(lay, g0 + ig) = tauray;
            }
    }
    // band 26 (:1414-1474)
    {
        const BandTab& B = T.b[26]; const int g0 = B.g0;
        const int laysolfr = laytrop;
        for (int lay = 1; lay <= laytrop; ++lay)
            for (int ig = 1; ig <= B.ng; ++ig) {
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, 1.0);
                G.tg(lay, g0 + ig) = 0.0;
                G.tr(lay, g0 + ig) = c.colmol[lay] * B.rayl[ig - 1];
            }
        for (int lay = laytrop + 1; lay <= nlay; ++lay)
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = 0.0;
                G.tr(lay, g0 + ig) = c.colmol[lay] * B.rayl[ig - 1];
            }
    }
    // band 27 (:1477-1565)
    {
        const BandTab& B = T.b[27]; const int g0 = B.g0; const int layreffr = 32;
        const double scalekur = 50.15 / 48.37;
        for (int lay = 1; lay <= laytrop; ++lay) {
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + 1;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + 1;
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * B.rayl[ig - 1];
                G.tg(lay, g0 + ig) = c.colo3[lay] * k4(c, lay, B.absa, 65, ind0, ind1, ig);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        int laysolfr = nlay;
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            for (int ig = 1; ig <= B.ng; ++ig) {
                const double tauray = c.colmol[lay] * B.rayl[ig - 1];
                G.tg(lay, g0 + ig) = c.colo3[lay] * k4(c, lay, B.absb, 235, ind0, ind1, ig);
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, scalekur);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 28 (:1568-1692)
    {
        const BandTab& B = T.b[28]; const int g0 = B.g0; const int layreffr = 42;
        const double strrat = 6.67029e-07;
        for (int lay = 1; lay <= laytrop; ++lay) {
            Spec s = spec(c.colo3[lay], strrat * c.colo2[lay], 8.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + s.js;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absa, 585, ind0, ind1, ig, 9);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        int laysolfr = nlay;
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
            Spec s = spec(c.colo3[lay], strrat * c.colo2[lay], 4.0, c.fac00[lay], c.fac01[lay], c.fac10[lay], c.fac11[lay]);
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + s.js;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + s.js;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = s.speccomb * k8(s, B.absb, 1175, ind0, ind1, ig, 5);
                if (lay == laysolfr) set_source(G, S, B, ig, true, s.js, s.fs, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
    // band 29 (:1695-1785)
    {
        const BandTab& B = T.b[29]; const int g0 = B.g0; const int layreffr = 49;
        for (int lay = 1; lay <= laytrop; ++lay) {
            const int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * B.nspa + 1;
            const int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * B.nspa + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = c.colh2o[lay] * ((k4(c, lay, B.absa, 65, ind0, ind1, ig)) + selfterm(c, lay, B, ig) + forterm(c, lay, B, ig)) +
                                     c.colco2[lay] * B.absco2[ig - 1];
                G.tr(lay, g0 + ig) = tauray;
            }
        }
        int laysolfr = nlay;
        for (int lay = laytrop + 1; lay <= nlay; ++lay) {
            if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
            const int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * B.nspb + 1;
            const int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * B.nspb + 1;
            const double tauray = c.colmol[lay] * B.rayl[0];
            for (int ig = 1; ig <= B.ng; ++ig) {
                G.tg(lay, g0 + ig) = c.colco2[lay] * k4(c, lay, B.absb, 235, ind0, ind1, ig) + c.colh2o[lay] * B.absh2o[ig - 1];
                if (lay == laysolfr) set_source(G, S, B, ig, false, 0, 0.0, 1.0);
                G.tr(lay, g0 + ig) = tauray;
            }
        }
    }
}

// ---------------------------------------------------------------- cldprmc
// cldprmc_sw (rrtmg_sw_cldprmc.f90:53-349).  Arrays are (ngpt, nlay) with
// element (ig, lay) at [(ig-1) + 112*(lay-1)].  taucmc/ssacmc/asmcmc are
// inout; taormc is out.
int cldprmc(int nlay, int inflag, int iceflag, int liqflag, const double* cldfmc,
            const double* ciwpmc, const double* clwpmc, const double* reicmc, const double* relqmc,
            double* taormc, double* taucmc, double* ssacmc, double* asmcmc, const double* fsfcmc) {
    const double eps = 1.e-06, cldmin = 1.e-20;
    for (int k = 0; k < nlay * NGPT; ++k) taormc[k] = taucmc[k];
    for (int lay = 1; lay <= nlay; ++lay) {
        for (int ig = 1; ig <= NGPT; ++ig) {
            const int k = (ig - 1) + NGPT * (lay - 1);
            const double cwp = ciwpmc[k] + clwpmc[k];
            if (!(cldfmc[k] >= cldmin && (cwp >= cldmin || taucmc[k] >= cldmin))) continue;
            if (inflag == 0) {
                const double taucldorig_a = taucmc[k];
                const double ffp = fsfcmc[k];
                const double ffp1 = 1.0 - ffp;
                const double ffpssa = 1.0 - ffp * ssacmc[k];
                const double ssacloud_a = ffp1 * ssacmc[k] / ffpssa;
                const double taucloud_a = ffpssa * taucldorig_a;
                taormc[k] = taucldorig_a;
                ssacmc[k] = ssacloud_a;
                taucmc[k] = taucloud_a;
                asmcmc[k] = (asmcmc[k] - ffp) / (ffp1);
            } else if (inflag == 1) {
                return ORC_ERR_INFLAG1;
            } else if (inflag == 2) {
                const double radice = reicmc[lay - 1];
                double extcoice = 0, ssacoice = 0, gice = 0, forwice = 0;
                double extcoliq = 0, ssacoliq = 0, gliq = 0, forwliq = 0;
                const int ib = T.ngb[ig - 1];
                if (ciwpmc[k] == 0.0) {
                    extcoice = 0.0; ssacoice = 0.0; gice = 0.0; forwice = 0.0;
                } else if (iceflag == 1) {
                    if (radice < 13.0 || radice > 130.0) return ORC_ERR_ICE_RADIUS;
                    const double w2 = T.wavenum2[ib - 16];
                    int icx = 0;
                    if (w2 > 1.43e04) icx = 1;
                    else if (w2 > 7.7e03) icx = 2;
                    else if (w2 > 5.3e03) icx = 3;
                    else if (w2 > 4.0e03) icx = 4;
                    else if (w2 >= 2.5e03) icx = 5;
                    extcoice = (T.abari[icx - 1] + T.bbari[icx - 1] / radice);
                    ssacoice = 1.0 - T.cbari[icx - 1] - T.dbari[icx - 1] * radice;
                    gice = T.ebari[icx - 1] + T.fbari[icx - 1] * radice;
                    if (gice >= 1.0) gice = 1.0 - eps;
                    forwice = gice * gice;
                    if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0)
                        return ORC_ERR_ICE_PROPS;
                } else if (iceflag == 2) {
                    if (radice < 5.0 || radice > 131.0) return ORC_ERR_ICE_RADIUS;
                    const double factor = (radice - 2.0) / 3.0;
                    int index = (int)factor;
                    if (index == 43) index = 42;
                    const double fint = factor - (double)index;
                    extcoice = A(T.extice2, 43, index, ib - 15) + fint * (A(T.extice2, 43, index + 1, ib - 15) - A(T.extice2, 43, index, ib - 15));
                    ssacoice = A(T.ssaice2, 43, index, ib - 15) + fint * (A(T.ssaice2, 43, index + 1, ib - 15) - A(T.ssaice2, 43, index, ib - 15));
                    gice = A(T.asyice2, 43, index, ib - 15) + fint * (A(T.asyice2, 43, index + 1, ib - 15) - A(T.asyice2, 43, index, ib - 15));
                    forwice = gice * gice;
                    if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0)
                        return ORC_ERR_ICE_PROPS;
                } else if (iceflag == 3) {
                    if (radice < 5.0 || radice > 140.0) return ORC_ERR_ICE_DGE;
                    const double factor = (radice - 2.0) / 3.0;
                    int index = (int)factor;
                    if (index == 46) index = 45;
                    const double fint = factor - (double)index;
                    const int jb = ib - 15;
                    extcoice = A(T.extice3, 46, index, jb) + fint * (A(T.extice3, 46, index + 1, jb) - A(T.extice3, 46, index, jb));
                    ssacoice = A(T.ssaice3, 46, index, jb) + fint * (A(T.ssaice3, 46, index + 1, jb) - A(T.ssaice3, 46, index, jb));
                    gice = A(T.asyice3, 46, index, jb) + fint * (A(T.asyice3, 46, index + 1, jb) - A(T.asyice3, 46, index, jb));
                    const double fdelta = A(T.fdlice3, 46, index, jb) + fint * (A(T.fdlice3, 46, index + 1, jb) - A(T.fdlice3, 46, index, jb));
                    if (fdelta < 0.0 || fdelta > 1.0) return ORC_ERR_ICE_PROPS;
                    forwice = fdelta + 0.5 / ssacoice;
                    if (forwice > gice) forwice = gice;
                    if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0)
                        return ORC_ERR_ICE_PROPS;
                }
                if (clwpmc[k] == 0.0) {
                    extcoliq = 0.0; ssacoliq = 0.0; gliq = 0.0; forwliq = 0.0;
                } else if (liqflag == 1) {
                    const double radliq = relqmc[lay - 1];
                    if (radliq < 2.5 || radliq > 60.0) return ORC_ERR_LIQ_RADIUS;
                    int index = (int)(radliq - 1.5);
                    if (index == 0) index = 1;
                    if (index == 58) index = 57;
                    const double fint = radliq - 1.5 - (double)index;
                    const int jb = ib - 15;
                    extcoliq = A(T.extliq1, 58, index, jb) + fint * (A(T.extliq1, 58, index + 1, jb) - A(T.extliq1, 58, index, jb));
                    ssacoliq = A(T.ssaliq1, 58, index, jb) + fint * (A(T.ssaliq1, 58, index + 1, jb) - A(T.ssaliq1, 58, index, jb));
                    if (fint < 0.0 && ssacoliq > 1.0) ssacoliq = A(T.ssaliq1, 58, index, jb);
                    gliq = A(T.asyliq1, 58, index, jb) + fint * (A(T.asyliq1, 58, index + 1, jb) - A(T.asyliq1, 58, index, jb));
                    forwliq = gliq * gliq;
                    if (extcoliq < 0.0 || ssacoliq > 1.0 || ssacoliq < 0.0 || gliq > 1.0 || gliq < 0.0)
                        return ORC_ERR_LIQ_PROPS;
                }
                const double tauliqorig = clwpmc[k] * extcoliq;
                const double tauiceorig = ciwpmc[k] * extcoice;
                taormc[k] = tauliqorig + tauiceorig;
                const double ssaliq = ssacoliq * (1.0 - forwliq) / (1.0 - forwliq * ssacoliq);
                const double tauliq = (1.0 - forwliq * ssacoliq) * tauliqorig;
                const double ssaice = ssacoice * (1.0 - forwice) / (1.0 - forwice * ssacoice);
                const double tauice = (1.0 - forwice * ssacoice) * tauiceorig;
                const double scatliq = ssaliq * tauliq;
                double scatice = ssaice * tauice;
                taucmc[k] = tauliq + tauice;
                if (taucmc[k] == 0.0) taucmc[k] = cldmin;
                if (scatice == 0.0) scatice = cldmin;
                ssacmc[k] = (scatliq + scatice) / taucmc[k];
                if (iceflag == 3) {
                    asmcmc[k] = (1.0 / (scatliq + scatice)) *
                                (scatliq * (gliq - forwliq) / (1.0 - forwliq) +
                                 scatice * ((gice - forwice) / (1.0 - forwice)));
                } else {
                    asmcmc[k] = (scatliq * (gliq - forwliq) / (1.0 - forwliq) +
                                 scatice * (gice - forwice) / (1.0 - forwice)) / (scatliq + scatice);
                }
            }
        }
    }
    return ORC_OK;
}

// ---------------------------------------------------------------- cldprop
// cldprop_sw (rrtmg_sw_cldprop.f90:53-374): cloud optics per (layer, band)
// for the non-McICA path.  Inputs cldfrac/ciwp/clwp/rei/rel (nlay) and
// tauc/ssac/asmc/fsfc (14, nlay) at [(ib-1) + 14*(lay-1)]; outputs
// (nlay, 14) at [(lay-1) + nlay*(ib-1)].  The reference's stops return
// their codes.
int cldprop(int nlay, int inflag, int iceflag, int liqflag, const double* cldfrac, const double* tauc,
            const double* ssac, const double* asmc, const double* fsfc, const double* ciwp, const double* clwp,
            const double* rei, const double* rel, double* taucldorig, double* taucloud, double* ssacloud,
            double* asmcloud) {
    const double eps = 1.e-06, cldmin = 1.e-20;
    auto at = [&](double* v, int lay, int ib) -> double& { return v[(lay - 1) + nlay * (ib - 1)]; };
    auto bi = [&](const double* v, int ib, int lay) { return v[(ib - 1) + 14 * (lay - 1)]; };
    std::vector<double> tauctot(nlay, 0.0);
    for (int lay = 1; lay <= nlay; ++lay)  // :140-147
        for (int ib = 1; ib <= NBND; ++ib) {
            at(taucldorig, lay, ib) = bi(tauc, ib, lay);
            at(taucloud, lay, ib) = 0.0;
            at(ssacloud, lay, ib) = 1.0;
            at(asmcloud, lay, ib) = 0.0;
            tauctot[lay - 1] = tauctot[lay - 1] + bi(tauc, ib, lay);
        }
    for (int lay = 1; lay <= nlay; ++lay) {
        const double cwp = ciwp[lay - 1] + clwp[lay - 1];
        if (!(cldfrac[lay - 1] >= cldmin && (cwp >= cldmin || tauctot[lay - 1] >= cldmin))) continue;
        if (inflag == 0) {  // :158-174
            for (int ib = 1; ib <= NBND; ++ib) {
                const double taucldorig_a = bi(tauc, ib, lay);
                const double ffp = bi(fsfc, ib, lay);
                const double ffp1 = 1.0 - ffp;
                const double ffpssa = 1.0 - ffp * bi(ssac, ib, lay);
                const double ssacloud_a = ffp1 * bi(ssac, ib, lay) / ffpssa;
                const double taucloud_a = ffpssa * taucldorig_a;
                at(taucldorig, lay, ib) = taucldorig_a;
                at(ssacloud, lay, ib) = ssacloud_a;
                at(taucloud, lay, ib) = taucloud_a;
                at(asmcloud, lay, ib) = (bi(asmc, ib, lay) - ffp) / (ffp1);
            }
        } else if (inflag == 2) {  // :177-366
            const double radice = rei[lay - 1];
            double extcoice[NBND] = {0}, ssacoice[NBND] = {0}, gice[NBND] = {0}, forwice[NBND] = {0};
            double extcoliq[NBND] = {0}, ssacoliq[NBND] = {0}, gliq[NBND] = {0}, forwliq[NBND] = {0};
            if (ciwp[lay - 1] == 0.0) {
            } else if (iceflag == 1) {
                if (radice < 13.0 || radice > 130.0) return ORC_ERR_ICE_RADIUS;
                for (int jb = 1; jb <= NBND; ++jb) {
                    const double w2 = T.wavenum2[jb - 1];
                    int icx = 0;
                    if (w2 > 1.43e04) icx = 1;
                    else if (w2 > 7.7e03) icx = 2;
                    else if (w2 > 5.3e03) icx = 3;
                    else if (w2 > 4.0e03) icx = 4;
                    else if (w2 >= 2.5e03) icx = 5;
                    extcoice[jb - 1] = T.abari[icx - 1] + T.bbari[icx - 1] / radice;
                    ssacoice[jb - 1] = 1.0 - T.cbari[icx - 1] - T.dbari[icx - 1] * radice;
                    gice[jb - 1] = T.ebari[icx - 1] + T.fbari[icx - 1] * radice;
                    if (gice[jb - 1] >= 1.0) gice[jb - 1] = 1.0 - eps;
                    forwice[jb - 1] = gice[jb - 1] * gice[jb - 1];
                    if (extcoice[jb - 1] < 0.0 || ssacoice[jb - 1] > 1.0 || ssacoice[jb - 1] < 0.0 ||
                        gice[jb - 1] > 1.0 || gice[jb - 1] < 0.0)
                        return ORC_ERR_ICE_PROPS;
                }
            } else if (iceflag == 2) {
                if (radice < 5.0 || radice > 131.0) return ORC_ERR_ICE_RADIUS;
                const double factor = (radice - 2.0) / 3.0;
                int index = (int)factor;
                if (index == 43) index = 42;
                const double fint = factor - (double)index;
                for (int jb = 1; jb <= NBND; ++jb) {
                    extcoice[jb - 1] = A(T.extice2, 43, index, jb) + fint * (A(T.extice2, 43, index + 1, jb) - A(T.extice2, 43, index, jb));
                    ssacoice[jb - 1] = A(T.ssaice2, 43, index, jb) + fint * (A(T.ssaice2, 43, index + 1, jb) - A(T.ssaice2, 43, index, jb));
                    gice[jb - 1] = A(T.asyice2, 43, index, jb) + fint * (A(T.asyice2, 43, index + 1, jb) - A(T.asyice2, 43, index, jb));
                    forwice[jb - 1] = gice[jb - 1] * gice[jb - 1];
                    if (extcoice[jb - 1] < 0.0 || ssacoice[jb - 1] > 1.0 || ssacoice[jb - 1] < 0.0 ||
                        gice[jb - 1] > 1.0 || gice[jb - 1] < 0.0)
                        return ORC_ERR_ICE_PROPS;
                }
            } else if (iceflag == 3) {
                if (radice < 5.0 || radice > 140.0) return ORC_ERR_ICE_DGE;
                const double factor = (radice - 2.0) / 3.0;
                int index = (int)factor;
                if (index == 46) index = 45;
                const double fint = factor - (double)index;
                for (int jb = 1; jb <= NBND; ++jb) {
                    extcoice[jb - 1] = A(T.extice3, 46, index, jb) + fint * (A(T.extice3, 46, index + 1, jb) - A(T.extice3, 46, index, jb));
                    ssacoice[jb - 1] = A(T.ssaice3, 46, index, jb) + fint * (A(T.ssaice3, 46, index + 1, jb) - A(T.ssaice3, 46, index, jb));
                    gice[jb - 1] = A(T.asyice3, 46, index, jb) + fint * (A(T.asyice3, 46, index + 1, jb) - A(T.asyice3, 46, index, jb));
                    const double fdelta = A(T.fdlice3, 46, index, jb) + fint * (A(T.fdlice3, 46, index + 1, jb) - A(T.fdlice3, 46, index, jb));
                    if (fdelta < 0.0 || fdelta > 1.0) return ORC_ERR_ICE_PROPS;
                    forwice[jb - 1] = fdelta + 0.5 / ssacoice[jb - 1];
                    if (forwice[jb - 1] > gice[jb - 1]) forwice[jb - 1] = gice[jb - 1];
                    if (extcoice[jb - 1] < 0.0 || ssacoice[jb - 1] > 1.0 || ssacoice[jb - 1] < 0.0 ||
                        gice[jb - 1] > 1.0 || gice[jb - 1] < 0.0)
                        return ORC_ERR_ICE_PROPS;
                }
            }
            if (clwp[lay - 1] == 0.0) {
            } else if (liqflag == 1) {
                const double radliq = rel[lay - 1];
                if (radliq < 2.5 || radliq > 60.0) return ORC_ERR_LIQ_RADIUS;
                int index = (int)(radliq - 1.5);
                if (index == 0) index = 1;
                if (index == 58) index = 57;
                const double fint = radliq - 1.5 - (double)index;
                for (int jb = 1; jb <= NBND; ++jb) {
                    extcoliq[jb - 1] = A(T.extliq1, 58, index, jb) + fint * (A(T.extliq1, 58, index + 1, jb) - A(T.extliq1, 58, index, jb));
                    ssacoliq[jb - 1] = A(T.ssaliq1, 58, index, jb) + fint * (A(T.ssaliq1, 58, index + 1, jb) - A(T.ssaliq1, 58, index, jb));
                    if (fint < 0.0 && ssacoliq[jb - 1] > 1.0) ssacoliq[jb - 1] = A(T.ssaliq1, 58, index, jb);
                    gliq[jb - 1] = A(T.asyliq1, 58, index, jb) + fint * (A(T.asyliq1, 58, index + 1, jb) - A(T.asyliq1, 58, index, jb));
                    forwliq[jb - 1] = gliq[jb - 1] * gliq[jb - 1];
                    if (extcoliq[jb - 1] < 0.0 || ssacoliq[jb - 1] > 1.0 || ssacoliq[jb - 1] < 0.0 ||
                        gliq[jb - 1] > 1.0 || gliq[jb - 1] < 0.0)
                        return ORC_ERR_LIQ_PROPS;
                }
            }
            for (int ib = 1; ib <= NBND; ++ib) {
                const int j = ib - 1;
                const double tauliqorig = clwp[lay - 1] * extcoliq[j];
                const double tauiceorig = ciwp[lay - 1] * extcoice[j];
                at(taucldorig, lay, ib) = tauliqorig + tauiceorig;
                const double ssaliq = ssacoliq[j] * (1.0 - forwliq[j]) / (1.0 - forwliq[j] * ssacoliq[j]);
                const double tauliq = (1.0 - forwliq[j] * ssacoliq[j]) * tauliqorig;
                const double ssaice = ssacoice[j] * (1.0 - forwice[j]) / (1.0 - forwice[j] * ssacoice[j]);
                const double tauice = (1.0 - forwice[j] * ssacoice[j]) * tauiceorig;
                const double scatliq = ssaliq * tauliq;
                double scatice = ssaice * tauice;
                at(taucloud, lay, ib) = tauliq + tauice;
                if (at(taucloud, lay, ib) == 0.0) at(taucloud, lay, ib) = cldmin;
                if (scatice == 0.0) scatice = cldmin;
                at(ssacloud, lay, ib) = (scatliq + scatice) / at(taucloud, lay, ib);
                if (iceflag == 3) {
                    at(asmcloud, lay, ib) = (1.0 / (scatliq + scatice)) *
                                            (scatliq * (gliq[j] - forwliq[j]) / (1.0 - forwliq[j]) +
                                             scatice * ((gice[j] - forwice[j]) / (1.0 - forwice[j])));
                } else {
                    at(asmcloud, lay, ib) = (scatliq * (gliq[j] - forwliq[j]) / (1.0 - forwliq[j]) +
                                             scatice * (gice[j] - forwice[j]) / (1.0 - forwice[j])) /
                                            (scatliq + scatice);
                }
            }
        }
    }
    return ORC_OK;
}

// ---------------------------------------------------------------- reftra
// exp(-x) through the lookup table, or the quadratic below od_lo
// (rrtmg_sw_reftra.f90:203-209)
inline double tbl_exp(double ze1) {
    const double od_lo = 0.06;
    if (ze1 <= od_lo) return 1.0 - ze1 + 0.5 * ze1 * ze1;
    const double tblind = ze1 / (T.bpade + ze1);
    const int itind = (int)(10000.0 * tblind + 0.5);
    return T.exp_tbl[itind];
}

// reftra_sw (rrtmg_sw_reftra.f90:48-329) for kmodts = 2; arrays 1-based
void reftra(int nlay, const std::vector<char>& lrtchk, const std::vector<double>& pgg, double prmuz,
            const std::vector<double>& ptau, const std::vector<double>& pw, std::vector<double>& pref,
            std::vector<double>& prefd, std::vector<double>& ptra, std::vector<double>& ptrad) {
    const double zwcrit = 0.9999995, eps = 1.e-08;
    for (int jk = 1; jk <= nlay; ++jk) {
        if (!lrtchk[jk]) {
            pref[jk] = 0.0; ptra[jk] = 1.0; prefd[jk] = 0.0; ptrad[jk] = 1.0;
            continue;
        }
        const double zto1 = ptau[jk], zw = pw[jk], zg = pgg[jk];
        const double zg3 = 3.0 * zg;
        const double zgamma1 = (8.0 - zw * (5.0 + zg3)) * 0.25;
        const double zgamma2 = 3.0 * (zw * (1.0 - zg)) * 0.25;
        const double zgamma3 = (2.0 - zg3 * prmuz) * 0.25;
        const double zgamma4 = 1.0 - zgamma3;
        double zwo = 0.0, denom = 1.0;
        if (zg != 1.0) {
            const double q = zg / (1.0 - zg);
            denom = (1.0 - (1.0 - zw) * (q * q));
        }
        if (zw > 0.0 && denom != 0.0) zwo = zw / denom;
        if (zwo >= zwcrit) {
            const double za = zgamma1 * prmuz;
            const double za1 = za - zgamma3;
            const double zgt = zgamma1 * zto1;
            const double ze1 = std::min(zto1 / prmuz, 500.0);
            const double ze2 = tbl_exp(ze1);
            pref[jk] = (zgt - za1 * (1.0 - ze2)) / (1.0 + zgt);
            ptra[jk] = 1.0 - pref[jk];
            prefd[jk] = zgt / (1.0 + zgt);
            ptrad[jk] = 1.0 - prefd[jk];
            if (ze2 == 1.0) { pref[jk] = 0.0; ptra[jk] = 1.0; prefd[jk] = 0.0; ptrad[jk] = 1.0; }
        } else {
            const double za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
            const double za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
            const double zrk = std::sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
            const double zrp = zrk * prmuz;
            const double zrp1 = 1.0 + zrp, zrm1 = 1.0 - zrp;
            const double zrk2 = 2.0 * zrk;
            const double zrpp = 1.0 - zrp * zrp;
            const double zrkg = zrk + zgamma1;
            const double zr1 = zrm1 * (za2 + zrk * zgamma3);
            const double zr2 = zrp1 * (za2 - zrk * zgamma3);
            const double zr3 = zrk2 * (zgamma3 - za2 * prmuz);
            const double zr4 = zrpp * zrkg;
            const double zr5 = zrpp * (zrk - zgamma1);
            const double zt1 = zrp1 * (za1 + zrk * zgamma4);
            const double zt2 = zrm1 * (za1 - zrk * zgamma4);
            const double zt3 = zrk2 * (zgamma4 + za1 * prmuz);
            const double zt4 = zr4, zt5 = zr5;
            const double zbeta = (zgamma1 - zrk) / zrkg;
            const double ze1 = std::min(zrk * zto1, 500.0);
            const double ze2 = std::min(zto1 / prmuz, 500.0);
            const double zem1 = tbl_exp(ze1);
            const double zep1 = 1.0 / zem1;
            const double zem2 = tbl_exp(ze2);
            const double zep2 = 1.0 / zem2;
            const double zdenr = zr4 * zep1 + zr5 * zem1;
            const double zdent = zt4 * zep1 + zt5 * zem1;
            if (zdenr >= -eps && zdenr <= eps) {
                pref[jk] = eps;
                ptra[jk] = zem2;
            } else {
                pref[jk] = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
                ptra[jk] = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
            }
            const double zemm = zem1 * zem1;
            const double zdend = 1.0 / ((1.0 - zbeta * zemm) * zrkg);
            prefd[jk] = zgamma2 * (1.0 - zemm) * zdend;
            ptrad[jk] = zrk2 * zem1 * zdend;
        }
    }
}

// ---------------------------------------------------------------- vrtqdr
// vrtqdr_sw (rrtmg_sw_vrtqdr.f90:47-171); arrays 1-based over 1..klev+1
void vrtqdr(int klev, const std::vector<double>& pref, const std::vector<double>& prefd,
            const std::vector<double>& ptra, const std::vector<double>& ptrad,
            const std::vector<double>& pdbt, std::vector<double>& prdnd, std::vector<double>& prup,
            std::vector<double>& prupd, const std::vector<double>& ptdbt, std::vector<double>& pfd,
            std::vector<double>& pfu) {
    std::vector<double> ztdn(klev + 2);
    double zreflect = 1.0 / (1.0 - prefd[klev + 1] * prefd[klev]);
    prup[klev] = pref[klev] + (ptrad[klev] * ((ptra[klev] - pdbt[klev]) * prefd[klev + 1] + pdbt[klev] * pref[klev + 1])) * zreflect;
    prupd[klev] = prefd[klev] + ptrad[klev] * ptrad[klev] * prefd[klev + 1] * zreflect;
    for (int jk = 1; jk <= klev - 1; ++jk) {
        const int ikp = klev + 1 - jk, ikx = ikp - 1;
        zreflect = 1.0 / (1.0 - prupd[ikp] * prefd[ikx]);
        prup[ikx] = pref[ikx] + (ptrad[ikx] * ((ptra[ikx] - pdbt[ikx]) * prupd[ikp] + pdbt[ikx] * prup[ikp])) * zreflect;
        prupd[ikx] = prefd[ikx] + ptrad[ikx] * ptrad[ikx] * prupd[ikp] * zreflect;
    }
    ztdn[1] = 1.0;
    prdnd[1] = 0.0;
    ztdn[2] = ptra[1];
    prdnd[2] = prefd[1];
    for (int jk = 2; jk <= klev; ++jk) {
        const int ikp = jk + 1;
        zreflect = 1.0 / (1.0 - prefd[jk] * prdnd[jk]);
        ztdn[ikp] = ptdbt[jk] * ptra[jk] + (ptrad[jk] * ((ztdn[jk] - ptdbt[jk]) + ptdbt[jk] * pref[jk] * prdnd[jk])) * zreflect;
        prdnd[ikp] = prefd[jk] + ptrad[jk] * ptrad[jk] * prdnd[jk] * zreflect;
    }
    for (int jk = 1; jk <= klev + 1; ++jk) {
        zreflect = 1.0 / (1.0 - prdnd[jk] * prupd[jk]);
        pfu[jk] = (ptdbt[jk] * prup[jk] + (ztdn[jk] - ptdbt[jk]) * prupd[jk]) * zreflect;
        pfd[jk] = ptdbt[jk] + (ztdn[jk] - ptdbt[jk] + ptdbt[jk] * prup[jk] * prdnd[jk]) * zreflect;
    }
}

// ---------------------------------------------------------------- spcvmc
struct Fluxes {  // level arrays 1..nlay+1, bottom to top
    std::vector<double> bbfd, bbfu, bbcd, bbcu, uvfd, uvcd, nifd, nicd;
    std::vector<double> bbfddir, bbcddir, uvfddir, uvcddir, nifddir, nicddir;
    // per band (ibm 1..14): total up, down, direct down, clear up, down at
    // [(ibm-1)*(n+2) + level]
    std::vector<double> bnd[5];
    int nlev2 = 0;
    void alloc(int n) {
        for (auto* v : {&bbfd, &bbfu, &bbcd, &bbcu, &uvfd, &uvcd, &nifd, &nicd, &bbfddir, &bbcddir,
                        &uvfddir, &uvcddir, &nifddir, &nicddir})
            v->assign(n + 2, 0.0);
        nlev2 = n + 2;
        for (auto& v : bnd) v.assign((size_t)14 * (n + 2), 0.0);
    }
};

struct ColumnOptics {
    // (lay 1..nlay, g 1..112) -> [(lay-1) + nlay*(g-1)], Fortran z* arrays of the driver
    std::vector<double> cldfmc, taucmc, asycmc, omgcmc, taormc;
    // (lay, band 1..14) -> [(lay-1) + nlay*(ib-1)]
    std::vector<double> taua, asya, omga;
};

// spcvrt_sw (rrtmg_sw_spcvrt.f90:53-667) differs from spcvmc_sw only in
// reading the cloud fraction per layer (pclfr, :429,453-454,547-548) and the
// cloud optics per (layer, band) (ptauc .. ptaucorig indexed by the band of
// the g-point, :473,503-515).  The oracle therefore runs spcvmc with the
// band values spread over their g-points and the layer fraction over all
// g-points.
void spread_bands(int nlay, const double* cldfrac, const double* taucloud, const double* taucldorig,
                  const double* ssacloud, const double* asmcloud, ColumnOptics& O) {
    for (int l = 1; l <= nlay; ++l)
        for (int ig = 1; ig <= NGPT; ++ig) {
            const int ib = T.ngb[ig - 1] - 15;
            const size_t d = (l - 1) + (size_t)nlay * (ig - 1);
            const size_t s = (l - 1) + (size_t)nlay * (ib - 1);
            O.cldfmc[d] = cldfrac[l - 1];
            O.taucmc[d] = taucloud[s];
            O.taormc[d] = taucldorig[s];
            O.asycmc[d] = asmcloud[s];
            O.omgcmc[d] = ssacloud[s];
        }
}

// spcvmc_sw (rrtmg_sw_spcvmc.f90:53-663); icpr = 1 (cloud properties from
// cldprmc, already delta-scaled)
void spcvmc(int nlay, int istart, int iend, int idelm, int iout, const double* palbd,
            const double* palbp, const ColumnOptics& O, double prmu0, const double* adjflux,
            const Solar& S, const Gas& G, Fluxes& F) {
    const int klev = nlay;
    const double repclc = 1.e-12;
    F.alloc(nlay);
    std::vector<char> lrtchkclr(klev + 2), lrtchkcld(klev + 2);
    std::vector<double> zdbt(klev + 2), zdbt_nodel(klev + 2), zgcc(klev + 2), zgco(klev + 2),
        zomcc(klev + 2), zomco(klev + 2), zrdnd(klev + 2), zrdndc(klev + 2), zref(klev + 2),
        zrefc(klev + 2), zrefo(klev + 2), zrefd(klev + 2), zrefdc(klev + 2), zrefdo(klev + 2),
        zrup(klev + 2), zrupd(klev + 2), zrupc(klev + 2), zrupdc(klev + 2), ztauc(klev + 2),
        ztauo(klev + 2), ztdbt(klev + 2), ztra(klev + 2), ztrac(klev + 2), ztrao(klev + 2),
        ztrad(klev + 2), ztradc(klev + 2), ztrado(klev + 2), zdbtc(klev + 2), ztdbtc(klev + 2),
        zdbtc_nodel(klev + 2), ztdbt_nodel(klev + 2), ztdbtc_nodel(klev + 2), zcd(klev + 2),
        zcu(klev + 2), zfd(klev + 2), zfu(klev + 2);
    auto cl = [&](const std::vector<double>& v, int lay, int ig) { return v[(lay - 1) + nlay * (ig - 1)]; };
    auto ab = [&](const std::vector<double>& v, int lay, int ib) { return v[(lay - 1) + nlay * (ib - 1)]; };
    int iw = 0;
    for (int jb = istart; jb <= iend; ++jb) {
        const int ibm = jb - 15;
        const int igt = kNG[ibm - 1];
        if (iout > 0 && ibm >= 2) {
            iw = 0;
            for (int k = 0; k < ibm - 1; ++k) iw += kNG[k];
        }
        for (int jg = 1; jg <= igt; ++jg) {
            iw = iw + 1;
            double zincflx;
            if (S.isolvar < 0) zincflx = adjflux[jb - 16] * G.sfluxzen[iw - 1] * prmu0;
            else zincflx = adjflux[jb - 16] * G.ssi[iw - 1] * prmu0;
            ztdbtc[1] = 1.0;
            ztdbtc_nodel[1] = 1.0;
            zdbtc[klev + 1] = 0.0;
            ztrac[klev + 1] = 0.0;
            ztradc[klev + 1] = 0.0;
            zrefc[klev + 1] = palbp[ibm - 1];
            zrefdc[klev + 1] = palbd[ibm - 1];
            zrupc[klev + 1] = palbp[ibm - 1];
            zrupdc[klev + 1] = palbd[ibm - 1];
            ztrao[klev + 1] = 0.0;
            ztrado[klev + 1] = 0.0;
            zrefo[klev + 1] = palbp[ibm - 1];
            zrefdo[klev + 1] = palbd[ibm - 1];
            ztdbt[1] = 1.0;
            ztdbt_nodel[1] = 1.0;
            zdbt[klev + 1] = 0.0;
            ztra[klev + 1] = 0.0;
            ztrad[klev + 1] = 0.0;
            zref[klev + 1] = palbp[ibm - 1];
            zrefd[klev + 1] = palbd[ibm - 1];
            zrup[klev + 1] = palbp[ibm - 1];
            zrupd[klev + 1] = palbd[ibm - 1];
            for (int jk = 1; jk <= klev; ++jk) {
                const int ikl = klev + 1 - jk;
                lrtchkclr[jk] = 1;
                lrtchkcld[jk] = cl(O.cldfmc, ikl, iw) > repclc;
                const double taur = G.taur[(ikl - 1) + nlay * (iw - 1)];
                const double taug = G.taug[(ikl - 1) + nlay * (iw - 1)];
                const double taua = ab(O.taua, ikl, ibm), omga = ab(O.omga, ikl, ibm), asya = ab(O.asya, ikl, ibm);
                ztauc[jk] = taur + taug + taua;
                zomcc[jk] = taur * 1.0 + taua * omga;
                zgcc[jk] = asya * omga * taua / zomcc[jk];
                zomcc[jk] = zomcc[jk] / ztauc[jk];
                if (idelm == 0) {
                    const double zclear = 1.0 - cl(O.cldfmc, ikl, iw);
                    const double zcloud = cl(O.cldfmc, ikl, iw);
                    const double zdbtmc = tbl_exp(ztauc[jk] / prmu0);
                    zdbtc_nodel[jk] = zdbtmc;
                    ztdbtc_nodel[jk + 1] = zdbtc_nodel[jk] * ztdbtc_nodel[jk];
                    const double tauorig = ztauc[jk] + cl(O.taormc, ikl, iw);
                    const double zdbtmo = tbl_exp(tauorig / prmu0);
                    zdbt_nodel[jk] = zclear * zdbtmc + zcloud * zdbtmo;
                    ztdbt_nodel[jk + 1] = zdbt_nodel[jk] * ztdbt_nodel[jk];
                }
                const double zf = zgcc[jk] * zgcc[jk];
                const double zwf = zomcc[jk] * zf;
                ztauc[jk] = (1.0 - zwf) * ztauc[jk];
                zomcc[jk] = (zomcc[jk] - zwf) / (1.0 - zwf);
                zgcc[jk] = (zgcc[jk] - zf) / (1.0 - zf);
                const double tc = cl(O.taucmc, ikl, iw), oc = cl(O.omgcmc, ikl, iw), gc = cl(O.asycmc, ikl, iw);
                ztauo[jk] = ztauc[jk] + tc;
                zomco[jk] = ztauc[jk] * zomcc[jk] + tc * oc;
                zgco[jk] = (tc * oc * gc + ztauc[jk] * zomcc[jk] * zgcc[jk]) / zomco[jk];
                zomco[jk] = zomco[jk] / ztauo[jk];
            }
            reftra(klev, lrtchkclr, zgcc, prmu0, ztauc, zomcc, zrefc, zrefdc, ztrac, ztradc);
            reftra(klev, lrtchkcld, zgco, prmu0, ztauo, zomco, zrefo, zrefdo, ztrao, ztrado);
            for (int jk = 1; jk <= klev; ++jk) {
                const int ikl = klev + 1 - jk;
                const double zclear = 1.0 - cl(O.cldfmc, ikl, iw);
                const double zcloud = cl(O.cldfmc, ikl, iw);
                zref[jk] = zclear * zrefc[jk] + zcloud * zrefo[jk];
                zrefd[jk] = zclear * zrefdc[jk] + zcloud * zrefdo[jk];
                ztra[jk] = zclear * ztrac[jk] + zcloud * ztrao[jk];
                ztrad[jk] = zclear * ztradc[jk] + zcloud * ztrado[jk];
                const double zdbtmc = tbl_exp(ztauc[jk] / prmu0);
                zdbtc[jk] = zdbtmc;
                ztdbtc[jk + 1] = zdbtc[jk] * ztdbtc[jk];
                const double zdbtmo = tbl_exp(ztauo[jk] / prmu0);
                zdbt[jk] = zclear * zdbtmc + zcloud * zdbtmo;
                ztdbt[jk + 1] = zdbt[jk] * ztdbt[jk];
            }
            vrtqdr(klev, zrefc, zrefdc, ztrac, ztradc, zdbtc, zrdndc, zrupc, zrupdc, ztdbtc, zcd, zcu);
            vrtqdr(klev, zref, zrefd, ztra, ztrad, zdbt, zrdnd, zrup, zrupd, ztdbt, zfd, zfu);
            for (int jk = 1; jk <= klev + 1; ++jk) {
                const int ikl = klev + 2 - jk;
                F.bbfu[ikl] = F.bbfu[ikl] + zincflx * zfu[jk];
                F.bbfd[ikl] = F.bbfd[ikl] + zincflx * zfd[jk];
                F.bbcu[ikl] = F.bbcu[ikl] + zincflx * zcu[jk];
                F.bbcd[ikl] = F.bbcd[ikl] + zincflx * zcd[jk];
                const double dirf = idelm == 0 ? ztdbt_nodel[jk] : ztdbt[jk];
                const double dirc = idelm == 0 ? ztdbtc_nodel[jk] : ztdbtc[jk];
                F.bbfddir[ikl] = F.bbfddir[ikl] + zincflx * dirf;
                F.bbcddir[ikl] = F.bbcddir[ikl] + zincflx * dirc;
                const size_t bo = (size_t)(ibm - 1) * F.nlev2 + ikl;
                F.bnd[0][bo] += zincflx * zfu[jk];
                F.bnd[1][bo] += zincflx * zfd[jk];
                F.bnd[2][bo] += zincflx * dirf;
                F.bnd[3][bo] += zincflx * zcu[jk];
                F.bnd[4][bo] += zincflx * zcd[jk];
                if (ibm >= 10 && ibm <= 13) {
                    F.uvcd[ikl] = F.uvcd[ikl] + zincflx * zcd[jk];
                    F.uvfd[ikl] = F.uvfd[ikl] + zincflx * zfd[jk];
                    F.uvfddir[ikl] = F.uvfddir[ikl] + zincflx * dirf;
                    F.uvcddir[ikl] = F.uvcddir[ikl] + zincflx * dirc;
                } else if (ibm == 14 || ibm <= 9) {
                    F.nicd[ikl] = F.nicd[ikl] + zincflx * zcd[jk];
                    F.nifd[ikl] = F.nifd[ikl] + zincflx * zfd[jk];
                    F.nifddir[ikl] = F.nifddir[ikl] + zincflx * dirf;
                    F.nicddir[ikl] = F.nicddir[ikl] + zincflx * dirc;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- McICA RNGs
// Mersenne Twister MT19937 (mcica_random_numbers.f90:77-306)
struct MT {
    uint32_t state[624];
    int cur;
    explicit MT(int32_t seed) {
        state[0] = (uint32_t)seed;
        for (int i = 1; i < 624; ++i)
            state[i] = 1812433253u * (state[i - 1] ^ (state[i - 1] >> 30)) + (uint32_t)i;
        cur = 624;
    }
    static uint32_t twist(uint32_t u, uint32_t v) {
        const uint32_t mix = (u & 0x80000000u) | (v & 0x7fffffffu);
        return (mix >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
    }
    void next_state() {
        for (int k = 0; k < 624 - 397; ++k) state[k] = state[k + 397] ^ twist(state[k], state[k + 1]);
        for (int k = 624 - 397; k < 623; ++k) state[k] = state[k + 397 - 624] ^ twist(state[k], state[k + 1]);
        state[623] = state[396] ^ twist(state[623], state[0]);
        cur = 0;
    }
    uint32_t next_int() {
        if (cur >= 624) next_state();
        uint32_t y = state[cur++];
        y ^= (y >> 11);
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= (y >> 18);
        return y;
    }
    // getRandomReal (:276-295): u32 / (2^32 - 1) in FP64
    double next_real() { return (double)next_int() / (4294967296.0 - 1.0); }
};

// KISS (mcica_subcol_gen_sw.f90:721-753), 32-bit wrapping arithmetic
struct Kiss {
    uint32_t s1, s2, s3, s4;
    double next() {
        s1 = 69069u * s1 + 1327217885u;
        uint32_t k = s2;
        k = k ^ (k << 13);
        k = k ^ (k >> 17);
        k = k ^ (k << 5);
        s2 = k;
        s3 = 18000u * (s3 & 65535u) + (s3 >> 16);
        s4 = 30903u * (s4 & 65535u) + (s4 >> 16);
        const int32_t kiss = (int32_t)(s1 + s2 + (s3 << 16) + s4);
        return (double)kiss * 2.328306e-10 + 0.5;
    }
};

// seed = int((pmid - int(pmid)) * 1e9) with pmid in Pa (mcica:475-478);
// the product is real and the conversion truncates toward zero
inline int32_t kiss_seed(double pmid) {
    const double frac = pmid - (double)(int64_t)pmid;
    return (int32_t)(int64_t)(frac * 1000000000.0);
}

std::string g_err;

inline int omp_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // namespace


// ====================================================================== API
extern "C" {

int orc_init(const char* path, double cpdair) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return ORC_ERR_TABLES;
    char magic[8];
    uint32_t n = 0;
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "RRSWTB01", 8) != 0 ||
        std::fread(&n, 4, 1, f) != 1) {
        std::fclose(f);
        return ORC_ERR_TABLES;
    }
    std::map<std::string, std::vector<double>> rec;
    for (uint32_t r = 0; r < n; ++r) {
        char name[32];
        uint32_t hdr[5];
        uint64_t cnt;
        if (std::fread(name, 1, 32, f) != 32 || std::fread(hdr, 4, 5, f) != 5 || std::fread(&cnt, 8, 1, f) != 1) {
            std::fclose(f);
            return ORC_ERR_TABLES;
        }
        std::vector<double> v(cnt);
        if (std::fread(v.data(), 8, cnt, f) != cnt) { std::fclose(f); return ORC_ERR_TABLES; }
        name[31] = 0;
        rec[name] = std::move(v);
    }
    std::fclose(f);
    auto get = [&](const std::string& k) -> const std::vector<double>& {
        static const std::vector<double> empty;
        auto it = rec.find(k);
        return it == rec.end() ? empty : it->second;
    };
    int g0 = 0;
    for (int band = 16; band <= 29; ++band) {
        BandTab& B = T.b[band];
        const std::string p = "b" + std::to_string(band) + ".";
        B.ng = kNG[band - 16];
        B.g0 = g0;
        g0 += B.ng;
        B.nspa = kNSPA[band - 16];
        B.nspb = kNSPB[band - 16];
        B.absa = get(p + "ka");
        B.absb = get(p + "kb");
        B.selfref = get(p + "selfref");
        B.forref = get(p + "forref");
        B.nfr = B.forref.empty() ? 3 : (int)(B.forref.size() / B.ng);
        B.sfluxref = get(p + "sfluxref");
        B.irradnce = get(p + "irradnce");
        B.facbrght = get(p + "facbrght");
        B.snsptdrk = get(p + "snsptdrk");
        B.rayl = get(p + "rayl");
        B.rayla = get(p + "rayla");
        B.raylb = get(p + "raylb");
        B.abso3a = get(p + "abso3a");
        B.abso3b = get(p + "abso3b");
        B.absch4 = get(p + "absch4");
        B.absco2 = get(p + "absco2");
        B.absh2o = get(p + "absh2o");
        if (B.sfluxref.empty()) return ORC_ERR_TABLES;
    }
    auto cp = [&](const char* k, double* dst, size_t nn) {
        const auto& v = get(k);
        if (v.size() != nn) return false;
        std::memcpy(dst, v.data(), nn * 8);
        return true;
    };
    bool ok = cp("pref", T.pref, 59) && cp("preflog", T.preflog, 59) && cp("tref", T.tref, 59) &&
              cp("abari", T.abari, 5) && cp("bbari", T.bbari, 5) && cp("cbari", T.cbari, 5) &&
              cp("dbari", T.dbari, 5) && cp("ebari", T.ebari, 5) && cp("fbari", T.fbari, 5) &&
              cp("rsrtaua", T.rsrtaua, 84) && cp("rsrpiza", T.rsrpiza, 84) && cp("rsrasya", T.rsrasya, 84) &&
              cp("wavenum1", T.wavenum1, 14) && cp("wavenum2", T.wavenum2, 14) &&
              cp("mgavgcyc", T.mgavgcyc, 134) && cp("sbavgcyc", T.sbavgcyc, 134);
    if (!ok) return ORC_ERR_TABLES;
    T.extliq1 = get("extliq1"); T.ssaliq1 = get("ssaliq1"); T.asyliq1 = get("asyliq1");
    T.extice2 = get("extice2"); T.ssaice2 = get("ssaice2"); T.asyice2 = get("asyice2");
    T.extice3 = get("extice3"); T.ssaice3 = get("ssaice3"); T.asyice3 = get("asyice3");
    T.fdlice3 = get("fdlice3");
    const auto& ngb = get("ngb");
    if (ngb.size() != NGPT) return ORC_ERR_TABLES;
    for (int i = 0; i < NGPT; ++i) T.ngb[i] = (int)ngb[i];
    // exp_tbl: rrtmg_sw_init.f90:115-123
    const double expeps = 1.e-20, pade = 0.278;
    T.exp_tbl[0] = 1.0;
    T.exp_tbl[NTBL] = expeps;
    T.bpade = 1.0 / pade;
    for (int itr = 1; itr <= NTBL - 1; ++itr) {
        const double tfn = (double)itr / (double)NTBL;
        const double tau_tbl = T.bpade * tfn / (1.0 - tfn);
        T.exp_tbl[itr] = std::exp(-tau_tbl);
        if (T.exp_tbl[itr] <= expeps) T.exp_tbl[itr] = expeps;
    }
    // heatfac: rrtmg_sw_init.f90:258 (grav, secdy :207-243)
    const double grav = 9.8066, secdy = 8.6400e4;
    T.heatfac = grav * secdy / (cpdair * 1.e2);
    T.oneminus = 1.0 - 1.e-06;  // rrtmg_sw_rad.f90:563-565
    T.pi = 2.0 * std::asin(1.0);
    T.ok = true;
    return ORC_OK;
}

int orc_exp_table(double* out) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    std::memcpy(out, T.exp_tbl, sizeof(T.exp_tbl));
    return ORC_OK;
}

double orc_heatfac(void) { return T.heatfac; }

int orc_setcoef_indices(int nlay, const double* pavel, const double* tavel, const double* coldry,
                        const double* wkl, int32_t* jp, int32_t* jt, int32_t* jt1, int32_t* indself,
                        int32_t* indfor, int32_t* laytrop) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    Coef c;
    setcoef(nlay, pavel, tavel, coldry, wkl, c);
    for (int l = 1; l <= nlay; ++l) {
        jp[l - 1] = c.jp[l]; jt[l - 1] = c.jt[l]; jt1[l - 1] = c.jt1[l];
        indself[l - 1] = c.indself[l]; indfor[l - 1] = c.indfor[l];
    }
    *laytrop = c.laytrop;
    return ORC_OK;
}

// setcoef_sw indices of GCM-interface columns: inatm_sw's layer amounts
// (rrtmg_sw_rad.f90:1527-1586, as in rrtmg_sw_impl below), then setcoef.
// Outputs (ncol, nlay) in column-major order, laytrop (ncol).
int orc_gcm_setcoef_indices(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                            const double* h2ovmr, const double* co2vmr, const double* o3vmr, const double* n2ovmr,
                            const double* ch4vmr, const double* o2vmr, int32_t* jp, int32_t* jt, int32_t* jt1,
                            int32_t* indself, int32_t* indfor, int32_t* laytrop) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    const double amd = 28.9660, amw = 18.0160, avogad = 6.02214199e+23, grav = 9.8066;
    for (int iplon = 0; iplon < ncol; ++iplon) {
        std::vector<double> pavel(nlay), tavel(nlay), pz(nlay + 1), coldry(nlay), wkl(7 * nlay, 0.0);
        pz[0] = plev[iplon];
        for (int l = 1; l <= nlay; ++l) {
            const size_t k = iplon + (size_t)ncol * (l - 1);
            pavel[l - 1] = play[k];
            tavel[l - 1] = tlay[k];
            pz[l] = plev[iplon + (size_t)ncol * l];
            double* w = &wkl[7 * (l - 1)];
            w[0] = h2ovmr[k]; w[1] = co2vmr[k]; w[2] = o3vmr[k]; w[3] = n2ovmr[k]; w[5] = ch4vmr[k]; w[6] = o2vmr[k];
            const double amm = (1.0 - w[0]) * amd + w[0] * amw;
            coldry[l - 1] = (pz[l - 1] - pz[l]) * 1.e3 * avogad / (1.e2 * grav * amm * (1.0 + w[0]));
        }
        for (int l = 1; l <= nlay; ++l)
            for (int m = 0; m < 7; ++m) wkl[7 * (l - 1) + m] = coldry[l - 1] * wkl[7 * (l - 1) + m];
        Coef c;
        setcoef(nlay, pavel.data(), tavel.data(), coldry.data(), wkl.data(), c);
        for (int l = 1; l <= nlay; ++l) {
            const size_t k = iplon + (size_t)ncol * (l - 1);
            jp[k] = c.jp[l]; jt[k] = c.jt[l]; jt1[k] = c.jt1[l];
            indself[k] = c.indself[l]; indfor[k] = c.indfor[l];
        }
        laytrop[iplon] = c.laytrop;
    }
    return ORC_OK;
}

// earth_sun (rrtmg_sw_rad.f90:844-868)
static double earth_sun(int idn) {
    const double gamma = 2.0 * T.pi * (idn - 1) / 365.0;
    return 1.000110 + .034221 * std::cos(gamma) + .001289 * std::sin(gamma) +
           .000719 * std::cos(2.0 * gamma) + .000077 * std::sin(2.0 * gamma);
}

// Solar variability settings of inatm_sw (rrtmg_sw_rad.f90:1245-1512).
static void solar_setup(const orc_rrtmg_sw_args* a, Solar& S, double* adjflux) {
    const double Iint = 1360.37, Fint = 0.996047, Sint = -0.511590;
    const double Foffset = 0.14959542, Soffset = 0.00066696;
    const double svar_f_avg = 0.1567652, svar_s_avg = 902.71260;
    const double solcycfrac_min = 0.0189, solcycfrac_max = 0.3750;
    const double fracdiff_min2max = 0.3561, fracdiff_max2min = 0.6439;
    const double rrsw_scon = 1.36822e+03;
    const int isolvar = a->isolvar;
    double solvar[NBND];
    for (int i = 0; i < NBND; ++i) {
        solvar[i] = 1.0;
        S.svar_f_bnd[i] = S.svar_s_bnd[i] = S.svar_i_bnd[i] = 1.0;
    }
    S.isolvar = isolvar;
    S.svar_f = S.svar_s = S.svar_i = 1.0;
    double indsolvar_scl[2] = {1.0, 1.0}, indsolvar_ndx[2] = {svar_f_avg, svar_s_avg};
    double solcycfr = 0.0;
    if (isolvar == 1 && a->indsolvar && a->solcycfrac) {
        const double scf = *a->solcycfrac;
        solcycfr = scf;
        const double* iv = a->indsolvar;
        if (iv[0] != 1.0 || iv[1] != 1.0) {
            if (scf >= 0.0 && scf < solcycfrac_min) {
                const double wgt = (scf + 1.0 - solcycfrac_max) / fracdiff_max2min;
                indsolvar_scl[0] = iv[0] + wgt * (1.0 - iv[0]);
                indsolvar_scl[1] = iv[1] + wgt * (1.0 - iv[1]);
            }
            if (scf >= solcycfrac_min && scf <= solcycfrac_max) {
                const double wgt = (scf - solcycfrac_min) / fracdiff_min2max;
                indsolvar_scl[0] = 1.0 + wgt * (iv[0] - 1.0);
                indsolvar_scl[1] = 1.0 + wgt * (iv[1] - 1.0);
            }
            if (scf > solcycfrac_max && scf <= 1.0) {
                const double wgt = (scf - solcycfrac_max) / fracdiff_max2min;
                indsolvar_scl[0] = iv[0] + wgt * (1.0 - iv[0]);
                indsolvar_scl[1] = iv[1] + wgt * (1.0 - iv[1]);
            }
        }
    }
    if (isolvar == 2 && a->indsolvar) {
        indsolvar_ndx[0] = a->indsolvar[0];
        indsolvar_ndx[1] = a->indsolvar[1];
    }
    double adjflx = a->adjes;
    if (a->dyofyr > 0) adjflx = earth_sun(a->dyofyr);
    // Mg / SB index tables of the mean solar cycle (rrtmg_sw_rad.f90:1172-1219)
    const double* kMgAvgCyc = T.mgavgcyc;
    const double* kSbAvgCyc = T.sbavgcyc;
    auto cycle_interp = [&](double& f0, double& s0) {
        const int nsolfrac = 134;
        if (solcycfr <= 0.0) { f0 = kMgAvgCyc[0]; s0 = kSbAvgCyc[0]; return; }
        if (solcycfr >= 1.0) { f0 = kMgAvgCyc[nsolfrac - 1]; s0 = kSbAvgCyc[nsolfrac - 1]; return; }
        const double intrvl_len = 1.0 / (nsolfrac - 2);
        const double intrvl_len_hf = 0.5 * intrvl_len;
        int sfid = 1;
        double fraclo = 0.0, frachi = intrvl_len_hf;
        if (solcycfr <= intrvl_len_hf) { sfid = 1; fraclo = 0.0; frachi = intrvl_len_hf; }
        if (solcycfr > intrvl_len_hf && solcycfr < 1.0 - intrvl_len_hf) {
            sfid = (int)std::floor((solcycfr - intrvl_len_hf) * (nsolfrac - 2)) + 2;
            fraclo = (sfid - 2) * intrvl_len + intrvl_len_hf;
            frachi = fraclo + intrvl_len;
        }
        if (solcycfr >= 1.0 - intrvl_len_hf) { sfid = (nsolfrac - 2) + 1; fraclo = 1.0 - intrvl_len_hf; frachi = 1.0; }
        const double intfrac = (solcycfr - fraclo) / (frachi - fraclo);
        f0 = kMgAvgCyc[sfid - 1] + intfrac * (kMgAvgCyc[sfid] - kMgAvgCyc[sfid - 1]);
        s0 = kSbAvgCyc[sfid - 1] + intfrac * (kSbAvgCyc[sfid] - kSbAvgCyc[sfid - 1]);
    };
    const double scon = a->scon;
    if (scon == 0.0) {
        if (isolvar == -1) {
            for (int i = 0; i < NBND; ++i) solvar[i] = a->bndsolvar ? a->bndsolvar[i] : 1.0;
        }
        if (isolvar == 0) { S.svar_f = S.svar_s = S.svar_i = 1.0; }
        if (isolvar == 1) {
            double f0, s0;
            cycle_interp(f0, s0);
            S.svar_f = indsolvar_scl[0] * (f0 - Foffset) / (svar_f_avg - Foffset);
            S.svar_s = indsolvar_scl[1] * (s0 - Soffset) / (svar_s_avg - Soffset);
            S.svar_i = 1.0;
        }
        if (isolvar == 2) {
            S.svar_f = (indsolvar_ndx[0] - Foffset) / (svar_f_avg - Foffset);
            S.svar_s = (indsolvar_ndx[1] - Soffset) / (svar_s_avg - Soffset);
            S.svar_i = 1.0;
        }
        if (isolvar == 3) {
            for (int i = 0; i < NBND; ++i) {
                solvar[i] = a->bndsolvar ? a->bndsolvar[i] : 1.0;
                S.svar_f_bnd[i] = S.svar_s_bnd[i] = S.svar_i_bnd[i] = solvar[i];
            }
        }
    }
    if (scon > 0.0) {
        if (isolvar == -1) {
            for (int i = 0; i < NBND; ++i)
                solvar[i] = a->bndsolvar ? a->bndsolvar[i] * scon / rrsw_scon : scon / rrsw_scon;
        }
        if (isolvar == 0) {
            const double svar_cprim = Fint + Sint + Iint;
            const double svar_r = scon / svar_cprim;
            S.svar_f = S.svar_s = S.svar_i = svar_r;
        }
        if (isolvar == 1) {
            double f0, s0;
            cycle_interp(f0, s0);
            S.svar_i = (scon - (indsolvar_scl[0] * Fint + indsolvar_scl[1] * Sint)) / Iint;
            S.svar_f = indsolvar_scl[0] * (f0 - Foffset) / (svar_f_avg - Foffset);
            S.svar_s = indsolvar_scl[1] * (s0 - Soffset) / (svar_s_avg - Soffset);
        }
        if (isolvar == 3) {
            const double svar_cprim = Fint + Sint + Iint;
            for (int i = 0; i < NBND; ++i) {
                solvar[i] = a->bndsolvar ? a->bndsolvar[i] * scon / svar_cprim : scon / svar_cprim;
                S.svar_f_bnd[i] = S.svar_s_bnd[i] = S.svar_i_bnd[i] = solvar[i];
            }
        }
    }
    for (int i = 0; i < NBND; ++i) adjflux[i] = isolvar < 0 ? adjflx * solvar[i] : adjflx;
}

// The column driver's solar settings (rrtmg_sw.1col.f90:1391-1436,1446-1660) are
// those of inatm_sw for isolvar 0..3: expose them for orc_column_mode.
int orc_solar_factors(int isolvar, double scon, double adjes, int dyofyr, const double* indsolvar,
                      const double* solcycfrac, const double* bndsolvar, double* svar, double* svar_bnd,
                      double* adjflux) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    orc_rrtmg_sw_args a{};
    a.isolvar = isolvar;
    a.scon = scon;
    a.adjes = adjes;
    a.dyofyr = dyofyr;
    a.indsolvar = indsolvar;
    a.solcycfrac = solcycfrac;
    a.bndsolvar = bndsolvar;
    Solar S;
    solar_setup(&a, S, adjflux);
    svar[0] = S.svar_f; svar[1] = S.svar_s; svar[2] = S.svar_i;
    for (int i = 0; i < NBND; ++i) {
        svar_bnd[i] = S.svar_f_bnd[i];
        svar_bnd[NBND + i] = S.svar_s_bnd[i];
        svar_bnd[2 * NBND + i] = S.svar_i_bnd[i];
    }
    return ORC_OK;
}

struct NomcicaClouds {
    const double *cldfr, *taucld, *ssacld, *asmcld, *fsfcld, *cicewp, *cliqwp, *reice, *reliq;
};

// rrtmg_sw (rrtmg_sw_rad.f90:561-841) and, with nm, its non-McICA twin
// (rrtmg_sw_rad.nomcica.f90:531-815).
static int rrtmg_sw_impl(const orc_rrtmg_sw_args* a, const NomcicaClouds* nm) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    const int ncol = a->ncol, nlay = a->nlay;
    if (ncol <= 0 || nlay <= 1) return ORC_ERR_ARGS;
    int icld = a->icld;
    if (icld < 0 || icld > 5) icld = 2;  // rad:589 clamps to 0..3; 4/5 accepted (1col semantics)
    int iaer = a->iaer;
    if (iaer != 0 && iaer != 6 && iaer != 10) iaer = 0;
    const int idelm = a->idelm;
    Solar S;
    double adjflux[NBND];
    solar_setup(a, S, adjflux);
    int err = ORC_OK;
    const int nthr = a->nthreads;
    (void)nthr;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthr > 0 ? nthr : omp_max_threads())
    for (int iplon = 0; iplon < ncol; ++iplon) {
        if (err != ORC_OK) continue;
        // ---- inatm_sw (rrtmg_sw_rad.f90:1527-1640)
        std::vector<double> pavel(nlay), tavel(nlay), pz(nlay + 1), pdp(nlay), coldry(nlay), wkl(7 * nlay, 0.0);
        const double amd = 28.9660, amw = 18.0160, avogad = 6.02214199e+23, grav = 9.8066;
        pz[0] = a->plev[iplon];
        for (int l = 1; l <= nlay; ++l) {
            const size_t k = iplon + (size_t)ncol * (l - 1);
            pavel[l - 1] = a->play[k];
            tavel[l - 1] = a->tlay[k];
            pz[l] = a->plev[iplon + (size_t)ncol * l];
            pdp[l - 1] = pz[l - 1] - pz[l];
            double* w = &wkl[7 * (l - 1)];
            w[0] = a->h2ovmr[k];
            w[1] = a->co2vmr[k];
            w[2] = a->o3vmr[k];
            w[3] = a->n2ovmr[k];
            w[5] = a->ch4vmr[k];
            w[6] = a->o2vmr[k];
            const double amm = (1.0 - w[0]) * amd + w[0] * amw;
            coldry[l - 1] = (pz[l - 1] - pz[l]) * 1.e3 * avogad / (1.e2 * grav * amm * (1.0 + w[0]));
        }
        for (int l = 1; l <= nlay; ++l)
            for (int m = 0; m < 7; ++m) wkl[7 * (l - 1) + m] = coldry[l - 1] * wkl[7 * (l - 1) + m];
        ColumnOptics O;
        const size_t nlg = (size_t)nlay * NGPT;
        O.cldfmc.assign(nlg, 0.0); O.taucmc.assign(nlg, 0.0); O.taormc.assign(nlg, 0.0);
        O.asycmc.assign(nlg, 0.0); O.omgcmc.assign(nlg, 1.0);
        O.taua.assign((size_t)nlay * NBND, 0.0); O.asya.assign((size_t)nlay * NBND, 0.0);
        O.omga.assign((size_t)nlay * NBND, 1.0);
        if (icld >= 1 && nm) {
            // clouds per layer and band, cldprop_sw, no partial cloud
            // (rrtmg_sw_rad.nomcica.f90:617-625, inatm :1588-1597)
            std::vector<double> cf(nlay), ci(nlay), cw(nlay), ri(nlay), rl(nlay), tc(14 * nlay), sc(14 * nlay),
                ac(14 * nlay), fc(14 * nlay);
            for (int l = 1; l <= nlay; ++l) {
                const size_t k = iplon + (size_t)ncol * (l - 1);
                cf[l - 1] = nm->cldfr[k];
                ci[l - 1] = nm->cicewp[k];
                cw[l - 1] = nm->cliqwp[k];
                ri[l - 1] = nm->reice[k];
                rl[l - 1] = nm->reliq[k];
                for (int b = 0; b < 14; ++b) {
                    const size_t kb = b + 14 * k;
                    tc[b + 14 * (l - 1)] = nm->taucld ? nm->taucld[kb] : 0.0;
                    sc[b + 14 * (l - 1)] = nm->ssacld ? nm->ssacld[kb] : 1.0;
                    ac[b + 14 * (l - 1)] = nm->asmcld ? nm->asmcld[kb] : 0.0;
                    fc[b + 14 * (l - 1)] = nm->fsfcld ? nm->fsfcld[kb] : 0.0;
                }
            }
            const double zepsec = 1.e-06, oneminus = 1.0 - zepsec;
            bool partial = false;
            for (int i = 0; i < nlay; ++i)
                if (cf[i] > zepsec && cf[i] < oneminus) partial = true;
            std::vector<double> tco((size_t)nlay * 14), tcl((size_t)nlay * 14), scl((size_t)nlay * 14),
                acl((size_t)nlay * 14);
            const int e = partial ? ORC_ERR_PARTIAL
                                  : cldprop(nlay, a->inflgsw, a->iceflgsw, a->liqflgsw, cf.data(), tc.data(), sc.data(),
                                            ac.data(), fc.data(), ci.data(), cw.data(), ri.data(), rl.data(), tco.data(),
                                            tcl.data(), scl.data(), acl.data());
            if (e != ORC_OK) {
#pragma omp critical
                err = e;
                continue;
            }
            spread_bands(nlay, cf.data(), tcl.data(), tco.data(), scl.data(), acl.data(), O);
        } else if (icld >= 1) {
            // cloud arrays (ig, lay) of the McICA inputs, then cldprmc_sw
            std::vector<double> cldf(nlg), tauc(nlg), ssac(nlg), asmc(nlg), fsfc(nlg), ciwp(nlg), clwp(nlg), taor(nlg);
            std::vector<double> rei(nlay), rel(nlay);
            for (int l = 1; l <= nlay; ++l) {
                for (int ig = 1; ig <= NGPT; ++ig) {
                    const size_t src = (ig - 1) + (size_t)NGPT * (iplon + (size_t)ncol * (l - 1));
                    const size_t dst = (ig - 1) + (size_t)NGPT * (l - 1);
                    cldf[dst] = a->cldfmcl[src];
                    tauc[dst] = a->taucmcl[src];
                    ssac[dst] = a->ssacmcl[src];
                    asmc[dst] = a->asmcmcl[src];
                    fsfc[dst] = a->fsfcmcl[src];
                    ciwp[dst] = a->ciwpmcl[src];
                    clwp[dst] = a->clwpmcl[src];
                }
                rei[l - 1] = a->reicmcl[iplon + (size_t)ncol * (l - 1)];
                rel[l - 1] = a->relqmcl[iplon + (size_t)ncol * (l - 1)];
            }
            const int e = cldprmc(nlay, a->inflgsw, a->iceflgsw, a->liqflgsw, cldf.data(), ciwp.data(), clwp.data(),
                                  rei.data(), rel.data(), taor.data(), tauc.data(), ssac.data(), asmc.data(), fsfc.data());
            if (e != ORC_OK) {
#pragma omp critical
                err = e;
                continue;
            }
            for (int l = 1; l <= nlay; ++l)
                for (int ig = 1; ig <= NGPT; ++ig) {
                    const size_t s = (ig - 1) + (size_t)NGPT * (l - 1);
                    const size_t d = (l - 1) + (size_t)nlay * (ig - 1);
                    O.cldfmc[d] = cldf[s];
                    O.taucmc[d] = tauc[s];
                    O.taormc[d] = taor[s];
                    O.asycmc[d] = asmc[s];
                    O.omgcmc[d] = ssac[s];
                }
        }
        if (iaer == 6) {
            for (int i = 1; i <= nlay; ++i)
                for (int ib = 1; ib <= NBND; ++ib) {
                    double ta = 0.0, as = 0.0, om = 0.0;
                    for (int ia = 1; ia <= 6; ++ia) {
                        const double ec = a->ecaer[iplon + (size_t)ncol * ((i - 1) + (size_t)nlay * (ia - 1))];
                        const double rt = T.rsrtaua[(ib - 1) + 14 * (ia - 1)], rp = T.rsrpiza[(ib - 1) + 14 * (ia - 1)],
                                     ra = T.rsrasya[(ib - 1) + 14 * (ia - 1)];
                        ta = ta + rt * ec;
                        om = om + rt * ec * rp;
                        as = as + rt * ec * rp * ra;
                    }
                    if (ta == 0.0) { ta = 0.0; as = 0.0; om = 1.0; }
                    else {
                        if (om != 0.0) as = as / om;
                        if (ta != 0.0) om = om / ta;
                    }
                    const size_t d = (i - 1) + (size_t)nlay * (ib - 1);
                    O.taua[d] = ta; O.asya[d] = as; O.omga[d] = om;
                }
        } else if (iaer == 10) {
            for (int i = 1; i <= nlay; ++i)
                for (int ib = 1; ib <= NBND; ++ib) {
                    const size_t s = iplon + (size_t)ncol * ((i - 1) + (size_t)nlay * (ib - 1));
                    const size_t d = (i - 1) + (size_t)nlay * (ib - 1);
                    O.taua[d] = a->tauaer[s];
                    O.asya[d] = a->asmaer[s];
                    O.omga[d] = a->ssaaer[s];
                }
        }
        Coef c;
        setcoef(nlay, pavel.data(), tavel.data(), coldry.data(), wkl.data(), c);
        if (c.laytrop < 1 || c.laytrop >= nlay) {
#pragma omp critical
            err = ORC_ERR_LAYTROP;
            continue;
        }
        double cossza = a->coszen[iplon];
        if (cossza < 1.e-10) cossza = 1.e-10;
        double albdir[NBND], albdif[NBND];
        for (int ib = 0; ib < 9; ++ib) { albdir[ib] = a->aldir[iplon]; albdif[ib] = a->aldif[iplon]; }
        albdir[13] = a->aldir[iplon];
        albdif[13] = a->aldif[iplon];
        for (int ib = 9; ib < 13; ++ib) { albdir[ib] = a->asdir[iplon]; albdif[ib] = a->asdif[iplon]; }
        Gas G;
        taumol(c, S, G);
        Fluxes F;
        spcvmc(nlay, 16, 29, idelm, 0, albdif, albdir, O, cossza, adjflux, S, G, F);
        std::vector<double> swnflx(nlay + 2), swnflxc(nlay + 2);
        for (int i = 1; i <= nlay + 1; ++i) {
            const size_t k = iplon + (size_t)ncol * (i - 1);
            a->swuflxc[k] = F.bbcu[i];
            a->swdflxc[k] = F.bbcd[i];
            a->swuflx[k] = F.bbfu[i];
            a->swdflx[k] = F.bbfd[i];
            if (a->uvdflx) a->uvdflx[k] = F.uvfd[i];
            if (a->nidflx) a->nidflx[k] = F.nifd[i];
            if (a->dirdflux) a->dirdflux[k] = F.bbfddir[i];
            if (a->difdflux) a->difdflux[k] = F.bbfd[i] - F.bbfddir[i];
            if (a->dirdnuv) a->dirdnuv[k] = F.uvfddir[i];
            if (a->difdnuv) a->difdnuv[k] = F.uvfd[i] - F.uvfddir[i];
            if (a->dirdnir) a->dirdnir[k] = F.nifddir[i];
            if (a->difdnir) a->difdnir[k] = F.nifd[i] - F.nifddir[i];
            swnflxc[i] = F.bbcd[i] - F.bbcu[i];
            swnflx[i] = F.bbfd[i] - F.bbfu[i];
            double* bo[5] = {a->bndfu, a->bndfd, a->bndfddir, a->bndcu, a->bndcd};
            for (int q = 0; q < 5; ++q)
                if (bo[q])
                    for (int ib = 0; ib < 14; ++ib)
                        bo[q][k + (size_t)ncol * (nlay + 1) * ib] = F.bnd[q][(size_t)ib * F.nlev2 + i];
        }
        for (int i = 1; i <= nlay; ++i) {
            const double zdpgcp = T.heatfac / pdp[i - 1];
            const size_t k = iplon + (size_t)ncol * (i - 1);
            a->swhrc[k] = (swnflxc[i + 1] - swnflxc[i]) * zdpgcp;
            a->swhr[k] = (swnflx[i + 1] - swnflx[i]) * zdpgcp;
        }
        a->swhrc[iplon + (size_t)ncol * (nlay - 1)] = 0.0;
        a->swhr[iplon + (size_t)ncol * (nlay - 1)] = 0.0;
    }
    return err;
}

int orc_rrtmg_sw(const orc_rrtmg_sw_args* a) { return rrtmg_sw_impl(a, nullptr); }

int orc_rrtmg_sw_nomcica(const orc_rrtmg_sw_args* a, const double* cldfr, const double* taucld, const double* ssacld,
                         const double* asmcld, const double* fsfcld, const double* cicewp, const double* cliqwp,
                         const double* reice, const double* reliq) {
    const NomcicaClouds nm{cldfr, taucld, ssacld, asmcld, fsfcld, cicewp, cliqwp, reice, reliq};
    if (a->icld != 0 && (!cldfr || !cicewp || !cliqwp || !reice || !reliq)) return ORC_ERR_ARGS;
    return rrtmg_sw_impl(a, &nm);
}

int orc_get_alpha(int ncol, int nlay, int icld, int idcor, double decorr_con, const double* dz,
                  const double* lat, int juldat, const double* cldfrac, double* alpha) {
    // mcica_subcol_gen_sw.f90:66-178 (literals are FP64 under -r8)
    const double am1 = 1.4315, am2 = 2.1219, am4 = -25.584, amr = 7.0, f_one = 1.0;
    std::vector<double> decorr_inv(ncol, f_one), decorr_len(ncol);
    if (icld == 4 || icld == 5) {
        if (idcor == 1) {
            double am3;
            if (juldat > 181) am3 = -4.0 * amr / 365.0 * (juldat - 272);
            else am3 = 4.0 * amr / 365.0 * (juldat - 91);
            for (int i = 0; i < ncol; ++i) {
                const double d = lat[i] - am3;
                const double decorr_lat = am1 + am2 * std::exp(-(d * d) / (am4 * am4));
                decorr_len[i] = decorr_lat * 1.e3;
            }
        } else {
            for (int i = 0; i < ncol; ++i) decorr_len[i] = decorr_con;
        }
        for (int i = 0; i < ncol; ++i)
            if (decorr_len[i] >= 0.0) decorr_inv[i] = f_one / decorr_len[i];
    }
    if (icld == 4 || icld == 5) {
        for (int i = 0; i < ncol; ++i) {
            alpha[i] = 0.0;
            for (int k = 2; k <= nlay; ++k) {
                const size_t kk = i + (size_t)ncol * (k - 1), km = i + (size_t)ncol * (k - 2);
                alpha[kk] = std::exp(-(0.5 * (dz[kk] + dz[km])) * decorr_inv[i]);
                if (icld == 5 && cldfrac[kk] == 0.0 && cldfrac[km] > 0.0) alpha[kk] = 0.0;
            }
        }
    }
    return ORC_OK;
}

int orc_mcica_subcol_sw(int ncol, int nlay, int icld, int permuteseed, int irng, const double* play,
                        const double* cldfrac, const double* ciwp, const double* clwp, const double* rei,
                        const double* rel, const double* tauc, const double* ssac, const double* asmc,
                        const double* fsfc, const double* alpha, double* cldfmcl, double* ciwpmcl,
                        double* clwpmcl, double* reicmcl, double* relqmcl, double* taucmcl,
                        double* ssacmcl, double* asmcmcl, double* fsfcmcl) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    if (icld == 0) return ORC_OK;
    if (icld < 0 || icld > 5) return ORC_ERR_ICLD;
    if (irng != 0) irng = 1;
    const double cldmin = 1.0e-20;
    const int ns = NGPT;
    for (size_t k = 0; k < (size_t)ncol * nlay; ++k) { reicmcl[k] = rei[k]; relqmcl[k] = rel[k]; }
    // CDF over (isub, col, lay)
    std::vector<double> cdf((size_t)ns * ncol * nlay), cdf2((size_t)ns * ncol * nlay);
    std::vector<double> cldf((size_t)ncol * nlay);
    for (size_t k = 0; k < (size_t)ncol * nlay; ++k) cldf[k] = cldfrac[k] < cldmin ? 0.0 : cldfrac[k];
    auto idx = [&](int is, int i, int l) { return (size_t)(is - 1) + (size_t)ns * ((size_t)i + (size_t)ncol * (l - 1)); };
    if (irng == 0) {
        // per-column KISS streams, seeded from pmid of the bottom four layers
        for (int i = 0; i < ncol; ++i) {
            const double p1 = play[i] * 1.e2, p2 = play[i + ncol] * 1.e2;
            if (p1 < p2) return ORC_ERR_KISS_SEED;
        }
        for (int i = 0; i < ncol; ++i) {
            Kiss k;
            k.s1 = (uint32_t)kiss_seed(play[i] * 1.e2);
            k.s2 = (uint32_t)kiss_seed(play[i + ncol] * 1.e2);
            k.s3 = (uint32_t)kiss_seed(play[i + 2 * ncol] * 1.e2);
            k.s4 = (uint32_t)kiss_seed(play[i + 3 * ncol] * 1.e2);
            for (int s = 0; s < permuteseed; ++s) k.next();
            if (icld == 1 || icld == 2) {
                for (int is = 1; is <= ns; ++is)
                    for (int l = 1; l <= nlay; ++l) cdf[idx(is, i, l)] = k.next();
            } else if (icld == 3) {
                for (int is = 1; is <= ns; ++is) {
                    const double r = k.next();
                    for (int l = 1; l <= nlay; ++l) cdf[idx(is, i, l)] = r;
                }
            } else {
                for (int is = 1; is <= ns; ++is)
                    for (int l = 1; l <= nlay; ++l) { cdf[idx(is, i, l)] = k.next(); cdf2[idx(is, i, l)] = k.next(); }
            }
        }
    } else {
        MT mt(permuteseed);
        if (icld == 1 || icld == 2) {
            for (int is = 1; is <= ns; ++is)
                for (int i = 0; i < ncol; ++i)
                    for (int l = 1; l <= nlay; ++l) cdf[idx(is, i, l)] = mt.next_real();
        } else if (icld == 3) {
            for (int is = 1; is <= ns; ++is)
                for (int i = 0; i < ncol; ++i) {
                    const double r = mt.next_real();
                    for (int l = 1; l <= nlay; ++l) cdf[idx(is, i, l)] = r;
                }
        } else {
            for (int is = 1; is <= ns; ++is)
                for (int i = 0; i < ncol; ++i)
                    for (int l = 1; l <= nlay; ++l) { cdf[idx(is, i, l)] = mt.next_real(); cdf2[idx(is, i, l)] = mt.next_real(); }
        }
    }
    if (icld == 2) {
        for (int l = 2; l <= nlay; ++l)
            for (int i = 0; i < ncol; ++i)
                for (int is = 1; is <= ns; ++is) {
                    const double cf = cldf[i + (size_t)ncol * (l - 2)];
                    if (cdf[idx(is, i, l - 1)] > 1.0 - cf) cdf[idx(is, i, l)] = cdf[idx(is, i, l - 1)];
                    else cdf[idx(is, i, l)] = cdf[idx(is, i, l)] * (1.0 - cf);
                }
    } else if (icld == 4 || icld == 5) {
        for (int l = 2; l <= nlay; ++l)
            for (int i = 0; i < ncol; ++i)
                for (int is = 1; is <= ns; ++is)
                    if (cdf2[idx(is, i, l)] < alpha[i + (size_t)ncol * (l - 1)]) cdf[idx(is, i, l)] = cdf[idx(is, i, l - 1)];
    }
    const int ngbm = T.ngb[0] - 1;
    for (int l = 1; l <= nlay; ++l)
        for (int i = 0; i < ncol; ++i)
            for (int is = 1; is <= ns; ++is) {
                const size_t k = idx(is, i, l);
                const size_t cl = i + (size_t)ncol * (l - 1);
                if (cdf[k] >= 1.0 - cldf[cl]) {
                    const int n = T.ngb[is - 1] - ngbm;
                    const size_t b = (size_t)(n - 1) + 14 * cl;
                    cldfmcl[k] = 1.0;
                    clwpmcl[k] = clwp[cl];
                    ciwpmcl[k] = ciwp[cl];
                    taucmcl[k] = tauc[b];
                    ssacmcl[k] = ssac[b];
                    asmcmcl[k] = asmc[b];
                    fsfcmcl[k] = fsfc[b];
                } else {
                    cldfmcl[k] = 0.0;
                    clwpmcl[k] = 0.0;
                    ciwpmcl[k] = 0.0;
                    taucmcl[k] = 0.0;
                    ssacmcl[k] = 1.0;
                    asmcmcl[k] = 0.0;
                    fsfcmcl[k] = 0.0;
                }
            }
    return ORC_OK;
}

void orc_mt_real(int seed, int n, double* out) {
    MT mt(seed);
    for (int i = 0; i < n; ++i) out[i] = mt.next_real();
}

void orc_kiss_real(int32_t s1, int32_t s2, int32_t s3, int32_t s4, int n, double* out) {
    Kiss k{(uint32_t)s1, (uint32_t)s2, (uint32_t)s3, (uint32_t)s4};
    for (int i = 0; i < n; ++i) out[i] = k.next();
}

// Column driver (rrtmg_sw.1col.f90:552-948), one column, nmca McICA samples
int orc_column_mode(const orc_column_case* cc) {
    if (!T.ok) return ORC_ERR_NOT_INITIALIZED;
    const int nlay = cc->nlay;
    Solar S;
    S.isolvar = cc->isolvar;
    S.svar_f = cc->svar_f; S.svar_s = cc->svar_s; S.svar_i = cc->svar_i;
    for (int i = 0; i < NBND; ++i) {
        S.svar_f_bnd[i] = cc->svar_f_bnd[i]; S.svar_s_bnd[i] = cc->svar_s_bnd[i]; S.svar_i_bnd[i] = cc->svar_i_bnd[i];
    }
    if (cc->imca == 0 && cc->icld >= 1)  // rrtmg_sw.1col.f90:612-617
        for (int i = 0; i < nlay; ++i)
            if (cc->cldfrac[i] != 0.0 && cc->cldfrac[i] != 1.0) return ORC_ERR_PARTIAL;
    const int nmca = cc->imca == 1 ? cc->nmca : 1;
    std::vector<double> usum(nlay + 1, 0.0), dsum(nlay + 1, 0.0), dirsum(nlay + 1, 0.0), difsum(nlay + 1, 0.0),
        fnsum(nlay + 1, 0.0), hsum(nlay + 1, 0.0);
    std::vector<double> pdp(nlay);
    for (int l = 1; l <= nlay; ++l) pdp[l - 1] = cc->pz[l - 1] - cc->pz[l];
    Coef c;
    setcoef(nlay, cc->pavel, cc->tavel, cc->coldry, cc->wkl, c);
    if (c.laytrop < 1 || c.laytrop >= nlay) return ORC_ERR_LAYTROP;
    Gas G;
    taumol(c, S, G);
    double cossza = cc->zenith;
    if (cossza == 0.0) cossza = 1.e-10;
    const size_t nlg = (size_t)nlay * NGPT;
    for (int ims = 1; ims <= nmca; ++ims) {
        ColumnOptics O;
        O.cldfmc.assign(nlg, 0.0); O.taucmc.assign(nlg, 0.0); O.taormc.assign(nlg, 0.0);
        O.asycmc.assign(nlg, 0.0); O.omgcmc.assign(nlg, 1.0);
        O.taua.assign((size_t)nlay * NBND, 0.0); O.asya.assign((size_t)nlay * NBND, 0.0);
        O.omga.assign((size_t)nlay * NBND, 1.0);
        if (cc->imca == 1 && cc->icld >= 1) {
            std::vector<double> alpha(nlay, 0.0);
            if (cc->icld == 4 || cc->icld == 5)
                orc_get_alpha(1, nlay, cc->icld, cc->idcor, cc->decorr_con, cc->dz, &cc->lat, cc->juldat,
                              cc->cldfrac, alpha.data());
            std::vector<double> cldf(nlg), ciwp(nlg), clwp(nlg), tauc(nlg), ssac(nlg), asmc(nlg), fsfc(nlg), taor(nlg);
            std::vector<double> rei(nlay), rel(nlay);
            const int permuteseed = (ims + 1) * NGPT;  // mcica_subcol_gen_sw.1col.f90:255
            int e = orc_mcica_subcol_sw(1, nlay, cc->icld, permuteseed, 1, cc->pavel, cc->cldfrac, cc->ciwp, cc->clwp,
                                        cc->rei, cc->rel, cc->tauc, cc->ssac, cc->asmc, cc->fsfc, alpha.data(),
                                        cldf.data(), ciwp.data(), clwp.data(), rei.data(), rel.data(), tauc.data(),
                                        ssac.data(), asmc.data(), fsfc.data());
            if (e) return e;
            e = cldprmc(nlay, cc->inflag, cc->iceflag, cc->liqflag, cldf.data(), ciwp.data(), clwp.data(), rei.data(),
                        rel.data(), taor.data(), tauc.data(), ssac.data(), asmc.data(), fsfc.data());
            if (e) return e;
            for (int l = 1; l <= nlay; ++l)
                for (int ig = 1; ig <= NGPT; ++ig) {
                    const size_t s = (ig - 1) + (size_t)NGPT * (l - 1);
                    const size_t d = (l - 1) + (size_t)nlay * (ig - 1);
                    O.cldfmc[d] = cldf[s]; O.taucmc[d] = tauc[s]; O.taormc[d] = taor[s];
                    O.asycmc[d] = asmc[s]; O.omgcmc[d] = ssac[s];
                }
        }
        if (cc->imca == 0 && cc->icld >= 1) {
            // cldprop_sw, then the cloudy layers' band optics (1col:618-620, 669-679)
            std::vector<double> tco((size_t)nlay * 14), tcl((size_t)nlay * 14), scl((size_t)nlay * 14),
                acl((size_t)nlay * 14);
            std::vector<double> z14(14 * nlay, 0.0), o14(14 * nlay, 1.0);
            const int e = cldprop(nlay, cc->inflag, cc->iceflag, cc->liqflag, cc->cldfrac, cc->tauc ? cc->tauc : z14.data(),
                                  cc->ssac ? cc->ssac : o14.data(), cc->asmc ? cc->asmc : z14.data(),
                                  cc->fsfc ? cc->fsfc : z14.data(), cc->ciwp, cc->clwp, cc->rei, cc->rel, tco.data(),
                                  tcl.data(), scl.data(), acl.data());
            if (e) return e;
            for (int i = 1; i <= nlay; ++i)
                if (!(cc->cldfrac[i - 1] >= 1.e-06))
                    for (int ib = 1; ib <= NBND; ++ib) {
                        const size_t s = (i - 1) + (size_t)nlay * (ib - 1);
                        tcl[s] = 0.0; tco[s] = 0.0; acl[s] = 0.0; scl[s] = 1.0;
                    }
            spread_bands(nlay, cc->cldfrac, tcl.data(), tco.data(), scl.data(), acl.data(), O);
        }
        if (cc->iaer == 10) {
            for (int i = 1; i <= nlay; ++i)
                for (int ib = 1; ib <= NBND; ++ib) {
                    const size_t s = (i - 1) + (size_t)nlay * (ib - 1);
                    O.taua[s] = cc->tauaer[s]; O.asya[s] = cc->asmaer[s]; O.omga[s] = cc->ssaaer[s];
                }
        }
        Fluxes F;
        spcvmc(nlay, cc->istart, cc->iend, cc->idelm, cc->istart == cc->iend ? cc->istart : 0, cc->albedo,
               cc->albedo, O, cossza, cc->adjflux, S, G, F);
        std::vector<double> tu(nlay + 1), td(nlay + 1), dd(nlay + 1), fn(nlay + 1), ht(nlay + 1);
        for (int i = 1; i <= nlay + 1; ++i) {
            tu[i - 1] = F.bbfu[i];
            td[i - 1] = F.bbfd[i];
            dd[i - 1] = F.bbfddir[i];
            fn[i - 1] = td[i - 1] - tu[i - 1];
        }
        for (int i = 1; i <= nlay; ++i) ht[i - 1] = (fn[i] - fn[i - 1]) * (T.heatfac / pdp[i - 1]);
        ht[nlay] = 0.0;
        for (int i = nlay; i >= 0; --i) {
            usum[i] = usum[i] + tu[i];
            dsum[i] = dsum[i] + td[i];
            dirsum[i] = dirsum[i] + dd[i];
            difsum[i] = difsum[i] + (td[i] - dd[i]);
            fnsum[i] = fnsum[i] + fn[i];
            hsum[i] = hsum[i] + ht[i];
        }
    }
    for (int i = 0; i <= nlay; ++i) {
        cc->uflx[i] = usum[i] / nmca;
        cc->dflx[i] = dsum[i] / nmca;
        cc->dirdflx[i] = dirsum[i] / nmca;
        cc->difdflx[i] = difsum[i] / nmca;
        cc->fnet[i] = fnsum[i] / nmca;
        cc->htr[i] = hsum[i] / nmca;
    }
    return ORC_OK;
}

}  // extern "C"
