// solve.cuh -- the fused per-column shortwave solve, templated on the
// arithmetic type of the bulk work (double: plain FP64 form; float: FP32
// form).  One CTA handles two columns; each of its 224 threads owns one
// (column, g-point) pair and walks the layers:
//
//   prep   (all threads, per column x layer): inatm_sw + setcoef_sw into
//          shared memory (rrtmg_sw_rad.f90:1527-1586, rrtmg_sw_setcoef.f90:49-305)
//   pass 1 (bottom -> top): gas optics (taumol16..29), cloud optics
//          (cldprmc_sw, McICA subcolumn mask generated in place when fused),
//          delta scaling, reftra_sw for clear and cloudy layers, direct beam,
//          and the upward adding recurrence of vrtqdr_sw; per level the
//          layer R/T and the upward albedos go to a per-CTA scratch slot
//   pass 2 (top -> bottom): downward adding recurrence, level fluxes,
//          incident-flux weighting and the g-point sums (rrtmg_sw_spcvmc.f90:
//          607-655) as a fixed-order shared-memory reduction
//   finish: net fluxes and heating rates (rrtmg_sw_rad.f90:805-836)
//
// Layer R/T never leave the CTA's scratch slot (L2-resident working set);
// the McICA subcolumn arrays of the fused path are never materialised.
#pragma once

#include "common.cuh"

namespace rrsw {

// --------------------------------------------------------------- params
struct SolveParams {
    int ncol, nlay, icld, iaer, idelm, isolvar, inflag, iceflag, liqflag;
    int fused;       // 1: McICA masks generated in the kernel (KISS)
    int extra;       // 1: also the 8 direct/diffuse/UV/NIR outputs
    int permuteseed;
    int npairs;
    double svar_f, svar_s, svar_i;
    double svar_f_bnd[NBND], svar_s_bnd[NBND], svar_i_bnd[NBND], adjflux[NBND];
    const double *play, *plev, *tlay, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *o2vmr;
    const double *asdir, *asdif, *aldir, *aldif, *coszen;
    const double *cldfmcl, *taucmcl, *ssacmcl, *asmcmcl, *fsfcmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl;
    const double *tauaer, *ssaaer, *asmaer, *ecaer;
    const double *cldfrac, *ciwp, *clwp, *rei, *rel, *tauc, *ssac, *asmc, *fsfc, *alpha;
    double *swuflx, *swdflx, *swhr, *swuflxc, *swdflxc, *swhrc;
    double *xout[8];  // dirdflux, difdflux, uvdflx, nidflx, dirdnuv, difdnuv, dirdnir, difdnir
    void *scratch;
    size_t slot_elems;
    int *err;
};

// shared-memory fields of the per-column coefficients
enum { F_FAC00, F_FAC01, F_FAC10, F_FAC11, F_H2O, F_CO2, F_O3, F_CH4, F_O2, F_MOL,
       F_SELFFAC, F_SELFFRAC, F_FORFAC, F_FORFRAC, F_PDP, NFR };

template <typename R>
struct Coef {
    const R* r;      // [NFR][L]
    const int* pk;   // [L] packed jp | jt<<8 | jt1<<12 | indself<<16 | indfor<<24 | below100hPa<<30
    int L, laytrop;
    __device__ R f(int fld, int lay) const { return r[fld * L + lay - 1]; }
    __device__ int jp(int lay) const { return pk[lay - 1] & 0xff; }
    __device__ int jt(int lay) const { return (pk[lay - 1] >> 8) & 0xf; }
    __device__ int jt1(int lay) const { return (pk[lay - 1] >> 12) & 0xf; }
    __device__ int indself(int lay) const { return (pk[lay - 1] >> 16) & 0xff; }
    __device__ int indfor(int lay) const { return (pk[lay - 1] >> 24) & 0xf; }   // bit 30: layer below 100 hPa
};

// ----------------------------------------------------- arithmetic helpers
// The FP64 form is compiled without FMA contraction, so a*b+c rounds twice
// as the reference's expressions do.  The FP32 form may contract.
template <typename R> __device__ inline R rcp(R x) { return R(1) / x; }

// exp(-x) through the lookup table, or the quadratic below od_lo
// (rrtmg_sw_reftra.f90:203-209; table built at rrtmg_sw_init.f90:115-123)
template <typename R>
__device__ inline R tbl_exp(R ze1, const R* __restrict__ tab) {
    const R od_lo = R(0.06);
    if (ze1 <= od_lo) return R(1) - ze1 + R(0.5) * ze1 * ze1;
    const R tblind = ze1 / (R(cT.bpade) + ze1);
    const int itind = (int)(R(10000) * tblind + R(0.5));
    return __ldg(tab + cT.exp_tbl + itind);
}

// --------------------------------------------------------------- taumol
template <typename R>
struct Spec {
    R speccomb, fs, f000, f001, f010, f011, f100, f101, f110, f111;
    int js;
};

// species-ratio interpolation factors (e.g. rrtmg_sw_taumol.f90:309-324)
template <typename R>
__device__ inline Spec<R> spec(R cola, R colb_scaled, R mult, const Coef<R>& c, int lay) {
    Spec<R> s;
    s.speccomb = cola + colb_scaled;
    R specparm = cola / s.speccomb;
    if (specparm >= R(cT.oneminus)) specparm = R(cT.oneminus);
    const R specmult = mult * (specparm);
    const int ij = (int)specmult;
    s.js = 1 + ij;
    s.fs = specmult - (R)ij;
    const R f00 = c.f(F_FAC00, lay), f01 = c.f(F_FAC01, lay), f10 = c.f(F_FAC10, lay), f11 = c.f(F_FAC11, lay);
    s.f000 = (R(1) - s.fs) * f00;
    s.f010 = (R(1) - s.fs) * f10;
    s.f100 = s.fs * f00;
    s.f110 = s.fs * f10;
    s.f001 = (R(1) - s.fs) * f01;
    s.f011 = (R(1) - s.fs) * f11;
    s.f101 = s.fs * f01;
    s.f111 = s.fs * f11;
    return s;
}

// k(ind, ig) of a transposed table: [(ind-1)*ng + ig-1]
template <typename R>
__device__ inline R K(const R* __restrict__ tab, int off, int ng, int ind, int ig) {
    return __ldg(tab + off + (ind - 1) * ng + (ig - 1));
}

template <typename R>
__device__ inline R k8(const Spec<R>& s, const R* __restrict__ tab, int off, int ng, int ind0, int ind1, int ig, int d1) {
    return (s.f000 * K(tab, off, ng, ind0, ig) + s.f100 * K(tab, off, ng, ind0 + 1, ig) +
            s.f010 * K(tab, off, ng, ind0 + d1, ig) + s.f110 * K(tab, off, ng, ind0 + d1 + 1, ig) +
            s.f001 * K(tab, off, ng, ind1, ig) + s.f101 * K(tab, off, ng, ind1 + 1, ig) +
            s.f011 * K(tab, off, ng, ind1 + d1, ig) + s.f111 * K(tab, off, ng, ind1 + d1 + 1, ig));
}

template <typename R>
__device__ inline R k4(const Coef<R>& c, int lay, const R* __restrict__ tab, int off, int ng, int ind0, int ind1, int ig) {
    return c.f(F_FAC00, lay) * K(tab, off, ng, ind0, ig) + c.f(F_FAC10, lay) * K(tab, off, ng, ind0 + 1, ig) +
           c.f(F_FAC01, lay) * K(tab, off, ng, ind1, ig) + c.f(F_FAC11, lay) * K(tab, off, ng, ind1 + 1, ig);
}

template <typename R>
__device__ inline R selfterm(const Coef<R>& c, int lay, const BandOff& B, const R* __restrict__ tab, int ig) {
    const int inds = c.indself(lay);
    const R a = K(tab, B.selfref, B.ng, inds, ig), b = K(tab, B.selfref, B.ng, inds + 1, ig);
    return c.f(F_SELFFAC, lay) * (a + c.f(F_SELFFRAC, lay) * (b - a));
}
template <typename R>
__device__ inline R forpart(const Coef<R>& c, int lay, const BandOff& B, const R* __restrict__ tab, int ig) {
    const int indf = c.indfor(lay);
    const R a = K(tab, B.forref, B.ng, indf, ig), b = K(tab, B.forref, B.ng, indf + 1, ig);
    return (a + c.f(F_FORFRAC, lay) * (b - a));
}
template <typename R>
__device__ inline R forterm(const Coef<R>& c, int lay, const BandOff& B, const R* __restrict__ tab, int ig) {
    return c.f(F_FORFAC, lay) * forpart(c, lay, B, tab, ig);
}
template <typename R>
__device__ inline R selffor(const Coef<R>& c, int lay, const BandOff& B, const R* __restrict__ tab, int ig) {
    return selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig);
}
template <typename R>
__device__ inline R V(const R* __restrict__ tab, int off, int i) { return __ldg(tab + off + i); }

// Lower/upper table base indices (taumol.f90:326-327, 357-358)
__device__ inline int ind_lo(int jp, int jt, int nsp, int js) { return ((jp - 1) * 5 + (jt - 1)) * nsp + js; }
__device__ inline int ind_lo1(int jp, int jt1, int nsp, int js) { return (jp * 5 + (jt1 - 1)) * nsp + js; }
__device__ inline int ind_up(int jp, int jt, int nsp, int js) { return ((jp - 13) * 5 + (jt - 1)) * nsp + js; }
__device__ inline int ind_up1(int jp, int jt1, int nsp, int js) { return ((jp - 12) * 5 + (jt1 - 1)) * nsp + js; }

// Gas (taug) and Rayleigh (taur) optical depth of g-point `ig` (1-based in
// its band) at layer `lay`: one g-point of taumol16..taumol29
// (rrtmg_sw_taumol.f90:275-1785), same expressions and association order.
template <typename R>
__device__ inline void taumol_g(int ib, int ig, int lay, const Coef<R>& c, const R* __restrict__ tab, R& taug, R& taur) {
    const BandOff& B = cT.b[ib];
    const bool low = lay <= c.laytrop;
    const R colh2o = c.f(F_H2O, lay), colco2 = c.f(F_CO2, lay), colo3 = c.f(F_O3, lay);
    const R colch4 = c.f(F_CH4, lay), colo2 = c.f(F_O2, lay), colmol = c.f(F_MOL, lay);
    const int jp = c.jp(lay), jt = c.jt(lay), jt1 = c.jt1(lay);
    switch (ib + 16) {
    case 16:
        if (low) {
            const Spec<R> s = spec(colh2o, R(252.131) * colch4, R(8), c, lay);
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colh2o * selffor(c, lay, B, tab, ig);
        } else {
            taug = colch4 * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    case 17:
        if (low) {
            const Spec<R> s = spec(colh2o, R(0.364641) * colco2, R(8), c, lay);
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colh2o * selffor(c, lay, B, tab, ig);
        } else {
            const Spec<R> s = spec(colh2o, R(0.364641) * colco2, R(4), c, lay);
            taug = s.speccomb * k8(s, tab, B.absb, B.ng, ind_up(jp, jt, 5, s.js), ind_up1(jp, jt1, 5, s.js), ig, 5) +
                   colh2o * c.f(F_FORFAC, lay) * forpart(c, lay, B, tab, ig);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    case 18:
    case 19: {
        const R colb = ib + 16 == 18 ? colch4 : colco2;
        if (low) {
            const Spec<R> s = spec(colh2o, R(ib + 16 == 18 ? 38.9589 : 5.49281) * colb, R(8), c, lay);
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colh2o * selffor(c, lay, B, tab, ig);
        } else {
            taug = colb * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    }
    case 20:
        if (low) {
            taug = colh2o * ((k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig)) +
                             selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig)) +
                   colch4 * V(tab, B.absch4, ig - 1);
        } else {
            taug = colh2o * (k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) +
                             forterm(c, lay, B, tab, ig)) +
                   colch4 * V(tab, B.absch4, ig - 1);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    case 21:
        if (low) {
            const Spec<R> s = spec(colh2o, R(0.0045321) * colco2, R(8), c, lay);
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colh2o * selffor(c, lay, B, tab, ig);
        } else {
            const Spec<R> s = spec(colh2o, R(0.0045321) * colco2, R(4), c, lay);
            taug = s.speccomb * k8(s, tab, B.absb, B.ng, ind_up(jp, jt, 5, s.js), ind_up1(jp, jt1, 5, s.js), ig, 5) +
                   colh2o * c.f(F_FORFAC, lay) * forpart(c, lay, B, tab, ig);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    case 22: {
        const R o2adj = R(1.6);
        const R o2cont = R(4.35e-4) * colo2 / (R(350.0) * R(2.0));
        if (low) {
            const Spec<R> s = spec(colh2o, o2adj * R(0.022708) * colo2, R(8), c, lay);
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colh2o * selffor(c, lay, B, tab, ig) + o2cont;
        } else {
            taug = colo2 * o2adj * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) + o2cont;
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    }
    case 23:
        if (low) {
            taug = colh2o * (R(1.029) * k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig) +
                             selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig));
        } else {
            taug = R(0);
        }
        taur = colmol * V(tab, B.rayl, ig - 1);
        break;
    case 24:
        if (low) {
            const Spec<R> s = spec(colh2o, R(0.124692) * colo2, R(8), c, lay);
            const R ra = V(tab, B.rayla, (s.js - 1) * B.ng + ig - 1), rb = V(tab, B.rayla, s.js * B.ng + ig - 1);
            taur = colmol * (ra + s.fs * (rb - ra));
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colo3 * V(tab, B.abso3a, ig - 1) + colh2o * selffor(c, lay, B, tab, ig);
        } else {
            taur = colmol * V(tab, B.raylb, ig - 1);
            taug = colo2 * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) +
                   colo3 * V(tab, B.abso3b, ig - 1);
        }
        break;
    case 25:
        taur = colmol * V(tab, B.rayl, ig - 1);
        if (low) {
            taug = colh2o * k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig) +
                   colo3 * V(tab, B.abso3a, ig - 1);
        } else {
            taug = colo3 * V(tab, B.abso3b, ig - 1);
        }
        break;
    case 26:
        taug = R(0);
        taur = colmol * V(tab, B.rayl, ig - 1);
        break;
    case 27:
        taur = colmol * V(tab, B.rayl, ig - 1);
        if (low) taug = colo3 * k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig);
        else taug = colo3 * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig);
        break;
    case 28:
        if (low) {
            const Spec<R> s = spec(colo3, R(6.67029e-07) * colo2, R(8), c, lay);
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9);
        } else {
            const Spec<R> s = spec(colo3, R(6.67029e-07) * colo2, R(4), c, lay);
            taug = s.speccomb * k8(s, tab, B.absb, B.ng, ind_up(jp, jt, 5, s.js), ind_up1(jp, jt1, 5, s.js), ig, 5);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    default:  // 29
        if (low) {
            taug = colh2o * ((k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig)) +
                             selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig)) +
                   colco2 * V(tab, B.absco2, ig - 1);
        } else {
            taug = colco2 * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) +
                   colh2o * V(tab, B.absh2o, ig - 1);
        }
        taur = colmol * V(tab, B.rayl, 0);
        break;
    }
}

// Layer at which each band takes its solar source (the laysolfr logic of
// taumol16..29): bands whose source sits below laytrop scan the lower loop,
// the others the upper loop; a later match overrides an earlier one.
template <typename R>
__device__ inline int solar_layer(int ib, const Coef<R>& c) {
    const int band = ib + 16;
    // layreffr per band (taumol.f90:306,417,548,666,782,883,1029,1148,1238,1357,-,1503,1595,1716)
    const int lref[14] = {18, 30, 6, 3, 3, 8, 2, 6, 1, 2, 0, 32, 42, 49};
    const int layreffr = lref[ib];
    const int L = c.L, lt = c.laytrop;
    int src = -1;
    if (band == 16 || band == 17 || band == 27 || band == 28 || band == 29) {
        int laysolfr = L;
        for (int lay = lt + 1; lay <= L; ++lay) {
            if (c.jp(lay - 1) < layreffr && c.jp(lay) >= layreffr) laysolfr = lay;
            if (lay == laysolfr) src = lay;
        }
    } else if (band == 26) {
        src = lt;
    } else {
        int laysolfr = lt;
        for (int lay = 1; lay <= lt; ++lay) {
            const int jpn = lay + 1 <= L ? c.jp(lay + 1) : -1000;
            if (c.jp(lay) < layreffr && jpn >= layreffr) laysolfr = min(lay + 1, lt);
            if (lay == laysolfr) src = lay;
        }
    }
    return src;
}

// Solar source of g-point ig at its reference layer: sfluxzen (isolvar<0)
// or ssi (isolvar>=0), e.g. taumol.f90:364-378 and 495-517.
template <typename R>
__device__ inline double solar_source(int ib, int ig, const Coef<R>& c, const SolveParams& P, const R* __restrict__ tab) {
    const BandOff& B = cT.b[ib];
    const int band = ib + 16;
    const int lay = solar_layer(ib, c);
    bool interp = false;
    double fs = 0.0;
    int js = 1;
    if (lay >= 1) {
        const R colh2o = c.f(F_H2O, lay), colco2 = c.f(F_CO2, lay), colo3 = c.f(F_O3, lay);
        const R colch4 = c.f(F_CH4, lay), colo2 = c.f(F_O2, lay);
        Spec<R> s;
        switch (band) {
        case 17: s = spec(colh2o, R(0.364641) * colco2, R(4), c, lay); interp = true; break;
        case 18: s = spec(colh2o, R(38.9589) * colch4, R(8), c, lay); interp = true; break;
        case 19: s = spec(colh2o, R(5.49281) * colco2, R(8), c, lay); interp = true; break;
        case 21: s = spec(colh2o, R(0.0045321) * colco2, R(8), c, lay); interp = true; break;
        case 22: s = spec(colh2o, R(1.6) * R(0.022708) * colo2, R(8), c, lay); interp = true; break;
        case 24: s = spec(colh2o, R(0.124692) * colo2, R(8), c, lay); interp = true; break;
        case 28: s = spec(colo3, R(6.67029e-07) * colo2, R(4), c, lay); interp = true; break;
        default: break;
        }
        if (interp) { js = s.js; fs = (double)s.fs; }
    }
    auto src = [&](int off) -> double {
        if (!interp) return (double)V(tab, off, ig - 1);
        const double a = (double)V(tab, off, (js - 1) * B.ng + ig - 1), b = (double)V(tab, off, js * B.ng + ig - 1);
        return a + fs * (b - a);
    };
    if (P.isolvar < 0) {
        const double sf = src(B.sfluxref);
        return band == 27 ? (50.15 / 48.37) * sf : sf;
    }
    const double fb = src(B.facbrght), sd = src(B.snsptdrk), ir = src(B.irradnce);
    if (P.isolvar == 3) return P.svar_f_bnd[ib] * fb + P.svar_s_bnd[ib] * sd + P.svar_i_bnd[ib] * ir;
    return P.svar_f * fb + P.svar_s * sd + P.svar_i * ir;
}

// --------------------------------------------------------------- cldprmc
// One (g-point, layer) of cldprmc_sw (rrtmg_sw_cldprmc.f90:53-349) for
// inflag = 0 or 2.  On input tauc/ssac/asmc are the subcolumn's values;
// on output the delta-scaled cloud properties and taor the unscaled depth.
template <typename R>
__device__ inline void cldprmc_g(int ib, int inflag, int iceflag, int liqflag, R cldf, R ciwp,
                                 R clwp, R rei, R rel, R fsfc, R& tauc,
                                 R& ssac, R& asmc, R& taor, const R* __restrict__ tab,
                                 int* err) {
    typedef R double_;
    const R eps = R(1.e-06), cldmin = R(1.e-20);
    taor = tauc;
    const double_ cwp = ciwp + clwp;
    if (!(cldf >= cldmin && (cwp >= cldmin || tauc >= cldmin))) return;
    if (inflag == 0) {
        const double_ taucldorig_a = tauc;
        const double_ ffp = fsfc;
        const double_ ffp1 = 1.0 - ffp;
        const double_ ffpssa = 1.0 - ffp * ssac;
        const double_ ssacloud_a = ffp1 * ssac / ffpssa;
        const double_ taucloud_a = ffpssa * taucldorig_a;
        taor = taucldorig_a;
        ssac = ssacloud_a;
        tauc = taucloud_a;
        asmc = (asmc - ffp) / (ffp1);
        return;
    }
    if (inflag != 2) { set_error(err, E_INFLAG1); return; }
    double_ extcoice = 0, ssacoice = 0, gice = 0, forwice = 0, extcoliq = 0, ssacoliq = 0, gliq = 0, forwliq = 0;
    const int jb = ib + 1;  // band column of the Fortran (index, 16:29) LUTs, 1-based
    auto lut = [&](int off, int n, int index) { return __ldg(tab + off + (jb - 1) * n + index - 1); };
    if (ciwp == 0.0) {
    } else if (iceflag == 1) {
        if (rei < 13.0 || rei > 130.0) { set_error(err, E_ICERAD); return; }
        const double_ w2 = __ldg(tab + cT.wavenum2 + ib);
        int icx = 0;
        if (w2 > 1.43e04) icx = 1;
        else if (w2 > 7.7e03) icx = 2;
        else if (w2 > 5.3e03) icx = 3;
        else if (w2 > 4.0e03) icx = 4;
        else if (w2 >= 2.5e03) icx = 5;
        extcoice = (__ldg(tab + cT.abari + icx - 1) + __ldg(tab + cT.bbari + icx - 1) / rei);
        ssacoice = 1.0 - __ldg(tab + cT.cbari + icx - 1) - __ldg(tab + cT.dbari + icx - 1) * rei;
        gice = __ldg(tab + cT.ebari + icx - 1) + __ldg(tab + cT.fbari + icx - 1) * rei;
        if (gice >= 1.0) gice = 1.0 - eps;
        forwice = gice * gice;
        if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) { set_error(err, E_ICEPROP); return; }
    } else if (iceflag == 2) {
        if (rei < 5.0 || rei > 131.0) { set_error(err, E_ICERAD); return; }
        const double_ factor = (rei - 2.0) / 3.0;
        int index = (int)factor;
        if (index == 43) index = 42;
        const double_ fint = factor - (double_)index;
        extcoice = lut(cT.extice2, 43, index) + fint * (lut(cT.extice2, 43, index + 1) - lut(cT.extice2, 43, index));
        ssacoice = lut(cT.ssaice2, 43, index) + fint * (lut(cT.ssaice2, 43, index + 1) - lut(cT.ssaice2, 43, index));
        gice = lut(cT.asyice2, 43, index) + fint * (lut(cT.asyice2, 43, index + 1) - lut(cT.asyice2, 43, index));
        forwice = gice * gice;
        if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) { set_error(err, E_ICEPROP); return; }
    } else if (iceflag == 3) {
        if (rei < 5.0 || rei > 140.0) { set_error(err, E_ICEDGE); return; }
        const double_ factor = (rei - 2.0) / 3.0;
        int index = (int)factor;
        if (index == 46) index = 45;
        const double_ fint = factor - (double_)index;
        extcoice = lut(cT.extice3, 46, index) + fint * (lut(cT.extice3, 46, index + 1) - lut(cT.extice3, 46, index));
        ssacoice = lut(cT.ssaice3, 46, index) + fint * (lut(cT.ssaice3, 46, index + 1) - lut(cT.ssaice3, 46, index));
        gice = lut(cT.asyice3, 46, index) + fint * (lut(cT.asyice3, 46, index + 1) - lut(cT.asyice3, 46, index));
        const double_ fdelta = lut(cT.fdlice3, 46, index) + fint * (lut(cT.fdlice3, 46, index + 1) - lut(cT.fdlice3, 46, index));
        if (fdelta < 0.0 || fdelta > 1.0) { set_error(err, E_ICEPROP); return; }
        forwice = fdelta + 0.5 / ssacoice;
        if (forwice > gice) forwice = gice;
        if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) { set_error(err, E_ICEPROP); return; }
    }
    if (clwp == 0.0) {
    } else if (liqflag == 1) {
        if (rel < 2.5 || rel > 60.0) { set_error(err, E_LIQRAD); return; }
        int index = (int)(rel - 1.5);
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        const double_ fint = rel - 1.5 - (double_)index;
        extcoliq = lut(cT.extliq1, 58, index) + fint * (lut(cT.extliq1, 58, index + 1) - lut(cT.extliq1, 58, index));
        ssacoliq = lut(cT.ssaliq1, 58, index) + fint * (lut(cT.ssaliq1, 58, index + 1) - lut(cT.ssaliq1, 58, index));
        if (fint < 0.0 && ssacoliq > 1.0) ssacoliq = lut(cT.ssaliq1, 58, index);
        gliq = lut(cT.asyliq1, 58, index) + fint * (lut(cT.asyliq1, 58, index + 1) - lut(cT.asyliq1, 58, index));
        forwliq = gliq * gliq;
        if (extcoliq < 0.0 || ssacoliq > 1.0 || ssacoliq < 0.0 || gliq > 1.0 || gliq < 0.0) { set_error(err, E_LIQPROP); return; }
    }
    const double_ tauliqorig = clwp * extcoliq;
    const double_ tauiceorig = ciwp * extcoice;
    taor = tauliqorig + tauiceorig;
    const double_ ssaliq = ssacoliq * (1.0 - forwliq) / (1.0 - forwliq * ssacoliq);
    const double_ tauliq = (1.0 - forwliq * ssacoliq) * tauliqorig;
    const double_ ssaice = ssacoice * (1.0 - forwice) / (1.0 - forwice * ssacoice);
    const double_ tauice = (1.0 - forwice * ssacoice) * tauiceorig;
    const double_ scatliq = ssaliq * tauliq;
    double_ scatice = ssaice * tauice;
    tauc = tauliq + tauice;
    if (tauc == 0.0) tauc = cldmin;
    if (scatice == 0.0) scatice = cldmin;
    ssac = (scatliq + scatice) / tauc;
    if (iceflag == 3) {
        asmc = (1.0 / (scatliq + scatice)) *
               (scatliq * (gliq - forwliq) / (1.0 - forwliq) + scatice * ((gice - forwice) / (1.0 - forwice)));
    } else {
        asmc = (scatliq * (gliq - forwliq) / (1.0 - forwliq) + scatice * (gice - forwice) / (1.0 - forwice)) /
               (scatliq + scatice);
    }
}

// --------------------------------------------------------------- reftra
// One layer of reftra_sw (rrtmg_sw_reftra.f90:151-326), kmodts = 2.
template <typename R>
struct RT { R ref, refd, tra, trad; };

template <typename R>
__device__ inline RT<R> reftra_g(R zto1, R zw, R zg, R prmuz, const R* __restrict__ tab);

// FP64 form: the reference's expressions verbatim
template <>
__device__ inline RT<double> reftra_g<double>(double zto1, double zw, double zg, double prmuz, const double* __restrict__ tab) {
    typedef double R;
    RT<R> o;
    const R zwcrit = 0.9999995, eps = 1.e-08;
    const R zg3 = 3.0 * zg;
    const R zgamma1 = (8.0 - zw * (5.0 + zg3)) * 0.25;
    const R zgamma2 = 3.0 * (zw * (1.0 - zg)) * 0.25;
    const R zgamma3 = (2.0 - zg3 * prmuz) * 0.25;
    const R zgamma4 = 1.0 - zgamma3;
    R zwo = 0.0, denom = 1.0;
    if (zg != 1.0) {
        const R q = zg / (1.0 - zg);
        denom = (1.0 - (1.0 - zw) * (q * q));
    }
    if (zw > 0.0 && denom != 0.0) zwo = zw / denom;
    if (zwo >= zwcrit) {
        const R za = zgamma1 * prmuz;
        const R za1 = za - zgamma3;
        const R zgt = zgamma1 * zto1;
        const R ze1 = fmin(zto1 / prmuz, 500.0);
        const R ze2 = tbl_exp(ze1, tab);
        o.ref = (zgt - za1 * (1.0 - ze2)) / (1.0 + zgt);
        o.tra = 1.0 - o.ref;
        o.refd = zgt / (1.0 + zgt);
        o.trad = 1.0 - o.refd;
        if (ze2 == 1.0) { o.ref = 0.0; o.tra = 1.0; o.refd = 0.0; o.trad = 1.0; }
    } else {
        const R za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
        const R za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
        const R zrk = sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
        const R zrp = zrk * prmuz;
        const R zrp1 = 1.0 + zrp, zrm1 = 1.0 - zrp;
        const R zrk2 = 2.0 * zrk;
        const R zrpp = 1.0 - zrp * zrp;
        const R zrkg = zrk + zgamma1;
        const R zr1 = zrm1 * (za2 + zrk * zgamma3);
        const R zr2 = zrp1 * (za2 - zrk * zgamma3);
        const R zr3 = zrk2 * (zgamma3 - za2 * prmuz);
        const R zr4 = zrpp * zrkg;
        const R zr5 = zrpp * (zrk - zgamma1);
        const R zt1 = zrp1 * (za1 + zrk * zgamma4);
        const R zt2 = zrm1 * (za1 - zrk * zgamma4);
        const R zt3 = zrk2 * (zgamma4 + za1 * prmuz);
        const R zbeta = (zgamma1 - zrk) / zrkg;
        const R ze1 = fmin(zrk * zto1, 500.0);
        const R ze2 = fmin(zto1 / prmuz, 500.0);
        const R zem1 = tbl_exp(ze1, tab);
        const R zep1 = 1.0 / zem1;
        const R zem2 = tbl_exp(ze2, tab);
        const R zep2 = 1.0 / zem2;
        const R zdenr = zr4 * zep1 + zr5 * zem1;
        const R zdent = zr4 * zep1 + zr5 * zem1;
        if (zdenr >= -eps && zdenr <= eps) {
            o.ref = eps;
            o.tra = zem2;
        } else {
            o.ref = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
            o.tra = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
        }
        const R zemm = zem1 * zem1;
        const R zdend = 1.0 / ((1.0 - zbeta * zemm) * zrkg);
        o.refd = zgamma2 * (1.0 - zemm) * zdend;
        o.trad = zrk2 * zem1 * zdend;
    }
    return o;
}

// ------------------------------------------------------------------ KISS
// KISS generator (mcica_subcol_gen_sw.f90:721-753) with O(log n) jumps:
// the congruential part is an affine map mod 2^32, the shift register is
// linear over GF(2) (precomputed M^(2^k) in cT.xs_jump), and each 16-bit
// multiply-with-carry part x' = a*(x & 0xffff) + (x >> 16) is the
// multiplicative congruential map x' = a*x mod (a*2^16 - 1).
struct Kiss {
    uint32_t s1, s2, s3, s4;
    __device__ double next() {
        s1 = 69069u * s1 + 1327217885u;
        uint32_t y = s2;
        y ^= y << 13;
        y ^= y >> 17;
        y ^= y << 5;
        s2 = y;
        s3 = 18000u * (s3 & 65535u) + (s3 >> 16);
        s4 = 30903u * (s4 & 65535u) + (s4 >> 16);
        const int32_t kiss = (int32_t)(s1 + s2 + (s3 << 16) + s4);
        return __dadd_rn(__dmul_rn((double)kiss, 2.328306e-10), 0.5);
    }
};

__device__ inline uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (a * b) % m; }
__device__ inline uint64_t powmod(uint64_t a, uint64_t n, uint64_t m) {
    uint64_t r = 1 % m;
    a %= m;
    while (n) {
        if (n & 1) r = mulmod(r, a, m);
        a = mulmod(a, a, m);
        n >>= 1;
    }
    return r;
}

__device__ inline void kiss_jump(Kiss& k, uint64_t n) {
    if (n == 0) return;
    // congruential: x -> 69069 x + 1327217885 (mod 2^32)
    uint32_t A = 1, C = 0, a = 69069u, c = 1327217885u;
    uint64_t m = n;
    while (m) {
        if (m & 1) { A = a * A; C = a * C + c; }
        c = a * c + c;
        a = a * a;
        m >>= 1;
    }
    k.s1 = A * k.s1 + C;
    // xorshift: y -> M^n y over GF(2)
    uint32_t y = k.s2;
    m = n;
    for (int b = 0; m; ++b, m >>= 1) {
        if (!(m & 1)) continue;
        uint32_t r = 0;
        for (int j = 0; j < 32; ++j)
            if (y >> j & 1u) r ^= cT.xs_jump[b][j];
        y = r;
    }
    k.s2 = y;
    // multiply-with-carry parts
    const uint64_t m3 = 18000ull * 65536ull - 1ull, m4 = 30903ull * 65536ull - 1ull;
    k.s3 = (uint32_t)mulmod(powmod(18000ull, n, m3), k.s3, m3);
    k.s4 = (uint32_t)mulmod(powmod(30903ull, n, m4), k.s4, m4);
}

// seed = int((pmid - int(pmid)) * 1e9), pmid in Pa (mcica:475-478)
__device__ inline uint32_t kiss_seed(double pmid) {
    const double frac = __dsub_rn(pmid, trunc(pmid));
    return (uint32_t)(int32_t)(long long)__dmul_rn(frac, 1000000000.0);
}

// Subcolumn cloud mask of one (column, subcolumn) walked bottom -> top
// (generate_stochastic_clouds_sw, KISS branch, mcica_subcol_gen_sw.f90:
// 466-659; icld 4/5 in the single-column generator's order,
// mcica_subcol_gen_sw.1col.f90:536-604).  Subcolumn g of a column uses the
// column's stream from position permuteseed + g*nlay (x2 for icld 4/5).
struct McicaKiss {
    Kiss k;
    double cdf_prev, cf_prev, cdf0;
    int icld;
    __device__ void init(const double* play, size_t ncol, int col, int g, int nlay, int icld_, int permuteseed,
                         int* err) {
        icld = icld_;
        cdf_prev = cf_prev = cdf0 = 0.0;
        const double p1 = __dmul_rn(play[col], 1.e2), p2 = __dmul_rn(play[col + ncol], 1.e2);
        if (p1 < p2) set_error(err, E_KISSSEED);
        k.s1 = kiss_seed(p1);
        k.s2 = kiss_seed(p2);
        k.s3 = kiss_seed(__dmul_rn(play[col + 2 * ncol], 1.e2));
        k.s4 = kiss_seed(__dmul_rn(play[col + 3 * ncol], 1.e2));
        uint64_t jump = (uint64_t)permuteseed;
        if (icld == 3) jump += (uint64_t)g;
        else if (icld >= 4) jump += 2ull * (uint64_t)g * (uint64_t)nlay;
        else jump += (uint64_t)g * (uint64_t)nlay;
        kiss_jump(k, jump);
        if (icld == 3) cdf0 = k.next();
    }
    // cf: layer cloud fraction; alpha: get_alpha value of this layer
    __device__ bool step(int lay, double cf, double alpha) {
        if (cf < 1.0e-20) cf = 0.0;
        double cdf;
        if (icld == 3) {
            cdf = cdf0;
        } else if (icld >= 4) {
            cdf = k.next();
            const double cdf2 = k.next();
            if (lay >= 2 && cdf2 < alpha) cdf = cdf_prev;
        } else {
            cdf = k.next();
            if (icld == 2 && lay >= 2) {
                if (cdf_prev > __dsub_rn(1.0, cf_prev)) cdf = cdf_prev;
                else cdf = __dmul_rn(cdf, __dsub_rn(1.0, cf_prev));
            }
        }
        cdf_prev = cdf;
        cf_prev = cf;
        return cdf >= __dsub_rn(1.0, cf);
    }
};

}  // namespace rrsw
