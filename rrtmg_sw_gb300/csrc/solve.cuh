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
    int fused;       // 1: McICA masks generated in the kernel
    int nomcica;     // 1: non-McICA path (cldprop_sw + spcvrt_sw): layer cloud fraction, band optics
    int extra;       // 1: also the 8 direct/diffuse/UV/NIR outputs
    int permuteseed;
    int npairs;
    double svar_f_bnd[NBND], svar_s_bnd[NBND], svar_i_bnd[NBND], adjflux[NBND];  // solar variability factors
    const double *play, *plev, *tlay, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *o2vmr;
    const double *asdir, *asdif, *aldir, *aldif, *coszen;
    const double *cldfmcl, *taucmcl, *ssacmcl, *asmcmcl, *fsfcmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl;
    const double *tauaer, *ssaaer, *asmaer, *ecaer;
    const double *cldfrac, *ciwp, *clwp, *rei, *rel, *tauc, *ssac, *asmc, *fsfc, *alpha;
    double *swuflx, *swdflx, *swhr, *swuflxc, *swdflxc, *swhrc;
    double *xout[8];  // dirdflux, difdflux, uvdflx, nidflx, dirdnuv, difdnuv, dirdnir, difdnir
    int bands;        // 1: per-band fluxes requested
    int irng;         // fused McICA generator: 0 KISS, 1 MT19937 (stream in mt)
    double *bout[5];  // bndfu, bndfd, bndfddir, bndcu, bndcd (ncol,nlay+1,nbnd)
    const int *colmap;   // batch: this instance's sunlit columns (nullptr: all columns in order)
    const int *mapcount; // batch: number of entries of colmap (device)
    void *scratch;
    size_t slot_elems;
    int *err;
    const uint32_t* mt;  // irng 1: tempered MT words of the call's stream (subcolumn, column, layer order)
    // tiled FP32 kernel: column pairs with more FP64 cells than its capacities
    // (list of pair indices, its length and capacity); the caller solves them
    // again with the scratch-based kernel.  tile_qcap > 0 lowers the capacity
    // of FP64 cells per pair (tests of that path).
    int* tovf;
    int* tovfcount;
    int tovfcap;
    int tile_qcap;
    int tile_slots;  // tiled FP32 kernel: pair slots (2 or 3) its shared memory was sized for
    // FP32 form's counters (nullptr: not kept): [0] cells redone in FP64,
    // [1] of those past the scratch kernel's queue (redone by their own
    // thread), [2] column pairs the tiled kernel handed back, [3] subcolumns
    // the tiled kernel swept a second time for their FP64 cells
    unsigned long long* stats;
    // tiled FP32 kernel: the pairs' prepared blocks (written by k_tiled_prep)
    void* tprep;
};

// Tangent-linear / adjoint request (solve_ad.cu): objective weights and
// the device arrays of the objective, its gradients or its direction.
struct AdParams {
    double w_toa, w_net, w_hr;   // objective weights
    int store;                   // 1: local Jacobians kept from pass 1, 0: recomputed in the reverse pass
    int tl;                      // 1: tangent-linear (dJ along dir), 0: adjoint (gradients)
    double* J;                   // (ncol)
    double* dJ;                  // (ncol), tangent-linear
    double* g[5];                // adjoint: dJ/d tlay, h2ovmr, o3vmr, clwp, ciwp (ncol,nlay)
    double* ga[4];               // adjoint: dJ/d asdir, asdif, aldir, aldif (ncol)
    const double* dir[5];        // tangent-linear direction, same layout
    const double* dira[4];
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

// Element type of the coefficient tables read by arithmetic type R: the
// table of R itself for float and double; derivative types read the FP64
// tables.
template <typename R>
struct TabOf { typedef R type; };
template <typename R>
using TabT = typename TabOf<R>::type;

// ----------------------------------------------------- arithmetic helpers
// The FP64 form is compiled without FMA contraction, so a*b+c rounds twice
// as the reference's expressions do.  The FP32 form may contract.
template <typename R> __device__ inline R rcp(R x) { return R(1) / x; }

template <typename R> __device__ inline R c_bpade();
template <> __device__ inline double c_bpade<double>() { return cT.bpade; }
template <> __device__ inline float c_bpade<float>() { return cT.bpade_f; }
template <typename R> __device__ inline R c_oneminus();
template <> __device__ inline double c_oneminus<double>() { return cT.oneminus; }
template <> __device__ inline float c_oneminus<float>() { return cT.oneminus_f; }

// exp(-x) through the lookup table, or the quadratic below od_lo
// (rrtmg_sw_reftra.f90:203-209; table built at rrtmg_sw_init.f90:115-123)
template <typename R>
__device__ inline R tbl_exp(R ze1, const R* __restrict__ tab) {
    const R od_lo = R(0.06);
    if (ze1 <= od_lo) return R(1) - ze1 + R(0.5) * ze1 * ze1;
    const R tblind = ze1 / (c_bpade<R>() + ze1);
    const int itind = (int)(R(10000) * tblind + R(0.5));
    return ldt(tab, cT.exp_tbl + itind);
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
    if (specparm >= c_oneminus<R>()) specparm = c_oneminus<R>();
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
__device__ inline R K(const TabT<R>* __restrict__ tab, int off, int ng, int ind, int ig) {
    return R(ldt(tab, off + (ind - 1) * ng + (ig - 1)));
}

template <typename R>
__device__ inline R k8(const Spec<R>& s, const TabT<R>* __restrict__ tab, int off, int ng, int ind0, int ind1, int ig, int d1) {
    return (s.f000 * K<R>(tab, off, ng, ind0, ig) + s.f100 * K<R>(tab, off, ng, ind0 + 1, ig) +
            s.f010 * K<R>(tab, off, ng, ind0 + d1, ig) + s.f110 * K<R>(tab, off, ng, ind0 + d1 + 1, ig) +
            s.f001 * K<R>(tab, off, ng, ind1, ig) + s.f101 * K<R>(tab, off, ng, ind1 + 1, ig) +
            s.f011 * K<R>(tab, off, ng, ind1 + d1, ig) + s.f111 * K<R>(tab, off, ng, ind1 + d1 + 1, ig));
}

template <typename R>
__device__ inline R k4(const Coef<R>& c, int lay, const TabT<R>* __restrict__ tab, int off, int ng, int ind0, int ind1, int ig) {
    return c.f(F_FAC00, lay) * K<R>(tab, off, ng, ind0, ig) + c.f(F_FAC10, lay) * K<R>(tab, off, ng, ind0 + 1, ig) +
           c.f(F_FAC01, lay) * K<R>(tab, off, ng, ind1, ig) + c.f(F_FAC11, lay) * K<R>(tab, off, ng, ind1 + 1, ig);
}

template <typename R>
__device__ inline R selfterm(const Coef<R>& c, int lay, const BandOff& B, const TabT<R>* __restrict__ tab, int ig) {
    const int inds = c.indself(lay);
    const R a = K<R>(tab, B.selfref, B.ng, inds, ig), b = K<R>(tab, B.selfref, B.ng, inds + 1, ig);
    return c.f(F_SELFFAC, lay) * (a + c.f(F_SELFFRAC, lay) * (b - a));
}
template <typename R>
__device__ inline R forpart(const Coef<R>& c, int lay, const BandOff& B, const TabT<R>* __restrict__ tab, int ig) {
    const int indf = c.indfor(lay);
    const R a = K<R>(tab, B.forref, B.ng, indf, ig), b = K<R>(tab, B.forref, B.ng, indf + 1, ig);
    return (a + c.f(F_FORFRAC, lay) * (b - a));
}
template <typename R>
__device__ inline R forterm(const Coef<R>& c, int lay, const BandOff& B, const TabT<R>* __restrict__ tab, int ig) {
    return c.f(F_FORFAC, lay) * forpart(c, lay, B, tab, ig);
}
template <typename R>
__device__ inline R selffor(const Coef<R>& c, int lay, const BandOff& B, const TabT<R>* __restrict__ tab, int ig) {
    return selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig);
}
template <typename R>
__device__ inline R V(const TabT<R>* __restrict__ tab, int off, int i) { return R(ldt(tab, off + i)); }

// Lower/upper table base indices (taumol.f90:326-327, 357-358)
__device__ inline int ind_lo(int jp, int jt, int nsp, int js) { return ((jp - 1) * 5 + (jt - 1)) * nsp + js; }
__device__ inline int ind_lo1(int jp, int jt1, int nsp, int js) { return (jp * 5 + (jt1 - 1)) * nsp + js; }
__device__ inline int ind_up(int jp, int jt, int nsp, int js) { return ((jp - 13) * 5 + (jt - 1)) * nsp + js; }
__device__ inline int ind_up1(int jp, int jt1, int nsp, int js) { return ((jp - 12) * 5 + (jt1 - 1)) * nsp + js; }

// Gas (taug) and Rayleigh (taur) optical depth of g-point `ig` (1-based in
// its band) at layer `lay`: one g-point of taumol16..taumol29
// (rrtmg_sw_taumol.f90:275-1785), same expressions and association order.
template <typename R>
__device__ inline void taumol_g(int ib, int ig, int lay, const Coef<R>& c, const TabT<R>* __restrict__ tab, R& taug, R& taur) {
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
        taur = colmol * V<R>(tab, B.rayl, 0);
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
        taur = colmol * V<R>(tab, B.rayl, 0);
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
        taur = colmol * V<R>(tab, B.rayl, 0);
        break;
    }
    case 20:
        if (low) {
            taug = colh2o * ((k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig)) +
                             selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig)) +
                   colch4 * V<R>(tab, B.absch4, ig - 1);
        } else {
            taug = colh2o * (k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) +
                             forterm(c, lay, B, tab, ig)) +
                   colch4 * V<R>(tab, B.absch4, ig - 1);
        }
        taur = colmol * V<R>(tab, B.rayl, 0);
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
        taur = colmol * V<R>(tab, B.rayl, 0);
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
        taur = colmol * V<R>(tab, B.rayl, 0);
        break;
    }
    case 23:
        if (low) {
            taug = colh2o * (R(1.029) * k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig) +
                             selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig));
        } else {
            taug = R(0);
        }
        taur = colmol * V<R>(tab, B.rayl, ig - 1);
        break;
    case 24:
        if (low) {
            const Spec<R> s = spec(colh2o, R(0.124692) * colo2, R(8), c, lay);
            const R ra = V<R>(tab, B.rayla, (s.js - 1) * B.ng + ig - 1), rb = V<R>(tab, B.rayla, s.js * B.ng + ig - 1);
            taur = colmol * (ra + s.fs * (rb - ra));
            taug = s.speccomb * k8(s, tab, B.absa, B.ng, ind_lo(jp, jt, 9, s.js), ind_lo1(jp, jt1, 9, s.js), ig, 9) +
                   colo3 * V<R>(tab, B.abso3a, ig - 1) + colh2o * selffor(c, lay, B, tab, ig);
        } else {
            taur = colmol * V<R>(tab, B.raylb, ig - 1);
            taug = colo2 * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) +
                   colo3 * V<R>(tab, B.abso3b, ig - 1);
        }
        break;
    case 25:
        taur = colmol * V<R>(tab, B.rayl, ig - 1);
        if (low) {
            taug = colh2o * k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig) +
                   colo3 * V<R>(tab, B.abso3a, ig - 1);
        } else {
            taug = colo3 * V<R>(tab, B.abso3b, ig - 1);
        }
        break;
    case 26:
        taug = R(0);
        taur = colmol * V<R>(tab, B.rayl, ig - 1);
        break;
    case 27:
        taur = colmol * V<R>(tab, B.rayl, ig - 1);
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
        taur = colmol * V<R>(tab, B.rayl, 0);
        break;
    default:  // 29
        if (low) {
            taug = colh2o * ((k4(c, lay, tab, B.absa, B.ng, ind_lo(jp, jt, 1, 1), ind_lo1(jp, jt1, 1, 1), ig)) +
                             selfterm(c, lay, B, tab, ig) + forterm(c, lay, B, tab, ig)) +
                   colco2 * V<R>(tab, B.absco2, ig - 1);
        } else {
            taug = colco2 * k4(c, lay, tab, B.absb, B.ng, ind_up(jp, jt, 1, 1), ind_up1(jp, jt1, 1, 1), ig) +
                   colh2o * V<R>(tab, B.absh2o, ig - 1);
        }
        taur = colmol * V<R>(tab, B.rayl, 0);
        break;
    }
}

// One g-point of taumol16..29 through the band/region descriptors (FP32
// form): same terms as taumol_g, one instruction stream for all bands.  The
// descriptors come from shared memory (sTm[band][region]).
__device__ inline void taumol_generic(int ib, int ig, int lay, const Coef<float>& c, const float* __restrict__ tab,
                                      const TmSmem* __restrict__ sTm, float& taug, float& taur, int& js_out,
                                      float& fs_out) {
    const TmSmem t = sTm[ib * 2 + (lay <= c.laytrop ? 0 : 1)];
    const TmRegion& d = t.r;
    const int ng = t.ng;
    const int jp = c.jp(lay) - d.jo, jt = c.jt(lay), jt1 = c.jt1(lay);
    const float colh2o = c.f(F_H2O, lay);
    float tg = 0.0f, fs = 0.0f;
    int js = 1;
    // A warp's 32 g-points span several bands, so the band kinds share one
    // path (branches would run one after the other): one species (kind 2)
    // is two species with fs = 0 and its column times fac; kind 0 has no
    // major absorber.
    if (d.kind != 0) {
        const bool two = d.kind == 1;
        const float ca = c.f(F_H2O + d.sa, lay);
        const float speccomb = two ? ca + d.strrat * c.f(F_H2O + d.sb, lay) : ca * d.fac;
        const float specmult = two ? d.mult * fminf(ca / speccomb, cT.oneminus_f) : 0.0f;
        const int ij = (int)specmult;
        js = 1 + ij;
        fs = specmult - (float)ij;
        const float f00 = c.f(F_FAC00, lay), f01 = c.f(F_FAC01, lay), f10 = c.f(F_FAC10, lay), f11 = c.f(F_FAC11, lay);
        const int nsp = d.nsp;
        const int i0 = ((jp * 5 + (jt - 1)) * nsp + js - 1) * ng + ig - 1;
        const int i1 = (((jp + 1) * 5 + (jt1 - 1)) * nsp + js - 1) * ng + ig - 1;
        const float gs = 1.0f - fs;
        // the fs terms exist for two species only (one species: fs = 0, and
        // i + (nsp + 1) ng would pass the table's end)
        const float a1 = two ? ldt(tab, d.ktab + i0 + ng) : 0.0f;
        const float a3 = two ? ldt(tab, d.ktab + i0 + (nsp + 1) * ng) : 0.0f;
        const float b1 = two ? ldt(tab, d.ktab + i1 + ng) : 0.0f;
        const float b3 = two ? ldt(tab, d.ktab + i1 + (nsp + 1) * ng) : 0.0f;
        const float k0 = gs * f00 * ldt(tab, d.ktab + i0) + fs * f00 * a1 + gs * f10 * ldt(tab, d.ktab + i0 + nsp * ng) +
                         fs * f10 * a3;
        const float k1 = gs * f01 * ldt(tab, d.ktab + i1) + fs * f01 * b1 + gs * f11 * ldt(tab, d.ktab + i1 + nsp * ng) +
                         fs * f11 * b3;
        tg = speccomb * (k0 + k1);
    }
    if (d.cont >= 1) {
        const int indf = c.indfor(lay);
        const float fa = ldt(tab, t.forref + (indf - 1) * ng + ig - 1), fb = ldt(tab, t.forref + indf * ng + ig - 1);
        float cont = c.f(F_FORFAC, lay) * (fa + c.f(F_FORFRAC, lay) * (fb - fa));
        if (d.cont == 1) {
            const int inds = c.indself(lay);
            const float sa = ldt(tab, t.selfref + (inds - 1) * ng + ig - 1);
            const float sb = ldt(tab, t.selfref + inds * ng + ig - 1);
            cont = c.f(F_SELFFAC, lay) * (sa + c.f(F_SELFFRAC, lay) * (sb - sa)) + cont;
        }
        tg += colh2o * cont;
    }
    if (d.minor == 9) tg += 4.35e-4f * c.f(F_O2, lay) / 700.0f;
    else if (d.minor >= 0) tg += c.f(F_H2O + d.minor, lay) * ldt(tab, d.mtab + ig - 1);
    const float colmol = c.f(F_MOL, lay);
    {
        // Rayleigh: one value (rtype 0), one per g-point (1), or interpolated
        // in the species ratio (2); one path, the second read only for rtype 2
        const int ir = d.rtab + (d.rtype == 2 ? (js - 1) * ng : 0) + (d.rtype >= 1 ? ig - 1 : 0);
        const float ra = ldt(tab, ir);
        const float rb = d.rtype == 2 ? ldt(tab, ir + ng) : ra;
        taur = colmol * (d.rtype == 2 ? ra + fs * (rb - ra) : ra);
    }
    taug = tg;
    js_out = js;
    fs_out = fs;
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
__device__ inline R solar_source(int ib, int ig, const Coef<R>& c, const SolveParams& P, const TabT<R>* __restrict__ tab) {
    const BandOff& B = cT.b[ib];
    const int band = ib + 16;
    const int lay = solar_layer(ib, c);
    bool interp = false;
    R fs = R(0);
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
        if (interp) { js = s.js; fs = s.fs; }
    }
    auto src = [&](int off) -> R {
        if (!interp) return V<R>(tab, off, ig - 1);
        const R a = V<R>(tab, off, (js - 1) * B.ng + ig - 1), b = V<R>(tab, off, js * B.ng + ig - 1);
        return a + fs * (b - a);
    };
    if (P.isolvar < 0) {
        const R sf = src(B.sfluxref);
        return band == 27 ? R(50.15 / 48.37) * sf : sf;
    }
    const R fb = src(B.facbrght), sd = src(B.snsptdrk), ir = src(B.irradnce);
    return R(P.svar_f_bnd[ib]) * fb + R(P.svar_s_bnd[ib]) * sd + R(P.svar_i_bnd[ib]) * ir;
}

// Solar source for the FP32 form through the descriptors: the species
// interpolation of the source tables applies where the source region is a
// kind-1 (speccomb) loop, as in taumol17,18,19,21,22,24,28.
__device__ inline float solar_source_generic(int ib, int ig, const Coef<float>& c, const SolveParams& P,
                                             const float* __restrict__ tab, const TmSmem* __restrict__ sTm) {
    const BandOff& B = cT.b[ib];
    const int band = ib + 16;
    const int lay = solar_layer(ib, c);
    const int up = (band == 16 || band == 17 || band == 27 || band == 28 || band == 29) ? 1 : 0;
    bool interp = false;
    int js = 1;
    float fs = 0.0f;
    if (lay >= 1 && cT.tm[ib][up].kind == 1) {
        float tg, tr;
        taumol_generic(ib, ig, lay, c, tab, sTm, tg, tr, js, fs);
        interp = true;
    }
    auto src = [&](int off) -> float {
        if (!interp) return ldt(tab, off + ig - 1);
        const float a = ldt(tab, off + (js - 1) * B.ng + ig - 1), b = ldt(tab, off + js * B.ng + ig - 1);
        return a + fs * (b - a);
    };
    if (P.isolvar < 0) {
        const float sf = src(B.sfluxref);
        return band == 27 ? float(50.15 / 48.37) * sf : sf;
    }
    const float fb = src(B.facbrght), sd = src(B.snsptdrk), ir = src(B.irradnce);
    return float(P.svar_f_bnd[ib]) * fb + float(P.svar_s_bnd[ib]) * sd + float(P.svar_i_bnd[ib]) * ir;
}

// --------------------------------------------------------------- cldprmc
// One (g-point, layer) of cldprmc_sw (rrtmg_sw_cldprmc.f90:53-349) for
// inflag = 0 or 2.  On input tauc/ssac/asmc are the subcolumn's values;
// on output the delta-scaled cloud properties and taor the unscaled depth.
template <typename R>
__device__ inline void cldprmc_g(int ib, int inflag, int iceflag, int liqflag, R cldf, R ciwp,
                                 R clwp, R rei, R rel, R fsfc, R& tauc,
                                 R& ssac, R& asmc, R& taor, R& co, const TabT<R>* __restrict__ tab,
                                 int* err, R ttest = R(-1)) {
    typedef R double_;
    const R eps = R((1.e-06)), cldmin = R((1.e-20));
    taor = tauc;
    co = R(1) - ssac;  // co-albedo (used by the FP32 form only)
    const double_ cwp = ciwp + clwp;
    // cldprmc tests the subcolumn's own depth; cldprop_sw (rrtmg_sw_cldprop.f90:153-154)
    // passes the layer's band-summed depth as ttest
    if (!(cldf >= cldmin && (cwp >= cldmin || (ttest < R(0) ? tauc : ttest) >= cldmin))) return;
    if (inflag == 0) {
        const double_ taucldorig_a = tauc;
        const double_ ffp = fsfc;
        const double_ ffp1 = R(1.0) - ffp;
        const double_ ffpssa = R(1.0) - ffp * ssac;
        const double_ ssacloud_a = ffp1 * ssac / ffpssa;
        const double_ taucloud_a = ffpssa * taucldorig_a;
        co = (R(1) - ssac) / ffpssa;
        taor = taucldorig_a;
        ssac = ssacloud_a;
        tauc = taucloud_a;
        asmc = (asmc - ffp) / (ffp1);
        return;
    }
    if (inflag != 2) { set_error(err, E_INFLAG1); return; }
    double_ extcoice = 0, ssacoice = 0, gice = 0, forwice = 0, extcoliq = 0, ssacoliq = 0, gliq = 0, forwliq = 0;
    double_ coice = 1, coliq = 1;  // 1 - ssacoice, 1 - ssacoliq from the co-albedo tables
    const int jb = ib + 1;  // band column of the Fortran (index, 16:29) LUTs, 1-based
    auto lut = [&](int off, int n, int index) { return R(ldt(tab, off + (jb - 1) * n + index - 1)); };
    if (ciwp == R(0.0)) {
    } else if (iceflag == 1) {
        if (rei < R(13.0) || rei > R(130.0)) { set_error(err, E_ICERAD); return; }
        const double_ w2 = R(ldt(tab, cT.wavenum2 + ib));
        int icx = 0;
        if (w2 > R(1.43e04)) icx = 1;
        else if (w2 > R(7.7e03)) icx = 2;
        else if (w2 > R(5.3e03)) icx = 3;
        else if (w2 > R(4.0e03)) icx = 4;
        else if (w2 >= R(2.5e03)) icx = 5;
        extcoice = (R(ldt(tab, cT.abari + icx - 1)) + R(ldt(tab, cT.bbari + icx - 1)) / rei);
        ssacoice = R(1.0) - R(ldt(tab, cT.cbari + icx - 1)) - R(ldt(tab, cT.dbari + icx - 1)) * rei;
        coice = R(ldt(tab, cT.cbari + icx - 1)) + R(ldt(tab, cT.dbari + icx - 1)) * rei;
        gice = R(ldt(tab, cT.ebari + icx - 1)) + R(ldt(tab, cT.fbari + icx - 1)) * rei;
        if (gice >= R(1.0)) gice = R(1.0) - eps;
        forwice = gice * gice;
        if (extcoice < R(0.0) || ssacoice > R(1.0) || ssacoice < R(0.0) || gice > R(1.0) || gice < R(0.0)) { set_error(err, E_ICEPROP); return; }
    } else if (iceflag == 2) {
        if (rei < R(5.0) || rei > R(131.0)) { set_error(err, E_ICERAD); return; }
        const double_ factor = (rei - R(2.0)) / R(3.0);
        int index = (int)factor;
        if (index == 43) index = 42;
        const double_ fint = factor - (double_)index;
        extcoice = lut(cT.extice2, 43, index) + fint * (lut(cT.extice2, 43, index + 1) - lut(cT.extice2, 43, index));
        ssacoice = lut(cT.ssaice2, 43, index) + fint * (lut(cT.ssaice2, 43, index + 1) - lut(cT.ssaice2, 43, index));
        coice = lut(cT.coice2, 43, index) + fint * (lut(cT.coice2, 43, index + 1) - lut(cT.coice2, 43, index));
        gice = lut(cT.asyice2, 43, index) + fint * (lut(cT.asyice2, 43, index + 1) - lut(cT.asyice2, 43, index));
        forwice = gice * gice;
        if (extcoice < R(0.0) || ssacoice > R(1.0) || ssacoice < R(0.0) || gice > R(1.0) || gice < R(0.0)) { set_error(err, E_ICEPROP); return; }
    } else if (iceflag == 3) {
        if (rei < R(5.0) || rei > R(140.0)) { set_error(err, E_ICEDGE); return; }
        const double_ factor = (rei - R(2.0)) / R(3.0);
        int index = (int)factor;
        if (index == 46) index = 45;
        const double_ fint = factor - (double_)index;
        extcoice = lut(cT.extice3, 46, index) + fint * (lut(cT.extice3, 46, index + 1) - lut(cT.extice3, 46, index));
        ssacoice = lut(cT.ssaice3, 46, index) + fint * (lut(cT.ssaice3, 46, index + 1) - lut(cT.ssaice3, 46, index));
        coice = lut(cT.coice3, 46, index) + fint * (lut(cT.coice3, 46, index + 1) - lut(cT.coice3, 46, index));
        gice = lut(cT.asyice3, 46, index) + fint * (lut(cT.asyice3, 46, index + 1) - lut(cT.asyice3, 46, index));
        const double_ fdelta = lut(cT.fdlice3, 46, index) + fint * (lut(cT.fdlice3, 46, index + 1) - lut(cT.fdlice3, 46, index));
        if (fdelta < R(0.0) || fdelta > R(1.0)) { set_error(err, E_ICEPROP); return; }
        forwice = fdelta + R(0.5) / ssacoice;
        if (forwice > gice) forwice = gice;
        if (extcoice < R(0.0) || ssacoice > R(1.0) || ssacoice < R(0.0) || gice > R(1.0) || gice < R(0.0)) { set_error(err, E_ICEPROP); return; }
    }
    if (clwp == R(0.0)) {
    } else if (liqflag == 1) {
        if (rel < R(2.5) || rel > R(60.0)) { set_error(err, E_LIQRAD); return; }
        int index = (int)(rel - R(1.5));
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        const double_ fint = rel - R(1.5) - (double_)index;
        extcoliq = lut(cT.extliq1, 58, index) + fint * (lut(cT.extliq1, 58, index + 1) - lut(cT.extliq1, 58, index));
        ssacoliq = lut(cT.ssaliq1, 58, index) + fint * (lut(cT.ssaliq1, 58, index + 1) - lut(cT.ssaliq1, 58, index));
        coliq = lut(cT.coliq1, 58, index) + fint * (lut(cT.coliq1, 58, index + 1) - lut(cT.coliq1, 58, index));
        if (fint < R(0.0) && ssacoliq > R(1.0)) {
            ssacoliq = lut(cT.ssaliq1, 58, index);
            coliq = lut(cT.coliq1, 58, index);
        }
        gliq = lut(cT.asyliq1, 58, index) + fint * (lut(cT.asyliq1, 58, index + 1) - lut(cT.asyliq1, 58, index));
        forwliq = gliq * gliq;
        if (extcoliq < R(0.0) || ssacoliq > R(1.0) || ssacoliq < R(0.0) || gliq > R(1.0) || gliq < R(0.0)) { set_error(err, E_LIQPROP); return; }
    }
    const double_ tauliqorig = clwp * extcoliq;
    const double_ tauiceorig = ciwp * extcoice;
    taor = tauliqorig + tauiceorig;
    const double_ ssaliq = ssacoliq * (R(1.0) - forwliq) / (R(1.0) - forwliq * ssacoliq);
    const double_ tauliq = (R(1.0) - forwliq * ssacoliq) * tauliqorig;
    const double_ ssaice = ssacoice * (R(1.0) - forwice) / (R(1.0) - forwice * ssacoice);
    const double_ tauice = (R(1.0) - forwice * ssacoice) * tauiceorig;
    const double_ scatliq = ssaliq * tauliq;
    double_ scatice = ssaice * tauice;
    tauc = tauliq + tauice;
    const bool zero = tauc == R(0.0);
    if (tauc == R(0.0)) tauc = cldmin;
    if (scatice == R(0.0)) scatice = cldmin;
    ssac = (scatliq + scatice) / tauc;
    // absorption depth tau*(1 - ssa) of each phase is invariant under the
    // delta scaling: tauliqorig*(1 - ssacoliq) + tauiceorig*(1 - ssacoice)
    co = zero ? R(0) : (tauliqorig * coliq + tauiceorig * coice) / tauc;
    if (iceflag == 3) {
        asmc = (R(1.0) / (scatliq + scatice)) *
               (scatliq * (gliq - forwliq) / (R(1.0) - forwliq) + scatice * ((gice - forwice) / (R(1.0) - forwice)));
    } else {
        asmc = (scatliq * (gliq - forwliq) / (R(1.0) - forwliq) + scatice * (gice - forwice) / (R(1.0) - forwice)) /
               (scatliq + scatice);
    }
}

// --------------------------------------------------------------- reftra
// One layer of reftra_sw (rrtmg_sw_reftra.f90:151-326), kmodts = 2.
template <typename R>
struct RT {
    R ref, refd, tra, trad;
    // FP32 form only: absorptances 1 - ref - tra (direct incidence) and
    // 1 - refd - trad (diffuse incidence), formed without cancellation
    R adir, adif;
    // FP32 form only: a discrete choice (table entry near resonance, the
    // conservative switch) is too close to call in FP32
    bool risky;
};

// zco = 1 - zw carried separately by the FP32 form (unused by FP64);
// tab64 is the FP64 table blob (the FP32 form's FP64 island needs it)
// force (FP32 form): 1 = also test every table lookup for an ambiguous entry
// (cloudy total sky), -1 = only near resonance
template <typename R>
__device__ inline RT<R> reftra_g(R zto1, R zw, R zco, R zg, R prmuz, const R* __restrict__ tab,
                                 const double* __restrict__ tab64, int force = -1);
// FP32 form: the same for a cloudy cell's total sky, compiled once (a few
// percent of the cells take it; inlined it only grows the kernels' code)
__device__ RT<float> reftra_f32_cloudy(float zto1, float zw, float zco, float zg, float prmuz,
                                       const float* __restrict__ tab, const double* __restrict__ tab64);

// FP64 form: the reference's expressions verbatim
namespace {
// out of line: one copy serves the clear-sky and the cloudy call
__device__ __noinline__ RT<double> reftra_fp64(double zto1, double zw, double zg, double prmuz,
                                               const double* __restrict__ tab) {
    typedef double R;
    RT<R> o;
    o.adir = o.adif = 0.0;
    o.risky = false;
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
}  // namespace

template <>
__device__ inline RT<double> reftra_g<double>(double zto1, double zw, double zco, double zg, double prmuz,
                                             const double* __restrict__ tab, const double* __restrict__ tab64,
                                             int force) {
    (void)zco;
    (void)tab64;
    (void)force;
    return reftra_fp64(zto1, zw, zg, prmuz, tab);
}

// ------------------------------------------------------------------ KISS
// KISS generator (mcica_subcol_gen_sw.f90:721-753).  Subcolumn g of a
// column consumes the column's stream from position n = permuteseed +
// g*nlay (x2 for icld 4/5, +g for icld 3), so each thread jumps there in
// O(1) per column: the congruential part is an affine map mod 2^32, the
// shift register is linear over GF(2) (M^n precomputed once per launch),
// and each 16-bit multiply-with-carry part x' = a*(x & 0xffff) + (x >> 16)
// is the multiplicative map x' = a*x mod (a*2^16 - 1).
struct Kiss {
    uint32_t s1, s2, s3, s4;
    __device__ int32_t next_int() {
        s1 = 69069u * s1 + 1327217885u;
        uint32_t y = s2;
        y ^= y << 13;
        y ^= y >> 17;
        y ^= y << 5;
        s2 = y;
        s3 = 18000u * (s3 & 65535u) + (s3 >> 16);
        s4 = 30903u * (s4 & 65535u) + (s4 >> 16);
        return (int32_t)(s1 + s2 + (s3 << 16) + s4);
    }
};

// ran_arr = kiss*2.328306e-10 + 0.5 (mcica:750), two FP64 roundings
__device__ inline double kiss_real(int32_t k) { return __dadd_rn(__dmul_rn((double)k, 2.328306e-10), 0.5); }

// Smallest k with kiss_real(k) >= x (kiss_real is increasing in k), in
// [INT_MIN, INT_MAX + 1].  Comparing the raw integer draw with this
// threshold is the reference's FP64 comparison, bit for bit.
__device__ inline long long kiss_threshold(double x) {
    const long long lo = -2147483648ll, hi = 2147483647ll;
    if (kiss_real((int32_t)lo) >= x) return lo;
    if (kiss_real((int32_t)hi) < x) return hi + 1;
    // first guess by a multiplication (the loops below make it exact)
    long long k = (long long)floor((x - 0.5) * (1.0 / 2.328306e-10));
    k = k < lo ? lo : (k > hi ? hi : k);
    while (k > lo && kiss_real((int32_t)(k - 1)) >= x) --k;
    while (kiss_real((int32_t)k) < x) ++k;
    return k;
}

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

constexpr uint64_t KISS_M3 = 18000ull * 65536ull - 1ull;
constexpr uint64_t KISS_M4 = 30903ull * 65536ull - 1ull;

// Per-subcolumn jump constants (depend on n only): computed once per launch.
struct KissJump {
    uint32_t A, C;      // s1 -> A*s1 + C
    uint32_t a3n, a4n;  // s3 -> a3n*s3 mod m3, s4 -> a4n*s4 mod m4
};

__device__ inline KissJump kiss_jump_consts(uint64_t n) {
    KissJump J;
    uint32_t A = 1, C = 0, a = 69069u, c = 1327217885u;
    for (uint64_t m = n; m; m >>= 1) {
        if (m & 1) { A = a * A; C = a * C + c; }
        c = a * c + c;
        a = a * a;
    }
    J.A = A;
    J.C = C;
    J.a3n = (uint32_t)powmod(18000ull, n, KISS_M3);
    J.a4n = (uint32_t)powmod(30903ull, n, KISS_M4);
    return J;
}

// columns of M^n for the xorshift component, from the M^(2^k) table
__device__ inline void xorshift_power(uint64_t n, uint32_t* col) {
    for (int j = 0; j < 32; ++j) col[j] = 1u << j;
    for (int b = 0; n; ++b, n >>= 1) {
        if (!(n & 1)) continue;
        for (int j = 0; j < 32; ++j) {
            uint32_t y = col[j], r = 0;
            for (int i = 0; i < 32; ++i)
                if (y >> i & 1u) r ^= cT.xs_jump[b][i];
            col[j] = r;
        }
    }
}

__device__ inline uint32_t gf2_apply(const uint32_t* col, uint32_t y) {
    uint32_t r = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i)
        if (y >> i & 1u) r ^= col[i];
    return r;
}

// seed = int((pmid - int(pmid)) * 1e9), pmid in Pa (mcica:475-478)
__device__ inline uint32_t kiss_seed(double pmid) {
    const double frac = __dsub_rn(pmid, trunc(pmid));
    return (uint32_t)(int32_t)(long long)__dmul_rn(frac, 1000000000.0);
}

// position of subcolumn g's first draw in its column's stream
__device__ inline uint64_t kiss_offset(int icld, int g, int nlay, int permuteseed) {
    uint64_t n = (uint64_t)permuteseed;
    if (icld == 3) n += (uint64_t)g;
    else if (icld >= 4) n += 2ull * (uint64_t)g * (uint64_t)nlay;
    else n += (uint64_t)g * (uint64_t)nlay;
    return n;
}

__device__ inline Kiss kiss_start(const uint32_t* seed, const KissJump& J, const uint32_t* xcol) {
    Kiss k;
    k.s1 = J.A * seed[0] + J.C;
    k.s2 = gf2_apply(xcol, seed[1]);
    k.s3 = (uint32_t)mulmod(J.a3n, seed[2], KISS_M3);
    k.s4 = (uint32_t)mulmod(J.a4n, seed[3], KISS_M4);
    return k;
}

// getRandomReal (mcica_random_numbers.f90:276-295): u32 / (2^32 - 1) in FP64
__device__ inline double mt_real(uint32_t y) { return __ddiv_rn((double)y, 4294967295.0); }

// MT draws are carried as signed words, u32 ^ 2^31 (same order as the u32
// value), so both generators fit the same 32-bit mask state.
__device__ inline int32_t mt_signed(uint32_t u) { return (int32_t)(u ^ 0x80000000u); }

// Smallest signed MT draw d with mt_real(d ^ 2^31) >= x, in [-2^31, 2^31]:
// comparing the draw with it is the reference's FP64 comparison (mt_real is
// increasing).
__device__ inline long long mt_threshold(double x) {
    const long long hi = 4294967295ll;
    long long k;
    if (mt_real(0u) >= x) {
        k = 0;
    } else if (mt_real(0xffffffffu) < x) {
        k = hi + 1;
    } else {
        k = (long long)floor(x * 4294967295.0);
        k = k < 0 ? 0 : (k > hi ? hi : k);
        while (k > 0 && mt_real((uint32_t)(k - 1)) >= x) --k;
        while (mt_real((uint32_t)k) < x) ++k;
    }
    return k - 2147483648ll;
}

// position of (subcolumn g, column col)'s first draw in the MT stream of a
// call: one stream in (subcolumn, column, layer) order (mcica_subcol_gen_sw.f90
// MT branch), two draws per layer for icld 4/5, one per column for icld 3
__device__ inline size_t mt_offset(int icld, int g, int col, int ncol, int nlay) {
    const size_t sc = (size_t)g * (size_t)ncol + (size_t)col;
    if (icld == 3) return sc;
    if (icld >= 4) return 2 * sc * (size_t)nlay;
    return sc * (size_t)nlay;
}

// Subcolumn cloud mask walked bottom -> top (generate_stochastic_clouds_sw,
// mcica_subcol_gen_sw.f90:492-659; icld 4/5 in the single-column
// generator's order, mcica_subcol_gen_sw.1col.f90:536-604).  Draws come from
// the KISS state (MT = false, irng 0) or from this subcolumn's run of a
// precomputed MT stream (MT = true, irng 1), whose address the KISS words
// hold (s1, s2) with the next layer's draws (s3, s4), loaded one layer
// ahead.  icld 1/3/4/5 compare the draws with per-layer thresholds (kc:
// 1 - cldf, ka: alpha, from kiss_threshold or mt_threshold); icld 2
// rescales the CDF in FP64.
template <bool MT>
struct McicaMask {
    Kiss k;
    int icld;
    int32_t prev, d0;
    double cdf_prev, omcf_prev;
    __device__ const uint32_t* run() const {
        return (const uint32_t*)(((uint64_t)k.s2 << 32) | (uint64_t)k.s1);
    }
    // MT draws of layer lay (two for icld 4/5: the run starts at an even
    // word, so the pair is 8-byte aligned).  The stream buffer carries two
    // words of padding, so the read one layer past the last run stays inside.
    __device__ void fetch(int lay) {
        const uint32_t* r = run();
        if (icld >= 4) {
            const uint2 v = __ldg((const uint2*)r + (lay - 1));
            k.s3 = v.x;
            k.s4 = v.y;
        } else {
            k.s3 = __ldg(r + (lay - 1));
        }
    }
    __device__ void start(const Kiss& k0, int icld_, const uint32_t* mt = nullptr) {
        icld = icld_;
        prev = 0;
        cdf_prev = 0.0;
        omcf_prev = 1.0;
        if constexpr (MT) {
            k.s1 = (uint32_t)(uint64_t)mt;
            k.s2 = (uint32_t)((uint64_t)mt >> 32);
            d0 = 0;
            if (icld == 3) d0 = mt_signed(__ldg(mt));
            else fetch(1);
        } else {
            k = k0;
            d0 = icld == 3 ? k.next_int() : 0;
        }
    }
    __device__ bool step(int lay, long long kc, long long ka, double omcf) {
        if constexpr (MT) {
            int32_t d = 0, d2 = 0;
            if (icld != 3) {
                d = mt_signed(k.s3);
                d2 = mt_signed(k.s4);
                fetch(lay + 1);
            }
            if (icld == 2) {
                double cdf = mt_real((uint32_t)d ^ 0x80000000u);
                if (lay >= 2) {
                    if (cdf_prev > omcf_prev) cdf = cdf_prev;
                    else cdf = __dmul_rn(cdf, omcf_prev);
                }
                cdf_prev = cdf;
                omcf_prev = omcf;
                return cdf >= omcf;
            }
            if (icld == 3) d = d0;
            else if (icld >= 4 && lay >= 2 && (long long)d2 < ka) d = prev;
            prev = d;
            return (long long)d >= kc;
        } else {
            if (icld == 2) {
                double cdf = kiss_real(k.next_int());
                if (lay >= 2) {
                    if (cdf_prev > omcf_prev) cdf = cdf_prev;
                    else cdf = __dmul_rn(cdf, omcf_prev);
                }
                cdf_prev = cdf;
                omcf_prev = omcf;
                return cdf >= omcf;
            }
            int32_t d;
            if (icld == 3) {
                d = d0;
            } else if (icld >= 4) {
                d = k.next_int();
                const int32_t d2 = k.next_int();
                if (lay >= 2 && (long long)d2 < ka) d = prev;
            } else {
                d = k.next_int();
            }
            prev = d;
            return (long long)d >= kc;
        }
    }
};

}  // namespace rrsw
