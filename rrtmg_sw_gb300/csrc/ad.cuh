// ad.cuh -- tangent-linear and adjoint of the column solve (FP64).
//
// Objective per column (total sky, rrtmg_sw_rad.f90:822-836):
//   J = w_toa_up * swuflx(top) + w_sfc_net * (swdflx(sfc) - swuflx(sfc))
//     + w_hr_sum * sum over layers 1..nlay-1 of swhr,
// differentiated with respect to tlay, h2ovmr, o3vmr, the McICA cloud
// water paths clwp, ciwp (masks frozen: they depend on cldfrac and the seeds
// only) and the four surface albedos.
//
// The model differentiated is the reference's with exp(-x) in place of the
// nearest-entry transmittance table and of its quadratic below od_lo
// (rrtmg_sw_reftra.f90:203-209, spcvmc:558-585): the table makes the
// reference piecewise constant in every optical depth, so its derivative is
// zero almost everywhere.  The value J returned is that of the smooth model,
// which is what finite differences of this entry point check.
//
// Structure (per column pair; one thread per (column, g-point)):
//   prep     setcoef_sw per layer with derivatives w.r.t. (tlay, h2ovmr, o3vmr)
//   pass 1   per cell (g-point, layer): gas optics, cloud optics and the
//            two-stream solution as 5-direction duals (tlay, h2ovmr, o3vmr,
//            clwp, ciwp of that layer) -- the cell's local Jacobian -- and the
//            up-sweep of vrtqdr_sw in FP64
//   pass 2   down-sweep and level fluxes; J is linear in each g-point's
//            fluxes, so its seeds are known per level
//   reverse  adjoint of the down-sweep (bottom to top), then of the up-sweep
//            (top to bottom); each cell's adjoint times its Jacobian is summed
//            over g-points into the layer's gradient.
// The tangent-linear mode runs the same forward with the Jacobians contracted
// with a direction and propagates tangents through both sweeps.
#pragma once

#include "kernel.cuh"

namespace rrsw {

// ---------------------------------------------------------------- duals
template <int N>
struct Dual {
    double v;
    double d[N];
    __host__ __device__ Dual() : v(0.0) {
        for (int i = 0; i < N; ++i) d[i] = 0.0;
    }
    __host__ __device__ Dual(double x) : v(x) {
        for (int i = 0; i < N; ++i) d[i] = 0.0;
    }
    __host__ __device__ explicit operator int() const { return (int)v; }
};
template <int N>
struct TabOf<Dual<N>> { typedef double type; };

#define DUAL_BIN(OP, VAL, DER)                                                                   \
    template <int N>                                                                             \
    __device__ inline Dual<N> operator OP(const Dual<N>& a, const Dual<N>& b) {                  \
        Dual<N> r;                                                                               \
        r.v = VAL;                                                                               \
        for (int i = 0; i < N; ++i) r.d[i] = DER;                                                \
        return r;                                                                                \
    }                                                                                            \
    template <int N>                                                                             \
    __device__ inline Dual<N> operator OP(const Dual<N>& a, double bv) { return a OP Dual<N>(bv); } \
    template <int N>                                                                             \
    __device__ inline Dual<N> operator OP(double av, const Dual<N>& b) { return Dual<N>(av) OP b; }
DUAL_BIN(+, a.v + b.v, a.d[i] + b.d[i])
DUAL_BIN(-, a.v - b.v, a.d[i] - b.d[i])
DUAL_BIN(*, a.v * b.v, a.d[i] * b.v + a.v * b.d[i])
DUAL_BIN(/, a.v / b.v, (a.d[i] - (a.v / b.v) * b.d[i]) / b.v)
#undef DUAL_BIN

template <int N>
__device__ inline Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r;
    r.v = -a.v;
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int N>
__device__ inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N>
__device__ inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { a = a - b; return a; }
template <int N>
__device__ inline Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { a = a * b; return a; }

#define DUAL_CMP(OP)                                                                                    \
    template <int N>                                                                                    \
    __device__ inline bool operator OP(const Dual<N>& a, const Dual<N>& b) { return a.v OP b.v; }       \
    template <int N>                                                                                    \
    __device__ inline bool operator OP(const Dual<N>& a, double b) { return a.v OP b; }                 \
    template <int N>                                                                                    \
    __device__ inline bool operator OP(double a, const Dual<N>& b) { return a OP b.v; }
DUAL_CMP(<)
DUAL_CMP(<=)
DUAL_CMP(>)
DUAL_CMP(>=)
DUAL_CMP(==)
DUAL_CMP(!=)
#undef DUAL_CMP

template <int N>
__device__ inline Dual<N> sqrt(const Dual<N>& a) {
    Dual<N> r;
    r.v = ::sqrt(a.v);
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / (2.0 * r.v);
    return r;
}
template <int N>
__device__ inline Dual<N> exp(const Dual<N>& a) {
    Dual<N> r;
    r.v = ::exp(a.v);
    for (int i = 0; i < N; ++i) r.d[i] = r.v * a.d[i];
    return r;
}
template <int N>
__device__ inline Dual<N> log(const Dual<N>& a) {
    Dual<N> r;
    r.v = ::log(a.v);
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v;
    return r;
}
template <int N>
__device__ inline Dual<N> fmin(const Dual<N>& a, double b) { return a.v <= b ? a : Dual<N>(b); }

template <> __device__ inline Dual<3> c_oneminus<Dual<3>>() { return Dual<3>(cT.oneminus); }
template <> __device__ inline Dual<5> c_oneminus<Dual<5>>() { return Dual<5>(cT.oneminus); }
template <> __device__ inline Dual<3> c_bpade<Dual<3>>() { return Dual<3>(cT.bpade); }
template <> __device__ inline Dual<5> c_bpade<Dual<5>>() { return Dual<5>(cT.bpade); }

__device__ inline double val(double x) { return x; }
template <int N>
__device__ inline double val(const Dual<N>& x) { return x.v; }

// Dual<5> holding the value and derivatives of a Dual<3> in its first slots
__device__ inline Dual<5> widen(const Dual<3>& a) {
    Dual<5> r(a.v);
    r.d[0] = a.d[0]; r.d[1] = a.d[1]; r.d[2] = a.d[2];
    return r;
}

// ------------------------------------------------- setcoef with derivatives
// inatm_sw (rrtmg_sw_rad.f90:1527-1586) and setcoef_sw
// (rrtmg_sw_setcoef.f90:158-301) for one (column, layer) with derivatives
// with respect to (tlay, h2ovmr, o3vmr) of that layer; the indices are those
// of the values.  Writes the NFR coefficients (Dual<3>, [NFR] with stride L
// starting at cf) and the packed indices; returns the layer's pressure
// thickness.
__device__ inline double prep_layer_dual(const SolveParams& P, int col, int lay, Dual<3>* cf, int L, int* pk,
                                         const double* __restrict__ tab64) {
    typedef Dual<3> D;
    const int i = lay - 1;
    const size_t n = (size_t)P.ncol;
    const size_t k = (size_t)col + n * (size_t)i;
    const double p = P.play[k];
    D t(P.tlay[k]);
    t.d[0] = 1.0;
    D h2o(P.h2ovmr[k]);
    h2o.d[1] = 1.0;
    D o3(P.o3vmr[k]);
    o3.d[2] = 1.0;
    const double pzb = P.plev[k], pzt = P.plev[k + n];
    const double amd = 28.9660, amw = 18.0160, avogad = 6.02214199e+23, grav = 9.8066;
    const D amm = (1.0 - h2o) * amd + h2o * amw;
    const D coldry = ((pzb - pzt) * 1.e3 * avogad) / ((1.e2 * grav) * amm * (1.0 + h2o));
    const D w0 = coldry * h2o, w2 = coldry * o3;
    const D w1 = coldry * P.co2vmr[k], w5 = coldry * P.ch4vmr[k], w6 = coldry * P.o2vmr[k];
    const double pdp = pzb - pzt;
    const double stpfac = 296.0 / 1013.0;
    const double plog = ::log(p);
    int jp = (int)(36.0 - 5.0 * (plog + 0.04));
    jp = jp < 1 ? 1 : (jp > 58 ? 58 : jp);
    const double fp = 5.0 * (ldt(tab64, cT.preflog + jp - 1) - plog);
    const double tr0 = ldt(tab64, cT.tref + jp - 1), tr1 = ldt(tab64, cT.tref + jp);
    int jt = (int)(3.0 + (t.v - tr0) / 15.0);
    jt = jt < 1 ? 1 : (jt > 4 ? 4 : jt);
    const D ft = (t - tr0) / 15.0 - (double)(jt - 3);
    int jt1 = (int)(3.0 + (t.v - tr1) / 15.0);
    jt1 = jt1 < 1 ? 1 : (jt1 > 4 ? 4 : jt1);
    const D ft1 = (t - tr1) / 15.0 - (double)(jt1 - 3);
    const D water = w0 / coldry;
    const D scalefac = (p * stpfac) / t;
    D forfac, forfrac, selffac, selffrac;
    int indfor, indself, low;
    if (plog > 4.56) {
        low = 1;
        forfac = scalefac / (1.0 + water);
        D factor = (332.0 - t) / 36.0;
        indfor = (int)factor;
        indfor = indfor < 1 ? 1 : (indfor > 2 ? 2 : indfor);
        forfrac = factor - (double)indfor;
        selffac = water * forfac;
        factor = (t - 188.0) / 7.2;
        indself = (int)factor - 7;
        indself = indself < 1 ? 1 : (indself > 9 ? 9 : indself);
        selffrac = factor - (double)(indself + 7);
    } else {
        low = 0;
        forfac = scalefac / (1.0 + water);
        const D factor = (t - 188.0) / 36.0;
        indfor = 3;
        forfrac = factor - 1.0;
        selffac = D(0.0);
        selffrac = D(0.0);
        indself = 0;
    }
    const D colh2o = 1.e-20 * w0;
    D colco2 = 1.e-20 * w1, colo3 = 1.e-20 * w2, colch4 = 1.e-20 * w5, colo2 = 1.e-20 * w6;
    const D colmol = 1.e-20 * coldry + colh2o;
    if (colco2 == 0.0) colco2 = 1.e-32 * coldry;
    if (colch4 == 0.0) colch4 = 1.e-32 * coldry;
    if (colo2 == 0.0) colo2 = 1.e-32 * coldry;
    const double compfp = 1.0 - fp;
    cf[F_FAC10 * L + i] = compfp * ft;
    cf[F_FAC00 * L + i] = compfp * (1.0 - ft);
    cf[F_FAC11 * L + i] = fp * ft1;
    cf[F_FAC01 * L + i] = fp * (1.0 - ft1);
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
    cf[F_PDP * L + i] = D(pdp);
    pk[i] = jp | (jt << 8) | (jt1 << 12) | (indself << 16) | (indfor << 24) | (low << 30);
    return pdp;
}

// --------------------------------------------------- smooth two-stream
// reftra_sw (rrtmg_sw_reftra.f90:151-326), kmodts = 2, with exp(-x) for
// every transmittance; T is double or a dual.
template <typename T>
struct RTs { T ref, refd, tra, trad; };

template <typename T>
__device__ inline RTs<T> reftra_sm(T zto1, T zw, T zg, double prmuz) {
    RTs<T> o;
    const double zwcrit = 0.9999995, eps = 1.e-08;
    const T zg3 = 3.0 * zg;
    const T zgamma1 = (8.0 - zw * (5.0 + zg3)) * 0.25;
    const T zgamma2 = 3.0 * (zw * (1.0 - zg)) * 0.25;
    const T zgamma3 = (2.0 - zg3 * prmuz) * 0.25;
    const T zgamma4 = 1.0 - zgamma3;
    T zwo(0.0), denom(1.0);
    if (zg != 1.0) {
        const T q = zg / (1.0 - zg);
        denom = 1.0 - (1.0 - zw) * (q * q);
    }
    if (zw > 0.0 && denom != 0.0) zwo = zw / denom;
    if (zwo >= zwcrit) {
        const T za1 = zgamma1 * prmuz - zgamma3;
        const T zgt = zgamma1 * zto1;
        const T ze2 = exp(-fmin(zto1 / prmuz, 500.0));
        o.ref = (zgt - za1 * (1.0 - ze2)) / (1.0 + zgt);
        o.tra = 1.0 - o.ref;
        o.refd = zgt / (1.0 + zgt);
        o.trad = 1.0 - o.refd;
        if (ze2 == 1.0) { o.ref = T(0.0); o.tra = T(1.0); o.refd = T(0.0); o.trad = T(1.0); }
        return o;
    }
    const T za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
    const T za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
    const T zrk = sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
    const T zrp = zrk * prmuz;
    const T zrp1 = 1.0 + zrp, zrm1 = 1.0 - zrp;
    const T zrk2 = 2.0 * zrk;
    const T zrpp = 1.0 - zrp * zrp;
    const T zrkg = zrk + zgamma1;
    const T zr1 = zrm1 * (za2 + zrk * zgamma3);
    const T zr2 = zrp1 * (za2 - zrk * zgamma3);
    const T zr3 = zrk2 * (zgamma3 - za2 * prmuz);
    const T zr4 = zrpp * zrkg;
    const T zr5 = zrpp * (zrk - zgamma1);
    const T zt1 = zrp1 * (za1 + zrk * zgamma4);
    const T zt2 = zrm1 * (za1 - zrk * zgamma4);
    const T zt3 = zrk2 * (zgamma4 + za1 * prmuz);
    const T zbeta = (zgamma1 - zrk) / zrkg;
    const T zem1 = exp(-fmin(zrk * zto1, 500.0));
    const T zep1 = 1.0 / zem1;
    const T zem2 = exp(-fmin(zto1 / prmuz, 500.0));
    const T zep2 = 1.0 / zem2;
    const T zdenr = zr4 * zep1 + zr5 * zem1;
    if (zdenr >= -eps && zdenr <= eps) {
        o.ref = T(eps);
        o.tra = zem2;
    } else {
        o.ref = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
        o.tra = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdenr;
    }
    const T zemm = zem1 * zem1;
    const T zdend = 1.0 / ((1.0 - zbeta * zemm) * zrkg);
    o.refd = zgamma2 * (1.0 - zemm) * zdend;
    o.trad = zrk2 * zem1 * zdend;
    return o;
}

// Total-sky optics of one cell for the objective (spcvmc:442-549 with the
// McICA cloud fraction 0 or 1): out[0..4] = pref, prefd, ptra, ptrad, zdbt.
template <typename T>
__device__ inline void cell_total(const CellIn<T>& ci, double prmu0, T out[5]) {
    T ztauc = ci.taur + ci.taug + ci.rta;
    T zomcc = ci.taur * 1.0 + ci.rta * ci.roa;
    T zgcc = ci.rga * ci.roa * ci.rta / zomcc;
    zomcc = zomcc / ztauc;
    const T zf = zgcc * zgcc;
    const T zwf = zomcc * zf;
    ztauc = (1.0 - zwf) * ztauc;
    zomcc = (zomcc - zwf) / (1.0 - zwf);
    zgcc = (zgcc - zf) / (1.0 - zf);
    T tau = ztauc, om = zomcc, g = zgcc;
    if (ci.cloudy) {
        const T ztauo = ztauc + ci.tc;
        T zomco = ztauc * zomcc + ci.tc * ci.oc;
        const T zgco = (ci.tc * ci.oc * ci.gc + ztauc * zomcc * zgcc) / zomco;
        zomco = zomco / ztauo;
        tau = ztauo;
        om = zomco;
        g = zgco;
    }
    const RTs<T> r = reftra_sm(tau, om, g, prmu0);
    out[0] = r.ref;
    out[1] = r.refd;
    out[2] = r.tra;
    out[3] = r.trad;
    out[4] = exp(-(tau / prmu0));
}

// ------------------------------------------------------------ AD kernel
// per-level scratch fields of one thread
enum { A_REF, A_REFD, A_TRA, A_TRAD, A_DBT, A_RUP, A_RUPD, A_TDBT, A_TDN, A_RDND,
       A_BREF, A_BREFD, A_BTRA, A_BTRAD, A_BDBT, A_BRUP, A_BRUPD, A_CLD, A_TRUP, A_TRUPD, A_JAC,
       A_NREC = A_JAC, A_NSTORE = A_JAC + 25 };

__host__ __device__ inline int ad_fields(int store) { return store ? A_NSTORE : A_NREC; }

// scratch elements (doubles) per CTA slot
__host__ __device__ inline size_t ad_slot_elems(int L, int store) {
    return (size_t)(L + 1) * ad_fields(store) * CTA_THREADS + (size_t)COLS_PER_CTA * NFR * L * 4;
}

struct AdSmem {
    size_t pk, pdp, hc, misc, kc, ka, omcf, cld, seed, xs, grad, galb, jsum, total;
};
__host__ __device__ inline AdSmem ad_smem_layout(int L) {
    AdSmem m;
    size_t o = 0;
    m.pk = o;   o = align16(o + COLS_PER_CTA * L * sizeof(int));
    m.pdp = o;  o = align16(o + COLS_PER_CTA * L * sizeof(double));
    m.hc = o;   o = align16(o + COLS_PER_CTA * L * sizeof(double));
    m.misc = o; o = align16(o + 8 * sizeof(int));
    m.kc = o;   o = align16(o + COLS_PER_CTA * L * sizeof(long long));
    m.ka = o;   o = align16(o + COLS_PER_CTA * L * sizeof(long long));
    m.omcf = o; o = align16(o + COLS_PER_CTA * L * sizeof(double));
    m.cld = o;  o = align16(o + COLS_PER_CTA * 4 * L * sizeof(double));
    m.seed = o; o = align16(o + COLS_PER_CTA * 4 * sizeof(uint32_t));
    m.xs = o;   o = align16(o + NGPT * 32 * sizeof(uint32_t));
    m.grad = o; o = align16(o + COLS_PER_CTA * L * 5 * sizeof(double));
    m.galb = o; o = align16(o + COLS_PER_CTA * 4 * sizeof(double));
    m.jsum = o; o = align16(o + COLS_PER_CTA * 2 * sizeof(double));
    m.total = o;
    return m;
}

// Optics of one cell with derivatives (pass 1 and the recomputing reverse
// pass).  Gas optics and aerosol depend on (tlay, h2ovmr, o3vmr) only, so
// they run in Dual<3> for every cell; a cloudy cell widens them to Dual<5>
// over (tlay, h2ovmr, o3vmr, clwp, ciwp) for cldprmc and the two-stream
// solution, a clear cell finishes in Dual<3> and is widened with zero
// water-path derivatives.  Each variant is compiled once (not inlined at
// its call sites): the kernel's instruction footprint, not its arithmetic,
// was what its warps waited on most.
__device__ inline Dual<5> widen5(const Dual<3>& a) { return widen(a); }

__device__ __noinline__ void ad_cell_clear(const CellIn<Dual<3>>& ci, double cossza, Dual<5> out[5]) {
    Dual<3> o[5];
    cell_total(ci, cossza, o);
    for (int k = 0; k < 5; ++k) out[k] = widen5(o[k]);
}

__device__ __noinline__ void ad_cell_cloudy(const SolveParams& P, const CellIn<Dual<3>>& c3, int col, int lay, int ib,
                                            const double* cld, int L, double cossza,
                                            const double* __restrict__ tab64, Dual<5> out[5]) {
    typedef Dual<5> D;
    CellIn<D> ci;
    ci.taug = widen5(c3.taug);
    ci.taur = widen5(c3.taur);
    ci.rta = widen5(c3.rta); ci.roa = widen5(c3.roa); ci.rga = widen5(c3.rga); ci.rcoa = widen5(c3.rcoa);
    ci.cloudy = true;
    ci.cldf = D(1.0);
    D ciwp(cld[0 * L + lay - 1]), clwp(cld[1 * L + lay - 1]);
    clwp.d[3] = 1.0;
    ciwp.d[4] = 1.0;
    const D rei(cld[2 * L + lay - 1]), rel(cld[3 * L + lay - 1]);
    D tc(0.0), oc(1.0), gc(0.0), fsfc(0.0), taor(0.0), coc(0.0);
    if (P.tauc) {
        const size_t kb = (size_t)ib + 14 * ((size_t)col + (size_t)P.ncol * (size_t)(lay - 1));
        tc = D(P.tauc[kb]); oc = D(P.ssac[kb]); gc = D(P.asmc[kb]); fsfc = D(P.fsfc[kb]);
    }
    cldprmc_g<D>(ib, P.inflag, P.iceflag, P.liqflag, D(1.0), ciwp, clwp, rei, rel, fsfc, tc, oc, gc, taor, coc,
                 tab64, P.err);
    ci.tc = tc; ci.oc = oc; ci.gc = gc; ci.coc = coc; ci.taor = taor;
    cell_total(ci, cossza, out);
}

__device__ __noinline__ void ad_cell(const SolveParams& P, const Dual<3>* coef3, const int* pk, int L, int laytrop,
                                     int col, int lay, int ib, int igb, bool cloudy, const double* cld,
                                     double cossza, const double* __restrict__ tab64, Dual<5> out[5]) {
    typedef Dual<3> D;
    D cf[NFR];
    for (int f = 0; f < NFR; ++f) cf[f] = coef3[f * L + lay - 1];
    const Coef<D> CN{cf, pk + lay - 1, 1, lay <= laytrop ? 1 : 0};
    CellIn<D> ci;
    taumol_g<D>(ib, igb, 1, CN, tab64, ci.taug, ci.taur);
    aerosol_in<D>(P, col, lay, ib, tab64, ci);
    ci.cloudy = false;
    ci.cldf = D(0.0);
    ci.tc = D(0.0); ci.oc = D(1.0); ci.gc = D(0.0); ci.coc = D(0.0); ci.taor = D(0.0);
    if (cloudy) ad_cell_cloudy(P, ci, col, lay, ib, cld, L, cossza, tab64, out);
    else ad_cell_clear(ci, cossza, out);
}

__global__ void __launch_bounds__(CTA_THREADS, 3)
k_adjoint(const SolveParams P, const AdParams A, const double* __restrict__ tab64) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = P.nlay;
    const AdSmem M = ad_smem_layout(L);
    int* sPk = (int*)(smem_raw + M.pk);
    double* sPdp = (double*)(smem_raw + M.pdp);
    double* sHc = (double*)(smem_raw + M.hc);
    int* sMisc = (int*)(smem_raw + M.misc);
    long long* sKc = (long long*)(smem_raw + M.kc);
    long long* sKa = (long long*)(smem_raw + M.ka);
    double* sOmcf = (double*)(smem_raw + M.omcf);
    double* sCld = (double*)(smem_raw + M.cld);
    uint32_t* sSeed = (uint32_t*)(smem_raw + M.seed);
    uint32_t* sXs = (uint32_t*)(smem_raw + M.xs);
    double* sGrad = (double*)(smem_raw + M.grad);
    double* sGalb = (double*)(smem_raw + M.galb);
    double* sJ = (double*)(smem_raw + M.jsum);

    const int tid = threadIdx.x;
    const int cc = thread_col<double>(tid), g = thread_g<double>(tid);
    const int ib = cT.ngb[g], igb = cT.gib[g];
    const bool nir = ib <= 8 || ib == 13;
    const bool fused = P.fused && P.icld >= 1;
    const int NA = ad_fields(A.store);
    double* slot = (double*)P.scratch + (size_t)blockIdx.x * P.slot_elems;
    Dual<3>* coef3 = (Dual<3>*)(slot + (size_t)(L + 1) * NA * CTA_THREADS);
    const size_t n = (size_t)P.ncol;
    const KissJump J = kiss_setup(P, sXs, g);

    for (int pair = blockIdx.x; pair < P.npairs; pair += gridDim.x) {
        __syncthreads();
        for (int i = tid; i < COLS_PER_CTA * L * 5; i += CTA_THREADS) sGrad[i] = 0.0;
        if (tid < COLS_PER_CTA * 4) sGalb[tid] = 0.0;
        if (tid < COLS_PER_CTA * 2) sJ[tid] = 0.0;
        // ---------------- prep
        for (int it = tid; it < COLS_PER_CTA * L; it += CTA_THREADS) {
            const int c2 = it / L, lay = it % L + 1;
            const int pcol = COLS_PER_CTA * pair + c2;
            const bool real = pcol < P.ncol;
            double pdp = 1.0;
            if (real) {
                pdp = prep_layer_dual(P, pcol, lay, coef3 + c2 * NFR * L, L, sPk + c2 * L, tab64);
            } else {
                for (int f = 0; f < NFR; ++f) coef3[c2 * NFR * L + f * L + lay - 1] = Dual<3>(0.0);
                sPk[c2 * L + lay - 1] = 1 | (1 << 8) | (1 << 12) | (1 << 16) | (1 << 24);
            }
            sPdp[c2 * L + lay - 1] = pdp;
            sHc[c2 * L + lay - 1] = cT.heatfac / pdp;
            const size_t kl = (size_t)pcol + n * (size_t)(lay - 1);
            double* cd = sCld + c2 * 4 * L;
            cd[0 * L + lay - 1] = real && P.icld >= 1 ? P.ciwp[kl] : 0.0;
            cd[1 * L + lay - 1] = real && P.icld >= 1 ? P.clwp[kl] : 0.0;
            cd[2 * L + lay - 1] = real && P.icld >= 1 ? P.rei[kl] : 0.0;
            cd[3 * L + lay - 1] = real && P.icld >= 1 ? P.rel[kl] : 0.0;
            if (fused) {
                double cf = real ? P.cldfrac[kl] : 0.0;
                if (cf < 1.0e-20) cf = 0.0;
                const double omcf = DS(1.0, cf);
                sOmcf[c2 * L + lay - 1] = omcf;
                sKc[c2 * L + lay - 1] = kiss_threshold(omcf);
                sKa[c2 * L + lay - 1] = (P.icld >= 4 && real) ? kiss_threshold(P.alpha[kl]) : 0ll;
                if (lay == 1) {
                    uint32_t* sd = sSeed + c2 * 4;
                    if (real) {
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
        }
        __syncthreads();
        if (g == 0) {
            int lt = 0;
            for (int i = 0; i < L; ++i) lt += (sPk[cc * L + i] >> 30) & 1;
            sMisc[cc] = lt;
        }
        __syncthreads();
        const int col = COLS_PER_CTA * pair + cc;
        const int laytrop = sMisc[cc];
        bool active = col < P.ncol;
        if (active && (laytrop < 1 || laytrop >= L)) {
            set_error(P.err, E_LAYTROP);
            active = false;
        }
        const Dual<3>* cf3 = coef3 + cc * NFR * L;
        const int* pk = sPk + cc * L;
        const double* cld = sCld + cc * 4 * L;
        double cossza = 1.0, albp = 0.0, albd = 0.0, talbp = 0.0, talbd = 0.0;
        Dual<3> zinc(0.0);
        int lsol = -1;
        McicaMask<false> mc;
        if (active) {
            cossza = P.coszen[col];
            if (cossza < 1.e-10) cossza = 1.e-10;
            albp = nir ? P.aldir[col] : P.asdir[col];
            albd = nir ? P.aldif[col] : P.asdif[col];
            if (A.tl) {
                talbp = A.dira[nir ? 2 : 0] ? A.dira[nir ? 2 : 0][col] : 0.0;
                talbd = A.dira[nir ? 3 : 1] ? A.dira[nir ? 3 : 1][col] : 0.0;
            }
            const Coef<Dual<3>> C3{cf3, pk, L, laytrop};
            zinc = Dual<3>(P.adjflux[ib]) * solar_source<Dual<3>>(ib, igb, C3, P, tab64) * cossza;
            lsol = solar_layer(ib, C3);
            if (fused) mc.start(kiss_start(sSeed + cc * 4, J, sXs + g * 32), P.icld);
        }
        auto at = [&](int jk, int fld) -> double& {  // level jk (1 = top .. L+1 = surface)
            return slot[((size_t)(jk - 1) * NA + fld) * CTA_THREADS + tid];
        };
        auto dirv = [&](int d, int lay) -> double {
            return A.dir[d] ? A.dir[d][(size_t)col + n * (size_t)(lay - 1)] : 0.0;
        };

        // ---------------- pass 1: cells and up-sweep, bottom -> top
        if (active) {
            double rup_b = albp, rupd_b = albd, trup_b = talbp, trupd_b = talbd;
            for (int lay = 1; lay <= L; ++lay) {
                const int jk = L + 1 - lay;
                bool cloudy = false;
                if (fused) cloudy = mc.step(lay, sKc[cc * L + lay - 1], sKa[cc * L + lay - 1], sOmcf[cc * L + lay - 1]);
                Dual<5> out[5];
                ad_cell(P, cf3, pk, L, laytrop, col, lay, ib, igb, cloudy, cld, cossza, tab64, out);
                for (int o = 0; o < 5; ++o) at(jk, A_REF + o) = out[o].v;
                at(jk, A_CLD) = cloudy ? 1.0 : 0.0;
                if (A.store)
                    for (int o = 0; o < 5; ++o)
                        for (int d = 0; d < 5; ++d) at(jk, A_JAC + 5 * o + d) = out[o].d[d];
                double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
                if (A.tl) {
                    double dv[5];
                    for (int d = 0; d < 5; ++d) dv[d] = dirv(d, lay);
                    for (int o = 0; o < 5; ++o) {
                        double s = 0.0;
                        for (int d = 0; d < 5; ++d) s += out[o].d[d] * dv[d];
                        t[o] = s;
                        at(jk, A_BREF + o) = s;  // tangent of the cell output
                    }
                }
                // up-sweep (vrtqdr:131-140) with tangents
                const double ref = out[0].v, refd = out[1].v, tra = out[2].v, trad = out[3].v, dbt = out[4].v;
                const double zr = 1.0 / (1.0 - rupd_b * refd);
                const double E = (tra - dbt) * rupd_b + dbt * rup_b;
                const double rup = ref + trad * E * zr;
                const double rupd = refd + trad * trad * rupd_b * zr;
                if (A.tl) {
                    const double tzr = zr * zr * (trupd_b * refd + rupd_b * t[1]);
                    const double tE = (t[2] - t[4]) * rupd_b + (tra - dbt) * trupd_b + t[4] * rup_b + dbt * trup_b;
                    const double trup = t[0] + t[3] * E * zr + trad * tE * zr + trad * E * tzr;
                    const double trupd = t[1] + 2.0 * trad * t[3] * rupd_b * zr + trad * trad * (trupd_b * zr + rupd_b * tzr);
                    trup_b = trup;
                    trupd_b = trupd;
                    at(jk, A_TRUP) = trup;
                    at(jk, A_TRUPD) = trupd;
                }
                rup_b = rup;
                rupd_b = rupd;
                at(jk, A_RUP) = rup;
                at(jk, A_RUPD) = rupd;
            }
        }

        // objective seeds of level m (0 = surface .. L = top), without zinc
        const double* hc = sHc + cc * L;
        auto seeds = [&](int m, double& sU, double& sD) {
            double an = 0.0;  // dJ/d net(m) through the heating-rate sum (layers 0 .. L-2)
            if (m >= 1 && m - 1 <= L - 2) an += A.w_hr * hc[m - 1];
            if (m <= L - 2) an -= A.w_hr * hc[m];
            sD = an + (m == 0 ? A.w_net : 0.0);
            sU = -an + (m == L ? A.w_toa : 0.0) - (m == 0 ? A.w_net : 0.0);
        };

        // ---------------- pass 2: down-sweep and level fluxes, top -> bottom
        double phi = 0.0, tphi = 0.0;
        if (active) {
            double tdbt = 1.0, tdn = 1.0, rdnd = 0.0, ttdbt = 0.0, ttdn = 0.0, trdnd = 0.0;
            for (int jk = 1; jk <= L + 1; ++jk) {
                const double rup = jk <= L ? at(jk, A_RUP) : albp, rupd = jk <= L ? at(jk, A_RUPD) : albd;
                at(jk, A_TDBT) = tdbt;
                at(jk, A_TDN) = tdn;
                at(jk, A_RDND) = rdnd;
                const double zr = 1.0 / (1.0 - rdnd * rupd);
                const double D = tdn - tdbt;
                const double Au = tdbt * rup + D * rupd;
                const double B = D + tdbt * rup * rdnd;
                const double fu = Au * zr, fd = tdbt + B * zr;
                double sU, sD;
                seeds(L + 1 - jk, sU, sD);
                phi += sU * fu + sD * fd;
                if (A.tl) {
                    const double trup = jk <= L ? at(jk, A_TRUP) : talbp, trupd = jk <= L ? at(jk, A_TRUPD) : talbd;
                    const double tzr = zr * zr * (trdnd * rupd + rdnd * trupd);
                    const double tD = ttdn - ttdbt;
                    const double tAu = ttdbt * rup + tdbt * trup + tD * rupd + D * trupd;
                    const double tB = tD + ttdbt * rup * rdnd + tdbt * trup * rdnd + tdbt * rup * trdnd;
                    const double tfu = tAu * zr + Au * tzr, tfd = ttdbt + tB * zr + B * tzr;
                    tphi += sU * tfu + sD * tfd;
                }
                if (jk <= L) {
                    const double ref = at(jk, A_REF), refd = at(jk, A_REFD), tra = at(jk, A_TRA), trad = at(jk, A_TRAD);
                    const double dbt = at(jk, A_DBT);
                    const double zr2 = 1.0 / (1.0 - refd * rdnd);
                    const double C = D + tdbt * ref * rdnd;
                    const double tdn1 = tdbt * tra + trad * C * zr2;
                    const double rdnd1 = refd + trad * trad * rdnd * zr2;
                    const double tdbt1 = dbt * tdbt;
                    if (A.tl) {
                        const double t0 = at(jk, A_BREF), t1 = at(jk, A_BREFD), t2 = at(jk, A_BTRA), t3 = at(jk, A_BTRAD);
                        const double t4 = at(jk, A_BDBT);
                        const double tzr2 = zr2 * zr2 * (t1 * rdnd + refd * trdnd);
                        const double tC = (ttdn - ttdbt) + ttdbt * ref * rdnd + tdbt * t0 * rdnd + tdbt * ref * trdnd;
                        const double ttdn1 = ttdbt * tra + tdbt * t2 + t3 * C * zr2 + trad * tC * zr2 + trad * C * tzr2;
                        const double trdnd1 = t1 + 2.0 * trad * t3 * rdnd * zr2 + trad * trad * (trdnd * zr2 + rdnd * tzr2);
                        const double ttdbt1 = t4 * tdbt + dbt * ttdbt;
                        ttdn = ttdn1;
                        trdnd = trdnd1;
                        ttdbt = ttdbt1;
                    }
                    tdn = tdn1;
                    rdnd = rdnd1;
                    tdbt = tdbt1;
                }
            }
            atomicAdd(&sJ[cc * 2 + 0], zinc.v * phi);
            if (A.tl) {
                double dz = 0.0;
                if (lsol >= 1)
                    for (int d = 0; d < 3; ++d) dz += zinc.d[d] * dirv(d, lsol);
                atomicAdd(&sJ[cc * 2 + 1], dz * phi + zinc.v * tphi);
            }
        }

        // ---------------- reverse: adjoint of the down-sweep (bottom -> top) and the up-sweep (top -> bottom)
        if (active && !A.tl) {
            const double zv = zinc.v;
            double a_tdbt = 0.0, a_tdn = 0.0, a_rdnd = 0.0, a_albp = 0.0, a_albd = 0.0;
            for (int jk = L + 1; jk >= 1; --jk) {
                const double tdbt = at(jk, A_TDBT), tdn = at(jk, A_TDN), rdnd = at(jk, A_RDND);
                const double rup = jk <= L ? at(jk, A_RUP) : albp, rupd = jk <= L ? at(jk, A_RUPD) : albd;
                double sU, sD;
                seeds(L + 1 - jk, sU, sD);
                const double afu = zv * sU, afd = zv * sD;
                const double zr = 1.0 / (1.0 - rdnd * rupd);
                const double D = tdn - tdbt;
                const double Au = tdbt * rup + D * rupd;
                const double B = D + tdbt * rup * rdnd;
                a_tdbt += afu * (rup - rupd) * zr + afd * (1.0 + (rup * rdnd - 1.0) * zr);
                a_tdn += afu * rupd * zr + afd * zr;
                a_rdnd += afu * Au * rupd * zr * zr + afd * (tdbt * rup * zr + B * rupd * zr * zr);
                const double a_rup = afu * tdbt * zr + afd * tdbt * rdnd * zr;
                const double a_rupd = afu * (D * zr + Au * rdnd * zr * zr) + afd * B * rdnd * zr * zr;
                if (jk == L + 1) {
                    a_albp += a_rup;
                    a_albd += a_rupd;
                } else {
                    at(jk, A_BRUP) = a_rup;
                    at(jk, A_BRUPD) = a_rupd;
                }
                if (jk >= 2) {
                    // state at level jk came from level jk-1 through layer jk-1 (vrtqdr:144-159)
                    const int lj = jk - 1;
                    const double t0 = at(lj, A_TDBT), n0 = at(lj, A_TDN), r0 = at(lj, A_RDND);
                    const double ref = at(lj, A_REF), refd = at(lj, A_REFD), tra = at(lj, A_TRA), trad = at(lj, A_TRAD);
                    const double dbt = at(lj, A_DBT);
                    const double zr2 = 1.0 / (1.0 - refd * r0);
                    const double C = (n0 - t0) + t0 * ref * r0;
                    const double b_tra = a_tdn * t0;
                    const double b_trad = a_tdn * C * zr2 + a_rdnd * 2.0 * trad * r0 * zr2;
                    const double b_ref = a_tdn * trad * t0 * r0 * zr2;
                    const double b_refd = a_tdn * trad * C * r0 * zr2 * zr2 + a_rdnd * (1.0 + trad * trad * r0 * r0 * zr2 * zr2);
                    const double b_dbt = a_tdbt * t0;
                    const double na_tdbt = a_tdn * (tra + trad * zr2 * (ref * r0 - 1.0)) + a_tdbt * dbt;
                    const double na_tdn = a_tdn * trad * zr2;
                    const double na_rdnd = a_tdn * trad * (t0 * ref * zr2 + C * refd * zr2 * zr2) +
                                           a_rdnd * trad * trad * (zr2 + r0 * refd * zr2 * zr2);
                    at(lj, A_BREF) = b_ref;
                    at(lj, A_BREFD) = b_refd;
                    at(lj, A_BTRA) = b_tra;
                    at(lj, A_BTRAD) = b_trad;
                    at(lj, A_BDBT) = b_dbt;
                    a_tdbt = na_tdbt;
                    a_tdn = na_tdn;
                    a_rdnd = na_rdnd;
                }
            }
            double c_rup = 0.0, c_rupd = 0.0;
            for (int jk = 1; jk <= L; ++jk) {
                const int lay = L + 1 - jk;
                const double ar = c_rup + at(jk, A_BRUP), ard = c_rupd + at(jk, A_BRUPD);
                const double rup_b = jk < L ? at(jk + 1, A_RUP) : albp, rupd_b = jk < L ? at(jk + 1, A_RUPD) : albd;
                const double ref = at(jk, A_REF), refd = at(jk, A_REFD), tra = at(jk, A_TRA), trad = at(jk, A_TRAD);
                const double dbt = at(jk, A_DBT);
                (void)ref;
                const double zr = 1.0 / (1.0 - rupd_b * refd);
                const double E = (tra - dbt) * rupd_b + dbt * rup_b;
                double b[5];
                b[0] = at(jk, A_BREF) + ar;
                b[1] = at(jk, A_BREFD) + ar * trad * E * rupd_b * zr * zr + ard * (1.0 + trad * trad * rupd_b * rupd_b * zr * zr);
                b[2] = at(jk, A_BTRA) + ar * trad * rupd_b * zr;
                b[3] = at(jk, A_BTRAD) + ar * E * zr + ard * 2.0 * trad * rupd_b * zr;
                b[4] = at(jk, A_BDBT) + ar * trad * (rup_b - rupd_b) * zr;
                c_rup = ar * trad * dbt * zr;
                c_rupd = ar * (trad * (tra - dbt) * zr + trad * E * refd * zr * zr) + ard * trad * trad * (zr + rupd_b * refd * zr * zr);
                double jac[25];
                if (A.store) {
                    for (int k = 0; k < 25; ++k) jac[k] = at(jk, A_JAC + k);
                } else {
                    Dual<5> out[5];
                    ad_cell(P, cf3, pk, L, laytrop, col, lay, ib, igb, at(jk, A_CLD) != 0.0, cld, cossza, tab64, out);
                    for (int o = 0; o < 5; ++o)
                        for (int d = 0; d < 5; ++d) jac[5 * o + d] = out[o].d[d];
                }
                for (int d = 0; d < 5; ++d) {
                    double s = 0.0;
                    for (int o = 0; o < 5; ++o) s += b[o] * jac[5 * o + d];
                    if (s != 0.0) atomicAdd(&sGrad[(cc * L + lay - 1) * 5 + d], s);
                }
            }
            a_albp += c_rup;
            a_albd += c_rupd;
            atomicAdd(&sGalb[cc * 4 + (nir ? 2 : 0)], a_albp);
            atomicAdd(&sGalb[cc * 4 + (nir ? 3 : 1)], a_albd);
            if (lsol >= 1)
                for (int d = 0; d < 3; ++d)
                    if (zinc.d[d] != 0.0) atomicAdd(&sGrad[(cc * L + lsol - 1) * 5 + d], phi * zinc.d[d]);
        }
        __syncthreads();
        // ---------------- outputs
        for (int it = tid; it < COLS_PER_CTA * L; it += CTA_THREADS) {
            const int c2 = it / L, l = it % L;
            const int ocol = COLS_PER_CTA * pair + c2;
            if (ocol >= P.ncol || A.tl) continue;
            const size_t o = (size_t)ocol + n * (size_t)l;
            for (int d = 0; d < 5; ++d)
                if (A.g[d]) A.g[d][o] = sGrad[(c2 * L + l) * 5 + d];
        }
        if (tid < COLS_PER_CTA) {
            const int ocol = COLS_PER_CTA * pair + tid;
            if (ocol < P.ncol) {
                if (A.J) A.J[ocol] = sJ[tid * 2 + 0];
                if (A.tl && A.dJ) {
                    double dj = sJ[tid * 2 + 1];
                    A.dJ[ocol] = dj;
                }
                if (!A.tl)
                    for (int a = 0; a < 4; ++a)
                        if (A.ga[a]) A.ga[a][ocol] = sGalb[tid * 4 + a];
            }
        }
    }
}

}  // namespace rrsw
