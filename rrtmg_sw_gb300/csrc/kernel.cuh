// kernel.cuh -- the fused solve kernel (see solve.cuh for the pieces).
#pragma once

#include "solve.cuh"

namespace rrsw {

constexpr int KLEV = 4;         // levels buffered per reduction round
constexpr int NQ_BASE = 6;      // fu, fd, cu, cd, fddir, cddir
constexpr int NQ_EXTRA = 14;    // + uvfd, uvcd, uvfddir, uvcddir, nifd, nicd, nifddir, nicddir

// scratch fields per level (pass 1 -> pass 2)
enum { S_REFC, S_REFDC, S_TRAC, S_TRADC, S_DBTC, S_RUPC, S_RUPDC,
       S_REF, S_REFD, S_TRA, S_TRAD, S_DBT, S_RUP, S_RUPD, S_DBTCN, S_DBTN, NS_MAX };

__device__ inline double DM(double a, double b) { return __dmul_rn(a, b); }
__device__ inline double DA(double a, double b) { return __dadd_rn(a, b); }
__device__ inline double DS(double a, double b) { return __dsub_rn(a, b); }

// inatm_sw (rrtmg_sw_rad.f90:1527-1586) and setcoef_sw
// (rrtmg_sw_setcoef.f90:158-301) for one (column, layer), in FP64 with
// explicit roundings so both arithmetic forms see identical indices.
template <typename R>
__device__ inline void prep_layer(const SolveParams& P, int col, int lay, R* cf, int* pk, double* pdp,
                                  int L, const double* __restrict__ tab64) {
    const int i = lay - 1;
    if (col >= P.ncol) {
        for (int f = 0; f < NFR; ++f) cf[f * L + i] = R(0);
        pk[i] = 1 | (1 << 8) | (1 << 12) | (1 << 16) | (1 << 24);
        pdp[i] = 1.0;
        return;
    }
    const size_t n = (size_t)P.ncol;
    const size_t k = (size_t)col + n * (size_t)i;
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
    const double fp = DM(5.0, DS(tab64[cT.preflog + jp - 1], plog));
    const double tr0 = tab64[cT.tref + jp - 1], tr1 = tab64[cT.tref + jp];
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
            const double rt = tab64[cT.rsrtaua + ib + 14 * ia], rp = tab64[cT.rsrpiza + ib + 14 * ia],
                         ra = tab64[cT.rsrasya + ib + 14 * ia];
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

template <typename R>
__device__ inline void warp_sum4(R& v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
}

template <typename R>
__global__ void __launch_bounds__(CTA_THREADS, 2)
k_solve(const SolveParams P, const R* __restrict__ tab, const double* __restrict__ tab64) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = P.nlay;
    const int NQ = P.extra ? NQ_EXTRA : NQ_BASE;
    double* sPdp = (double*)smem_raw;                      // [2][L]
    R* sCoef = (R*)(sPdp + COLS_PER_CTA * L);              // [2][NFR][L]
    int* sPk = (int*)(sCoef + COLS_PER_CTA * NFR * L);     // [2][L]
    int* sMisc = sPk + COLS_PER_CTA * L;                   // [4]
    size_t off = (size_t)((unsigned char*)(sMisc + 4) - smem_raw);
    off = (off + 15) & ~(size_t)15;
    R* sRed = (R*)(smem_raw + off);                        // [KLEV][NQ][224]
    R* sFlux = sRed + KLEV * NQ * CTA_THREADS;              // [2][NQ][L+1]

    const int tid = threadIdx.x;
    const int cc = tid / NGPT, g = tid % NGPT;
    const int ib = cT.ngb[g], igb = cT.gib[g];
    const bool uv = ib >= 9 && ib <= 12;  // bands 25-28 (spcvmc:629)
    const int NS = P.idelm == 0 ? NS_MAX : S_DBTCN;
    R* scr = (R*)P.scratch + (size_t)blockIdx.x * P.slot_elems;
    const size_t n = (size_t)P.ncol;

    for (int pair = blockIdx.x; pair < P.npairs; pair += gridDim.x) {
        __syncthreads();
        // ---------------- prep
        for (int it = tid; it < COLS_PER_CTA * L; it += CTA_THREADS) {
            const int c2 = it / L, lay = it % L + 1;
            prep_layer<R>(P, COLS_PER_CTA * pair + c2, lay, sCoef + c2 * NFR * L, sPk + c2 * L, sPdp + c2 * L, L, tab64);
        }
        __syncthreads();
        if (g == 0) {
            int lt = 0;
            for (int i = 0; i < L; ++i) lt += (sPk[cc * L + i] >> 30) & 1;
            sMisc[cc] = lt;
        }
        __syncthreads();
        const int col = COLS_PER_CTA * pair + cc;
        const Coef<R> C{sCoef + cc * NFR * L, sPk + cc * L, L, sMisc[cc]};
        bool active = col < P.ncol;
        if (active && (C.laytrop < 1 || C.laytrop >= L)) {
            set_error(P.err, E_LAYTROP);
            active = false;
        }

        // ---------------- per (column, g-point) setup
        double zincflx = 0.0, albp = 0.0, albd = 0.0, cossza = 1.0;
        McicaKiss mc;
        if (active) {
            cossza = P.coszen[col];
            if (cossza < 1.e-10) cossza = 1.e-10;
            const bool nir = ib <= 8 || ib == 13;
            albp = nir ? P.aldir[col] : P.asdir[col];
            albd = nir ? P.aldif[col] : P.asdif[col];
            zincflx = DM(DM(P.adjflux[ib], solar_source<R>(ib, igb, C, P, tab)), cossza);
            if (P.fused && P.icld >= 1) mc.init(P.play, n, col, g, L, P.icld, P.permuteseed, P.err);
        }
        const R prmu0 = (R)cossza;

        // ---------------- pass 1: bottom -> top
        R rupc_b = (R)albp, rupdc_b = (R)albd, rup_b = (R)albp, rupd_b = (R)albd;
        for (int lay = 1; lay <= L; ++lay) {
            const int jk = L + 1 - lay;
            R* sv = scr + (size_t)(jk - 1) * NS * CTA_THREADS + tid;
            if (!active) continue;
            R taug, taur;
            taumol_g<R>(ib, igb, lay, C, tab, taug, taur);
            double ta, oa, ga;
            aerosol(P, col, lay, ib, tab64, ta, oa, ga);
            // cloud of this subcolumn (McICA) at this layer
            double cldf = 0.0, ciwp = 0.0, clwp = 0.0, tauc = 0.0, ssac = 1.0, asmc = 0.0, fsfc = 0.0, rei = 0.0, rel = 0.0;
            if (P.icld >= 1) {
                const size_t kl = (size_t)col + n * (size_t)(lay - 1);
                if (P.fused) {
                    if (mc.step(lay, P.cldfrac[kl], P.icld >= 4 ? P.alpha[kl] : 0.0)) {
                        const size_t kb = (size_t)ib + 14 * kl;
                        cldf = 1.0;
                        ciwp = P.ciwp[kl];
                        clwp = P.clwp[kl];
                        if (P.tauc) {
                            tauc = P.tauc[kb];
                            ssac = P.ssac[kb];
                            asmc = P.asmc[kb];
                            fsfc = P.fsfc[kb];
                        }
                    }
                    rei = P.rei[kl];
                    rel = P.rel[kl];
                } else {
                    const size_t kg = (size_t)g + NGPT * kl;
                    cldf = P.cldfmcl[kg];
                    tauc = P.taucmcl[kg];
                    ssac = P.ssacmcl[kg];
                    asmc = P.asmcmcl[kg];
                    fsfc = P.fsfcmcl[kg];
                    ciwp = P.ciwpmcl[kg];
                    clwp = P.clwpmcl[kg];
                    rei = P.reicmcl[kl];
                    rel = P.relqmcl[kl];
                }
            }
            R tc = (R)tauc, oc = (R)ssac, gc = (R)asmc, taor = (R)tauc;
            if (P.icld >= 1)
                cldprmc_g<R>(ib, P.inflag, P.iceflag, P.liqflag, (R)cldf, (R)ciwp, (R)clwp, (R)rei, (R)rel, (R)fsfc,
                             tc, oc, gc, taor, tab, P.err);
            // clear-sky optics including aerosols (spcvmc:442-445)
            const R rta = (R)ta, roa = (R)oa, rga = (R)ga;
            R ztauc = taur + taug + rta;
            R zomcc = taur * R(1) + rta * roa;
            R zgcc = rga * roa * rta / zomcc;
            zomcc = zomcc / ztauc;
            const R zclear = R(1) - (R)cldf, zcloud = (R)cldf;
            if (P.idelm == 0) {
                const R zdbtmc = tbl_exp<R>(ztauc / prmu0, tab);
                const R tauorig = ztauc + taor;
                const R zdbtmo = tbl_exp<R>(tauorig / prmu0, tab);
                sv[S_DBTCN * CTA_THREADS] = zdbtmc;
                sv[S_DBTN * CTA_THREADS] = zclear * zdbtmc + zcloud * zdbtmo;
            }
            // delta scaling, clear (spcvmc:492-496)
            const R zf = zgcc * zgcc;
            const R zwf = zomcc * zf;
            ztauc = (R(1) - zwf) * ztauc;
            zomcc = (zomcc - zwf) / (R(1) - zwf);
            zgcc = (zgcc - zf) / (R(1) - zf);
            const RT<R> rc = reftra_g<R>(ztauc, zomcc, zgcc, prmu0, tab);
            const R zdbtc = tbl_exp<R>(ztauc / prmu0, tab);
            RT<R> rt = rc;
            R zdbt = zdbtc;
            if (cldf != 0.0) {
                // total sky: clear + delta-scaled cloud (spcvmc:500-505), reftra
                // only where cldf > repclc (:427), mixed by cloud fraction (:546-549)
                const R ztauo = ztauc + tc;
                R zomco = ztauc * zomcc + tc * oc;
                const R zgco = (tc * oc * gc + ztauc * zomcc * zgcc) / zomco;
                zomco = zomco / ztauo;
                RT<R> ro;
                if (cldf > 1.e-12) ro = reftra_g<R>(ztauo, zomco, zgco, prmu0, tab);
                else { ro.ref = R(0); ro.tra = R(1); ro.refd = R(0); ro.trad = R(1); }
                rt.ref = zclear * rc.ref + zcloud * ro.ref;
                rt.refd = zclear * rc.refd + zcloud * ro.refd;
                rt.tra = zclear * rc.tra + zcloud * ro.tra;
                rt.trad = zclear * rc.trad + zcloud * ro.trad;
                const R zdbtmo = tbl_exp<R>(ztauo / prmu0, tab);
                zdbt = zclear * zdbtc + zcloud * zdbtmo;
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
            sv[S_REFC * CTA_THREADS] = rc.ref;
            sv[S_REFDC * CTA_THREADS] = rc.refd;
            sv[S_TRAC * CTA_THREADS] = rc.tra;
            sv[S_TRADC * CTA_THREADS] = rc.trad;
            sv[S_DBTC * CTA_THREADS] = zdbtc;
            sv[S_RUPC * CTA_THREADS] = rupc_b;
            sv[S_RUPDC * CTA_THREADS] = rupdc_b;
            sv[S_REF * CTA_THREADS] = rt.ref;
            sv[S_REFD * CTA_THREADS] = rt.refd;
            sv[S_TRA * CTA_THREADS] = rt.tra;
            sv[S_TRAD * CTA_THREADS] = rt.trad;
            sv[S_DBT * CTA_THREADS] = zdbt;
            sv[S_RUP * CTA_THREADS] = rup_b;
            sv[S_RUPD * CTA_THREADS] = rupd_b;
        }

        // ---------------- pass 2: top -> bottom, level fluxes and g sums
        R tdbtc = R(1), tdnc = R(1), rdndc = R(0);
        R tdbt = R(1), tdn = R(1), rdnd = R(0);
        R tdbtcn = R(1), tdbtn = R(1);
        const R zinc = (R)zincflx;
        for (int jk = 1; jk <= L + 1; ++jk) {
            R q[NQ_EXTRA];
#pragma unroll
            for (int i = 0; i < NQ_EXTRA; ++i) q[i] = R(0);
            R refc = R(0), refdc = R(0), trac = R(0), tradc = R(0), dbtc = R(0), rupc, rupdc;
            R ref = R(0), refd = R(0), tra = R(0), trad = R(0), dbt = R(0), rup, rupd, dbtcn = R(0), dbtn = R(0);
            if (jk <= L) {
                const R* sv = scr + (size_t)(jk - 1) * NS * CTA_THREADS + tid;
                refc = sv[S_REFC * CTA_THREADS]; refdc = sv[S_REFDC * CTA_THREADS];
                trac = sv[S_TRAC * CTA_THREADS]; tradc = sv[S_TRADC * CTA_THREADS];
                dbtc = sv[S_DBTC * CTA_THREADS];
                rupc = sv[S_RUPC * CTA_THREADS]; rupdc = sv[S_RUPDC * CTA_THREADS];
                ref = sv[S_REF * CTA_THREADS]; refd = sv[S_REFD * CTA_THREADS];
                tra = sv[S_TRA * CTA_THREADS]; trad = sv[S_TRAD * CTA_THREADS];
                dbt = sv[S_DBT * CTA_THREADS];
                rup = sv[S_RUP * CTA_THREADS]; rupd = sv[S_RUPD * CTA_THREADS];
                if (P.idelm == 0) { dbtcn = sv[S_DBTCN * CTA_THREADS]; dbtn = sv[S_DBTN * CTA_THREADS]; }
            } else {
                rupc = (R)albp; rupdc = (R)albd; rup = (R)albp; rupd = (R)albd;
            }
            if (active) {
                // level fluxes (vrtqdr:163-169)
                const R zrc = R(1) / (R(1) - rdndc * rupdc);
                const R cu = (tdbtc * rupc + (tdnc - tdbtc) * rupdc) * zrc;
                const R cd = tdbtc + (tdnc - tdbtc + tdbtc * rupc * rdndc) * zrc;
                const R zrt = R(1) / (R(1) - rdnd * rupd);
                const R fu = (tdbt * rup + (tdn - tdbt) * rupd) * zrt;
                const R fd = tdbt + (tdn - tdbt + tdbt * rup * rdnd) * zrt;
                const R dirf = P.idelm == 0 ? tdbtn : tdbt;
                const R dirc = P.idelm == 0 ? tdbtcn : tdbtc;
                q[0] = zinc * fu;
                q[1] = zinc * fd;
                q[2] = zinc * cu;
                q[3] = zinc * cd;
                q[4] = zinc * dirf;
                q[5] = zinc * dirc;
                if (P.extra) {
                    if (uv) { q[6] = q[1]; q[7] = q[3]; q[8] = q[4]; q[9] = q[5]; }
                    else { q[10] = q[1]; q[11] = q[3]; q[12] = q[4]; q[13] = q[5]; }
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
            const int slot = (jk - 1) % KLEV;
#pragma unroll
            for (int i = 0; i < NQ_EXTRA; ++i)
                if (i < NQ) sRed[(slot * NQ + i) * CTA_THREADS + tid] = q[i];
            if (slot == KLEV - 1 || jk == L + 1) {
                __syncthreads();
                const int nlev = slot + 1;
                const int items = COLS_PER_CTA * NQ * nlev;
                for (int base = 0; base < items * 4; base += CTA_THREADS) {
                    const int t = base + tid;
                    const int item = t >> 2, part = t & 3;
                    R v = R(0);
                    int c2 = 0, qi = 0, s = 0;
                    if (item < items) {
                        c2 = item / (NQ * nlev);
                        qi = (item / nlev) % NQ;
                        s = item % nlev;
                        const R* src = sRed + (s * NQ + qi) * CTA_THREADS + c2 * NGPT + part * 28;
                        for (int j = 0; j < 28; ++j) v += src[j];
                    }
                    warp_sum4(v);
                    if (item < items && part == 0) {
                        const int jl = jk - slot + s;  // level (1 = top)
                        sFlux[(c2 * NQ + qi) * (L + 1) + (L + 1 - jl)] = v;
                    }
                }
                __syncthreads();
            }
        }

        // ---------------- outputs (level 0 = surface)
        for (int it = tid; it < COLS_PER_CTA * (L + 1); it += CTA_THREADS) {
            const int c2 = it / (L + 1), l = it % (L + 1);
            const int ocol = COLS_PER_CTA * pair + c2;
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
                    const double fu1 = (double)F[0 * (L + 1) + l + 1], fd1 = (double)F[1 * (L + 1) + l + 1];
                    const double cu1 = (double)F[2 * (L + 1) + l + 1], cd1 = (double)F[3 * (L + 1) + l + 1];
                    const double zdpgcp = cT.heatfac / pdp[l];
                    hrc = DM(DS(DS(cd1, cu1), DS(cd, cu)), zdpgcp);
                    hr = DM(DS(DS(fd1, fu1), DS(fd, fu)), zdpgcp);
                }
                P.swhr[o] = hr;
                P.swhrc[o] = hrc;
            }
            if (P.extra) {
                const double fddir = (double)F[4 * (L + 1) + l];
                const double uvfd = (double)F[6 * (L + 1) + l], uvfddir = (double)F[8 * (L + 1) + l];
                const double nifd = (double)F[10 * (L + 1) + l], nifddir = (double)F[12 * (L + 1) + l];
                const double vals[8] = {fddir, DS(fd, fddir), uvfd, nifd, uvfddir, DS(uvfd, uvfddir), nifddir,
                                        DS(nifd, nifddir)};
                for (int x = 0; x < 8; ++x)
                    if (P.xout[x]) P.xout[x][o] = vals[x];
            }
        }
    }
}

}  // namespace rrsw
