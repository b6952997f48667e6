// kernel.cuh -- the fused solve kernel (see solve.cuh for the pieces).
#pragma once

#include "solve.cuh"

namespace rrsw {

constexpr int KLEV = 4;         // levels buffered per reduction round
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

// FP32 form: when the FP32 estimate of 1 - zwo for a cloudy layer lies
// within 3e-5 (relative) of the switch 1 - zwcrit = 5e-7, the reference's
// discontinuous conservative/non-conservative choice (reftra:188) is made
// again from FP64 cloud optics (cldprmc in FP64 from the FP64 inputs) and
// the co-albedo, so thick clouds take the reference's branch.
static __device__ __noinline__ int decide_conservative64(const SolveParams& P, int col, int g, int lay, int ib, float ztauc,
                                                  float zomcc, float zgcc, float zcoc, const double* __restrict__ tab64) {
    const size_t n = (size_t)P.ncol;
    const size_t kl = (size_t)col + n * (size_t)(lay - 1);
    double cldf = 1.0, ciwp, clwp, rei, rel, tauc = 0.0, ssac = 1.0, asmc = 0.0, fsfc = 0.0;
    if (P.fused) {
        ciwp = P.ciwp[kl]; clwp = P.clwp[kl]; rei = P.rei[kl]; rel = P.rel[kl];
        if (P.tauc) {
            const size_t kb = (size_t)ib + 14 * kl;
            tauc = P.tauc[kb]; ssac = P.ssac[kb]; asmc = P.asmc[kb]; fsfc = P.fsfc[kb];
        }
    } else {
        const size_t kg = (size_t)g + NGPT * kl;
        cldf = P.cldfmcl[kg]; tauc = P.taucmcl[kg]; ssac = P.ssacmcl[kg]; asmc = P.asmcmcl[kg];
        fsfc = P.fsfcmcl[kg]; ciwp = P.ciwpmcl[kg]; clwp = P.clwpmcl[kg];
        rei = P.reicmcl[kl]; rel = P.relqmcl[kl];
    }
    double taor, coc;
    cldprmc_g<double>(ib, P.inflag, P.iceflag, P.liqflag, cldf, ciwp, clwp, rei, rel, fsfc, tauc, ssac, asmc, taor,
                      coc, tab64, nullptr);
    const double tc = (double)ztauc, oc = (double)zomcc, gcl = (double)zgcc;
    const double ztauo = tc + tauc;
    const double scat = tc * oc + tauc * ssac;
    const double zgco = (tauc * ssac * asmc + tc * oc * gcl) / scat;
    const double zomco = scat / ztauo;
    const double zcoo = (tc * (double)zcoc + tauc * coc) / ztauo;
    return one_minus_zwo<double>(zomco, zcoo, zgco) <= 5.0e-7 ? 1 : 0;
}

// Whether the FP32 estimate of 1 - zwo (reftra:183-188) is too close to the
// 5e-7 switch to trust its branch.  The window is an error bound from the
// FP32 optics: 2e-6 relative on the co-albedo and on the asymmetry.  Near
// zg = 0.5, where the reference's q = zg / (1 - zg) reaches 1, 1 - zwo
// falls steeply with zg and the window widens accordingly.
__device__ inline bool near_conservative_edge(float zw, float zco, float zg) {
    if (zg == 1.0f || !(zw > 0.0f)) return false;
    const float r = one_minus_zwo(zw, zco, zg);
    const float q = zg / (1.0f - zg);
    const float den = 1.0f - zco * q * q;
    if (den == 0.0f) return true;
    const float d_dg = 2.0f * zco * q * (1.0f - zco) / (den * den * (1.0f - zg) * (1.0f - zg));
    const float d_dco = fabsf(1.0f - q * q) / (den * den);
    const float tol = d_dg * (2.0e-6f * fabsf(zg) + 1.0e-9f) + d_dco * 2.0e-6f * zco + 1.0e-13f;
    return fabsf(r - 5.0e-7f) <= tol;
}

template <typename R>
__device__ inline void warp_sum4(R& v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
}

// Shared-memory carve-up of one CTA (two columns); the host sizes the
// launch with the same function.
struct Smem {
    size_t pdp, coef, pk, misc, kc, ka, omcf, cld, seed, aer, xs, red, flux, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline Smem smem_layout(int L, int nq, bool fused, bool aer_stage, size_t rsz) {
    Smem m;
    size_t o = 0;
    m.pdp = o;  o = align16(o + COLS_PER_CTA * L * sizeof(double));
    m.coef = o; o = align16(o + COLS_PER_CTA * NFR * L * rsz);
    m.pk = o;   o = align16(o + COLS_PER_CTA * L * sizeof(int));
    m.misc = o; o = align16(o + 8 * sizeof(int));
    m.kc = m.ka = m.omcf = m.cld = m.seed = m.xs = m.aer = o;
    if (fused) {
        m.kc = o;   o = align16(o + COLS_PER_CTA * L * sizeof(long long));
        m.ka = o;   o = align16(o + COLS_PER_CTA * L * sizeof(long long));
        m.omcf = o; o = align16(o + COLS_PER_CTA * L * sizeof(double));
        m.cld = o;  o = align16(o + COLS_PER_CTA * 4 * L * rsz);
        m.seed = o; o = align16(o + COLS_PER_CTA * 4 * sizeof(uint32_t));
        m.xs = o;   o = align16(o + NGPT * 32 * sizeof(uint32_t));
    }
    if (aer_stage) {
        m.aer = o;  o = align16(o + COLS_PER_CTA * 3 * NBND * L * rsz);
    }
    m.red = o;  o = align16(o + KLEV * nq * CTA_THREADS * rsz);
    m.flux = o; o = align16(o + COLS_PER_CTA * nq * (L + 1) * rsz);
    m.total = o;
    return m;
}

template <typename R>
__host__ __device__ inline bool stage_aerosol(int iaer) {
    // the FP32 form converts the FP64 aerosol inputs once per (column, layer, band)
    return sizeof(R) == 4 && iaer != 0;
}

template <typename R>
__global__ void __launch_bounds__(CTA_THREADS, 2)
k_solve(const SolveParams P, const R* __restrict__ tab, const double* __restrict__ tab64) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = P.nlay;
    const int NQ = num_q<R>(P.extra != 0);
    constexpr int QX = 6 + num_abs<R>();  // first extra-output sum
    const bool fused = P.fused && P.icld >= 1;
    const bool aer_stage = stage_aerosol<R>(P.iaer);
    const Smem M = smem_layout(L, NQ, fused, aer_stage, sizeof(R));
    double* sPdp = (double*)(smem_raw + M.pdp);        // [2][L]
    R* sCoef = (R*)(smem_raw + M.coef);                // [2][NFR][L]
    int* sPk = (int*)(smem_raw + M.pk);                // [2][L]
    int* sMisc = (int*)(smem_raw + M.misc);            // laytrop [2]
    long long* sKc = (long long*)(smem_raw + M.kc);    // [2][L] McICA threshold of 1 - cldf
    long long* sKa = (long long*)(smem_raw + M.ka);    // [2][L] McICA threshold of alpha
    double* sOmcf = (double*)(smem_raw + M.omcf);      // [2][L] 1 - cldf (icld 2)
    R* sCld = (R*)(smem_raw + M.cld);                  // [2][4][L] ciwp, clwp, rei, rel
    uint32_t* sSeed = (uint32_t*)(smem_raw + M.seed);  // [2][4]
    uint32_t* sXs = (uint32_t*)(smem_raw + M.xs);      // [112][32] columns of M^n
    R* sAer = (R*)(smem_raw + M.aer);                  // [2][3][14][L] tau, ssa, asym
    R* sRed = (R*)(smem_raw + M.red);                  // [KLEV][NQ][224]
    R* sFlux = (R*)(smem_raw + M.flux);                // [2][NQ][L+1]

    const int tid = threadIdx.x;
    const int cc = tid / NGPT, g = tid % NGPT;
    const int ib = cT.ngb[g], igb = cT.gib[g];
    const bool uv = ib >= 9 && ib <= 12;  // bands 25-28 (spcvmc:629)
    const int NS = P.idelm == 0 ? NS_MAX : S_DBTCN;
    R* scr = (R*)P.scratch + (size_t)blockIdx.x * P.slot_elems;
    const size_t n = (size_t)P.ncol;

    // McICA stream jump of this subcolumn: once per launch
    KissJump J{1u, 0u, 1u, 1u};
    if (fused) {
        const uint64_t off = kiss_offset(P.icld, g, L, P.permuteseed);
        J = kiss_jump_consts(off);
        if (cc == 0) xorshift_power(off, sXs + g * 32);
    }

    for (int pair = blockIdx.x; pair < P.npairs; pair += gridDim.x) {
        __syncthreads();
        // ---------------- prep: one (column, layer) per item, FP64
        for (int it = tid; it < COLS_PER_CTA * L; it += CTA_THREADS) {
            const int c2 = it / L, lay = it % L + 1;
            const int pcol = COLS_PER_CTA * pair + c2;
            prep_layer<R>(P, pcol, lay, sCoef + c2 * NFR * L, sPk + c2 * L, sPdp + c2 * L, L, tab64);
            const bool real = pcol < P.ncol;
            const size_t kl = (size_t)pcol + n * (size_t)(lay - 1);
            if (fused) {
                double cf = real ? P.cldfrac[kl] : 0.0;
                if (cf < 1.0e-20) cf = 0.0;
                const double omcf = DS(1.0, cf);
                sOmcf[c2 * L + lay - 1] = omcf;
                sKc[c2 * L + lay - 1] = kiss_threshold(omcf);
                sKa[c2 * L + lay - 1] = (P.icld >= 4 && real) ? kiss_threshold(P.alpha[kl]) : 0ll;
                R* cd = sCld + c2 * 4 * L;
                cd[0 * L + lay - 1] = real ? (R)P.ciwp[kl] : R(0);
                cd[1 * L + lay - 1] = real ? (R)P.clwp[kl] : R(0);
                cd[2 * L + lay - 1] = real ? (R)P.rei[kl] : R(0);
                cd[3 * L + lay - 1] = real ? (R)P.rel[kl] : R(0);
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
        R zinc = R(0), albp = R(0), albd = R(0);
        double cossza = 1.0;
        McicaMask mc;
        if (active) {
            cossza = P.coszen[col];
            if (cossza < 1.e-10) cossza = 1.e-10;
            const bool nir = ib <= 8 || ib == 13;
            albp = (R)(nir ? P.aldir[col] : P.asdir[col]);
            albd = (R)(nir ? P.aldif[col] : P.asdif[col]);
            // zincflx = adjflux * ssi * prmu0 (spcvmc:349-356)
            R src;
            if constexpr (sizeof(R) == 4) src = solar_source_generic(ib, igb, C, P, tab);
            else src = solar_source<R>(ib, igb, C, P, tab);
            zinc = R(P.adjflux[ib]) * src * (R)cossza;
            if (fused) mc.start(kiss_start(sSeed + cc * 4, J, sXs + g * 32), P.icld);
        }
        const R prmu0 = (R)cossza;
        const R* cld = sCld + cc * 4 * L;
        const R* aer = sAer + cc * 3 * NBND * L;

        // ---------------- pass 1: bottom -> top
        R rupc_b = albp, rupdc_b = albd, rup_b = albp, rupd_b = albd;
        for (int lay = 1; lay <= L; ++lay) {
            const int jk = L + 1 - lay;
            R* sv = scr + (size_t)(jk - 1) * NS * CTA_THREADS + tid;
            if (!active) continue;
            R taug, taur;
            if constexpr (sizeof(R) == 4) {
                int js;
                float fs;
                taumol_generic(ib, igb, lay, C, tab, taug, taur, js, fs);
            } else {
                taumol_g<R>(ib, igb, lay, C, tab, taug, taur);
            }
            R rta, roa, rga, rcoa;
            if (aer_stage) {
                rta = aer[(0 * NBND + ib) * L + lay - 1];
                rcoa = aer[(1 * NBND + ib) * L + lay - 1];
                roa = R(1) - rcoa;
                rga = aer[(2 * NBND + ib) * L + lay - 1];
            } else if (P.iaer == 0) {
                rta = R(0); roa = R(1); rga = R(0); rcoa = R(0);
            } else {
                double ta, oa, ga;
                aerosol(P, col, lay, ib, tab64, ta, oa, ga);
                rta = (R)ta; roa = (R)oa; rga = (R)ga; rcoa = (R)DS(1.0, oa);
            }
            // cloud of this subcolumn (McICA) at this layer
            bool cloudy = false;
            R cldf = R(0), tc = R(0), oc = R(1), gc = R(0), fsfc = R(0), ciwp = R(0), clwp = R(0), rei = R(0),
              rel = R(0);
            if (P.icld >= 1) {
                const size_t kl = (size_t)col + n * (size_t)(lay - 1);
                if (fused) {
                    cloudy = mc.step(lay, sKc[cc * L + lay - 1], sKa[cc * L + lay - 1], sOmcf[cc * L + lay - 1]);
                    if (cloudy) {
                        cldf = R(1);
                        ciwp = cld[0 * L + lay - 1];
                        clwp = cld[1 * L + lay - 1];
                        if (P.tauc) {
                            const size_t kb = (size_t)ib + 14 * kl;
                            tc = (R)P.tauc[kb];
                            oc = (R)P.ssac[kb];
                            gc = (R)P.asmc[kb];
                            fsfc = (R)P.fsfc[kb];
                        }
                    }
                    rei = cld[2 * L + lay - 1];
                    rel = cld[3 * L + lay - 1];
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
                cldprmc_g<R>(ib, P.inflag, P.iceflag, P.liqflag, cldf, ciwp, clwp, rei, rel, fsfc, tc, oc, gc, taor,
                             coc, tab, P.err);
            // clear-sky optics including aerosols (spcvmc:442-445)
            R ztauc = taur + taug + rta;
            R zomcc = taur * R(1) + rta * roa;
            R zgcc = rga * roa * rta / zomcc;
            R zcoc = R(0);
            if constexpr (sizeof(R) == 4) zcoc = (taug + rta * rcoa) / ztauc;  // co-albedo
            zomcc = zomcc / ztauc;
            const R zclear = R(1) - cldf, zcloud = cldf;
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
            if constexpr (sizeof(R) == 4) zcoc = zcoc / (R(1) - zwf);
            const RT<R> rc = reftra_g<R>(ztauc, zomcc, zcoc, zgcc, prmu0, tab, tab64);
            const R zdbtc = tbl_exp<R>(ztauc / prmu0, tab);
            RT<R> rt = rc;
            R zdbt = zdbtc;
            if (cloudy) {
                // total sky: clear + delta-scaled cloud (spcvmc:500-505); reftra
                // only where cldf > repclc (:427); mixed by cloud fraction (:546-549)
                const R ztauo = ztauc + tc;
                R zomco = ztauc * zomcc + tc * oc;
                const R zgco = (tc * oc * gc + ztauc * zomcc * zgcc) / zomco;
                R zcoo = R(0);
                if constexpr (sizeof(R) == 4) zcoo = (ztauc * zcoc + tc * coc) / ztauo;
                zomco = zomco / ztauo;
                RT<R> ro;
                if (cldf > R(1.e-12)) {
                    int force = -1;
                    if constexpr (sizeof(R) == 4) {
                        if (near_conservative_edge(zomco, zcoo, zgco))
                            force = decide_conservative64(P, col, g, lay, ib, ztauc, zomcc, zgcc, zcoc, tab64);
                    }
                    ro = reftra_g<R>(ztauo, zomco, zcoo, zgco, prmu0, tab, tab64, force);
                }
                else { ro.ref = R(0); ro.tra = R(1); ro.refd = R(0); ro.trad = R(1); ro.adir = R(0); ro.adif = R(0); }
                rt.ref = zclear * rc.ref + zcloud * ro.ref;
                rt.refd = zclear * rc.refd + zcloud * ro.refd;
                rt.tra = zclear * rc.tra + zcloud * ro.tra;
                rt.trad = zclear * rc.trad + zcloud * ro.trad;
                if constexpr (sizeof(R) == 4) {
                    rt.adir = zclear * rc.adir + zcloud * ro.adir;
                    rt.adif = zclear * rc.adif + zcloud * ro.adif;
                }
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
            // the FP32 form keeps the absorptances in the transmittance slots
            // and rebuilds ptra = 1 - pref - adir, ptrad = 1 - prefd - adif
            constexpr bool keep_abs = sizeof(R) == 4;
            sv[S_REFC * CTA_THREADS] = rc.ref;
            sv[S_REFDC * CTA_THREADS] = rc.refd;
            sv[S_TRAC * CTA_THREADS] = keep_abs ? rc.adir : rc.tra;
            sv[S_TRADC * CTA_THREADS] = keep_abs ? rc.adif : rc.trad;
            sv[S_DBTC * CTA_THREADS] = zdbtc;
            sv[S_RUPC * CTA_THREADS] = rupc_b;
            sv[S_RUPDC * CTA_THREADS] = rupdc_b;
            sv[S_REF * CTA_THREADS] = rt.ref;
            sv[S_REFD * CTA_THREADS] = rt.refd;
            sv[S_TRA * CTA_THREADS] = keep_abs ? rt.adir : rt.tra;
            sv[S_TRAD * CTA_THREADS] = keep_abs ? rt.adif : rt.trad;
            sv[S_DBT * CTA_THREADS] = zdbt;
            sv[S_RUP * CTA_THREADS] = rup_b;
            sv[S_RUPD * CTA_THREADS] = rupd_b;
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
                const R* sv = scr + (size_t)(jk - 1) * NS * CTA_THREADS + tid;
                refc = sv[S_REFC * CTA_THREADS]; refdc = sv[S_REFDC * CTA_THREADS];
                trac = sv[S_TRAC * CTA_THREADS]; tradc = sv[S_TRADC * CTA_THREADS];
                dbtc = sv[S_DBTC * CTA_THREADS];
                rupc = sv[S_RUPC * CTA_THREADS]; rupdc = sv[S_RUPDC * CTA_THREADS];
                ref = sv[S_REF * CTA_THREADS]; refd = sv[S_REFD * CTA_THREADS];
                tra = sv[S_TRA * CTA_THREADS]; trad = sv[S_TRAD * CTA_THREADS];
                dbt = sv[S_DBT * CTA_THREADS];
                if constexpr (sizeof(R) == 4) {
                    adirc = trac; adifc = tradc; adirt = tra; adift = trad;
                    trac = R(1) - refc - adirc;
                    tradc = R(1) - refdc - adifc;
                    tra = R(1) - ref - adirt;
                    trad = R(1) - refd - adift;
                }
                rup = sv[S_RUP * CTA_THREADS]; rupd = sv[S_RUPD * CTA_THREADS];
                if (P.idelm == 0) { dbtcn = sv[S_DBTCN * CTA_THREADS]; dbtn = sv[S_DBTN * CTA_THREADS]; }
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
            const int slot = (jk - 1) % KLEV;
#pragma unroll
            for (int i = 0; i < NQ_MAX; ++i)
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
}

}  // namespace rrsw
