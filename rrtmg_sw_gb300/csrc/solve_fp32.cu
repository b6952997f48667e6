// solve_fp32.cu -- FP32 form of the solve (FMA contraction allowed).
#include "kernel.cuh"
#include "launch.h"
#include "tiled.cuh"

namespace rrsw {

// exp(-x) from the table together with 1 - exp(-x) free of cancellation
// below od_lo, where the table is replaced by the quadratic 1 - x + x^2/2
// (rrtmg_sw_reftra.f90:203-209)
__device__ inline float tbl_exp_om(float x, const float* __restrict__ tab, float& om) {
    if (x <= 0.06f) {
        om = x * (1.0f - 0.5f * x);
        return 1.0f - om;
    }
    const float tblind = x / (cT.bpade_f + x);
    const int itind = (int)(10000.0f * tblind + 0.5f);
    const float e = ldt(tab, cT.exp_tbl + itind);
    om = 1.0f - e;
    return e;
}

// reftra_sw (rrtmg_sw_reftra.f90:151-326), kmodts = 2, in FP32 with the
// single-scattering co-albedo zco = 1 - zw carried from the optics so that
// no step cancels as zw -> 1 or as the layer gets thin:
//   gamma1 - gamma2 = 2 zco, so k = sqrt(2 zco (gamma1 + gamma2));
//   1 - zwo = zco (1 - q^2) / (1 - zco q^2) decides the conservative branch;
//   zrk - gamma1 = -gamma2^2 / (zrk + gamma1), zbeta = gamma2^2 / (zrk + gamma1)^2;
//   with om = 1 - exp(-x) and p = exp(x) - 1 = om / exp(-x):
//     zdenr = zrpp (2 zrk + (zrk + gamma1) p1 + gamma2^2 / (zrk + gamma1) om1),
//     zr1 zep1 - zr2 zem1 - zr3 zem2 = zr1 p1 + zr2 om1 + zr3 om2,
//     zt1 zep1 - zt2 zem1 - zt3 zep2 = zt1 p1 + zt2 om1 - zt3 p2
//   (zr1 - zr2 - zr3 = zt1 - zt2 - zt3 = 0), and
//     1 - zbeta zem1^2 = 2 zrk / (zrk + gamma1) + zbeta om1 (1 + zem1);
//   1 - exp(-x) is taken from the quadratic itself below od_lo.
// The absorptances follow from the same pieces:
//   1 - pref - ptra   = om2 - zw (Nr - zem2 Nt) / zdenr,
//   1 - prefd - ptrad = om1 (zrk om1 + 2 zco (1 + zem1)) zdend,
// so a heating rate can be summed from layer absorption instead of being
// differenced from level fluxes.  Mathematically these are the reference's
// expressions; they only avoid FP32 cancellation.
// Near resonance, k mu0 = 1 (zrpp = 1 - (k mu0)^2 -> 0), the solution has a
// removable singularity: the numerators of pref/ptra and zdenr vanish
// together, so the result hinges on zem1 and zem2 coming from consistent
// table entries.  The scattered part carries a factor zw, so the rounding
// error of an FP32 cell grows like zw / |zrpp|.  Cells with
// |zrpp| < RESONANCE_TOL zw, or with |zrpp| < RESONANCE_WIDE and a table
// lookup too close to an entry edge to be sure of, are flagged risky; the
// caller then recomputes the cell as the FP64 form does.  So are cells
// whose conservative switch is too close.  The edge window near resonance
// is RESONANCE_EPS relative in the lookup's argument, about four times the
// FP32 optical depth's own error: strongly absorbing clear layers under a
// sun near 60 degrees (k ~ 2, mu0 ~ 0.5) sit at resonance, and with a
// narrower window (5e-7) a flipped entry there moved one UV layer's heating
// rate by 0.01 K/day.  The amplification reaches well beyond |zrpp| = 0.05:
// a hazy surface layer with |zrpp| = 0.07 (k mu0 = 1.03) whose exp(-k tau)
// lookup sat 2.4e-6 (in entries) from an edge had its direct absorptance
// moved by 6 %, the surface flux by 0.1 W/m2; hence RESONANCE_WIDE = 0.15.
constexpr float RESONANCE_TOL = 2.0e-3f;
constexpr float RESONANCE_WIDE = 0.15f;
constexpr float RESONANCE_EPS = 2.0e-6f;
constexpr float CLOUD_EDGE_EPS = 2.0e-7f;  // window of the cloudy total-sky lookups

// Whether exp(-x) from the table could come from the neighbouring entry
// under a relative uncertainty eps of x.
__device__ inline bool entry_edge(float x, float eps) {
    if (x <= 0.06f) return false;
    const float b = cT.bpade_f;
    const float bx = b + x;
    const float t = 10000.0f * x / bx + 0.5f;
    const float fr = t - floorf(t);
    return fminf(fr, 1.0f - fr) < 10000.0f * b * x / (bx * bx) * eps;
}

template <>
__device__ __forceinline__ RT<float> reftra_g<float>(float zto1, float zw, float zco, float zg, float prmuz,
                                           const float* __restrict__ tab, const double* __restrict__ tab64,
                                           int force) {
    RT<float> o;
    const float eps = 1.e-08f;
    const float zg3 = 3.0f * zg;
    const float zgamma1 = (8.0f - zw * (5.0f + zg3)) * 0.25f;
    const float zgamma2 = 3.0f * (zw * (1.0f - zg)) * 0.25f;
    const float zgamma3 = (2.0f - zg3 * prmuz) * 0.25f;
    const float zgamma4 = 1.0f - zgamma3;
    // zwo >= zwcrit  <=>  1 - zwo <= 5e-7  (reftra:183-188)
    (void)tab64;
    bool edge;
    const bool cons = conservative_test(zw, zco, zg, edge) <= 5.0e-7f;
    o.adir = 0.0f;
    o.adif = 0.0f;
    o.risky = edge;
    if (cons) {
        // conservative scattering (reftra:191-228); ptra = 1 - pref and
        // ptrad = 1 - prefd written without the subtraction; no absorption
        const float za1 = zgamma1 * prmuz - zgamma3;
        const float zgt = zgamma1 * zto1;
        float om;
        const float ze2 = tbl_exp_om(fminf(zto1 / prmuz, 500.0f), tab, om);
        const float r1 = 1.0f / (1.0f + zgt);
        o.ref = (zgt - za1 * om) * r1;
        o.tra = (1.0f + za1 * om) * r1;
        o.refd = zgt * r1;
        o.trad = r1;
        if (ze2 == 1.0f) { o.ref = 0.0f; o.tra = 1.0f; o.refd = 0.0f; o.trad = 1.0f; }
        return o;
    }
    const float za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
    const float za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
    const float zrk = sqrtf(2.0f * zco * (zgamma1 + zgamma2));
    const float zrp = zrk * prmuz;
    const float zrp1 = 1.0f + zrp, zrm1 = 1.0f - zrp;
    const float zrk2 = 2.0f * zrk;
    const float zrpp = zrm1 * zrp1;
    if (fabsf(zrpp) < RESONANCE_TOL * zw) o.risky = true;
    const float zrkg = zrk + zgamma1;
    const float r_kg = 1.0f / zrkg;
    const float g2k = zgamma2 * zgamma2 * r_kg;  // gamma1 - zrk
    const float zr1 = zrm1 * (za2 + zrk * zgamma3);
    const float zr2 = zrp1 * (za2 - zrk * zgamma3);
    const float zr3 = zrk2 * (zgamma3 - za2 * prmuz);
    const float zt1 = zrp1 * (za1 + zrk * zgamma4);
    const float zt2 = zrm1 * (za1 - zrk * zgamma4);
    const float zt3 = zrk2 * (zgamma4 + za1 * prmuz);
    const float zbeta = g2k * r_kg;
    float om1, om2;
    const float zem1 = tbl_exp_om(fminf(zrk * zto1, 500.0f), tab, om1);
    const float zem2 = tbl_exp_om(fminf(zto1 / prmuz, 500.0f), tab, om2);
    // force = 1 (cloudy total sky): a neighbouring table entry moves pref/ptra
    // of a thick layer enough to show in the fluxes, so every lookup is tested
    if ((force == 1 || fabsf(zrpp) < RESONANCE_WIDE) && !o.risky) {
        const float eps = fabsf(zrpp) < RESONANCE_WIDE ? RESONANCE_EPS : CLOUD_EDGE_EPS;
        o.risky = entry_edge(fminf(zrk * zto1, 500.0f), eps) || entry_edge(fminf(zto1 / prmuz, 500.0f), eps);
    }
    const float p1 = om1 / zem1;  // zep1 - 1
    const float p2 = om2 / zem2;  // zep2 - 1
    const float zdenr = zrpp * (zrk2 + zrkg * p1 + g2k * om1);
    if (zdenr >= -eps && zdenr <= eps) {
        o.ref = eps;
        o.tra = zem2;
        o.adir = om2 - eps;
    } else {
        const float rd = 1.0f / zdenr;
        const float nr = zr1 * p1 + zr2 * om1 + zr3 * om2;
        const float nt = zt1 * p1 + zt2 * om1 - zt3 * p2;
        o.ref = zw * nr * rd;
        o.tra = zem2 - zem2 * zw * nt * rd;
        o.adir = om2 - zw * rd * (nr - zem2 * nt);
    }
    const float omm = om1 * (1.0f + zem1);  // 1 - zem1^2
    const float zdend = 1.0f / ((zrk2 * r_kg + zbeta * omm) * zrkg);
    o.refd = zgamma2 * omm * zdend;
    o.trad = zrk2 * zem1 * zdend;
    o.adif = om1 * (zrk * om1 + 2.0f * zco * (1.0f + zem1)) * zdend;
    return o;
}

__device__ __noinline__ RT<float> reftra_f32_cloudy(float zto1, float zw, float zco, float zg, float prmuz,
                                                    const float* __restrict__ tab,
                                                    const double* __restrict__ tab64) {
    return reftra_g<float>(zto1, zw, zco, zg, prmuz, tab, tab64, 1);
}

// setcoef of the FP32 form for every (column, layer): the diagnostic export
// of its table indices (rrtmg_sw_setcoef_c)
static __global__ void __launch_bounds__(256) k_setcoef_f32(const SolveParams P, const float* __restrict__ tab,
                                                            const double* __restrict__ tab64, float* cf, int* pk,
                                                            double* pdp) {
    const size_t n = (size_t)P.ncol, L = (size_t)P.nlay;
    const size_t it = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n * L) return;
    const int col = (int)(it % n), lay = (int)(it / n) + 1;
    prep_layer_f32(P, col, lay, cf + (size_t)col * NFR * L, pk + (size_t)col * L, pdp + (size_t)col * L, (int)L,
                   tab, tab64);
}

cudaError_t launch_setcoef_f32(const SolveParams& P, const float* tab, const double* tab64, float* cf, int* pk,
                               double* pdp, cudaStream_t s) {
    const size_t n = (size_t)P.ncol * P.nlay;
    k_setcoef_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, tab, tab64, cf, pk, pdp);
    return cudaGetLastError();
}

cudaError_t upload_tables_fp32(const DevTables& t) { return cudaMemcpyToSymbol(cT, &t, sizeof(DevTables)); }

LaunchInfo plan_fp32(const SolveParams& P, int num_sms, bool allow_tiled) {
    LaunchInfo li;
    static int smem_optin = -1;
    if (smem_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    if (allow_tiled && tiled_supports(P, (size_t)smem_optin)) {
        // one CTA per SM, persistent over the column pairs
        const bool fused = P.fused && P.icld >= 1, nomc = P.nomcica && P.icld >= 1;
        li.tiled = true;
        li.tile_slots = tiled_slots(P, (size_t)smem_optin);
        li.smem = tiled_smem(P.nlay, P.extra ? 16 : 8, fused, fused || nomc, li.tile_slots).total;
        cudaFuncSetAttribute(k_solve_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)li.smem);
        li.grid = num_sms < P.npairs ? num_sms : P.npairs;
        if (li.grid < 1) li.grid = 1;
        li.slot_bytes = tiled_glob(P.nlay).total;
        // the preparation kernel: persistent over the pairs at the occupancy it reaches
        li.prep_smem = tiled_prep_smem(P.nlay).total;
        li.prep_bytes = tiled_prep_layout(P.nlay, fused, fused || nomc, P.iaer != 0).total;
        const auto prep = P.mt ? k_tiled_prep<true> : k_tiled_prep<false>;
        cudaFuncSetAttribute(prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)li.prep_smem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prep, CTA_THREADS, li.prep_smem);
        if (per_sm < 1) per_sm = 1;
        li.prep_grid = num_sms * per_sm < P.npairs ? num_sms * per_sm : P.npairs;
        if (li.prep_grid < 1) li.prep_grid = 1;
        return li;
    }
    li.smem = smem_layout(P.nlay, num_q<float>(P.extra != 0), stages_clouds(P),
                          stage_aerosol<float>(P.iaer), sizeof(float)).total;
    const auto kern = P.mt ? k_solve<float, true> : k_solve<float, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)li.smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CTA_THREADS, li.smem);
    if (per_sm < 1) per_sm = 1;
    li.grid = num_sms * per_sm;
    if (li.grid > P.npairs) li.grid = P.npairs;
    if (li.grid < 1) li.grid = 1;
    li.slot_bytes = slot_elems(P.nlay, P.idelm, true) * sizeof(float);
    return li;
}

cudaError_t launch_solve_fp32(const SolveParams& P, const float* tab, const double* tab64, const LaunchInfo& li,
                              cudaStream_t s) {
    if (li.tiled) {
        if (P.mt) k_tiled_prep<true><<<li.prep_grid, CTA_THREADS, li.prep_smem, s>>>(P, tab, tab64);
        else k_tiled_prep<false><<<li.prep_grid, CTA_THREADS, li.prep_smem, s>>>(P, tab, tab64);
        k_solve_tiled<<<li.grid, T_THREADS, li.smem, s>>>(P, tab, tab64);
    } else {
        if (P.mt) k_solve<float, true><<<li.grid, CTA_THREADS, li.smem, s>>>(P, tab, tab64);
        else k_solve<float, false><<<li.grid, CTA_THREADS, li.smem, s>>>(P, tab, tab64);
    }
    return cudaGetLastError();
}

size_t solve_smem_fp32(const SolveParams& P, int nc) {
    return smem_layout(P.nlay, num_q<float>(P.extra != 0), stages_clouds(P), stage_aerosol<float>(P.iaer),
                       sizeof(float), nc).total;
}

int batch_blocks_per_sm_fp32(size_t smem, int nc) {
    const auto kern = nc == 4 ? k_solve_batch<float, 4> : k_solve_batch<float, 2>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nc * NGPT, smem);
    return per_sm;
}

cudaError_t launch_batch_fp32(const SolveParams* dPb, int n, const int* counts, const float* tab,
                              const double* tab64, int grid, size_t smem, int nc, cudaStream_t s) {
    if (nc == 4) k_solve_batch<float, 4><<<grid, 4 * NGPT, smem, s>>>(dPb, n, counts, tab, tab64);
    else k_solve_batch<float, 2><<<grid, 2 * NGPT, smem, s>>>(dPb, n, counts, tab, tab64);
    return cudaGetLastError();
}

}  // namespace rrsw
