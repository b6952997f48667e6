// solve_fp32.cu -- FP32 form of the solve (FMA contraction allowed).
#include "kernel.cuh"
#include "launch.h"

namespace rrsw {

// reftra_sw (rrtmg_sw_reftra.f90:151-326) with FP32 bulk arithmetic.  The
// near-conservative branch (zwo >= zwcrit, :188-228) is evaluated in FP64.
template <>
__device__ inline RT<float> reftra_g<float>(float zto1, float zw, float zg, float prmuz, const float* __restrict__ tab) {
    typedef float R;
    RT<R> o;
    const R eps = 1.e-08f;
    const R zg3 = 3.0f * zg;
    const R zgamma1 = (8.0f - zw * (5.0f + zg3)) * 0.25f;
    const R zgamma2 = 3.0f * (zw * (1.0f - zg)) * 0.25f;
    const R zgamma3 = (2.0f - zg3 * prmuz) * 0.25f;
    const R zgamma4 = 1.0f - zgamma3;
    R zwo = 0.0f, denom = 1.0f;
    if (zg != 1.0f) {
        const R q = zg / (1.0f - zg);
        denom = (1.0f - (1.0f - zw) * (q * q));
    }
    if (zw > 0.0f && denom != 0.0f) zwo = zw / denom;
    if (zwo >= 0.9999995f) {
        const double g1 = (double)zgamma1, mu = (double)prmuz;
        const double za1 = g1 * mu - (double)zgamma3;
        const double zgt = g1 * (double)zto1;
        const R ze1 = fminf(zto1 / prmuz, 500.0f);
        const double ze2 = (double)tbl_exp<R>(ze1, tab);
        o.ref = (R)((zgt - za1 * (1.0 - ze2)) / (1.0 + zgt));
        o.tra = 1.0f - o.ref;
        o.refd = (R)(zgt / (1.0 + zgt));
        o.trad = 1.0f - o.refd;
        if (ze2 == 1.0) { o.ref = 0.0f; o.tra = 1.0f; o.refd = 0.0f; o.trad = 1.0f; }
    } else {
        const R za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
        const R za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
        const R zrk = sqrtf(zgamma1 * zgamma1 - zgamma2 * zgamma2);
        const R zrp = zrk * prmuz;
        const R zrp1 = 1.0f + zrp, zrm1 = 1.0f - zrp;
        const R zrk2 = 2.0f * zrk;
        const R zrpp = 1.0f - zrp * zrp;
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
        const R ze1 = fminf(zrk * zto1, 500.0f);
        const R ze2 = fminf(zto1 / prmuz, 500.0f);
        const R zem1 = tbl_exp<R>(ze1, tab);
        const R zep1 = 1.0f / zem1;
        const R zem2 = tbl_exp<R>(ze2, tab);
        const R zep2 = 1.0f / zem2;
        const R zdenr = zr4 * zep1 + zr5 * zem1;
        if (zdenr >= -eps && zdenr <= eps) {
            o.ref = eps;
            o.tra = zem2;
        } else {
            o.ref = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
            o.tra = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdenr;
        }
        const R zemm = zem1 * zem1;
        const R zdend = 1.0f / ((1.0f - zbeta * zemm) * zrkg);
        o.refd = zgamma2 * (1.0f - zemm) * zdend;
        o.trad = zrk2 * zem1 * zdend;
    }
    return o;
}

cudaError_t upload_tables_fp32(const DevTables& t) { return cudaMemcpyToSymbol(cT, &t, sizeof(DevTables)); }

static size_t smem_bytes32(int L, int extra) {
    const int NQ = extra ? NQ_EXTRA : NQ_BASE;
    size_t off = (size_t)COLS_PER_CTA * L * sizeof(double) + (size_t)COLS_PER_CTA * NFR * L * sizeof(float) +
                 (size_t)COLS_PER_CTA * L * sizeof(int) + 4 * sizeof(int);
    off = (off + 15) & ~(size_t)15;
    return off + (size_t)KLEV * NQ * CTA_THREADS * sizeof(float) + (size_t)COLS_PER_CTA * NQ * (L + 1) * sizeof(float);
}

LaunchInfo plan_fp32(const SolveParams& P, int num_sms) {
    LaunchInfo li;
    li.smem = smem_bytes32(P.nlay, P.extra);
    cudaFuncSetAttribute(k_solve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)li.smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve<float>, CTA_THREADS, li.smem);
    if (per_sm < 1) per_sm = 1;
    li.grid = num_sms * per_sm;
    if (li.grid > P.npairs) li.grid = P.npairs;
    if (li.grid < 1) li.grid = 1;
    return li;
}

cudaError_t launch_solve_fp32(const SolveParams& P, const float* tab, const double* tab64, const LaunchInfo& li,
                              cudaStream_t s) {
    k_solve<float><<<li.grid, CTA_THREADS, li.smem, s>>>(P, tab, tab64);
    return cudaGetLastError();
}

}  // namespace rrsw
