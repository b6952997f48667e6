// solve_fp64.cu -- plain FP64 form.  Built with --fmad=false so that every
// multiply and add rounds separately, as the reference's expressions do;
// together with the reference's operation order this makes the device
// results agree with the FP64 oracle to rounding of log/exp only.
#include "kernel.cuh"
#include "launch.h"

namespace rrsw {

cudaError_t upload_tables_fp64(const DevTables& t) { return cudaMemcpyToSymbol(cT, &t, sizeof(DevTables)); }

size_t slot_elems(int nlay, int idelm, bool fp32, int nc) {
    (void)fp32;  // the same level fields in both forms (elements of the form's type)
    return (size_t)nlay * (size_t)(idelm == 0 ? NS_MAX : S_DBTCN) * (size_t)(nc * NGPT);
}

LaunchInfo plan_fp64(const SolveParams& P, int num_sms) {
    LaunchInfo li;
    li.smem = smem_layout(P.nlay, num_q<double>(P.extra != 0), stages_clouds(P),
                          stage_aerosol<double>(P.iaer), sizeof(double)).total;
    const auto kern = P.mt ? k_solve<double, true> : k_solve<double, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)li.smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CTA_THREADS, li.smem);
    if (per_sm < 1) per_sm = 1;
    li.grid = num_sms * per_sm;
    if (li.grid > P.npairs) li.grid = P.npairs;
    if (li.grid < 1) li.grid = 1;
    return li;
}

cudaError_t launch_solve_fp64(const SolveParams& P, const double* tab, const LaunchInfo& li, cudaStream_t s) {
    if (P.mt) k_solve<double, true><<<li.grid, CTA_THREADS, li.smem, s>>>(P, tab, tab);
    else k_solve<double, false><<<li.grid, CTA_THREADS, li.smem, s>>>(P, tab, tab);
    return cudaGetLastError();
}

cudaError_t launch_compact(const SolveParams* dPb, int n, int* map_all, const long long* map_off, int* counts,
                           cudaStream_t s) {
    k_compact<<<n, 1024, 0, s>>>(dPb, map_all, map_off, counts);
    return cudaGetLastError();
}

size_t solve_smem_fp64(const SolveParams& P, int nc) {
    return smem_layout(P.nlay, num_q<double>(P.extra != 0), stages_clouds(P), stage_aerosol<double>(P.iaer),
                       sizeof(double), nc).total;
}

int batch_blocks_per_sm_fp64(size_t smem, int nc) {
    const auto kern = nc == 4 ? k_solve_batch<double, 4> : k_solve_batch<double, 2>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nc * NGPT, smem);
    return per_sm;
}

cudaError_t launch_batch_fp64(const SolveParams* dPb, int n, const int* counts, const double* tab, int grid,
                              size_t smem, int nc, cudaStream_t s) {
    if (nc == 4) k_solve_batch<double, 4><<<grid, 4 * NGPT, smem, s>>>(dPb, n, counts, tab, tab);
    else k_solve_batch<double, 2><<<grid, 2 * NGPT, smem, s>>>(dPb, n, counts, tab, tab);
    return cudaGetLastError();
}

// ------------------------------------------------------------ get_alpha
// mcica_subcol_gen_sw.f90:119-176, one thread per column (the layer loop
// is sequential in the reference only through alpha(i,1) = 0).
__global__ void k_get_alpha(int ncol, int nlay, int icld, int idcor, double decorr_con, const double* dz,
                            const double* lat, int juldat, const double* cldfrac, double* alpha) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncol) return;
    const double am1 = 1.4315, am2 = 2.1219, am4 = -25.584, amr = 7.0;
    if (icld != 4 && icld != 5) return;
    double decorr_inv = 1.0, decorr_len;
    if (idcor == 1) {
        const double am3 = juldat > 181 ? -4.0 * amr / 365.0 * (double)(juldat - 272)
                                        : 4.0 * amr / 365.0 * (double)(juldat - 91);
        const double d = lat[i] - am3;
        decorr_len = (am1 + am2 * exp(-(d * d) / (am4 * am4))) * 1.e3;
    } else {
        decorr_len = decorr_con;
    }
    if (decorr_len >= 0.0) decorr_inv = 1.0 / decorr_len;
    const size_t n = (size_t)ncol;
    alpha[i] = 0.0;
    for (int k = 2; k <= nlay; ++k) {
        const size_t kk = (size_t)i + n * (size_t)(k - 1), km = kk - n;
        double a = exp(-(0.5 * (dz[kk] + dz[km])) * decorr_inv);
        if (icld == 5 && cldfrac[kk] == 0.0 && cldfrac[km] > 0.0) a = 0.0;
        alpha[kk] = a;
    }
}

cudaError_t launch_get_alpha(int ncol, int nlay, int icld, int idcor, double decorr_con, const double* dz,
                             const double* lat, int juldat, const double* cldfrac, double* alpha, cudaStream_t s) {
    k_get_alpha<<<(ncol + 127) / 128, 128, 0, s>>>(ncol, nlay, icld, idcor, decorr_con, dz, lat, juldat, cldfrac,
                                                  alpha);
    return cudaGetLastError();
}

// ------------------------------------------------------------- McICA
// Fill of the seven subcolumn arrays (mcica_subcol_gen_sw.f90:666-690).
__device__ inline void mcica_fill(bool cloudy, int g, size_t kl, size_t kg, const double* ciwp, const double* clwp,
                                  const double* tauc, const double* ssac, const double* asmc, const double* fsfc,
                                  double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* taucmcl,
                                  double* ssacmcl, double* asmcmcl, double* fsfcmcl) {
    if (cloudy) {
        const size_t kb = (size_t)cT.ngb[g] + 14 * kl;
        cldfmcl[kg] = 1.0;
        clwpmcl[kg] = clwp[kl];
        ciwpmcl[kg] = ciwp[kl];
        taucmcl[kg] = tauc ? tauc[kb] : 0.0;
        ssacmcl[kg] = tauc ? ssac[kb] : 1.0;
        asmcmcl[kg] = tauc ? asmc[kb] : 0.0;
        fsfcmcl[kg] = tauc ? fsfc[kb] : 0.0;
    } else {
        cldfmcl[kg] = 0.0;
        clwpmcl[kg] = 0.0;
        ciwpmcl[kg] = 0.0;
        taucmcl[kg] = 0.0;
        ssacmcl[kg] = 1.0;
        asmcmcl[kg] = 0.0;
        fsfcmcl[kg] = 0.0;
    }
}

// one thread per (column, subcolumn), g fastest for coalesced stores
__global__ void k_mcica_kiss(int ncol, int nlay, int icld, int permuteseed, const double* play,
                             const double* cldfrac, const double* ciwp, const double* clwp, const double* tauc,
                             const double* ssac, const double* asmc, const double* fsfc, const double* alpha,
                             double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* taucmcl, double* ssacmcl,
                             double* asmcmcl, double* fsfcmcl, int* err) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)ncol * NGPT) return;
    const int g = (int)(t % NGPT), col = (int)(t / NGPT);
    const size_t n = (size_t)ncol;
    const uint64_t off = kiss_offset(icld, g, nlay, permuteseed);
    uint32_t xcol[32];
    xorshift_power(off, xcol);
    uint32_t seed[4];
    const double p1 = __dmul_rn(play[col], 1.e2), p2 = __dmul_rn(play[col + n], 1.e2);
    if (p1 < p2) set_error(err, E_KISSSEED);
    seed[0] = kiss_seed(p1);
    seed[1] = kiss_seed(p2);
    seed[2] = kiss_seed(__dmul_rn(play[col + 2 * n], 1.e2));
    seed[3] = kiss_seed(__dmul_rn(play[col + 3 * n], 1.e2));
    McicaMask<false> mc;
    mc.start(kiss_start(seed, kiss_jump_consts(off), xcol), icld);
    for (int lay = 1; lay <= nlay; ++lay) {
        const size_t kl = (size_t)col + n * (size_t)(lay - 1);
        double cf = cldfrac[kl];
        if (cf < 1.0e-20) cf = 0.0;
        const double omcf = __dsub_rn(1.0, cf);
        const bool cloudy = mc.step(lay, kiss_threshold(omcf), icld >= 4 ? kiss_threshold(alpha[kl]) : 0ll, omcf);
        mcica_fill(cloudy, g, kl, (size_t)g + NGPT * kl, ciwp, clwp, tauc, ssac, asmc, fsfc, cldfmcl, ciwpmcl,
                   clwpmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl);
    }
}

cudaError_t launch_mcica_kiss(int ncol, int nlay, int icld, int permuteseed, const double* play,
                              const double* cldfrac, const double* ciwp, const double* clwp, const double* tauc,
                              const double* ssac, const double* asmc, const double* fsfc, const double* alpha,
                              double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* taucmcl,
                              double* ssacmcl, double* asmcmcl, double* fsfcmcl, int* err, cudaStream_t s) {
    const size_t nt = (size_t)ncol * NGPT;
    k_mcica_kiss<<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(ncol, nlay, icld, permuteseed, play, cldfrac, ciwp,
                                                              clwp, tauc, ssac, asmc, fsfc, alpha, cldfmcl, ciwpmcl,
                                                              clwpmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl, err);
    return cudaGetLastError();
}

// McICA from the call's MT19937 stream (irng = 1; tempered words in the
// reference's (subcolumn, column, layer) order, from launch_mt_jump), with
// the same mask walk as the fused solve.
__global__ void k_mcica_stream(int ncol, int nlay, int icld, const uint32_t* rs, const double* cldfrac,
                               const double* ciwp, const double* clwp, const double* tauc, const double* ssac,
                               const double* asmc, const double* fsfc, const double* alpha, double* cldfmcl,
                               double* ciwpmcl, double* clwpmcl, double* taucmcl, double* ssacmcl, double* asmcmcl,
                               double* fsfcmcl) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)ncol * NGPT) return;
    const int g = (int)(t % NGPT), col = (int)(t / NGPT);
    const size_t n = (size_t)ncol;
    McicaMask<true> mc;
    mc.start(Kiss{1u, 1u, 1u, 1u}, icld, rs + mt_offset(icld, g, col, ncol, nlay));
    for (int lay = 1; lay <= nlay; ++lay) {
        const size_t kl = (size_t)col + n * (size_t)(lay - 1);
        double cf = cldfrac[kl];
        if (cf < 1.0e-20) cf = 0.0;
        const double omcf = __dsub_rn(1.0, cf);
        const bool cloudy = mc.step(lay, mt_threshold(omcf), icld >= 4 ? mt_threshold(alpha[kl]) : 0ll, omcf);
        mcica_fill(cloudy, g, kl, (size_t)g + NGPT * kl, ciwp, clwp, tauc, ssac, asmc, fsfc, cldfmcl,
                   ciwpmcl, clwpmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl);
    }
}

cudaError_t launch_mcica_stream(int ncol, int nlay, int icld, const uint32_t* stream, const double* cldfrac,
                                const double* ciwp, const double* clwp, const double* tauc, const double* ssac,
                                const double* asmc, const double* fsfc, const double* alpha, double* cldfmcl,
                                double* ciwpmcl, double* clwpmcl, double* taucmcl, double* ssacmcl,
                                double* asmcmcl, double* fsfcmcl, cudaStream_t s) {
    const size_t nt = (size_t)ncol * NGPT;
    k_mcica_stream<<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(ncol, nlay, icld, stream, cldfrac, ciwp, clwp, tauc,
                                                                ssac, asmc, fsfc, alpha, cldfmcl, ciwpmcl, clwpmcl,
                                                                taucmcl, ssacmcl, asmcmcl, fsfcmcl);
    return cudaGetLastError();
}


// setcoef_sw's integer outputs as the solve computes them: one thread per
// (column, layer) through prep_layer, the routine both forms' kernels call;
// pk (ncol, nlay) holds the packed jp | jt<<8 | jt1<<12 | indself<<16 |
// indfor<<24 | below-100-hPa<<30 word.
static __global__ void __launch_bounds__(256) k_setcoef(const SolveParams P, const double* __restrict__ tab64,
                                                        double* cf, int* pk, double* pdp) {
    const size_t n = (size_t)P.ncol, L = (size_t)P.nlay;
    const size_t it = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n * L) return;
    const int col = (int)(it % n), lay = (int)(it / n) + 1;
    int* pc = pk + (size_t)col * L;
    prep_layer<double>(P, col, lay, cf + (size_t)col * NFR * L, pc, pdp + (size_t)col * L, (int)L, tab64);
}

cudaError_t launch_setcoef(const SolveParams& P, const double* tab64, double* cf, int* pk, double* pdp,
                           cudaStream_t s) {
    const size_t n = (size_t)P.ncol * P.nlay;
    k_setcoef<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, tab64, cf, pk, pdp);
    return cudaGetLastError();
}

}  // namespace rrsw
