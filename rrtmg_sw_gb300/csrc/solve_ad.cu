// solve_ad.cu -- tangent-linear and adjoint of the FP64 column solve (see ad.cuh).
#include "ad.cuh"
#include "launch.h"

namespace rrsw {

// every translation unit has its own copy of the constant tables
cudaError_t upload_tables_ad(const DevTables& t) { return cudaMemcpyToSymbol(cT, &t, sizeof(DevTables)); }

size_t adjoint_slot_elems(int nlay, int store) { return ad_slot_elems(nlay, store); }

cudaError_t launch_adjoint(const SolveParams& P, const AdParams& A, const double* tab64, int num_sms, int* grid_out,
                           cudaStream_t s) {
    const size_t smem = ad_smem_layout(P.nlay).total;
    cudaError_t e = cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint, CTA_THREADS, smem);
    if (per_sm < 1) per_sm = 1;
    int grid = num_sms * per_sm;
    if (grid > P.npairs) grid = P.npairs;
    if (grid < 1) grid = 1;
    if (grid_out) *grid_out = grid;
    k_adjoint<<<grid, CTA_THREADS, smem, s>>>(P, A, tab64);
    return cudaGetLastError();
}

int adjoint_grid(const SolveParams& P, int num_sms) {
    const size_t smem = ad_smem_layout(P.nlay).total;
    cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint, CTA_THREADS, smem);
    if (per_sm < 1) per_sm = 1;
    int grid = num_sms * per_sm;
    if (grid > P.npairs) grid = P.npairs;
    return grid < 1 ? 1 : grid;
}

}  // namespace rrsw
