// launch.h -- interface between the host C-ABI (api.cu) and the kernel
// translation units (solve_fp64.cu built without FMA contraction,
// solve_fp32.cu built with it).
#pragma once

#include <cuda_runtime.h>

#include "solve.cuh"

namespace rrsw {

struct LaunchInfo {
    int grid;            // CTAs (persistent: each loops over column pairs)
    size_t smem;         // dynamic shared memory per CTA
    bool tiled = false;  // FP32 form: the tiled kernel (layer R/T in shared memory)
    size_t slot_bytes = 0;  // global scratch per CTA
    // tiled kernel: its preparation kernel's grid and shared memory, and the
    // bytes of one pair's prepared block (P.tprep holds npairs of them)
    int prep_grid = 0;
    size_t prep_smem = 0, prep_bytes = 0;
    int tile_slots = 2;  // pair slots of the tiled kernel (SolveParams::tile_slots)
};

// FP64 form
cudaError_t upload_tables_fp64(const DevTables& t);
LaunchInfo plan_fp64(const SolveParams& P, int num_sms);
cudaError_t launch_solve_fp64(const SolveParams& P, const double* tab, const LaunchInfo& li, cudaStream_t s);
// FP32 form
cudaError_t upload_tables_fp32(const DevTables& t);
// setcoef of the FP32 form (FP32 arithmetic, the FP64 form's indices) over all (column, layer)
cudaError_t launch_setcoef_f32(const SolveParams& P, const float* tab, const double* tab64, float* cf, int* pk,
                               double* pdp, cudaStream_t s);
// allow_tiled = false keeps the scratch-based kernel (k_solve<float>)
LaunchInfo plan_fp32(const SolveParams& P, int num_sms, bool allow_tiled = true);
cudaError_t launch_solve_fp32(const SolveParams& P, const float* tab, const double* tab64, const LaunchInfo& li,
                              cudaStream_t s);
// batch of instances (device array of SolveParams, sunlit lists built by
// launch_compact); smem is the largest instance's dynamic shared memory
cudaError_t launch_compact(const SolveParams* dPb, int n, int* map_all, const long long* map_off, int* counts,
                           cudaStream_t s);
// batch kernel with tiles of nc columns (2 or 4) x 112 g-points per CTA
size_t solve_smem_fp64(const SolveParams& P, int nc);
size_t solve_smem_fp32(const SolveParams& P, int nc);
int batch_blocks_per_sm_fp64(size_t smem, int nc);
int batch_blocks_per_sm_fp32(size_t smem, int nc);
cudaError_t launch_batch_fp64(const SolveParams* dPb, int n, const int* counts, const double* tab, int grid,
                              size_t smem, int nc, cudaStream_t s);
cudaError_t launch_batch_fp32(const SolveParams* dPb, int n, const int* counts, const float* tab,
                              const double* tab64, int grid, size_t smem, int nc, cudaStream_t s);
// tangent-linear / adjoint (solve_ad.cu)
cudaError_t upload_tables_ad(const DevTables& t);
size_t adjoint_slot_elems(int nlay, int store);
int adjoint_grid(const SolveParams& P, int num_sms);
cudaError_t launch_adjoint(const SolveParams& P, const AdParams& A, const double* tab64, int num_sms, int* grid_out,
                           cudaStream_t s);
// scratch elements (of the form's type) per CTA slot of nc columns
size_t slot_elems(int nlay, int idelm, bool fp32, int nc = COLS_PER_CTA);

// setcoef_sw indices of every (column, layer) through the solve's prep_layer:
// cf (ncol x NFR x nlay), pk and pdp (ncol x nlay), column-major by column
cudaError_t launch_setcoef(const SolveParams& P, const double* tab64, double* cf, int* pk, double* pdp,
                           cudaStream_t s);
// get_alpha (mcica_subcol_gen_sw.f90:66-178) on the device
cudaError_t launch_get_alpha(int ncol, int nlay, int icld, int idcor, double decorr_con, const double* dz,
                             const double* lat, int juldat, const double* cldfrac, double* alpha, cudaStream_t s);
// mcica_subcol_sw with KISS streams (irng = 0) on the device
cudaError_t launch_mcica_kiss(int ncol, int nlay, int icld, int permuteseed, const double* play,
                              const double* cldfrac, const double* ciwp, const double* clwp, const double* tauc,
                              const double* ssac, const double* asmc, const double* fsfc, const double* alpha,
                              double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* taucmcl,
                              double* ssacmcl, double* asmcmcl, double* fsfcmcl, int* err, cudaStream_t s);
// MT19937 stream of the reference generator seeded with seed: n tempered
// words, segments of 2^log_seg words generated in parallel after a
// jump-ahead (log_seg <= 0: chosen from n and num_sms) (mt19937.cu)
cudaError_t launch_mt_jump(uint32_t seed, uint64_t n, uint32_t* out, int num_sms, int log_seg, cudaStream_t s);
// raw (untempered) words behind outputs offset .. offset+623, on the host;
// 0 or -1 (offset >= 2^48 or jump tables unavailable)
int mt_window_host(uint32_t seed, uint64_t offset, uint32_t* window);
// free the device copies of the jump table (rebuilt on next use)
void mt_release_device_tables();
// mcica_subcol_sw from the call's MT stream (irng = 1, GCM order)
cudaError_t launch_mcica_stream(int ncol, int nlay, int icld, const uint32_t* stream, const double* cldfrac,
                                const double* ciwp, const double* clwp, const double* tauc, const double* ssac,
                                const double* asmc, const double* fsfc, const double* alpha, double* cldfmcl,
                                double* ciwpmcl, double* clwpmcl, double* taucmcl, double* ssacmcl,
                                double* asmcmcl, double* fsfcmcl, cudaStream_t s);

}  // namespace rrsw
