// common.cuh -- device-side tables and shared definitions of the GB300
// RRTMG_SW solver.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rrsw {

constexpr int NBND = 14;
constexpr int NGPT = 112;
constexpr int NTBL = 10000;
constexpr int COLS_PER_CTA = 2;                  // 2 columns x 112 g-points = 7 warps
constexpr int CTA_THREADS = COLS_PER_CTA * NGPT;  // 224
constexpr int MAX_NLAY = 1000;

// Offsets (in elements) of one band's reduced tables inside the table blob.
// Absorption-type tables are stored transposed so that consecutive
// g-points of a band are contiguous: absa(ind, ig) -> [(ind-1)*ng + ig-1].
struct BandOff {
    int ng, g0, nspa, nspb, nfr;
    int absa, absb, selfref, forref;
    int sfluxref, irradnce, facbrght, snsptdrk;  // (ng, js): [(js-1)*ng + ig-1]
    int rayl, rayla, raylb, abso3a, abso3b, absch4, absco2, absh2o;
};

// Gas optics of one band and region (below / above laytrop) in the form
// used by the FP32 solve: every taumolNN loop is one of
//   kind 1: speccomb * 8-point k (binary species parameter, taumol.f90:309-338)
//   kind 2: column(sa) * fac * 4-point k
// plus an optional water-vapour continuum, one minor-species term and the
// Rayleigh depth, so all bands run one code path.
struct TmRegion {
    int8_t kind, sa, sb, cont, minor, rtype, nsp, jo;
    float strrat, fac, mult;
    int ktab, mtab, rtab;
};

// One band/region descriptor with the band's continuum offsets, as the FP32
// solve keeps it in shared memory: a warp's g-points span several bands, and
// indexing the constant bank by band serialises; three 16-byte shared loads
// per layer replace those constant loads.
struct alignas(16) TmSmem {
    TmRegion r;
    int selfref, forref, ng, pad;
};

struct DevTables {
    BandOff b[NBND];
    int pref, preflog, tref;
    // cloud LUTs, Fortran order (index, band): [(ib-16)*n + index-1]
    int extliq1, ssaliq1, asyliq1, extice2, ssaice2, asyice2;
    int extice3, ssaice3, asyice3, fdlice3;
    int abari, bbari, cbari, dbari, ebari, fbari;
    int coliq1, coice2, coice3;     // 1 - ssa of the cloud LUTs, formed in FP64 (FP32 form)
    int rsrtaua, rsrpiza, rsrasya;  // (14, 6)
    int wavenum2;
    int exp_tbl;                    // (0:10000)
    int total;                      // blob size
    int8_t ngb[NGPT];               // band index 0..13 of each g-point
    uint8_t gib[NGPT];              // g index within its band, 1-based
    // FP64 solve and adjoint CTAs: thread -> column slot (bit 7) and g-point
    // (bits 0-6).  The g-points of a band sit together with both columns'
    // copies, so a warp spans 2 (at most 3) bands and band-dependent
    // branches diverge less.
    uint8_t thr_cg[CTA_THREADS];
    // bounds-check builds (RRTMG_BOUNDS_CHECK): word set to E_BOUNDS when a
    // table index falls outside the blob
    int* bounds_err;
    double heatfac, bpade, oneminus;
    float bpade_f, oneminus_f;
    TmRegion tm[NBND][2];
    // GF(2) jump matrices of the KISS xorshift component: column j of
    // M^(2^k) at xs_jump[k][j]
    uint32_t xs_jump[32][32];
};

// every translation unit that launches kernels holds its own copy, filled by
// its upload function (no relocatable device code needed)
static __constant__ DevTables cT;

// Table read of element i of a coefficient blob (FP64 or FP32 copy, both
// cT.total elements).  A bounds-check build (-DRRTMG_BOUNDS_CHECK) tests i
// against the blob, records E_BOUNDS in cT.bounds_err and reads a clamped
// element instead of leaving the blob.
template <typename T>
__device__ __forceinline__ T ldt(const T* __restrict__ tab, int i) {
#ifdef RRTMG_BOUNDS_CHECK
    if (i < 0 || i >= cT.total) {
        if (cT.bounds_err) atomicCAS(cT.bounds_err, 0, 40);
        i = i < 0 ? 0 : cT.total - 1;
    }
#endif
    return __ldg(tab + i);
}

// Error word: first error code wins.
__device__ inline void set_error(int* err, int code) {
    if (err) atomicCAS(err, 0, code);
}

constexpr int MAX_BATCH = 1024;  // instances per batch launch

// Error codes (mirror include/rrtmg_sw_gb300.h)
enum {
    E_OK = 0, E_INFLAG1 = 10, E_ICERAD = 11, E_ICEDGE = 12, E_ICEPROP = 13,
    E_LIQRAD = 14, E_LIQPROP = 15, E_ICLD = 20, E_KISSSEED = 21, E_LAYTROP = 30, E_PARTIAL = 32,
    E_BOUNDS = 40, E_TIMEOUT = 41
};

}  // namespace rrsw
