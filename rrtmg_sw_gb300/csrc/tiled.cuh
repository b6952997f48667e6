// tiled.cuh -- FP32 form of the solve with every layer's reflectance and
// transmittance kept on chip.  Included by solve_fp32.cu (FMA contraction,
// approximate FP32 division).
//
// One persistent CTA per SM works through column pairs.  A pair's 224
// subcolumns (column x g-point) are cut into 7 tiles of 32.  A tile holds,
// for its 32 subcolumns and every layer, the clear and total layer
// reflectance, absorptance and direct transmittance of spcvmc_sw /
// reftra_sw (rrtmg_sw_spcvmc.f90:442-585, rrtmg_sw_reftra.f90:151-326) in
// shared memory, two tiles double-buffered.  Warp roles:
//
//   optics warps (T_OPT): per pair, the pair's prepared block (below) into
//     shared memory; then per tile the cells (g-point, layer) -- gas optics, clouds, aerosol,
//     delta scaling, the two-stream layer solution -- layer rows taken from
//     a shared counter, the 32 subcolumns of a row in one warp (32
//     consecutive g-points: coalesced table reads).
//   adding warps (2): per tile, the vertical adding method of vrtqdr_sw
//     (rrtmg_sw_vrtqdr.f90:122-169), one lane per subcolumn, one warp for
//     the clear sky and one for the total sky (the two recurrences are
//     independent): up-sweep from the surface (upward albedos kept in shared
//     memory), down-sweep with the weighted level fluxes written into the
//     tile slots the warp has just read; then the g-point sums of spcvmc_sw
//     (:607-655), one lane per level, half of the levels per warp.
//   FP64 warps (2, pairs in turn): redo in FP64 the cells whose FP32 discrete
//     choices (transmittance table entry, conservative switch, resonance)
//     are too close to call, for the whole pair at once (FP64 runs at a small
//     fraction of the FP32 rate, so its cells are processed 32 at a time);
//     then finish the pair (below) and write its outputs.
//
// A separate kernel, k_tiled_prep, prepares each pair beforehand at full
// occupancy: setcoef in FP32 with the FP64 form's table indices, the McICA subcolumn masks
// (one walk per subcolumn), the solar source and albedos, the cloud and
// aerosol inputs in FP32 -- about 16 KB per pair in HBM (60 layers, no
// aerosol).  In the solve kernel that work would stall the optics warps;
// read back it costs a few vector loads per pair.  setcoef in FP64 (as the
// scratch-based kernel does it) would cost more than a tenth of the solve
// at GB300's FP64 rate.
//
// A subcolumn with such a cell is left out of its tile's sums; the optics
// warps copy its R/T column aside (global, per CTA) once the tile is done,
// and the FP64 warp sweeps it again with the FP64 cells, its contribution
// added before the pair's outputs are written.  Handoffs use mbarriers
// (tile full / empty; per pair slot: pair produced, swept, finished) whose
// waits give up after ~2^33 cycles with an error code instead of hanging.  A pair with more such cells than the
// capacities below is listed for the caller, which solves it again with the
// scratch-based kernel (k_solve<float>).
#pragma once

#include "kernel.cuh"

#ifndef RRSW_TILED_OPT
#define RRSW_TILED_OPT 20
#endif
#ifndef RRSW_TILED_F64
#define RRSW_TILED_F64 2
#endif

namespace rrsw {

constexpr int TW = 32;                                   // subcolumns per tile
constexpr int TILES = COLS_PER_CTA * NGPT / TW;          // 7 tiles per pair
constexpr int T_OPT = RRSW_TILED_OPT;                    // optics warps
constexpr int T_F64 = RRSW_TILED_F64;                    // FP64 warps (pairs taken in turn)
// (a third FP64 warp could wait on a slot's barrier two phases early when
// there are only two pair slots)
static_assert(T_F64 == 1 || T_F64 == 2, "one or two FP64 warps");
constexpr int T_REDO = T_OPT;                            // first FP64 warp
constexpr int T_ADDC = T_OPT + T_F64;                    // adding warp, clear sky
constexpr int T_ADDT = T_OPT + T_F64 + 1;                // adding warp, total sky
constexpr int T_THREADS = (T_OPT + T_F64 + 2) * 32;
constexpr int T_QCAP = 128;                              // FP64 cells per pair
constexpr int T_RCAP = 64;                               // subcolumns with such cells per pair
constexpr int T_NF = 10;                                 // tile fields per cell
constexpr int T_MAXL = 64;                               // layers (two mask words per subcolumn)
enum { TF_REFC, TF_REFDC, TF_ADIRC, TF_ADIFC, TF_DBTC, TF_REF, TF_REFD, TF_ADIR, TF_ADIF, TF_DBT };
// Pair slots: the per-pair state (solar source and albedos, active flags,
// FP64 queue, set-aside marks, level sums) of pair lp sits in slot
// lp % nslot, nslot = 3 when shared memory allows (else 2), so the optics
// and adding warps can start pair lp while pairs lp - 1 and lp - 2 are still
// swept or finished.
constexpr int T_SLOTS = 3;
// mbarriers: tile buffers (FULL, EMPTY per buffer), then per pair slot the
// pair produced (PAIR), swept (SWEPT) and finished (FIN)
enum { TB_FULL0, TB_FULL1, TB_EMPTY0, TB_EMPTY1, TB_PAIR0, TB_SWEPT0 = TB_PAIR0 + T_SLOTS,
       TB_FIN0 = TB_SWEPT0 + T_SLOTS, TB_N = TB_FIN0 + T_SLOTS };
// control words in shared memory: row counters per tile buffer; per slot the
// FP64 queue length and (TC_ACT0 + 2 * slot + column) the active flags
enum { TC_ROW0, TC_ROW1, TC_ABORT, TC_LT0, TC_LT1, TC_QN0, TC_ACT0 = TC_QN0 + T_SLOTS,
       TC_N = TC_ACT0 + 2 * T_SLOTS };

// Shared-memory carve-up of the tiled kernel; the host sizes the launch with
// the same function.
struct TSmem {
    size_t bar, ctl, tm, tile, rup, coef, pk, hrf, mu, cld, mask, sub, risky, queue, recof, flux, scr, scr2,
        total;
};

__host__ __device__ inline TSmem tiled_smem(int L, int nq, bool fused, bool cloud_stage, int nslot) {
    TSmem m;
    size_t o = 0;
    m.bar = o;   o = align16(o + TB_N * sizeof(unsigned long long));
    m.ctl = o;   o = align16(o + TC_N * sizeof(int));
    m.tm = o;    o = align16(o + NBND * 2 * sizeof(TmSmem));
    m.tile = o;  o = align16(o + (size_t)2 * T_NF * L * TW * sizeof(float));
    m.rup = o;   o = align16(o + (size_t)4 * L * TW * sizeof(float));
    m.coef = o;  o = align16(o + (size_t)COLS_PER_CTA * NFR * L * sizeof(float));
    m.pk = o;    o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(int));
    m.hrf = o;   o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(float));
    m.mu = o;    o = align16(o + (size_t)COLS_PER_CTA * sizeof(float));
    m.cld = m.mask = o;
    if (cloud_stage) { m.cld = o; o = align16(o + (size_t)COLS_PER_CTA * 4 * L * sizeof(float)); }
    if (fused) { m.mask = o; o = align16(o + (size_t)COLS_PER_CTA * NGPT * 2 * sizeof(uint32_t)); }
    // per pair slot
    m.sub = o;   o = align16(o + (size_t)nslot * 3 * COLS_PER_CTA * NGPT * sizeof(float));   // [slot][zinc,albp,albd][224]
    m.risky = o; o = align16(o + (size_t)nslot * TILES * sizeof(uint32_t));
    m.queue = o; o = align16(o + (size_t)nslot * T_QCAP * sizeof(int));
    m.recof = o; o = align16(o + (size_t)nslot * COLS_PER_CTA * NGPT * sizeof(short));
    m.flux = o;  o = align16(o + (size_t)nslot * COLS_PER_CTA * nq * (L + 1) * sizeof(float));
    // adding warps: surface-level sums and lane keys of a tile
    m.scr = o;   o = align16(o + (size_t)16 * TW * sizeof(float));
    // FP64 warp: reduction scratch of the set-aside subcolumns (rows 6-7: 64-bit keys)
    m.scr2 = o;  o = align16(o + (size_t)T_F64 * 16 * TW * sizeof(float));
    m.total = o;
    return m;
}

// Per-CTA global area of the tiled kernel (bytes): the FP64 warps' albedo
// scratch and, per pair slot, the FP64 cells and the set-aside subcolumns.
struct TGlob {
    size_t rrup, par, corr, rec, rec_stride, par_stride, total;
};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

__host__ __device__ inline TGlob tiled_glob(int L) {
    TGlob g;
    size_t o = 0;
    g.rrup = o; o = align256(o + (size_t)T_F64 * 4 * L * TW * sizeof(float));   // FP64 warps: record sweeps' albedos
    g.par = o;
    size_t p = 0;
    g.corr = p;   p = align256(p + (size_t)T_QCAP * T_NF * sizeof(float));
    // record: s, column slot, zinc, albp, albd, pad[3], then T_NF x L fields
    g.rec_stride = align256((8 + (size_t)T_NF * L) * sizeof(float));
    g.rec = p;    p = align256(p + (size_t)T_RCAP * g.rec_stride);
    g.par_stride = p;
    o += T_SLOTS * p;
    g.total = o;
    return g;
}

// A pair's prepared block in global memory (bytes), written by
// k_tiled_prep and read by k_solve_tiled: setcoef's FP32 coefficients and
// packed indices, heatfac / dp, dp in FP64, the cloud inputs and the
// aerosol (FP32), per subcolumn zinc, direct and diffuse albedo, the McICA
// mask bits, and per column laytrop, the active flag and mu0.
struct TPrep {
    size_t coef, pk, hrf, pdp, cld, aer, sub, mask, misc, total;
};
enum { TP_LT0, TP_LT1, TP_ACT0, TP_ACT1, TP_MU0, TP_MU1, TP_N };

__host__ __device__ inline TPrep tiled_prep_layout(int L, bool fused, bool cloud_stage, bool aerosol) {
    TPrep b;
    size_t o = 0;
    b.coef = o; o = align16(o + (size_t)COLS_PER_CTA * NFR * L * sizeof(float));
    b.pk = o;   o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(int));
    b.hrf = o;  o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(float));
    b.pdp = o;  o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(double));
    b.cld = b.aer = b.mask = o;
    if (cloud_stage) { b.cld = o; o = align16(o + (size_t)COLS_PER_CTA * 4 * L * sizeof(float)); }
    if (aerosol) { b.aer = o; o = align16(o + (size_t)COLS_PER_CTA * 3 * NBND * L * sizeof(float)); }
    b.sub = o;  o = align16(o + (size_t)3 * COLS_PER_CTA * NGPT * sizeof(float));
    if (fused) { b.mask = o; o = align16(o + (size_t)COLS_PER_CTA * NGPT * 2 * sizeof(uint32_t)); }
    b.misc = o; o = align16(o + (size_t)TP_N * sizeof(int));
    b.total = align256(o);
    return b;
}

// Shared memory of k_tiled_prep (bytes).
struct TPrepSmem {
    size_t xs, tm, coef, pk, kc, ka, omcf, seed, misc, total;
};
__host__ __device__ inline TPrepSmem tiled_prep_smem(int L) {
    TPrepSmem m;
    size_t o = 0;
    m.xs = o;   o = align16(o + (size_t)NGPT * 32 * sizeof(uint32_t));
    m.tm = o;   o = align16(o + (size_t)NBND * 2 * sizeof(TmSmem));
    m.coef = o; o = align16(o + (size_t)COLS_PER_CTA * NFR * L * sizeof(float));
    m.pk = o;   o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(int));
    m.kc = o;   o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(long long));
    m.ka = o;   o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(long long));
    m.omcf = o; o = align16(o + (size_t)COLS_PER_CTA * L * sizeof(double));
    m.seed = o; o = align16(o + (size_t)COLS_PER_CTA * 4 * sizeof(uint32_t));
    m.misc = o; o = align16(o + (size_t)TP_N * sizeof(int));
    m.total = o;
    return m;
}

// ------------------------------------------------------------- mbarriers
__device__ inline uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ inline void mbar_init(unsigned long long* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}

__device__ inline void mbar_arrive(unsigned long long* b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(b))
                 : "memory");
}

__device__ inline bool mbar_test(unsigned long long* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the completion of the phase of parity `parity`.  Gives up after
// ~2^33 cycles (seconds; a tile takes microseconds): records E_TIMEOUT and
// the CTA's abort flag, after which every later wait returns at once, so a
// fault in the handoff ends the kernel with an error instead of a hang.
__device__ inline void mbar_wait(unsigned long long* b, unsigned parity, volatile int* abort, int* err) {
    if (*abort) return;
    const long long t0 = clock64();
    while (!mbar_test(b, parity)) {
        if (*abort) return;
        if (clock64() - t0 > (1ll << 33)) {
            *abort = 1;
            set_error(err, E_TIMEOUT);
            return;
        }
    }
}

// named barriers: the optics warps; the two adding warps
__device__ inline void opt_sync() { asm volatile("bar.sync 1, %0;" ::"n"(T_OPT * 32) : "memory"); }
__device__ inline void add_sync() { asm volatile("bar.sync 2, 64;" ::: "memory"); }

// ------------------------------------------------------------- helpers
struct TileView {
    unsigned long long* bar;
    int* ctl;
    const TmSmem* tm;
    float* tile;      // [2][T_NF][L][TW]
    float* rup;       // [4][L][TW]
    float* coef;      // [2][NFR][L]
    int* pk;          // [2][L]
    float* hrf;       // [2][L]
    float* mu;        // [2]
    float* cld;       // [2][4][L]
    uint32_t* mask;   // [224][2]
    float* sub;       // [slot][3][224]
    uint32_t* risky;  // [slot][TILES]
    int* queue;       // [slot][T_QCAP]
    short* recof;     // [slot][224]
    float* flux;      // [slot][2][NQ][L+1]
    float* scr;       // [16][TW] adding warps
    float* scr2;      // [T_F64][16][TW] FP64 warps
};

__device__ inline TileView tile_view(unsigned char* raw, const TSmem& M) {
    TileView v;
    v.bar = (unsigned long long*)(raw + M.bar);
    v.ctl = (int*)(raw + M.ctl);
    v.tm = (const TmSmem*)(raw + M.tm);
    v.tile = (float*)(raw + M.tile);
    v.rup = (float*)(raw + M.rup);
    v.coef = (float*)(raw + M.coef);
    v.pk = (int*)(raw + M.pk);
    v.hrf = (float*)(raw + M.hrf);
    v.mu = (float*)(raw + M.mu);
    v.cld = (float*)(raw + M.cld);
    v.mask = (uint32_t*)(raw + M.mask);
    v.sub = (float*)(raw + M.sub);
    v.risky = (uint32_t*)(raw + M.risky);
    v.queue = (int*)(raw + M.queue);
    v.recof = (short*)(raw + M.recof);
    v.flux = (float*)(raw + M.flux);
    v.scr = (float*)(raw + M.scr);
    v.scr2 = (float*)(raw + M.scr2);
    return v;
}

// Tile buffer layout (T_NF * L * TW floats): per sky (0 clear, 1 total) the
// fields ref, refd, adir, adif of each (layer index i, lane) as one float4
// -- one 16-byte access for the adding warps, whose sweeps are bound by
// instruction issue -- then per sky the direct transmittances.
__device__ inline float4* tquad(float* tb, int L, int sky, int i) { return (float4*)tb + ((size_t)sky * L + i) * TW; }
__device__ inline float* tdbt(float* tb, int L, int sky, int i) {
    return tb + (size_t)8 * L * TW + ((size_t)sky * L + i) * TW;
}
// tile field f (TF_*) of layer index i (0 = surface layer), lane l
__device__ inline float& tfield(float* tb, int L, int f, int i, int l) {
    const int sky = f >= 5 ? 1 : 0, c = f - 5 * sky;
    return c < 4 ? ((float*)tquad(tb, L, sky, i))[4 * l + c] : tdbt(tb, L, sky, i)[l];
}

// ---------------------------------------------------------- adding method
// One sky's layer fields in a tile: reflectance, diffuse reflectance,
// absorptance (direct, diffuse incidence), direct transmittance.

// State of one sky's down-sweep of one subcolumn, plus the absorption of the
// layer above the current level for the heating rate.
struct Down1 {
    float tdbt, tdn, rdnd, abs, adif_up;
};

__device__ inline void down1_init(Down1& s) {
    s.tdbt = s.tdn = 1.0f;
    s.rdnd = s.abs = s.adif_up = 0.0f;
}

// Fluxes at a level whose upward albedos (below it) are rup, rupd (vrtqdr:
// 163-169), weighted by zinc: q = up, down, direct down, absorption of the
// layer above the level (its lower face's upward flux added here); dif is
// the diffuse down flux, for the layer step.
__device__ inline void level1(const Down1& s, float rup, float rupd, float zinc, float* q, float& dif) {
    const float zr = 1.0f / (1.0f - s.rdnd * rupd);
    const float u = (s.tdbt * rup + (s.tdn - s.tdbt) * rupd) * zr;
    dif = (s.tdn - s.tdbt + s.tdbt * rup * s.rdnd) * zr;
    q[0] = zinc * u;
    q[1] = zinc * (s.tdbt + dif);
    q[2] = zinc * s.tdbt;
    q[3] = zinc * (s.abs + u * s.adif_up);
}

// Through one layer downward (vrtqdr:144-159, direct beam spcvmc:575-585);
// f = the sky's 5 fields.  The layer's absorption is carried to the next level.
__device__ inline void down1(Down1& s, const float* f, float dif) {
    const float ref = f[0], refd = f[1], adir = f[2], adif = f[3], dbt = f[4];
    const float tra = 1.0f - ref - adir, trad = 1.0f - refd - adif;
    s.abs = s.tdbt * adir + dif * adif;
    s.adif_up = adif;
    const float zr = 1.0f / (1.0f - refd * s.rdnd);
    const float tdn_n = s.tdbt * tra + (trad * ((s.tdn - s.tdbt) + s.tdbt * ref * s.rdnd)) * zr;
    s.rdnd = refd + trad * trad * s.rdnd * zr;
    s.tdn = tdn_n;
    s.tdbt = dbt * s.tdbt;
}

// One up-sweep step of one sky through a layer (vrtqdr:122-140).
__device__ inline void up1(const float* f, float& rup, float& rupd) {
    const float ref = f[0], refd = f[1], dbt = f[4];
    const float tra = 1.0f - ref - f[2], trad = 1.0f - refd - f[3];
    const float zr = 1.0f / (1.0f - rupd * refd);
    const float r = ref + (trad * ((tra - dbt) * rupd + dbt * rup)) * zr;
    rupd = refd + trad * trad * rupd * zr;
    rup = r;
}

// ------------------------------------------------------------ the kernel
struct TCtx {
    TileView V;
    TGlob G;
    TPrep B;
    unsigned char* glob;        // this CTA's global area
    const unsigned char* prep;  // the prepared blocks of all pairs
    int L, nmapped, qcap, nlocal, nslot;
    bool fused, nomc, cstage;
    volatile int* abort;
};

__device__ inline const unsigned char* tblk(const TCtx& X, int pair) { return X.prep + (size_t)pair * X.B.total; }

__device__ inline unsigned char* tpar(const TCtx& X, int slot) {
    return X.glob + X.G.par + (size_t)slot * X.G.par_stride;
}
__device__ inline float* trec(const TCtx& X, int slot, int r) {
    return (float*)(tpar(X, slot) + X.G.rec + (size_t)r * X.G.rec_stride);
}
__device__ inline int tpair(int lp) { return blockIdx.x + lp * gridDim.x; }
// pair lp's slot, and the phase parity of the slot's barriers for it
__device__ inline int tslot(const TCtx& X, int lp) { return lp % X.nslot; }
__device__ inline unsigned tphase(const TCtx& X, int lp) { return (unsigned)(lp / X.nslot) & 1u; }

// ---- k_tiled_prep: one CTA (2 columns x 112 g-points) per pair at a time,
// persistent.  setcoef (FP32, the FP64 form's indices), McICA
// thresholds, cloud and aerosol inputs; then per column laytrop; then per
// subcolumn the solar source, the albedos and the McICA mask bits
// (rrtmg_sw_setcoef.f90:158-301, mcica_subcol_gen_sw.f90:472-600,
// rrtmg_sw_spcvmc.f90:349-356).
template <bool MT>
__global__ void __launch_bounds__(CTA_THREADS, 4)
k_tiled_prep(const SolveParams P, const float* __restrict__ tab, const double* __restrict__ tab64) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int L = P.nlay, tid = threadIdx.x;
    const size_t n = (size_t)P.ncol;
    const bool fused = P.fused && P.icld >= 1, nomc = P.nomcica && P.icld >= 1, cstage = fused || nomc;
    const TPrep B = tiled_prep_layout(L, fused, cstage, P.iaer != 0);
    const TPrepSmem M = tiled_prep_smem(L);
    uint32_t* xs = (uint32_t*)(sm + M.xs);
    TmSmem* tm = (TmSmem*)(sm + M.tm);
    float* scoef = (float*)(sm + M.coef);
    int* spk = (int*)(sm + M.pk);
    long long* skc = (long long*)(sm + M.kc);
    long long* ska = (long long*)(sm + M.ka);
    double* somcf = (double*)(sm + M.omcf);
    uint32_t* sseed = (uint32_t*)(sm + M.seed);
    int* smisc = (int*)(sm + M.misc);
    for (int i = tid; i < NBND * 2; i += CTA_THREADS) {
        TmSmem d;
        d.r = cT.tm[i / 2][i % 2];
        d.selfref = cT.b[i / 2].selfref;
        d.forref = cT.b[i / 2].forref;
        d.ng = cT.b[i / 2].ng;
        d.pad = 0;
        tm[i] = d;
    }
    // KISS: the xorshift part of each subcolumn's stream jump (depends on g)
    if (fused && !MT && tid < NGPT) xorshift_power(kiss_offset(P.icld, tid, L, P.permuteseed), xs + tid * 32);
    const int s = tid, c2s = s / NGPT, g = s % NGPT;
    const int ib = cT.ngb[g], igb = cT.gib[g];
    KissJump J{1u, 0u, 1u, 1u};
    if (fused && !MT) J = kiss_jump_consts(kiss_offset(P.icld, g, L, P.permuteseed));
    __syncthreads();
    for (int pair = blockIdx.x; pair < P.npairs; pair += gridDim.x) {
        unsigned char* blk = (unsigned char*)P.tprep + (size_t)pair * B.total;
        double* pdp = (double*)(blk + B.pdp);
        float* hrf = (float*)(blk + B.hrf);
        for (int it = tid; it < COLS_PER_CTA * L; it += CTA_THREADS) {
            const int c2 = it / L, lay = it % L + 1, i = lay - 1;
            const int pcol = COLS_PER_CTA * pair + c2;
            prep_layer_f32(P, pcol, lay, scoef + c2 * NFR * L, spk + c2 * L, pdp + c2 * L, L, tab, tab64);
            hrf[c2 * L + i] = (float)cT.heatfac / (float)pdp[c2 * L + i];  // risk thresholds only
            const bool real = pcol < P.ncol;
            const size_t kl = (size_t)pcol + n * (size_t)i;
            if (fused) {
                double cf = real ? P.cldfrac[kl] : 0.0;
                if (cf < 1.0e-20) cf = 0.0;
                const double omcf = DS(1.0, cf);
                somcf[c2 * L + i] = omcf;
                if constexpr (MT) {
                    skc[c2 * L + i] = mt_threshold(omcf);
                    ska[c2 * L + i] = (P.icld >= 4 && real) ? mt_threshold(P.alpha[kl]) : 0ll;
                } else {
                    skc[c2 * L + i] = kiss_threshold(omcf);
                    ska[c2 * L + i] = (P.icld >= 4 && real) ? kiss_threshold(P.alpha[kl]) : 0ll;
                }
                if (lay == 1) {
                    uint32_t* sd = sseed + c2 * 4;
                    if (real && !MT) {
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
            if (nomc) {
                // spcvrt_sw takes clear or overcast layers only (rrtmg_sw_rad.nomcica.f90:617-621)
                const double cf = real ? P.cldfrac[kl] : 0.0;
                if (cf > 1.e-6 && cf < 1.0 - 1.e-6) set_error(P.err, E_PARTIAL);
            }
            if (cstage) {
                float* cd = (float*)(blk + B.cld) + c2 * 4 * L;
                cd[0 * L + i] = real ? (float)P.ciwp[kl] : 0.0f;
                cd[1 * L + i] = real ? (float)P.clwp[kl] : 0.0f;
                cd[2 * L + i] = real ? (float)P.rei[kl] : 0.0f;
                cd[3 * L + i] = real ? (float)P.rel[kl] : 0.0f;
            }
            if (P.iaer != 0) {
                float* ad = (float*)(blk + B.aer) + c2 * 3 * NBND * L;
                for (int b = 0; b < NBND; ++b) {
                    double ta = 0.0, oa = 1.0, ga = 0.0;
                    if (real) aerosol(P, pcol, lay, b, tab64, ta, oa, ga);
                    ad[(0 * NBND + b) * L + i] = (float)ta;
                    ad[(1 * NBND + b) * L + i] = (float)DS(1.0, oa);  // co-albedo, formed in FP64
                    ad[(2 * NBND + b) * L + i] = (float)ga;
                }
            }
        }
        __syncthreads();
        if (tid < COLS_PER_CTA) {
            const int c2 = tid;
            int lt = 0;
            for (int i = 0; i < L; ++i) lt += (spk[c2 * L + i] >> 30) & 1;
            const int pcol = COLS_PER_CTA * pair + c2;
            int act = pcol < P.ncol;
            if (act && (lt < 1 || lt >= L)) {
                set_error(P.err, E_LAYTROP);
                act = 0;
            }
            double cz = act ? P.coszen[pcol] : 1.0;
            if (cz < 1.e-10) cz = 1.e-10;
            smisc[TP_LT0 + c2] = lt;
            smisc[TP_ACT0 + c2] = act;
            smisc[TP_MU0 + c2] = __float_as_int((float)cz);
        }
        __syncthreads();
        {
            const int c2 = c2s;
            const int pcol = COLS_PER_CTA * pair + c2;
            const bool act = smisc[TP_ACT0 + c2] != 0;
            float zinc = 0.0f, albp = 0.0f, albd = 0.0f;
            if (act) {
                const bool nir = ib <= 8 || ib == 13;
                albp = (float)(nir ? P.aldir[pcol] : P.asdir[pcol]);
                albd = (float)(nir ? P.aldif[pcol] : P.asdif[pcol]);
                const Coef<float> C{scoef + c2 * NFR * L, spk + c2 * L, L, smisc[TP_LT0 + c2]};
                // zincflx = adjflux * ssi * prmu0 (spcvmc:349-356)
                const float src = solar_source_generic(ib, igb, C, P, tab, tm);
                zinc = float(P.adjflux[ib]) * src * __int_as_float(smisc[TP_MU0 + c2]);
            }
            float* sub = (float*)(blk + B.sub);
            sub[s] = zinc;
            sub[COLS_PER_CTA * NGPT + s] = albp;
            sub[2 * COLS_PER_CTA * NGPT + s] = albd;
            if (fused) {
                uint32_t w0 = 0u, w1 = 0u;
                if (act) {
                    McicaMask<MT> mc;
                    Kiss k0{1u, 1u, 1u, 1u};
                    if constexpr (!MT) k0 = kiss_start(sseed + c2 * 4, J, xs + g * 32);
                    mc.start(k0, P.icld, MT ? P.mt + mt_offset(P.icld, g, pcol, P.ncol, L) : nullptr);
                    for (int lay = 1; lay <= L; ++lay) {
                        const int i = lay - 1;
                        if (mc.step(lay, skc[c2 * L + i], ska[c2 * L + i], somcf[c2 * L + i])) {
                            if (i < 32) w0 |= 1u << i;
                            else w1 |= 1u << (i - 32);
                        }
                    }
                }
                uint32_t* mk = (uint32_t*)(blk + B.mask);
                mk[s * 2] = w0;
                mk[s * 2 + 1] = w1;
            }
        }
        // the coefficients, indices and column words to the block
        float* cfo = (float*)(blk + B.coef);
        for (int i = tid; i < COLS_PER_CTA * NFR * L; i += CTA_THREADS) cfo[i] = scoef[i];
        int* pko = (int*)(blk + B.pk);
        for (int i = tid; i < COLS_PER_CTA * L; i += CTA_THREADS) pko[i] = spk[i];
        if (tid < TP_N) ((int*)(blk + B.misc))[tid] = smisc[tid];
        __syncthreads();
    }
}

// 16-byte copy of n bytes (n a multiple of 16) by the optics warps
__device__ inline void opt_copy(void* dst, const void* src, size_t n) {
    const float4* a = (const float4*)src;
    float4* d = (float4*)dst;
    for (size_t i = threadIdx.x; i < n / 16; i += T_OPT * 32) d[i] = a[i];
}

// ---- optics warps: pair lp's prepared block into shared memory
__device__ void tiled_load(const SolveParams& P, const TCtx& X, int lp) {
    const TileView& V = X.V;
    const int L = X.L, slot = tslot(X, lp);
    const unsigned char* blk = tblk(X, tpair(lp));
    opt_copy(V.coef, blk + X.B.coef, align16((size_t)COLS_PER_CTA * NFR * L * sizeof(float)));
    opt_copy(V.pk, blk + X.B.pk, align16((size_t)COLS_PER_CTA * L * sizeof(int)));
    opt_copy(V.hrf, blk + X.B.hrf, align16((size_t)COLS_PER_CTA * L * sizeof(float)));
    if (X.cstage) opt_copy(V.cld, blk + X.B.cld, align16((size_t)COLS_PER_CTA * 4 * L * sizeof(float)));
    if (X.fused) opt_copy(V.mask, blk + X.B.mask, (size_t)COLS_PER_CTA * NGPT * 2 * sizeof(uint32_t));
    opt_copy(V.sub + slot * 3 * COLS_PER_CTA * NGPT, blk + X.B.sub, (size_t)3 * COLS_PER_CTA * NGPT * sizeof(float));
    const int* misc = (const int*)(blk + X.B.misc);
    if (threadIdx.x < COLS_PER_CTA) {
        const int c2 = threadIdx.x;
        V.ctl[TC_LT0 + c2] = misc[TP_LT0 + c2];
        V.ctl[TC_ACT0 + 2 * slot + c2] = misc[TP_ACT0 + c2];
        V.mu[c2] = __int_as_float(misc[TP_MU0 + c2]);
    }
    opt_sync();
}

// ---- optics warps: the cells of tile t of pair lp into buffer b
__device__ void tiled_optics(const SolveParams& P, const TCtx& X, int lp, int t, int b,
                             const float* __restrict__ tab, const double* __restrict__ tab64) {
    const TileView& V = X.V;
    const int L = X.L, slot = tslot(X, lp), pair = tpair(lp), lane = threadIdx.x & 31;
    float* tb = V.tile + (size_t)b * T_NF * L * TW;
    const int s = TW * t + lane, c2 = s / NGPT, g = s % NGPT;
    const int ib = cT.ngb[g], igb = cT.gib[g];
    const int pcol = pair_col(P, pair, c2, X.nmapped);
    const bool act = V.ctl[TC_ACT0 + 2 * slot + c2] != 0;
    const Coef<float> C{V.coef + c2 * NFR * L, V.pk + c2 * L, L, V.ctl[TC_LT0 + c2]};
    const float zinc = V.sub[slot * 3 * COLS_PER_CTA * NGPT + s];
    const float mu = V.mu[c2];
    const float* aer = (const float*)(tblk(X, pair) + X.B.aer) + c2 * 3 * NBND * L;
    const float* cld = X.cstage ? V.cld + c2 * 4 * L : nullptr;
    while (true) {
        int r = 0;
        if (lane == 0) r = atomicAdd(&V.ctl[TC_ROW0 + b], 1);
        r = __shfl_sync(0xffffffffu, r, 0);
        if (r >= L) break;
        const int lay = r + 1;
        float f[T_NF] = {0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f};
        if (act) {
            float taug, taur, fs;
            int js;
            taumol_generic(ib, igb, lay, C, tab, V.tm, taug, taur, js, fs);
            CellIn<float> ci;
            ci.taug = taug;
            ci.taur = taur;
            if (P.iaer != 0) {
                ci.rta = aer[(0 * NBND + ib) * L + r];
                ci.rcoa = aer[(1 * NBND + ib) * L + r];
                ci.roa = 1.0f - ci.rcoa;
                ci.rga = aer[(2 * NBND + ib) * L + r];
            } else {
                ci.rta = 0.0f; ci.roa = 1.0f; ci.rga = 0.0f; ci.rcoa = 0.0f;
            }
            bool cloudy = false;
            if (X.fused) cloudy = (V.mask[s * 2 + (r >> 5)] >> (r & 31)) & 1u;
            cloud_in<float>(P, pcol, g, lay, ib, X.fused, cloudy, cld, ci, tab);
            const float hrs = zinc * V.hrf[c2 * L + r];
            const CellOpt<float> co = cell_optics<float>(ci, 1, mu, tab, tab64, hrs, zinc);
            f[TF_REFC] = co.rc.ref; f[TF_REFDC] = co.rc.refd; f[TF_ADIRC] = co.rc.adir; f[TF_ADIFC] = co.rc.adif;
            f[TF_DBTC] = co.zdbtc;
            f[TF_REF] = co.rt.ref; f[TF_REFD] = co.rt.refd; f[TF_ADIR] = co.rt.adir; f[TF_ADIF] = co.rt.adif;
            f[TF_DBT] = co.zdbt;
            if (co.risky) {
                // an FP32 choice too close to call: the FP64 warp redoes the
                // cell, and the subcolumn is swept apart from its tile
                const int q = atomicAdd(&V.ctl[TC_QN0 + slot], 1);
                if (q < X.qcap) V.queue[slot * T_QCAP + q] = (s << 12) | (lay << 1) | (ci.cloudy ? 1 : 0);
                atomicOr(&V.risky[slot * TILES + t], 1u << lane);
            }
        }
        tquad(tb, L, 0, r)[lane] = make_float4(f[TF_REFC], f[TF_REFDC], f[TF_ADIRC], f[TF_ADIFC]);
        tdbt(tb, L, 0, r)[lane] = f[TF_DBTC];
        tquad(tb, L, 1, r)[lane] = make_float4(f[TF_REF], f[TF_REFD], f[TF_ADIR], f[TF_ADIF]);
        tdbt(tb, L, 1, r)[lane] = f[TF_DBT];
    }
}

// Record slots of tile t's set-aside subcolumns start after those of the
// pair's earlier tiles (their risky masks are final once tile t is).
__device__ inline int tiled_rec_base(const TileView& V, int slot, int t) {
    int base = 0;
    for (int tt = 0; tt < t; ++tt) base += __popc(V.risky[slot * TILES + tt]);
    return base;
}

// ---- optics warps, after tile t's cells (buffer b) are all written: the
// subcolumns with FP64 cells are copied aside (global, per CTA) for the FP64
// warp's second sweep -- header (subcolumn, column, zinc, albedos) and all
// ten fields of every layer, spread over the optics warps' threads
__device__ void tiled_set_aside(const TCtx& X, int lp, int t, int b) {
    const TileView& V = X.V;
    const int L = X.L, slot = tslot(X, lp);
    const uint32_t rm = V.risky[slot * TILES + t];
    if (!rm) return;
    const int base = tiled_rec_base(V, slot, t), nr = __popc(rm);
    const float* tb = V.tile + (size_t)b * T_NF * L * TW;
    const float* sub = V.sub + slot * 3 * COLS_PER_CTA * NGPT;
    const int per = T_NF * L;
    for (int it = threadIdx.x; it < nr * (per + 1); it += T_OPT * 32) {
        const int j = it / (per + 1), rem = it % (per + 1);
        const int idx = base + j;
        if (idx >= T_RCAP) continue;  // the pair overflows; the FP64 warp hands it back
        uint32_t m = rm;  // its j-th set bit
        for (int k = 0; k < j; ++k) m &= m - 1u;
        const int lane = __ffs(m) - 1;
        float* rp = trec(X, slot, idx);
        if (rem < per) {
            rp[8 + rem] = tfield((float*)tb, L, rem / L, rem % L, lane);  // record order: field, layer
        } else {
            const int s = TW * t + lane;
            rp[0] = (float)s;
            rp[1] = (float)(s / NGPT);
            rp[2] = sub[s];
            rp[3] = sub[COLS_PER_CTA * NGPT + s];
            rp[4] = sub[2 * COLS_PER_CTA * NGPT + s];
            V.recof[slot * COLS_PER_CTA * NGPT + s] = (short)idx;
        }
    }
}

// ---- FP64 warp: the pair's queued cells, 32 at a time
__device__ void tiled_redo(const SolveParams& P, const TCtx& X, int lp, const double* __restrict__ tab64) {
    const TileView& V = X.V;
    const int L = X.L, slot = tslot(X, lp), pair = tpair(lp), lane = threadIdx.x & 31;
    unsigned char* pb = tpar(X, slot);
    float* corr = (float*)(pb + X.G.corr);
    const int* misc = (const int*)(tblk(X, pair) + X.B.misc);
    const int qn = min(V.ctl[TC_QN0 + slot], X.qcap);
    (void)L;
    for (int k = lane; k < qn; k += 32) {
        const int e = V.queue[slot * T_QCAP + k];
        const int s = e >> 12, lay = (e >> 1) & 127, c2 = s / NGPT, g = s % NGPT;
        const int pcol = pair_col(P, pair, c2, X.nmapped);
        Coef64At b;
        const Coef<double> C64 = coef64_at(P, pcol, lay, misc[TP_LT0 + c2], tab64, b);
        double cz = P.coszen[pcol];
        if (cz < 1.e-10) cz = 1.e-10;
        const CellOpt<float> co =
            cell_optics_fp64(P, C64, pcol, g, lay, cT.ngb[g], cT.gib[g], X.fused, (e & 1) != 0, cz, tab64, 1);
        float* o = corr + k * T_NF;
        o[TF_REFC] = co.rc.ref; o[TF_REFDC] = co.rc.refd; o[TF_ADIRC] = co.rc.adir; o[TF_ADIFC] = co.rc.adif;
        o[TF_DBTC] = co.zdbtc;
        o[TF_REF] = co.rt.ref; o[TF_REFD] = co.rt.refd; o[TF_ADIR] = co.rt.adir; o[TF_ADIF] = co.rt.adif;
        o[TF_DBT] = co.zdbt;
    }
}

// Where a tile keeps the weighted fluxes of a level after the sweeps: level
// v >= 1 in each sky's float4 of layer v-1 that the sweeps have read (up,
// down, direct, absorption of the layer above), the surface level in scr as
// float4 [sky][lane].  Order of the 8 sums: fu, fd, cu, cd, direct total,
// direct clear, absorption total, absorption clear.
__device__ __forceinline__ void q_order(const float4& c, const float4& t, float* x) {
    x[0] = t.x; x[1] = t.y; x[2] = c.x; x[3] = c.y; x[4] = t.z; x[5] = c.z; x[6] = t.w; x[7] = c.w;
}

// ---- adding warps: the vertical sweeps of tile t (buffer b) of pair lp,
// sky SKY (0 clear, 1 total); then the g-point sums of half the levels
template <int SKY, int NQ>
__device__ void tiled_sweep(const SolveParams& P, const TCtx& X, int lp, int t, int b) {
    const TileView& V = X.V;
    const int L = X.L, ps = tslot(X, lp), pair = tpair(lp), lane = threadIdx.x & 31;
    const size_t n = (size_t)P.ncol, L1 = (size_t)L + 1;
    float* tb = V.tile + (size_t)b * T_NF * L * TW;
    const int s = TW * t + lane, c2 = s / NGPT, g = s % NGPT;
    const int ib = cT.ngb[g];
    const float* sub = V.sub + ps * 3 * COLS_PER_CTA * NGPT;
    const float zinc = sub[s], albp = sub[COLS_PER_CTA * NGPT + s], albd = sub[2 * COLS_PER_CTA * NGPT + s];
    const bool act = V.ctl[TC_ACT0 + 2 * ps + c2] != 0;
    const bool risky = (V.risky[ps * TILES + t] >> lane) & 1u;
    const bool use = act && !risky;
    const float zinc_use = use ? zinc : 0.0f;  // the lanes left out of the sums get zero level fluxes
    // subcolumns with FP64 cells were copied aside by the optics warps
    // (tiled_set_aside); they stay out of this tile's sums
    float* R = V.rup + (size_t)2 * SKY * L * TW;  // [2][L][TW]: rup, rupd of this sky
    // up-sweep from the surface (vrtqdr:122-140), the next layer's fields
    // loaded while this one is swept
    float ru = albp, rud = albd;
    float f[5], fn[5];
    auto load5 = [&](int i, float* g5) {
        const float4 a = tquad(tb, L, SKY, i)[lane];
        g5[0] = a.x; g5[1] = a.y; g5[2] = a.z; g5[3] = a.w;
        g5[4] = tdbt(tb, L, SKY, i)[lane];
    };
    load5(0, f);
#pragma unroll 2  // (by 4 the code outgrows the instruction cache)
    for (int i = 0; i < L; ++i) {
        const int in = i + 1 < L ? i + 1 : i;
        load5(in, fn);
        up1(f, ru, rud);
        R[i * TW + lane] = ru;
        R[(L + i) * TW + lane] = rud;
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] = fn[k];
    }
    // down-sweep: this sky's 4 weighted fluxes of level i+1 replace its
    // first 4 fields of layer i, read just before
    Down1 st;
    down1_init(st);
    float q[4], rr[2], rn[2], dif;
    load5(L - 1, f);
    rr[0] = R[(L - 1) * TW + lane];
    rr[1] = R[(2 * L - 1) * TW + lane];
#pragma unroll 2
    for (int i = L - 1; i >= 0; --i) {
        const int in = i > 0 ? i - 1 : 0;
        load5(in, fn);
        rn[0] = R[in * TW + lane];
        rn[1] = R[(L + in) * TW + lane];
        level1(st, rr[0], rr[1], zinc_use, q, dif);
        down1(st, f, dif);
        tquad(tb, L, SKY, i)[lane] = make_float4(q[0], q[1], q[2], q[3]);
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] = fn[k];
        rr[0] = rn[0];
        rr[1] = rn[1];
    }
    level1(st, albp, albd, zinc_use, q, dif);  // surface
    ((float4*)V.scr)[SKY * TW + lane] = make_float4(q[0], q[1], q[2], q[3]);
    int* key = (int*)(V.scr + 8 * TW);
    if (SKY == 1) key[lane] = c2 * 16 + ib;
    const bool uv = ib >= 9 && ib <= 12;  // bands 25-28 (spcvmc:629)
    const unsigned uvm = __ballot_sync(0xffffffffu, uv);
    add_sync();  // both skies' fluxes of every level are in place
    // g-point sums, one lane per level, levels split between the two warps;
    // lanes of the tile's two columns (tile 3 holds the end of column 0 and
    // the start of column 1) summed apart
    const int c0 = (TW * t) / NGPT;
    const int cb = ((TW * t + TW - 1) / NGPT == c0) ? TW : NGPT * (c0 + 1) - TW * t;  // first lane of column 1
    for (int v = lane + 32 * SKY; v <= L; v += 64) {
        const float4* sc = v ? tquad(tb, L, 0, v - 1) : (const float4*)V.scr;      // clear sky
        const float4* stt = v ? tquad(tb, L, 1, v - 1) : (const float4*)V.scr + TW;  // total sky
        float a0[8], a1[8], e0[8], e1[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a0[k] = a1[k] = e0[k] = e1[k] = 0.0f;
        // (not unrolled: the kernel's largest stall is instruction fetch)
#pragma unroll 1
        for (int m = 0; m < TW; ++m) {
            const int j = (m + lane) & 31;  // rotated: a quarter warp's lanes read 8 different 16-byte groups
            const bool lo = j < cb;
            float x[8];
            q_order(sc[j], stt[j], x);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (lo) a0[k] += x[k];
                else a1[k] += x[k];
            }
            if constexpr (NQ > 8) {
                // UV (bands 25-28) / near-IR split of fd, cd and the direct fluxes
                const int o = ((uvm >> j) & 1u) ? 0 : 4;
                float* e = lo ? e0 : e1;
                e[o] += x[1]; e[o + 1] += x[3]; e[o + 2] += x[4]; e[o + 3] += x[5];
            }
        }
        float* Fl0 = V.flux + ((size_t)(ps * COLS_PER_CTA + c0) * NQ) * L1;
#pragma unroll
        for (int k = 0; k < 8; ++k) Fl0[k * L1 + v] += a0[k];
        if constexpr (NQ > 8) {
#pragma unroll
            for (int k = 0; k < 8; ++k) Fl0[(8 + k) * L1 + v] += e0[k];
        }
        if (cb < TW) {
            float* Fl1 = Fl0 + (size_t)NQ * L1;
#pragma unroll
            for (int k = 0; k < 8; ++k) Fl1[k * L1 + v] += a1[k];
            if constexpr (NQ > 8) {
#pragma unroll
                for (int k = 0; k < 8; ++k) Fl1[(8 + k) * L1 + v] += e1[k];
            }
        }
        if (P.bands) {
            // per-band fluxes (the band loop of spcvmc:619-630): lanes of one
            // (column, band) in order, added to the FP64 outputs (zeroed at
            // the pair's first tile)
            int j = 0;
            while (j < TW) {
                const int kj = key[j];
                float a[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
                int e = j;
                for (; e < TW && key[e] == kj; ++e) {
                    float x[8];
                    q_order(sc[e], stt[e], x);
                    a[0] += x[0]; a[1] += x[1]; a[2] += x[4]; a[3] += x[2]; a[4] += x[3];  // fu, fd, fddir, cu, cd
                }
                const int pc = pair_col(P, pair, kj >> 4, X.nmapped);
                if (pc < P.ncol) {
                    const size_t idx = (size_t)pc + n * ((size_t)v + L1 * (size_t)(kj & 15));
#pragma unroll
                    for (int k = 0; k < 5; ++k)
                        if (P.bout[k]) P.bout[k][idx] += (double)a[k];
                }
                j = e;
            }
        }
    }
    // both warps are done reading this tile's surface rows and keys (scr),
    // which the next tile's sweeps overwrite
    add_sync();
}

// ---- FP64 warp: sweeps of the set-aside subcolumns r0 .. r0+31 of pair lp
// (their FP64 cells already patched in), added to the pair's level sums;
// R: 4 x L x TW albedo scratch, scr: 16 x TW reduction scratch
template <int NQ>
__device__ void tiled_records(const SolveParams& P, const TCtx& X, int lp, int r0, int rn, float* R, float* scr) {
    const TileView& V = X.V;
    const int L = X.L, slot = tslot(X, lp), pair = tpair(lp), lane = threadIdx.x & 31;
    const size_t n = (size_t)P.ncol, L1 = (size_t)L + 1;
    const int r = r0 + lane;
    const bool on = r < rn;
    const float* rp = trec(X, slot, on ? r : r0);
    const int s = (int)rp[0], c2 = (int)rp[1], g = s % NGPT, ib = cT.ngb[g];
    const bool uv = ib >= 9 && ib <= 12;
    const float zinc = on ? rp[2] : 0.0f, albp = rp[3], albd = rp[4];
    const int pcol = pair_col(P, pair, c2, X.nmapped);
    const float* fl = rp + 8;
    float rupc = albp, rupdc = albd, rup = albp, rupd = albd;
    // the records sit in global memory, one per lane: each layer's ten
    // fields are loaded while the previous layer is swept
    float fc[5], ft[5], nc[5], nt[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        fc[k] = fl[(TF_REFC + k) * L];
        ft[k] = fl[(TF_REF + k) * L];
    }
#pragma unroll 1  // (FP64 warps' loops kept small: they share instruction caches with optics warps)
    for (int i = 0; i < L; ++i) {
        const int in = i + 1 < L ? i + 1 : i;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            nc[k] = fl[(TF_REFC + k) * L + in];
            nt[k] = fl[(TF_REF + k) * L + in];
        }
        up1(fc, rupc, rupdc);
        up1(ft, rup, rupd);
        R[(0 * L + i) * TW + lane] = rupc;
        R[(1 * L + i) * TW + lane] = rupdc;
        R[(2 * L + i) * TW + lane] = rup;
        R[(3 * L + i) * TW + lane] = rupd;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            fc[k] = nc[k];
            ft[k] = nt[k];
        }
    }
    const unsigned m0 = __ballot_sync(0xffffffffu, on && c2 == 0);
    const unsigned m1 = __ballot_sync(0xffffffffu, on && c2 == 1);
    Down1 sc, stt;
    down1_init(sc);
    down1_init(stt);
    float q[16];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        fc[k] = fl[(TF_REFC + k) * L + L - 1];
        ft[k] = fl[(TF_REF + k) * L + L - 1];
    }
    float ra[4], rb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ra[k] = R[(k * L + L - 1) * TW + lane];
#pragma unroll 1
    for (int i = L - 1; i >= -1; --i) {
        float qc[4], qt[4], difc, dift;
        if (i >= 0) {
            const int in = i > 0 ? i - 1 : 0;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                nc[k] = fl[(TF_REFC + k) * L + in];
                nt[k] = fl[(TF_REF + k) * L + in];
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) rb[k] = R[(k * L + in) * TW + lane];
            level1(sc, ra[0], ra[1], zinc, qc, difc);
            level1(stt, ra[2], ra[3], zinc, qt, dift);
            down1(sc, fc, difc);
            down1(stt, ft, dift);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                fc[k] = nc[k];
                ft[k] = nt[k];
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) ra[k] = rb[k];
        } else {
            level1(sc, albp, albd, zinc, qc, difc);
            level1(stt, albp, albd, zinc, qt, dift);
        }
        q[0] = qt[0]; q[1] = qt[1]; q[2] = qc[0]; q[3] = qc[1];
        q[4] = qt[2]; q[5] = qc[2]; q[6] = qt[3]; q[7] = qc[3];
        if constexpr (NQ > 8) {
            const int o = uv ? 8 : 12, z = uv ? 12 : 8;
            q[o] = q[1]; q[o + 1] = q[3]; q[o + 2] = q[4]; q[o + 3] = q[5];
            q[z] = q[z + 1] = q[z + 2] = q[z + 3] = 0.0f;
        }
        const int l = i + 1;
#pragma unroll
        for (int k = 0; k < NQ; ++k) scr[k * TW + lane] = on ? q[k] : 0.0f;
        __syncwarp();
        if (lane < 2 * NQ) {
            // one lane per (column, quantity), subcolumns in record order
            const int c = lane / NQ, k = lane % NQ;
            unsigned m = c ? m1 : m0;
            if (m) {
                float v = 0.0f;
                while (m) {
                    const int j = __ffs(m) - 1;
                    m &= m - 1;
                    v += scr[k * TW + j];
                }
                V.flux[((size_t)(slot * COLS_PER_CTA + c) * NQ + k) * L1 + l] += v;
            }
        }
        __syncwarp();
        if (P.bands) {
            const float bv[5] = {q[0], q[1], q[4], q[2], q[3]};
#pragma unroll
            for (int k = 0; k < 5; ++k) scr[k * TW + lane] = on ? bv[k] : 0.0f;
            long long* key = (long long*)(scr + 6 * TW);
            key[lane] = on && pcol < P.ncol ? (long long)((size_t)pcol + n * ((size_t)l + L1 * (size_t)ib)) : -1ll;
            __syncwarp();
            if (lane < 5 && P.bout[lane]) {
                // records in order, one lane per output array
                for (int j = 0; j < TW; ++j)
                    if (key[j] >= 0) P.bout[lane][key[j]] += (double)scr[lane * TW + j];
            }
            __syncwarp();
        }
    }
}

// ---- FP64 warp: pair lp's set-aside subcolumns, outputs, reset (after both
// adding warps have summed the pair's last tile)
template <int NQ>
__device__ void tiled_finish(const SolveParams& P, const TCtx& X, int lp) {
    const TileView& V = X.V;
    const int L = X.L, slot = tslot(X, lp), pair = tpair(lp), lane = threadIdx.x & 31;
    const size_t n = (size_t)P.ncol;
    const int qn = V.ctl[TC_QN0 + slot], rn = tiled_rec_base(V, slot, TILES);
    const bool ovf = qn > X.qcap || rn > T_RCAP;
    if (!ovf && rn > 0) {
        const float* corr = (const float*)(tpar(X, slot) + X.G.corr);
        for (int k = lane; k < qn; k += 32) {
            const int e = V.queue[slot * T_QCAP + k];
            const int s = e >> 12, lay = (e >> 1) & 127;
            const int r = V.recof[slot * COLS_PER_CTA * NGPT + s];
            if (r >= 0 && r < T_RCAP) {
                float* rp = trec(X, slot, r) + 8;
#pragma unroll
                for (int f = 0; f < T_NF; ++f) rp[f * L + lay - 1] = corr[k * T_NF + f];
            }
        }
        __syncwarp();
        const int w = (threadIdx.x >> 5) - T_REDO;  // this FP64 warp
        float* R = (float*)(X.glob + X.G.rrup) + (size_t)w * 4 * L * TW;
        for (int r0 = 0; r0 < rn; r0 += TW) tiled_records<NQ>(P, X, lp, r0, rn, R, V.scr2 + w * 16 * TW);
    }
    if (lane == 0 && P.stats) {
        if (ovf) atomicAdd(P.stats + 2, 1ull);
        else {
            atomicAdd(P.stats, (unsigned long long)qn);
            atomicAdd(P.stats + 3, (unsigned long long)rn);
        }
    }
    if (ovf && lane == 0 && P.tovfcount) {
        // too many FP64 cells for the capacities: the caller solves the pair again
        const int k = atomicAdd(P.tovfcount, 1);
        if (k < P.tovfcap) P.tovf[k] = pair;
    }
    // outputs (level 0 = surface)
    const double* pdpg = (const double*)(tblk(X, pair) + X.B.pdp);
    constexpr int QX = 8;
#pragma unroll 1
    for (int it = lane; it < COLS_PER_CTA * (L + 1); it += 32) {
        const int c2 = it / (L + 1), l = it % (L + 1);
        const int ocol = pair_col(P, pair, c2, X.nmapped);
        if (ocol >= P.ncol) continue;
        const float* F = V.flux + (size_t)(slot * COLS_PER_CTA + c2) * NQ * (L + 1);
        const size_t o = (size_t)ocol + n * (size_t)l;
        const double fu = (double)F[0 * (L + 1) + l], fd = (double)F[1 * (L + 1) + l];
        P.swuflx[o] = fu;
        P.swdflx[o] = fd;
        P.swuflxc[o] = (double)F[2 * (L + 1) + l];
        P.swdflxc[o] = (double)F[3 * (L + 1) + l];
        if (l < L) {
            double hr = 0.0, hrc = 0.0;
            if (l < L - 1) {
                // summed layer absorption (= net-flux divergence) (rrtmg_sw_rad.f90:829-836)
                const double zdpgcp = cT.heatfac / pdpg[c2 * L + l];
                hr = (double)F[6 * (L + 1) + l] * zdpgcp;
                hrc = (double)F[7 * (L + 1) + l] * zdpgcp;
            }
            P.swhr[o] = hr;
            P.swhrc[o] = hrc;
        }
        if constexpr (NQ > 8) {
            const double fddir = (double)F[4 * (L + 1) + l];
            const double uvfd = (double)F[(QX + 0) * (L + 1) + l], uvfddir = (double)F[(QX + 2) * (L + 1) + l];
            const double nifd = (double)F[(QX + 4) * (L + 1) + l], nifddir = (double)F[(QX + 6) * (L + 1) + l];
            const double vals[8] = {fddir, DS(fd, fddir), uvfd, nifd, uvfddir, DS(uvfd, uvfddir), nifddir,
                                    DS(nifd, nifddir)};
            for (int x = 0; x < 8; ++x)
                if (P.xout[x]) P.xout[x][o] = vals[x];
        }
    }
    __syncwarp();
    // this slot's per-pair state, ready for pair lp + nslot
    float* F = V.flux + (size_t)slot * COLS_PER_CTA * NQ * (L + 1);
    for (int k = lane; k < COLS_PER_CTA * NQ * (L + 1); k += 32) F[k] = 0.0f;
    for (int k = lane; k < COLS_PER_CTA * NGPT; k += 32) V.recof[slot * COLS_PER_CTA * NGPT + k] = -1;
    if (lane < TILES) V.risky[slot * TILES + lane] = 0u;
    if (lane == 0) {
        V.ctl[TC_QN0 + slot] = 0;
    }
    __syncwarp();
}

// ---- adding warp: the pair's per-band outputs start at zero
__device__ void tiled_zero_bands(const SolveParams& P, const TCtx& X, int lp) {
    const int L = X.L, pair = tpair(lp), lane = threadIdx.x & 31;
    const size_t n = (size_t)P.ncol, L1 = (size_t)L + 1;
    for (int it = lane; it < COLS_PER_CTA * (L + 1) * NBND; it += 32) {
        const int c2 = it / ((L + 1) * NBND), rem = it % ((L + 1) * NBND), l = rem % (L + 1), b = rem / (L + 1);
        const int pcol = pair_col(P, pair, c2, X.nmapped);
        if (pcol >= P.ncol) continue;
        const size_t o = (size_t)pcol + n * ((size_t)l + L1 * (size_t)b);
        for (int k = 0; k < 5; ++k)
            if (P.bout[k]) P.bout[k][o] = 0.0;
    }
    __syncwarp();
}

__global__ void __launch_bounds__(T_THREADS, 1)
k_solve_tiled(const SolveParams P, const float* __restrict__ tab, const double* __restrict__ tab64) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = P.nlay;
    const int NQ = P.extra ? 16 : 8;
    TCtx X;
    X.fused = P.fused && P.icld >= 1;
    X.nomc = P.nomcica && P.icld >= 1;
    X.cstage = X.fused || X.nomc;
    X.nslot = P.tile_slots == T_SLOTS ? T_SLOTS : 2;
    const TSmem M = tiled_smem(L, NQ, X.fused, X.cstage, X.nslot);
    X.V = tile_view(smem_raw, M);
    X.G = tiled_glob(L);
    X.B = tiled_prep_layout(L, X.fused, X.cstage, P.iaer != 0);
    X.glob = (unsigned char*)P.scratch + (size_t)blockIdx.x * P.slot_elems * sizeof(float);
    X.prep = (const unsigned char*)P.tprep;
    X.L = L;
    X.nmapped = P.colmap ? *P.mapcount : 0;
    X.qcap = (P.tile_qcap > 0 && P.tile_qcap < T_QCAP) ? P.tile_qcap : T_QCAP;
    X.nlocal = (int)blockIdx.x < P.npairs ? (P.npairs - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    X.abort = (volatile int*)&X.V.ctl[TC_ABORT];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    TmSmem* tm = (TmSmem*)X.V.tm;
    for (int i = tid; i < NBND * 2; i += T_THREADS) {
        TmSmem d;
        d.r = cT.tm[i / 2][i % 2];
        d.selfref = cT.b[i / 2].selfref;
        d.forref = cT.b[i / 2].forref;
        d.ng = cT.b[i / 2].ng;
        d.pad = 0;
        tm[i] = d;
    }
    for (int i = tid; i < TC_N; i += T_THREADS) X.V.ctl[i] = 0;
    for (int i = tid; i < X.nslot * TILES; i += T_THREADS) X.V.risky[i] = 0u;
    for (int i = tid; i < X.nslot * COLS_PER_CTA * NGPT; i += T_THREADS) X.V.recof[i] = -1;
    for (int i = tid; i < X.nslot * COLS_PER_CTA * NQ * (L + 1); i += T_THREADS) X.V.flux[i] = 0.0f;
    if (tid == 0) {
        mbar_init(&X.V.bar[TB_FULL0], T_OPT);
        mbar_init(&X.V.bar[TB_FULL1], T_OPT);
        mbar_init(&X.V.bar[TB_EMPTY0], 2);
        mbar_init(&X.V.bar[TB_EMPTY1], 2);
        for (int k = 0; k < T_SLOTS; ++k) {
            mbar_init(&X.V.bar[TB_PAIR0 + k], T_OPT);
            mbar_init(&X.V.bar[TB_SWEPT0 + k], 2);
            mbar_init(&X.V.bar[TB_FIN0 + k], 1);
        }
    }
    __syncthreads();
    // Handoffs per pair lp (slot lp % nslot; a slot's barriers complete one
    // phase per pair, so the parity of pair lp's phase is (lp / nslot) & 1):
    // the optics warps arrive PAIR when its cells are all made, the adding
    // warps SWEPT when its tiles are all swept, the FP64 warp FIN when its
    // outputs are written.  No barrier can run two phases ahead of a waiter:
    // the optics and adding warps start pair lp + nslot only after FIN of
    // pair lp.
    if (warp < T_OPT) {
        for (int lp = 0; lp < X.nlocal; ++lp) {
            // pair lp - nslot is finished: the slot's per-pair state is free
            if (lp >= X.nslot) {
                const int q = lp - X.nslot;
                mbar_wait(&X.V.bar[TB_FIN0 + tslot(X, q)], tphase(X, q), X.abort, P.err);
            }
            opt_sync();  // the previous pair's cells are all written
            tiled_load(P, X, lp);
            for (int t = 0; t < TILES; ++t) {
                const int T = TILES * lp + t, b = T & 1;
                if (T >= 2) mbar_wait(&X.V.bar[TB_EMPTY0 + b], ((T - 2) >> 1) & 1, X.abort, P.err);
                tiled_optics(P, X, lp, t, b, tab, tab64);
                opt_sync();  // the tile's cells and risky bits are all written
                tiled_set_aside(X, lp, t, b);
                __syncwarp();
                __threadfence_block();
                if (lane == 0) {
                    mbar_arrive(&X.V.bar[TB_FULL0 + b]);
                    if (t == TILES - 1) mbar_arrive(&X.V.bar[TB_PAIR0 + tslot(X, lp)]);
                }
            }
        }
    } else if (warp < T_REDO + T_F64) {
        for (int lp = warp - T_REDO; lp < X.nlocal; lp += T_F64) {
            const int slot = tslot(X, lp);
            const unsigned ph = tphase(X, lp);
            mbar_wait(&X.V.bar[TB_PAIR0 + slot], ph, X.abort, P.err);
            tiled_redo(P, X, lp, tab64);
            __syncwarp();
            mbar_wait(&X.V.bar[TB_SWEPT0 + slot], ph, X.abort, P.err);
            if (NQ > 8) tiled_finish<16>(P, X, lp);
            else tiled_finish<8>(P, X, lp);
            __threadfence_block();
            if (lane == 0) mbar_arrive(&X.V.bar[TB_FIN0 + slot]);
        }
    } else {
        const int sky = warp == T_ADDT ? 1 : 0;
        for (int lp = 0; lp < X.nlocal; ++lp) {
            const int slot = tslot(X, lp);
            // pair lp - nslot is finished: the slot's level sums are free
            if (lp >= X.nslot) {
                const int q = lp - X.nslot;
                mbar_wait(&X.V.bar[TB_FIN0 + tslot(X, q)], tphase(X, q), X.abort, P.err);
            }
            if (P.bands && sky == 1) tiled_zero_bands(P, X, lp);
            for (int t = 0; t < TILES; ++t) {
                const int T = TILES * lp + t, b = T & 1;
                mbar_wait(&X.V.bar[TB_FULL0 + b], (T >> 1) & 1, X.abort, P.err);
                if (sky) {
                    if (NQ > 8) tiled_sweep<1, 16>(P, X, lp, t, b);
                    else tiled_sweep<1, 8>(P, X, lp, t, b);
                } else {
                    if (NQ > 8) tiled_sweep<0, 16>(P, X, lp, t, b);
                    else tiled_sweep<0, 8>(P, X, lp, t, b);
                }
                __syncwarp();
                if (lane == 0) {
                    if (sky == 1) X.V.ctl[TC_ROW0 + b] = 0;
                    __threadfence_block();
                    mbar_arrive(&X.V.bar[TB_EMPTY0 + b]);
                    if (t == TILES - 1) mbar_arrive(&X.V.bar[TB_SWEPT0 + slot]);
                }
                __syncwarp();
            }
        }
    }
}

// Whether the tiled kernel takes a call: FP32 form, delta-scaled direct
// fluxes (idelm = 1), at most T_MAXL layers whose tiles fit in shared
// memory, no batch column map.
__host__ inline bool tiled_supports(const SolveParams& P, size_t smem_max) {
    if (P.idelm != 1 || P.nlay > T_MAXL || P.colmap) return false;
    const bool fused = P.fused && P.icld >= 1, nomc = P.nomcica && P.icld >= 1;
    return tiled_smem(P.nlay, P.extra ? 16 : 8, fused, fused || nomc, 2).total <= smem_max;
}

// Pair slots of a call the tiled kernel takes: 3 when their shared memory
// fits, else 2.
__host__ inline int tiled_slots(const SolveParams& P, size_t smem_max) {
    const bool fused = P.fused && P.icld >= 1, nomc = P.nomcica && P.icld >= 1;
    return tiled_smem(P.nlay, P.extra ? 16 : 8, fused, fused || nomc, T_SLOTS).total <= smem_max ? T_SLOTS : 2;
}

}  // namespace rrsw
