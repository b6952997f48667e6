/*
 * rrtmg_sw_gb300.h -- C ABI of the GB300 (sm_103a) RRTMG_SW shortwave solver.
 *
 * Drop-in boundary for the GCM interface of RRTMG_SW.  Every entry point
 * names the reference routine it replaces (paths relative to the RRTMG_SW
 * source tree).  Arrays use the reference's Fortran (column-major) layout,
 * so a Fortran caller passes c_loc(x(1,1)) of its contiguous arrays
 * unchanged:
 *   (ncol,nlay)        element (i,l)   at [i + ncol*l]
 *   (ngpt,ncol,nlay)   element (g,i,l) at [g + 112*(i + ncol*l)]
 *   (ncol,nlay,nbnd)   element (i,l,b) at [i + ncol*(l + nlay*b)]
 *   (nbnd,ncol,nlay)   element (b,i,l) at [b + 14*(i + ncol*l)]
 * Layer 1 is the surface layer (rrtmg_sw_rad.f90:1527-1529).  Units as in
 * the reference: hPa, K, volume mixing ratio, g m-2, microns; outputs W m-2
 * and K d-1.
 *
 * All entry points return 0 on success or one of the RRTMG_SW_E* codes
 * below; rrtmg_sw_errstr_c gives the message the reference would `stop`
 * with.  A call with ncol = 0 does nothing and returns 0, as the
 * reference's column loop does (a batch instance must have columns).
 * Outputs are fully overwritten.  The caller owns every array.  The
 * library owns its device tables (rrtmg_sw_ini_c) and a reusable device
 * workspace, released by rrtmg_sw_finalize_c.  Calls are serialised
 * internally; one process drives one GPU: every entry point that uses the
 * device returns RRTMG_SW_ENOTINIT when the current device is not the one
 * rrtmg_sw_ini_c loaded the tables on.  Host-array entry points run on a
 * non-blocking stream of the library's own and return when their outputs
 * are back in host memory.
 */
#ifndef RRTMG_SW_GB300_H
#define RRTMG_SW_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Arguments of rrtmg_sw, in the order of rrtmg_sw_rad.f90:99-111
 * (declarations :220-388).  Optional Fortran arguments (bndsolvar,
 * indsolvar, solcycfrac) are nullable.  The eight extra output pointers are
 * the direct/diffuse and UV/near-IR fluxes that spcvmc_sw computes but the
 * reference driver keeps local (rrtmg_sw_rad.f90:810-820); each is
 * (ncol,nlay+1) or NULL.  idelm selects delta-scaled (1, the reference's
 * hard-coded value, rrtmg_sw_rad.f90:605) or unscaled (0) direct fluxes. */
typedef struct rrtmg_sw_args {
    int32_t ncol, nlay, icld, iaer;
    const double *play, *plev, *tlay, *tlev, *tsfc;
    const double *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr, *o2vmr;
    const double *asdir, *asdif, *aldir, *aldif;
    const double *coszen;
    double adjes;
    int32_t dyofyr;
    double scon;
    int32_t isolvar;
    int32_t inflgsw, iceflgsw, liqflgsw;
    const double *cldfmcl, *taucmcl, *ssacmcl, *asmcmcl, *fsfcmcl;   /* (ngpt,ncol,nlay) */
    const double *ciwpmcl, *clwpmcl;                                  /* (ngpt,ncol,nlay) */
    const double *reicmcl, *relqmcl;                                  /* (ncol,nlay) */
    const double *tauaer, *ssaaer, *asmaer;                           /* (ncol,nlay,nbnd) */
    const double *ecaer;                                              /* (ncol,nlay,6) */
    double *swuflx, *swdflx, *swhr, *swuflxc, *swdflxc, *swhrc;
    const double *bndsolvar;   /* (14) or NULL */
    const double *indsolvar;   /* (2)  or NULL */
    const double *solcycfrac;  /* scalar or NULL */
    double *dirdflux, *difdflux, *uvdflx, *nidflx, *dirdnuv, *difdnuv, *dirdnir, *difdnir;
    int32_t idelm;
    int32_t nthreads;          /* unused by the GPU library (kept for layout) */
    /* Per-band fluxes (ncol,nlay+1,nbnd) or NULL: total-sky up, down and
     * direct down, clear-sky up and down, summed over each band's g-points
     * (the band loop of rrtmg_sw_spcvmc.f90:619-630 that the column driver
     * prints with iout = 98, rrtmg_sw.1col.f90:573-578). */
    double *bndfu, *bndfd, *bndfddir, *bndcu, *bndcd;
} rrtmg_sw_args;

/* Physical cloud inputs for the fused path: the arguments of
 * mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-185) that rrtmg_sw_mcica_c
 * consumes on the device instead of the seven (ngpt,ncol,nlay) subcolumn
 * arrays.  irng = 0: KISS, per-column streams; irng = 1: MT19937, one
 * stream for the call in (subcolumn, column, layer) order seeded with
 * permuteseed, generated on the device before the solve (rrtmg_sw_mcica_c /
 * _dev_c only; the static, batch and TL/AD entry points return
 * RRTMG_SW_EIRNG). */
typedef struct rrtmg_sw_clouds {
    int32_t permuteseed, irng;
    const double *cldfrac, *ciwp, *clwp, *rei, *rel;   /* (ncol,nlay) */
    const double *tauc, *ssac, *asmc, *fsfc;           /* (nbnd,ncol,nlay), used when inflgsw = 0 */
    const double *alpha;                               /* (ncol,nlay), icld = 4 or 5 (get_alpha) */
} rrtmg_sw_clouds;

/* Arithmetic form of the solve. */
enum {
    RRTMG_SW_FORM_FP64 = 0,    /* plain FP64, reference operation order */
    RRTMG_SW_FORM_FP32 = 1     /* FP32 bulk (co-albedo carried, cancellation-free two-stream,
                                  heating from layer absorption); FP64 in setcoef, the
                                  outputs and cells whose table entry, conservative switch
                                  or resonance is ambiguous in FP32 */
};

enum {
    RRTMG_SW_OK = 0,
    RRTMG_SW_ENOTINIT = 1,     /* rrtmg_sw_ini_c not called */
    RRTMG_SW_ETABLES = 2,      /* coefficient table file missing or corrupt */
    RRTMG_SW_EARGS = 3,        /* bad sizes or NULL required pointer */
    RRTMG_SW_ECUDA = 4,        /* CUDA runtime error (see rrtmg_sw_last_cuda_error_c) */
    RRTMG_SW_ESCRATCH = 5,     /* rrtmg_sw_static_dev_c: request larger than its fixed scratch */
    RRTMG_SW_EINFLAG1 = 10,    /* cldprmc:166  INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA */
    RRTMG_SW_EICERAD = 11,     /* cldprmc:183,204  ICE RADIUS OUT OF BOUNDS */
    RRTMG_SW_EICEDGE = 12,     /* cldprmc:227  ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS */
    RRTMG_SW_EICEPROP = 13,    /* cldprmc:196-260  ice optical property outside physical limits */
    RRTMG_SW_ELIQRAD = 14,     /* cldprmc:273  LIQUID EFFECTIVE RADIUS OUT OF BOUNDS */
    RRTMG_SW_ELIQPROP = 15,    /* cldprmc:290-294  liquid optical property outside physical limits */
    RRTMG_SW_EICLD = 20,       /* mcica_subcol_gen_sw.f90:262-264  INVALID ICLD */
    RRTMG_SW_EKISSSEED = 21,   /* mcica_subcol_gen_sw.f90:472-474  KISSVEC SEED GENERATOR REQUIRES
                                  PMID FROM BOTTOM FOUR LAYERS */
    RRTMG_SW_ELAYTROP = 30,    /* profile without layers on both sides of the ~100 hPa switch */
    RRTMG_SW_EIRNG = 31,       /* irng = 1 (MT19937) on the static, batch or TL/AD entry points */
    RRTMG_SW_EPARTIAL = 32,    /* rrtmg_sw_rad.nomcica.f90:619-621  PARTIAL CLOUD NOT ALLOWED */
    RRTMG_SW_EBOUNDS = 40,     /* bounds-check build only: a table index left its coefficient blob */
    RRTMG_SW_ETIMEOUT = 41     /* FP32 form, tiled kernel: a wait between its warps gave up after seconds
                                  (the kernel ends with this code instead of hanging; outputs invalid) */
};

/* rrtmg_sw_ini (rrtmg_sw_init.f90:47-173): load the 112-g-point tables
 * (rrtmg_sw_tables.bin next to the library, or $RRTMG_SW_TABLES), build the
 * transmittance lookup table and heatfac = grav*secdy/(cpdair*1e2)
 * (rrtmg_sw_init.f90:258) and upload everything to the current GPU.
 * Idempotent; a later call only changes cpdair. */
int rrtmg_sw_ini_c(double cpdair);

/* rrtmg_sw (rrtmg_sw_rad.f90:99-841) with host arrays: copies inputs to the
 * device, solves every column, copies the outputs back.  icld outside 0..5
 * becomes 2 and iaer outside {0,6,10} becomes 0 (rrtmg_sw_rad.f90:589,597;
 * icld 4/5 are accepted).  Any nlay from 1 to 1000 is accepted; the profile
 * must have layers on both sides of the 100 hPa switch (RRTMG_SW_ELAYTROP),
 * and KISS subcolumns (fused McICA, irng = 0) need nlay >= 4
 * (RRTMG_SW_EKISSSEED), as their seeds come from the bottom four layers. */
int rrtmg_sw_c(const rrtmg_sw_args *a);

/* Same, all array pointers are device pointers; work is queued on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and the call returns after
 * the launch; the status of the device-side input checks is read back. */
int rrtmg_sw_dev_c(const rrtmg_sw_args *a, void *stream);

/* Fused McICA + rrtmg_sw: mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-296)
 * and rrtmg_sw in one pass; the subcolumn cloud masks are generated per
 * (column, g-point) inside the solve and never stored.  a->cldfmcl ..
 * a->clwpmcl are ignored; a->reicmcl/relqmcl are ignored too (c->rei, c->rel
 * are used, as mcica_subcol_sw copies them).  Host / device variants. */
int rrtmg_sw_mcica_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c);
int rrtmg_sw_mcica_dev_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c, void *stream);

/* rrtmg_sw without McICA (rrtmg_sw_rad.nomcica.f90:97-109): clouds are
 * given per layer and band, their optics come from cldprop_sw
 * (rrtmg_sw_cldprop.f90:53-374) and the solve is spcvrt_sw
 * (rrtmg_sw_spcvrt.f90:53-667).  The cloud arguments cldfr, cicewp, cliqwp,
 * reice, reliq (ncol,nlay) and taucld, ssacld, asmcld, fsfcld (nbnd,ncol,nlay)
 * are c->cldfrac, c->ciwp, c->clwp, c->rei, c->rel and c->tauc .. c->fsfc;
 * the McICA fields of `a` and c->permuteseed, irng, alpha are ignored.  A
 * layer cloud fraction strictly between 1e-6 and 1 - 1e-6 returns
 * RRTMG_SW_EPARTIAL, as the reference stops.  Host / device variants. */
int rrtmg_sw_nomcica_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c);
int rrtmg_sw_nomcica_dev_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c, void *stream);

/* Tangent-linear and adjoint (rrtmg_sw_tl / rrtmg_sw_ad; no counterpart in
 * the reference).  Objective per column, total sky:
 *   J = w_toa_up * swuflx(top) + w_sfc_net * (swdflx(sfc) - swuflx(sfc))
 *     + w_hr_sum * (sum of swhr over layers 1 .. nlay-1)
 * as a function of tlay, h2ovmr, o3vmr, the in-cloud water paths clwp and
 * ciwp of the fused McICA clouds (subcolumn masks frozen: they depend on
 * cldfrac and the seeds only) and the surface albedos.  The model is the
 * FP64 form with exp(-x) in place of the nearest-entry transmittance table
 * (whose derivative is zero almost everywhere); J is that model's value.
 * Host arrays; c is the fused McICA cloud input (irng = 0) or NULL for
 * clear sky (icld = 0).  rrtmg_sw_ad_c writes J and the gradient arrays
 * (any may be NULL); rrtmg_sw_tl_c reads the same arrays as a direction and
 * writes J and dJ = dJ/dx . direction.  store = 1 keeps each cell's local
 * Jacobian from the forward pass (more memory), 0 recomputes it in the
 * reverse pass, -1 chooses by memory: stored when that scratch fits in half
 * of the free device memory; rrtmg_sw_last_ad_store_c reports the choice. */
typedef struct rrtmg_sw_ad_args {
    double w_toa_up, w_sfc_net, w_hr_sum;
    int32_t store, pad;
    double *J;                                    /* (ncol) */
    double *dJ;                                   /* (ncol), rrtmg_sw_tl_c */
    double *tlay, *h2ovmr, *o3vmr, *clwp, *ciwp;  /* (ncol,nlay) gradients / direction */
    double *asdir, *asdif, *aldir, *aldif;        /* (ncol) gradients / direction */
} rrtmg_sw_ad_args;
int rrtmg_sw_ad_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c, const rrtmg_sw_ad_args *ad);
int rrtmg_sw_tl_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c, const rrtmg_sw_ad_args *ad);

/* Batches: many independent rrtmg_sw calls (ncol and nlay may differ) in
 * one persistent launch.  a[0..n) and, for instances with icld >= 1, c[0..n)
 * (fused McICA, irng = 0; c may be NULL when every instance is clear) hold
 * device pointers, as for rrtmg_sw_mcica_dev_c; they must stay valid, and
 * their contents may change, between runs.  The plan lists each instance's
 * sunlit columns (coszen > 0) on the device before the solve and skips the
 * others, whose outputs are set to zero (the reference solves them with mu0
 * clamped to 1e-10, i.e. 1e-10 of a daytime flux).  Planning runs an
 * autotuner (CTA tile of 2 or 4 columns x 112 g-points, instance order as
 * given or deepest first, 1 .. n resident CTAs per SM as shared memory
 * allows; one timed trial each, on the current data) and captures the
 * compaction and the solve in a CUDA graph; a run
 * replays the graph on `stream` and returns the device error status.  The
 * arithmetic form is the one current at planning.  No counterpart in the
 * reference (a GCM calls rrtmg_sw per chunk of columns). */
int rrtmg_sw_batch_plan_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c, int32_t n, void *stream,
                          void **plan);
int rrtmg_sw_batch_run_c(void *plan, void *stream);
/* The autotuner's choice (grid size, deepest-first order) and its trial
 * times in ms, in trial order (tile 2 then 4 columns; per tile the given
 * order then deepest first; per order 1, 2, .. CTAs per SM; tiles whose
 * shared memory does not fit are skipped); ntrials holds the capacity of
 * trial_ms on entry. */
int rrtmg_sw_batch_info_c(void *plan, int32_t *grid, int32_t *deepest_first, float *trial_ms,
                          int32_t *ntrials);
/* The chosen CTA tile (cols columns x gpoints g-points, one thread per
 * (column, g-point)) and each trial's candidate, in the trial order of
 * rrtmg_sw_batch_info_c, as cols << 16 | deepest_first << 8 | CTAs per SM;
 * ntrials holds the capacity of trial_cfg on entry. */
int rrtmg_sw_batch_tile_c(void *plan, int32_t *cols, int32_t *gpoints, int32_t *trial_cfg, int32_t *ntrials);
int rrtmg_sw_batch_free_c(void *plan);

/* Allocation-free device solve.  No counterpart in the reference: it exists
 * for callers that must not allocate device memory while they run -- a
 * model whose memory pool owns the whole GPU, or a time step that forbids
 * allocation after start-up.  It computes what rrtmg_sw_dev_c (c == NULL)
 * or rrtmg_sw_mcica_dev_c (c != NULL) computes, on device pointers, in the
 * current form, but its per-CTA scratch is a fixed 256 MiB area compiled
 * into the library instead of the growable workspace the other entry points
 * allocate with cudaMalloc; the call itself allocates nothing, on the device
 * or the host.
 *   - The first call on each device looks up the area's address once
 *     (cudaGetSymbolAddress with that device current) and loads the module
 *     that holds it; make that first call before any stream capture.
 *     rrtmg_sw_finalize_c forgets the address, so a later first call looks
 *     it up again.
 *   - Memory: with lazy CUDA module loading (the default since CUDA 12) the
 *     area is reserved on a device when that first call loads its module;
 *     with CUDA_MODULE_LOADING=EAGER every device the process creates a
 *     context on reserves the 256 MiB at context creation, even if this
 *     entry point is never called.
 *   - Limit: the area must hold one scratch slot per SM, or per column pair
 *     when the call has fewer pairs than SMs.  A slot is nlay * (16 with
 *     idelm = 0, else 14) * 224 values of the form's type, so 256 MiB
 *     takes nlay <= 140 (FP32) or <= 70 (FP64) with idelm = 1 on a 152-SM
 *     GPU and at least 304 columns.  Larger requests return
 *     RRTMG_SW_ESCRATCH, nothing runs.  The FP32 form's tiled kernel needs
 *     instead its per-SM areas plus one prepared block per column pair
 *     (about 16 KB at 60 layers); calls whose blocks do not fit take the
 *     scratch-based kernel.
 *     Fewer resident CTAs than rrtmg_sw_dev_c may run when the slots that
 *     fit are fewer than its grid; results are identical, only slower.
 *   - Nothing needs to start at zero: every scratch value is written before
 *     it is read; the device error word is cleared by the call itself.
 *   - One area per device and process, shared by every call: two solves
 *     that use it at the same time race and corrupt each other.  The
 *     library serialises its own calls and each call waits for its kernel
 *     before returning, so calls made one after another are safe; do not
 *     arrange for two of its kernels to be in flight at once.
 *   - Tables must have been loaded on the current device by rrtmg_sw_ini_c
 *     (RRTMG_SW_ENOTINIT otherwise). */
int rrtmg_sw_static_dev_c(const rrtmg_sw_args *a, const rrtmg_sw_clouds *c, void *stream);

/* mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-296), host arrays, outputs
 * (ngpt,ncol,nlay) and (ncol,nlay).  irng = 0: KISS with per-column streams
 * (seeded from the bottom four layer pressures, mcica:466-485); irng = 1:
 * Mersenne Twister, one stream in (subcolumn, column, layer) order seeded
 * with permuteseed.  icld 4/5 follow mcica_subcol_gen_sw.1col.f90:536-604. */
int mcica_subcol_sw_c(int32_t ncol, int32_t nlay, int32_t icld, int32_t permuteseed, int32_t irng,
                      const double *play, const double *cldfrac, const double *ciwp,
                      const double *clwp, const double *rei, const double *rel,
                      const double *tauc, const double *ssac, const double *asmc,
                      const double *fsfc, const double *alpha,
                      double *cldfmcl, double *ciwpmcl, double *clwpmcl, double *reicmcl,
                      double *relqmcl, double *taucmcl, double *ssacmcl, double *asmcmcl,
                      double *fsfcmcl);

/* MT19937 streams of the McICA generator (mcica_random_numbers.f90:77-306)
 * with jump-ahead; no reference counterpart (the reference draws its stream
 * sequentially).  The fused entry points (rrtmg_sw_mcica_c / _dev_c with
 * clouds->irng = 1) and mcica_subcol_sw_c use the device generator
 * internally; these two expose it, e.g. to split one GCM-order stream over
 * several processes.
 *   rrtmg_sw_mt_window_c: the 624 raw (untempered) state words behind
 *     outputs offset .. offset+623 of the stream seeded with seed, computed on
 *     the host (no GPU needed; offset < 2^48).  Tempering window[0] gives
 *     output number offset.
 *   rrtmg_sw_mt_stream_dev_c: outputs 0 .. n-1 (tempered u32, getRandomReal
 *     = u32 / (2^32 - 1)) into device memory `out`, generated as segments of
 *     2^log_seg words (log_seg <= 0: chosen from n), each started by a
 *     jump-ahead; same words for every log_seg. */
int rrtmg_sw_mt_window_c(int32_t seed, uint64_t offset, uint32_t *window);
int rrtmg_sw_mt_stream_dev_c(int32_t seed, uint64_t n, uint32_t *out, int32_t log_seg, void *stream);

/* setcoef_sw's integer outputs (rrtmg_sw_setcoef.f90:158-200) for the
 * layers of a GCM call, as the solve kernels of both forms compute them (the
 * same device routine, after inatm_sw's layer amounts,
 * rrtmg_sw_rad.f90:1527-1586): jp, jt, jt1, indself, indfor (ncol,nlay) and
 * laytrop (ncol), host arrays.  Only the state inputs of `a` are read (play,
 * plev, tlay and the gas mixing ratios).  A diagnostic for checking the
 * table indices bit for bit against another implementation.  Computed as
 * the current arithmetic form computes them: the FP32 form's setcoef (FP32
 * arithmetic, each index re-evaluated in FP64 where its FP32 value is within
 * 1e-4 of an integer or threshold) returns the FP64 form's indices. */
int rrtmg_sw_setcoef_c(const rrtmg_sw_args *a, int32_t *jp, int32_t *jt, int32_t *jt1, int32_t *indself,
                       int32_t *indfor, int32_t *laytrop);

/* get_alpha (mcica_subcol_gen_sw.f90:66-178), host arrays. */
int get_alpha_c(int32_t ncol, int32_t nlay, int32_t icld, int32_t idcor, double decorr_con,
                const double *dz, const double *lat, int32_t juldat, const double *cldfrac,
                double *alpha);

/* Select the arithmetic form used by subsequent solves (default FP64).  The
 * switch takes the library's lock, so a solve in progress on another thread
 * finishes in the form it started with. */
int rrtmg_sw_set_form_c(int32_t form);
int rrtmg_sw_get_form_c(void);

/* Number of kernels the most recent solve launched (for launch accounting). */
int rrtmg_sw_last_launch_count_c(void);
/* Kernel of the most recent solve's main launch: RRTMG_SW_KERNEL_FP64, the
 * FP32 form's scratch-based kernel (RRTMG_SW_KERNEL_FP32) or its tiled kernel
 * (RRTMG_SW_KERNEL_FP32_TILED: nlay <= 64, idelm = 1, shared memory
 * permitting); -1 before the first solve. */
#define RRTMG_SW_KERNEL_FP64 0
#define RRTMG_SW_KERNEL_FP32 1
#define RRTMG_SW_KERNEL_FP32_TILED 2
int rrtmg_sw_last_kernel_c(void);
/* Pair slots of the most recent solve's tiled kernel: 3 when their shared
 * memory fits (60 layers without the extra outputs, for instance), else 2;
 * 0 when the most recent solve did not run the tiled kernel. */
int rrtmg_sw_last_tile_slots_c(void);
/* Counters of the FP32 form over the most recent solve through
 * rrtmg_sw_c / rrtmg_sw_mcica_c / their _dev_ forms (zeros for the FP64
 * form): stats[0] cells whose FP32 optics were too close to a discrete
 * choice of the reference (table entry, conservative switch, resonance)
 * and were redone in FP64; stats[1] of those, cells past the scratch-based
 * kernel's redo queue (redone by their own thread); stats[2] column pairs
 * the tiled kernel handed back to the scratch-based kernel (capacity of
 * FP64 cells exceeded); stats[3] subcolumns the tiled kernel swept a
 * second time for their FP64 cells. */
int rrtmg_sw_last_fp32_stats_c(int64_t* stats);
/* Checkpointing of the most recent rrtmg_sw_ad_c / rrtmg_sw_tl_c call:
 * 1 stored Jacobians, 0 recomputed, -1 none yet. */
int rrtmg_sw_last_ad_store_c(void);

/* Reference message for an error code; last CUDA error string. */
const char *rrtmg_sw_errstr_c(int32_t code);
const char *rrtmg_sw_last_cuda_error_c(void);

/* Release the device tables and workspace (rrtmg_sw_ini_c may be called
 * again afterwards). */
int rrtmg_sw_finalize_c(void);

#ifdef __cplusplus
}
#endif

#endif
