/*
 * rrtmg_sw_oracle.h -- FP64 CPU restatement of the RRTMG_SW shortwave solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the GPU
 * implementation in rrtmg_sw_gb300/ is tested against: it is loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
 * product path.  It restates, in plain C++ compiled with -ffp-contract=off,
 * the reference Fortran routines cited next to each function in
 * rrtmg_sw_oracle.cpp, and it is pinned against the reference's committed
 * golden outputs (run_examples_std_atm/output_rrtm_*, fixtures under
 * tests/golden/).
 *
 * Array layout: every array argument uses the reference's Fortran
 * (column-major) layout.  A Fortran array a(ncol,nlay) is passed as a flat
 * buffer with element (i,l) at [i + ncol*l]; a(ngpt,ncol,nlay) has
 * (g,i,l) at [g + 112*(i + ncol*l)]; a(ncol,nlay,nbnd) has (i,l,b) at
 * [i + ncol*(l + nlay*b)].  Layer 1 is the surface layer.
 */
#ifndef RRTMG_SW_ORACLE_H
#define RRTMG_SW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Arguments of the GCM entry point rrtmg_sw (rrtmg_sw_rad.f90:99-111), in
 * the same order.  Optional Fortran arguments are nullable pointers. */
typedef struct orc_rrtmg_sw_args {
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
    const double *cldfmcl, *taucmcl, *ssacmcl, *asmcmcl, *fsfcmcl;
    const double *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl;
    const double *tauaer, *ssaaer, *asmaer, *ecaer;
    double *swuflx, *swdflx, *swhr, *swuflxc, *swdflxc, *swhrc;
    const double *bndsolvar;   /* (14) or NULL */
    const double *indsolvar;   /* (2)  or NULL */
    const double *solcycfrac;  /* scalar or NULL */
    /* Extra outputs (computed by spcvmc_sw but local in the GCM driver,
     * rrtmg_sw_rad.f90:810-820); each is (ncol,nlay+1) or NULL. */
    double *dirdflux, *difdflux, *uvdflx, *nidflx, *dirdnuv, *difdnuv, *dirdnir, *difdnir;
    int32_t idelm;             /* reference hard-codes 1 (rrtmg_sw_rad.f90:605) */
    int32_t nthreads;          /* OpenMP threads over columns, <=0: default */
    double *bndfu, *bndfd, *bndfddir, *bndcu, *bndcd;  /* (ncol,nlay+1,14) per-band fluxes or NULL */
} orc_rrtmg_sw_args;

/* Error codes: 0 = success; values mirror the reference's `stop` sites. */
enum {
    ORC_OK = 0,
    ORC_ERR_NOT_INITIALIZED = 1,
    ORC_ERR_TABLES = 2,
    ORC_ERR_ARGS = 3,
    ORC_ERR_INFLAG1 = 10,          /* cldprmc:166  INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA */
    ORC_ERR_ICE_RADIUS = 11,       /* cldprmc:183,204  ICE RADIUS OUT OF BOUNDS */
    ORC_ERR_ICE_DGE = 12,          /* cldprmc:227  ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS */
    ORC_ERR_ICE_PROPS = 13,        /* cldprmc:196-200,213-217,250-260  ice extinction/ssa/asym/fdelta limits */
    ORC_ERR_LIQ_RADIUS = 14,       /* cldprmc:273  LIQUID EFFECTIVE RADIUS OUT OF BOUNDS */
    ORC_ERR_LIQ_PROPS = 15,        /* cldprmc:290-294  liquid extinction/ssa/asym limits */
    ORC_ERR_ICLD = 20,             /* mcica:262-264  INVALID ICLD */
    ORC_ERR_KISS_SEED = 21,        /* mcica:472-474  KISSVEC SEED GENERATOR REQUIRES PMID FROM BOTTOM FOUR LAYERS */
    ORC_ERR_LAYTROP = 30,          /* profile with no layer above or below the 100 hPa switch */
    ORC_ERR_PARTIAL = 32           /* rad.nomcica:619-621 / 1col:612-617  PARTIAL CLOUD NOT ALLOWED */
};

/* rrtmg_sw_ini (rrtmg_sw_init.f90:47-173): load the reduced tables written
 * by rrtmg_sw_gb300/data/extract_tables.py and build exp_tbl and heatfac. */
int orc_init(const char *table_path, double cpdair);

/* rrtmg_sw (rrtmg_sw_rad.f90:99-841). */
int orc_rrtmg_sw(const orc_rrtmg_sw_args *a);

/* rrtmg_sw without McICA (rrtmg_sw_rad.nomcica.f90:97-841): cloud fraction
 * cldfr, ice/liquid paths cicewp/cliqwp and sizes reice/reliq (ncol,nlay),
 * and taucld/ssacld/asmcld/fsfcld (14,ncol,nlay); the McICA fields of `a`
 * are ignored.  Cloud optics from cldprop_sw, solve by spcvrt_sw. */
int orc_rrtmg_sw_nomcica(const orc_rrtmg_sw_args *a, const double *cldfr, const double *taucld,
                         const double *ssacld, const double *asmcld, const double *fsfcld,
                         const double *cicewp, const double *cliqwp, const double *reice,
                         const double *reliq);

/* get_alpha (mcica_subcol_gen_sw.f90:66-178). */
int orc_get_alpha(int ncol, int nlay, int icld, int idcor, double decorr_con,
                  const double *dz, const double *lat, int juldat,
                  const double *cldfrac, double *alpha);

/* mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-296) with
 * generate_stochastic_clouds_sw (:300-717).  irng=0 (KISS) gives every column
 * its own stream; irng=1 (Mersenne Twister) uses one stream in the
 * reference's (subcolumn, column, layer) order.  icld 4/5 follow the
 * single-column generator's loop order (mcica_subcol_gen_sw.1col.f90:536-604)
 * because the GCM file's icld 4/5 branches do not compile. */
int orc_mcica_subcol_sw(int ncol, int nlay, int icld, int permuteseed, int irng,
                        const double *play, const double *cldfrac,
                        const double *ciwp, const double *clwp,
                        const double *rei, const double *rel,
                        const double *tauc, const double *ssac,
                        const double *asmc, const double *fsfc,
                        const double *alpha,
                        double *cldfmcl, double *ciwpmcl, double *clwpmcl,
                        double *reicmcl, double *relqmcl,
                        double *taucmcl, double *ssacmcl, double *asmcmcl,
                        double *fsfcmcl);

/* Mersenne Twister stream (mcica_random_numbers.f90): n values of
 * getRandomReal after new_RandomNumberSequence(seed). */
void orc_mt_real(int seed, int n, double *out);
/* KISS (mcica_subcol_gen_sw.f90:721-753) on one seed quadruple: n draws. */
void orc_kiss_real(int32_t s1, int32_t s2, int32_t s3, int32_t s4, int n, double *out);

/* One single-column case of the column driver (rrtmg_sw.1col.f90:552-948):
 * inputs are the already-parsed INPUT_RRTM / IN_CLD_RRTM / IN_AER_RRTM
 * records (column amounts in molecules/cm^2, bands 16..29 as 0..13).
 * With imca=1 the McICA samples use the Mersenne Twister with seed
 * (ims+1)*112 and are averaged over nmca samples. */
typedef struct orc_column_case {
    int32_t nlay, icld, iaer, idelm, imca, nmca, idcor, juldat;
    int32_t inflag, iceflag, liqflag, isolvar;
    int32_t istart, iend;       /* band range 16..29 (per-band output) */
    double zenith;              /* cosine of solar zenith angle */
    double decorr_con, lat;
    double svar_f, svar_s, svar_i;
    const double *svar_f_bnd, *svar_s_bnd, *svar_i_bnd, *adjflux;  /* (14) */
    const double *albedo;       /* (14): 1 - semiss */
    const double *pavel, *tavel, *pz, *tz, *coldry;  /* pz,tz: (0:nlay) */
    const double *wkl;          /* (7,nlay) molecules/cm^2 */
    const double *dz;           /* (nlay) m */
    const double *cldfrac, *ciwp, *clwp, *rei, *rel;  /* (nlay) */
    const double *tauc, *ssac, *asmc, *fsfc;         /* (14,nlay) */
    const double *tauaer, *ssaaer, *asmaer;          /* (nlay,14) */
    /* outputs, index 0..nlay (level 0 = surface) */
    double *uflx, *dflx, *dirdflx, *difdflx, *fnet, *htr;
} orc_column_case;

int orc_column_mode(const orc_column_case *c);

/* Solar-variability factors of one solar record, for orc_column_mode: the
 * settings of inatm_sw (rrtmg_sw_rad.f90:1245-1512), which the column driver
 * repeats for isolvar 0..3 (rrtmg_sw.1col.f90:1391-1436,1446-1660).
 * indsolvar (2), solcycfrac and bndsolvar (14) may be NULL as in
 * orc_rrtmg_sw_args.  Outputs: svar = {f, s, i}, svar_bnd = {f[14], s[14],
 * i[14]}, adjflux (14). */
int orc_solar_factors(int isolvar, double scon, double adjes, int dyofyr,
                      const double *indsolvar, const double *solcycfrac, const double *bndsolvar,
                      double *svar, double *svar_bnd, double *adjflux);

/* Diagnostics of setcoef_sw for parity tests of the integer indices:
 * jp, jt, jt1, indself, indfor (nlay each) and laytrop for one column. */
int orc_setcoef_indices(int nlay, const double *pavel, const double *tavel,
                        const double *coldry, const double *wkl,
                        int32_t *jp, int32_t *jt, int32_t *jt1,
                        int32_t *indself, int32_t *indfor, int32_t *laytrop);
/* setcoef_sw indices of GCM-interface columns (inatm_sw amounts first);
 * outputs (ncol, nlay) column-major, laytrop (ncol) */
int orc_gcm_setcoef_indices(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                            const double* h2ovmr, const double* co2vmr, const double* o3vmr, const double* n2ovmr,
                            const double* ch4vmr, const double* o2vmr, int32_t* jp, int32_t* jt, int32_t* jt1,
                            int32_t* indself, int32_t* indfor, int32_t* laytrop);

/* exp_tbl (0:10000) as built by rrtmg_sw_ini, for tests. */
int orc_exp_table(double *out10001);
double orc_heatfac(void);

#ifdef __cplusplus
}
#endif

#endif
