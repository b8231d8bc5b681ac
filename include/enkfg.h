/*
 * enkfg.h -- C ABI of the GB300 EnKF-C analysis hot path (libenkfg.so).
 *
 * The library replaces two host stages of EnKF-C with sm_103a CUDA kernels:
 *   enkf_calc   : das_calctransforms  (reference calc/transforms.c:991-1637)
 *   enkf_update : das_updatefields / das_updatebg  (update/update.c:92-814)
 * together with the routines they call (obs_findlocal, calc_wT_etkf,
 * calc_wT_denkf, calc_G/calc_w, das_calcinnandspread, das_standardise,
 * das_sethybridensemble).  Each entry point below names the reference
 * interface it stands in for.
 *
 * Conventions (unlike the reference, nothing aborts):
 *   - every call returns an enkfg_status; enkfg_last_error() explains it;
 *   - host buffers are owned by the caller, device buffers by the context;
 *   - a context is bound to one GPU and is used from one host thread;
 *   - array layouts are the reference's: S [nmem][nobs], transforms
 *     T [nj][ni][m_dyn][m] and w [nj][ni][m] (transforms.nc, transforms.c:
 *     54-94), fields [nmem][jsize][mni] per field-layer (update.c:92).
 *   - device-pointer entry points (suffix _dev) take and return plain device
 *     addresses and a cudaStream_t passed as void*; nothing is synchronised
 *     on the host by them.
 */
#ifndef ENKFG_H
#define ENKFG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ENKFG_API __attribute__((visibility("default")))
#else
#define ENKFG_API
#endif

typedef enum {
    ENKFG_OK = 0,
    ENKFG_EINVAL = 1,           /* bad argument or inconsistent sizes */
    ENKFG_ECUDA = 2,            /* a CUDA runtime call failed */
    ENKFG_ENOMEM = 3,           /* device allocation failed */
    ENKFG_ETIMEOUT = 4,         /* a bounded device wait gave up */
    ENKFG_ENUMERIC = 5,         /* a per-point factorisation failed (info in last_error) */
    ENKFG_ECAPACITY = 6,        /* an output or scratch capacity is too small */
    ENKFG_ESTATE = 7,           /* call order: required inputs not set */
    ENKFG_EUNSUPPORTED = 8      /* option not implemented on the device path */
} enkfg_status;

enum { ENKFG_MODE_ENKF = 0, ENKFG_MODE_ENOI = 1, ENKFG_MODE_HYBRID = 2 };        /* dasystem.h MODE_* */
enum { ENKFG_SCHEME_DENKF = 0, ENKFG_SCHEME_ETKF = 1 };                          /* dasystem.h SCHEME_* */
enum { ENKFG_PATH_PLAIN = 0, ENKFG_PATH_BATCHED = 1 };
enum { ENKFG_PREC_FP64 = 0, ENKFG_PREC_MIXED = 1 };

#define ENKFG_MAXLOCRAD 8
#define ENKFG_MAXTYPES 32
#define ENKFG_MAXMEM 160

typedef struct enkfg_ctx enkfg_ctx;

/* Context on CUDA device `device`.  Replaces the per-rank state EnKF-C keeps
 * in dasystem/observations (dasystem.h:60-128) for the hot path. */
ENKFG_API enkfg_status enkfg_create(int device, enkfg_ctx** ctx);
ENKFG_API void enkfg_destroy(enkfg_ctx* ctx);

/* Bound on each device wait of this context, in nanoseconds (0: the default,
 * 2 s).  No counterpart in the reference, which has no device waits: the
 * mixed-precision transform kernel waits on mbarriers for its tensor-core
 * MMAs; a wait that exceeds the bound makes the point's status a timeout,
 * the kernel drains its MMAs (at most 2 s more) and releases its tensor
 * memory, and enkfg_calc_transforms returns ENKFG_ETIMEOUT.  The context
 * stays usable. */
ENKFG_API enkfg_status enkfg_set_wait_limit(enkfg_ctx* ctx, unsigned long long ns);
/* A drill of that timeout path, off by default; no counterpart in the
 * reference.  With `on`, every CTA of the mixed-precision transform kernel
 * first waits (within the bound above) on an mbarrier that nothing arrives
 * at, so the wait expires: the call returns ENKFG_ETIMEOUT without a fault
 * or a hang, and the context stays usable once the drill is off. */
ENKFG_API enkfg_status enkfg_set_wait_drill(enkfg_ctx* ctx, int on);
ENKFG_API const char* enkfg_last_error(const enkfg_ctx* ctx);
ENKFG_API const char* enkfg_status_string(enkfg_status st);
ENKFG_API int enkfg_version(void);

/* Observation types: LOCRAD/LOCWEIGHT/RFACTOR per type (obstypes.c:170-560,
 * used by obstype_calclcoeff obstypes.c:800 and das_standardise ensobs.c:849).
 * locrad/locweight are [ntypes][ENKFG_MAXLOCRAD]; geographic selects 3-D
 * distances on the sphere (ll2xyz, utils.c:1449). */
ENKFG_API enkfg_status enkfg_set_obstypes(enkfg_ctx* ctx, int ntypes, const int* nlocrad, const double* locrad, const double* locweight, const double* rfactor, int geographic);

/* NLOBSMAX per observation type (obstype NLOBSMAX, obstypes.c:432 and 547;
 * applied in obs_findlocal, observations.c:1899-1901, with the distance sort
 * of kd_findnodeswithinrange, kdtree.c:558-574): a point keeps, of each type
 * t with nlobsmax[t] > 0, the nlobsmax[t] observations nearest to it (exact
 * FP64 squared distance; equal distances in order of observation index).
 * nlobsmax[t] <= 0: no limit (the default).  nlobsmax NULL clears every
 * limit.  Applies to enkfg_local_obs, the transforms and the adjoint;
 * enkfg_set_obstypes clears the limits. */
ENKFG_API enkfg_status enkfg_set_obstype_nlobsmax(enkfg_ctx* ctx, int ntypes, const int* nlobsmax);

/* Which observation types the current grid sees (obstype DOMAINS against the
 * grid's domain name: observations.c:1877-1892, where a type whose domain
 * list does not hold the grid's domain is skipped by obs_findlocal).  The
 * caller compares the names; visible[t] = 0 hides type t from the local
 * search (enkfg_local_obs, the transforms, the adjoint) until it is set
 * again.  visible NULL shows every type (the default, and the state after
 * enkfg_set_obstypes). */
ENKFG_API enkfg_status enkfg_set_obstype_visible(enkfg_ctx* ctx, int ntypes, const int* visible);

/* Observations (observation fields used on the path, observations.h:47-100):
 * float lon/lat, type, status (0 = STATUS_OK), float estd and value. */
ENKFG_API enkfg_status enkfg_set_obs(enkfg_ctx* ctx, int nobs, const float* lon, const float* lat, const short* type, const short* status, const float* estd, const float* value);

/* Forecast ensemble observations HE [nmem][nobs] (das->S in S_MODE_HE_f,
 * dasystem.h:95).  nmem_dynamic < nmem for hybrid ensembles. */
ENKFG_API enkfg_status enkfg_set_HE(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* HE);

/* ---- forward operator on the device (das_getHE, calc/ensobs.c:46-490) ----
 * Instead of enkfg_set_HE, HE can be built on the device from the ensemble
 * fields: enkfg_set_obs_positions once, enkfg_begin_HE, one enkfg_map_obs per
 * observation type and member block (the reference calls H per type and
 * member, ensobs.c:181-300), then enkfg_finish_HE. */

/* Fractional grid positions of the observations (observation.fij[0..1],
 * double, and observation.fk, float; observations.h:47-100).  fk may be NULL
 * when no observation type is 3-D. */
ENKFG_API enkfg_status enkfg_set_obs_positions(enkfg_ctx* ctx, const double* fi, const double* fj, const float* fk);

/* das_getHE set-up (ensobs.c:72-83): HE [nmem][nobs] in the context filled
 * with NaN, plus, when with_background (EnOI), the background row Hx. */
ENKFG_API enkfg_status enkfg_begin_HE(enkfg_ctx* ctx, int nmem, int nmem_dynamic, int with_background);

typedef struct {
    int ni, nj, nk;             /* the variable's grid; nk = 1 for a 2-D field */
    int three_d;                /* 0: H_surf_standard (2-D interpolation of one layer), 1: H_subsurf_standard */
    int ksurf;                  /* grid_getsurflayerid: 0 or nk - 1 (3-D) */
    int periodic_i;
    int offset_kind;            /* "<type>:OFFSET" data: 0 none, 1 [nk], 2 [nj][ni], 3 [nk][nj][ni] */
    int skip_bad;               /* --skip-bad-forecast-obs */
} enkfg_hop_params;

/* H_surf_standard / H_subsurf_standard (model2obs.c:127-181, 256-348) with
 * evaluate_2d_obs / interpolate_3d_obs (model2obs.c:37-124), footprint 0, on a
 * structured grid (interpolate2d_structured / interpolate3d_structured,
 * utils.c:1140-1366), for members mem0 .. mem0 + nfield - 1 at once
 * (mem0 = -1 with nfield = 1: the EnOI background row).  fields is
 * [nfield][nk][nj][ni] (3-D) or [nfield][nj][ni] (2-D: the layer the
 * reference reads), numlevels [nj][ni], offset laid out per offset_kind (or
 * NULL).  The observations are ids[nids] (all of type obstype), or, when ids
 * is NULL, every observation of type obstype with status 0 (obs_find_bytype,
 * observations.c:1543).  A forecast that is not finite or exceeds 999999 in
 * magnitude is ENKFG_ENUMERIC unless skip_bad (then NaN); a position off the
 * grid is ENKFG_EINVAL. */
ENKFG_API enkfg_status enkfg_map_obs(enkfg_ctx* ctx, const enkfg_hop_params* p, int obstype, int nids, const int* ids, int mem0, int nfield, const float* fields, const int* numlevels, const float* offset);
/* Device-resident form: ids/fields/numlevels/offset are device addresses;
 * nothing is synchronised, and errors (an id outside 0..nobs-1 included)
 * surface in enkfg_finish_HE. */
ENKFG_API enkfg_status enkfg_map_obs_dev(enkfg_ctx* ctx, const enkfg_hop_params* p, int obstype, int nids, const int* ids_dev, int mem0, int nfield, const float* fields_dev, const int* numlevels_dev, const float* offset_dev, void* stream);

/* End of das_getHE (ensobs.c:372-490): with skip_bad, observations with a NaN
 * forecast in any member (or in Hx) get status 10 (STATUS_BADFC); then for
 * ENKFG_MODE_ENOI every member is recentred on the background (S_e += Hx -
 * mean, float) and for ENKFG_MODE_HYBRID the dynamic and static anomalies are
 * scaled by k_d = sqrt((m-1)/(m_d-1)) and k_s = sqrt(gamma (m-1)/(m_s-1)) about
 * the dynamic mean.  nbad (or NULL) receives the number of observations with
 * status 10 and status (or NULL) the statuses [nobs].  HE is then ready for
 * enkfg_calc_innovations. */
ENKFG_API enkfg_status enkfg_finish_HE(enkfg_ctx* ctx, int mode, double gamma, int skip_bad, int* nbad, short* status);

/* das_calcinnandspread (ensobs.c:541-690): HE -> HA in place on the device,
 * innovations s_f = y - Hx and spread std_f; either output may be NULL. */
ENKFG_API enkfg_status enkfg_calc_innovations(enkfg_ctx* ctx, double* s_f, double* std_f);

/* das_standardise (ensobs.c:849-898): S and s_f divided by
 * estd * sqrt(rfactor) * sqrt(nmem - 1), on the device. */
ENKFG_API enkfg_status enkfg_standardise(enkfg_ctx* ctx);

/* Set standardised S [nmem][nobs] and s [nobs] directly (the state
 * das_calctransforms works on after das_standardise, S_MODE_S_f). */
ENKFG_API enkfg_status enkfg_set_S(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* S, const double* s);
/* Copy the device S / s back (either may be NULL). */
ENKFG_API enkfg_status enkfg_get_S(enkfg_ctx* ctx, float* S, double* s);

/* Model grid of the analysed variables (rectangular: x[mni], y[mnj];
 * curvilinear: x2d/y2d [mnj][mni], x/y NULL) with the transform stride and
 * the periodic-i flag (grid_getstride, grid_isperiodic_i; hgrid_ij2xy,
 * hgrid.c:457-472).  A strided point without coordinates (NaN: a grid of
 * type NONE, where obs_findlocal takes every observation) is refused with
 * ENKFG_EUNSUPPORTED. */
typedef struct {
    int mni, mnj;
    const double* x;
    const double* y;
    const double* x2d;
    const double* y2d;
    int stride;
    int periodic_i;
} enkfg_grid;
ENKFG_API enkfg_status enkfg_set_grid(enkfg_ctx* ctx, const enkfg_grid* grid);

/* Strided transform grid size: nj = (mnj-1)/stride+1, ni = (mni-1)/stride+1
 * (transforms.c:1065-1072). */
ENKFG_API enkfg_status enkfg_transform_dims(const enkfg_ctx* ctx, int* nj, int* ni);

/* obs_findlocal (observations.c:1837-1927) for every strided grid point.
 * counts [nj*ni] receives the local obs count per point.  If ids is not
 * NULL, offsets [nj*ni+1] receives the CSR offsets and ids/coeffs the local
 * observation ids (sorted by id) and their taper coefficients, up to
 * `capacity` entries (ENKFG_ECAPACITY if the total exceeds it). */
ENKFG_API enkfg_status enkfg_local_obs(enkfg_ctx* ctx, int* counts, long long* offsets, int* ids, double* coeffs, long long capacity);

typedef struct {
    int mode;                   /* ENKFG_MODE_* */
    int scheme;                 /* ENKFG_SCHEME_* */
    double alpha;               /* relaxation to prior, transforms.c:1270-1286 */
    int path;                   /* ENKFG_PATH_PLAIN or ENKFG_PATH_BATCHED */
    int precision;              /* ENKFG_PREC_FP64 or ENKFG_PREC_MIXED */
    int want_diag;              /* fill the enkf_diag.nc outputs */
    int tune;                   /* batched path: autotune the chunk size per local-obs count bin on first use */
} enkfg_calc_params;

typedef struct {
    int* nlobs;                 /* [nj][ni] */
    float* dfs;                 /* [nj][ni] */
    float* srf;                 /* [nj][ni] */
    int* pnlobs;                /* [ntypes][nj][ni] */
    float* pdfs;                /* [ntypes][nj][ni] */
    float* psrf;                /* [ntypes][nj][ni] */
} enkfg_diag;

/* das_calctransforms (transforms.c:991-1637): for every strided point find
 * the local obs, taper, form I + S'S, solve (ETKF eigen / DEnKF Cholesky /
 * EnOI), relax to prior and write T [nj][ni][m_dyn][m] (NULL for EnOI) and
 * w [nj][ni][m] as float, plus, if not NULL, the same in double before the
 * float cast (T64, w64) and the diagnostics (enkf_diag.nc, transforms.c:
 * 1298-1345).  Results stay resident on the device for enkfg_update_*. */
ENKFG_API enkfg_status enkfg_calc_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, float* T, float* w, double* T64, double* w64, const enkfg_diag* diag);

/* Device-resident form: computes into the context's device buffers on
 * `stream` (NULL = the context stream) without host copies. */
ENKFG_API enkfg_status enkfg_calc_transforms_dev(enkfg_ctx* ctx, const enkfg_calc_params* p, void* stream);
/* Device addresses of the resident transforms (valid until the next calc). */
ENKFG_API enkfg_status enkfg_transforms_dev_ptr(enkfg_ctx* ctx, float** T, float** w);
/* Load transforms (e.g. read back from transforms.nc) into the context. */
ENKFG_API enkfg_status enkfg_set_transforms(enkfg_ctx* ctx, int mode, int nmem, int nmem_dynamic, const float* T, const float* w);

typedef struct {
    int mode;                   /* ENKF / HYBRID: das_updatefields; ENOI: das_updatebg */
    int nmem, nmem_dynamic;
    int surfk;                  /* grid_getsurflayerid */
    int issurfacevar;
    float inflation;            /* INFLATION (model_getvarinflation) */
    double inf_ratio;           /* NaN: plain multiplicative inflation */
    int output_increment;       /* --output-increment */
    int applylog;               /* variable stored as log10 */
    int j1, j2;                 /* field tile rows (FIELDSPLIT), j1 % stride == 0; j2 < 0: all */
    int precision;              /* ENKFG_PREC_FP64 (float CUDA cores) or ENKFG_PREC_MIXED */
} enkfg_update_params;

/* das_updatefields (update.c:92-564) for nfield field-layers sharing the
 * grid: fields [nfield][nmem][jsize][mni] updated in place (host), levels
 * [nfield] their layer index, numlevels [mnj][mni] the grid's wet-level
 * count.  infl (or NULL) receives [nfield][jsize][mni] inflation
 * (--write-inflation).  For ENKFG_MODE_ENOI the call is das_updatebg
 * (update.c:568-814) and fields are [nfield][nmem+1][jsize][mni] with the
 * background in slot nmem.  Uses the transforms resident in the context.
 * The field-layers stream through the device in groups (as the reference's
 * FIELDBUFFERSIZE batches, update/update.c:1552-2132), each group in blocks
 * of model rows (about 512 MB, a multiple of the stride), three device
 * buffers in turn: the copies in and out of neighbouring blocks run on the
 * context's copy streams while a block is updated, so with pinned host
 * buffers the transfers overlap the update and the device holds three
 * blocks, not the whole ensemble.  The result does not depend on the
 * grouping. */
ENKFG_API enkfg_status enkfg_update_fields(enkfg_ctx* ctx, const enkfg_update_params* p, const int* numlevels, int nfield, const int* levels, float* fields, float* infl);

/* Field-layers per group of the host-buffer update (FIELDBUFFERSIZE,
 * common/enkfprm.c:381-388); 0 (the default) picks groups of about 3 GB. */
ENKFG_API enkfg_status enkfg_set_field_buffer_size(enkfg_ctx* ctx, int nfield);

/* Local analyses per batch of the batched solves (the transform kernel
 * hands each batch's points to the solve kernels through a scratch slot of
 * each point; the host outputs of enkfg_calc_transforms leave batch by
 * batch).  0 (the default) sizes batches by their scratch: about 8 GB for
 * the refined ETKF solve, 2 GB for the FP64 ones.  Taken to at least 256
 * and, from 1024 on, to a multiple of 1024.  No counterpart in the
 * reference; the result does not depend on it. */
ENKFG_API enkfg_status enkfg_set_solve_batch(enkfg_ctx* ctx, int points);

/* Model rows per block of the host-buffer update, rounded up to a multiple
 * of the stride; 0 (the default) picks blocks of about 512 MB.  No
 * counterpart in the reference (it reads whole fields); the result does
 * not depend on it. */
ENKFG_API enkfg_status enkfg_set_field_block_rows(enkfg_ctx* ctx, int rows);

/* RANDOMISE ("propagate") for the next enkfg_update_fields or
 * enkfg_update_fields_dev call (addnoise, update/update.c:46-87, which
 * das_updatefields applies to each of its fields after the update,
 * :552-563): field-layer f with a non-NaN deflation[f] (DEFLATION of its
 * model variable) becomes, in every cell of member e,
 *     v * (float)deflation + mult * (random[f][e] - mean_e random[f][e]),
 *     mult = (float)(sqrt(1 - deflation^2) * sigma[f])   (SIGMA),
 * in the reference's precisions.  random [nfield][nmem] are the standard
 * normals the host draws for the field (get_normalpair, utils.c:1477-1484,
 * in the reference's order: (nmem + 1) / 2 pairs, the first nmem used).
 * The noise covers the rows the update call covers (its j1..j2 tile).
 * A deflation outside [0, 1] or a non-finite sigma is refused (the
 * reference's model parameter check, common/model.c:253-256).
 * nfield and nmem must be the next call's; ENOI updates take no noise.
 * nfield 0 or deflation NULL: none.  The next update call uses it up. */
ENKFG_API enkfg_status enkfg_set_field_noise(enkfg_ctx* ctx, int nfield, int nmem, const double* deflation, const double* sigma, const double* random);

/* Device-resident form: fields/infl are device addresses. */
ENKFG_API enkfg_status enkfg_update_fields_dev(enkfg_ctx* ctx, const enkfg_update_params* p, const int* numlevels_dev, int nfield, const int* levels, float* fields_dev, float* infl_dev, void* stream);

/* das_sethybridensemble (dasystem.c:775-819) on v [nmem][nij] (host, in
 * place): dynamic anomalies scaled by k_d, static by k_s, both recentred on
 * the dynamic mean. */
ENKFG_API enkfg_status enkfg_set_hybrid_ensemble(enkfg_ctx* ctx, int nmem, int nmem_dynamic, double gamma, int nij, float* v);
ENKFG_API enkfg_status enkfg_set_hybrid_ensemble_dev(enkfg_ctx* ctx, int nmem, int nmem_dynamic, double gamma, int nij, float* v_dev, void* stream);

/* Run all later work of this context on `stream` (a cudaStream_t; NULL
 * restores the context's own stream). */
ENKFG_API enkfg_status enkfg_set_stream(enkfg_ctx* ctx, void* stream);

/* Device-resident HE [nmem][nobs] (a device address): copied on the device
 * into the context, as enkfg_set_HE does from the host. */
ENKFG_API enkfg_status enkfg_set_HE_dev(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* HE_dev);

/* Rebuild the spatial index now, on the context's stream (obs_createkdtrees
 * is part of every enkf_calc run, observations.c:1616).  The build reads
 * bucket counts back to the host, so it stays outside CUDA-graph capture; the
 * calls after it (innovations, standardisation, transforms, update) can be
 * captured, and the index's device buffers keep their addresses while the
 * observation count does not grow. */
ENKFG_API enkfg_status enkfg_rebuild_index(enkfg_ctx* ctx);

/* Observation impact: adjoint of the local analysis (no counterpart in the
 * reference; it differentiates das_calctransforms, transforms.c:1150-1360).
 * Given wbar = dJ/dw [nj][ni][m] (and optionally Tbar = dJ/dT
 * [nj][ni][m_dyn][m], NULL if J does not depend on T) for the transforms of
 * the current inputs, computes, in FP64 (p->precision ENKFG_PREC_FP64) or
 * in FP32 arithmetic with FP64 accumulators (ENKFG_PREC_MIXED, the
 * production form),
 *   dJ_dinnovation [nobs]  dJ/d(y - Hx) per observation,
 *   dJ_dvariance   [nobs]  dJ/d(estd^2) per observation,
 *   dJ_dradius     [1]     dJ/d(rho), rho a common scale of all LOCRAD
 *                          values (dJ/dr = dJ/drho / r for one radius).
 * Each point's eigendecomposition is recomputed; the T term uses the
 * Daleckii-Krein form.  nmem <= 96. */
ENKFG_API enkfg_status enkfg_adjoint_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, const double* wbar, const double* Tbar, double* dJ_dinnovation, double* dJ_dvariance, double* dJ_dradius);

/* Adjoint of the analysis-mean update of one field-layer (update.c:380-410)
 * and of the stride interpolation of w (update.c:195-272): field [nmem]
 * [mnj][mni] is the forecast ensemble, dJ_dmean [mnj][mni] the gradient with
 * respect to the analysis mean (0 on masked cells); wbar [nj][ni][m]
 * receives dJ/dw at the strided points. */
ENKFG_API enkfg_status enkfg_adjoint_mean(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* field, const double* dJ_dmean, double* wbar);

/* The chunk sizes (observations per contraction step) the autotuner chose
 * per local-obs count bin (bin b holds counts in [2^b - 1, 2^(b+1) - 1));
 * table[16].  Returns ENKFG_ESTATE before the first tuned batched call. */
ENKFG_API enkfg_status enkfg_autotune_table(const enkfg_ctx* ctx, int* table);
/* Forget the tuned table (the next tuned batched call tunes again). */
ENKFG_API enkfg_status enkfg_autotune_reset(enkfg_ctx* ctx);

/* Number of kernels this context has launched (for launch accounting). */
ENKFG_API long long enkfg_kernel_launches(const enkfg_ctx* ctx);
/* Last stage timings in milliseconds, measured with CUDA events on the
 * launching stream: [0] index build, [1] count/queue, [2] transforms,
 * [3] update.  Read after the stream has finished the work (the _dev entry
 * points return before it ends); stages run inside a CUDA graph keep the
 * values of their last eager run. */
ENKFG_API enkfg_status enkfg_stage_times(const enkfg_ctx* ctx, float* ms4);
/* The last transform stage split in milliseconds (CUDA events on the
 * launching stream, summed over the stage's batches): [0] the transform
 * kernels (local observations, S'S and S's), [1] the solve kernels after
 * them (the batched eigensolver, refined solve or inverse).  No reference
 * counterpart: it refines stage [2] of enkfg_stage_times. */
ENKFG_API enkfg_status enkfg_kernel_times(const enkfg_ctx* ctx, float* ms2);

/* No counterpart in the reference.  CSR offsets of local-observation
 * counts (offsets[k] = counts[0] + ... + counts[k-1], offsets[n] = total; the
 * same offsets enkfg_local_obs returns) for callers that cannot allocate
 * device memory: code whose device memory is owned by a pool or another
 * framework, hosts that forbid allocation after start-up, or callers that
 * must avoid the implicit synchronisation of cudaMalloc/cudaFree.  It needs
 * no context and allocates nothing: counts_dev [n] and offsets_dev [n+1] are
 * the caller's device buffers, and the scan's block sums live in a fixed
 * 512 KiB array inside the library that every GPU using the library keeps
 * until the process exits.  Limit: n <= 134,217,728 (32768 scan blocks of
 * 4096 counts), else ENKFG_ECAPACITY.  Outside stream capture each call
 * looks up the array's device address in the current CUDA context
 * (cudaGetSymbolAddress; a lookup, no allocation) and records it for that
 * context; a call made while `stream` is being captured uses the recorded
 * address, so the first call in a context, and the first after a device
 * reset, must come before any capture (else ENKFG_ESTATE).  All calls share the
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  counts_dev may be NULL when n = 0.  Work is queued on `stream`
 * (NULL: the legacy default stream). */
ENKFG_API enkfg_status enkfg_local_offsets_noalloc(const int* counts_dev, long long n, long long* offsets_dev, void* stream);

/* ---- NetCDF classic files around the path (the reference reads and writes
 * them through NetCDF-C: common/ncw.c, common/ncutils.c) ----
 * Host only: these calls need no context and no GPU.  Formats: CDF-1,
 * CDF-2 (64-bit offset) and CDF-5 (64-bit data) are read; files are written
 * as CDF-2, or CDF-5 when a variable exceeds 4 GiB.  NetCDF-4 (HDF5) files
 * are not handled.  Errors: enkfg_nc_last_error() (per thread). */
#define ENKFG_NC_MAXDIMS 8
ENKFG_API const char* enkfg_nc_last_error(void);

/* transforms.nc as nc_createtransforms / nc_writetransforms write it
 * (calc/transforms.c:54-131): dimensions j, i, m_dyn, m; float T
 * [j][i][m_dyn][m] and w [j][i][m]; global attributes stride (int) and
 * grid_name (text).  T NULL (EnOI): no m_dyn and no T. */
ENKFG_API enkfg_status enkfg_nc_write_transforms(const char* path, int nj, int ni, int nmem_dynamic, int nmem, const float* T, const float* w, int stride, const char* grid_name);

/* The same file row by row, as the reference fills it: nc_createtransforms
 * (calc/transforms.c:54-94) makes the file with its variables' space
 * reserved; nc_writetransforms (calc/transforms.c:98-131) writes strided row
 * j: Tj [ni][m_dyn][m] (NULL for a file without T) and wj [ni][m]. */
ENKFG_API enkfg_status enkfg_nc_create_transforms(const char* path, int nj, int ni, int nmem_dynamic, int nmem, int with_T, int stride, const char* grid_name);
ENKFG_API enkfg_status enkfg_nc_write_transforms_row(const char* path, int j, const float* Tj, const float* wj);

/* enkf_diag.nc (calc/transforms.c:380-470): dimensions nobstypes, j, i; int
 * nlobs [j][i], float dfs and srf [j][i], int pnlobs and float pdfs, psrf
 * [nobstypes][j][i] with the reference's long_name / comment attributes;
 * global attributes stride and, per observation type, <name> = its index. */
ENKFG_API enkfg_status enkfg_nc_write_diag(const char* path, int nj, int ni, int ntypes, const char* const* type_names, int stride, const int* nlobs, const float* dfs, const float* srf, const int* pnlobs, const float* pdfs, const float* psrf);

/* Shape of a variable: ndims, dims [ENKFG_NC_MAXDIMS] (the record dimension
 * at its current length), its NetCDF type code, and whether the first
 * dimension is the record dimension.  Any output may be NULL. */
ENKFG_API enkfg_status enkfg_nc_inq_var(const char* path, const char* var, int* ndims, long long* dims, int* type, int* has_record);

/* A hyperslab [start, start + count) of a numeric variable as float (the
 * native type converted as nc_get_vara_float does; doubles beyond the float
 * range read as NaN, ncw_get_vara_float_fixerange, common/ncw.c:1078), no
 * attributes applied. */
ENKFG_API enkfg_status enkfg_nc_get_vara_float(const char* path, const char* var, const long long* start, const long long* count, float* out);

/* ncu_readfield (common/ncutils.c:102-530) on a structured grid: layer k of
 * record r (r < 0: the only record) of `var` laid out [r][k][j][i],
 * [k][j][i], [r][j][i] or [j][i], into v [nj][ni]; fill values (_FillValue
 * or the type's default), missing_value and values outside valid_min /
 * valid_max / valid_range become NaN, then scale_factor and add_offset are
 * applied in float. */
ENKFG_API enkfg_status enkfg_nc_read_layer(const char* path, const char* var, int r, int k, int ni, int nj, int nk, float* v);

/* ncu_read3dfield (common/ncutils.c:923-1245) on a structured grid: the
 * whole field of record r (r < 0: the only record) of `var` laid out
 * [r][k][j][i] or [k][j][i], into v [nk][nj][ni]; the value rules of
 * enkfg_nc_read_layer, except that values are masked only when one of
 * _FillValue, missing_value, valid_min, valid_max or valid_range is present,
 * and a double beyond the float range is an error. */
ENKFG_API enkfg_status enkfg_nc_read_field3d(const char* path, const char* var, int r, int ni, int nj, int nk, float* v);

/* ncu_writefield (common/ncutils.c:537-700) on a structured grid, into an
 * existing file: layer k (or the last record) of a numeric variable;
 * add_offset and scale_factor undone, values clamped to the valid range, NaN
 * written as the fill value (or missing_value), then stored in the
 * variable's type (integers by truncation toward zero, as NetCDF's put
 * conversion; a value outside the type's range is ENKFG_EINVAL). */
ENKFG_API enkfg_status enkfg_nc_write_layer(const char* path, const char* var, int k, int ni, int nj, int nk, const float* v);

#ifdef __cplusplus
}
#endif
#endif
