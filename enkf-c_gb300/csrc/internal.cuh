// internal.cuh -- shared definitions of libenkfg (GB300 EnKF-C hot path).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include "../../include/enkfg.h"

#define ENKFG_VERSION 1

struct CalcArgs;

// default bound on a device wait (mixed path: waits for the tensor cores)
#define ENKFG_DEFAULT_WAIT_NS 2000000000ull
// per-point status a transform kernel records when a bounded wait expired
#define ENKFG_POINT_TIMEOUT 99

// ---------------------------------------------------------------------------
// Per-type spatial index description (device copy lives in ctx->d_types).
// The observations of one type are bucketed on a uniform grid of cells of
// edge >= the type's maximum localisation radius; buckets are numbered in
// Morton (Z) order of their cell coordinates, so a query point visits the
// 3x3 (2-D) or 3x3x3 (3-D) cells around it.
// ---------------------------------------------------------------------------
struct TypeIndex {
    double x0, y0, z0;          // origin of the cell grid
    double inv_cell;            // 1 / cell edge
    int ncx, ncy, ncz;          // cells per axis (ncz = 1 in 2-D)
    int mbits;                  // Morton bits per axis
    long long bucket_base;      // first bucket of this type in the global bucket array
    long long nbuckets;         // 2^(ndim*mbits)
    int pos_begin, pos_end;     // range of this type in the sorted obs arrays
    int nlocrad;
    double locrad[ENKFG_MAXLOCRAD];
    double locweight[ENKFG_MAXLOCRAD];
    double rmax;                // max(locrad)
    double rmax2;               // rmax * rmax (rounded as the reference rounds range*range)
    // FP32 copies for the mixed path's search and taper: radii, squared
    // radii, weights, and the band [rmax2_lo, rmax2_hi] around rmax2 inside
    // which the FP32 distance cannot decide membership (exact FP64 test)
    float locrad_f[ENKFG_MAXLOCRAD];
    float r2_f[ENKFG_MAXLOCRAD];      // r^2 as a double-float r2_f + r2_fl
    float r2_fl[ENKFG_MAXLOCRAD];
    float locweight_f[ENKFG_MAXLOCRAD];
    float rmax2_lo, rmax2_hi;
    // NLOBSMAX of the type (0: no limit): a point keeps its nlobsmax nearest
    // observations of the type, those at or before the point's cut key
    int nlobsmax;
};

// Cut of a point's local observations of one type under NLOBSMAX: an
// observation in range is kept when (d2, id) <= (d2, id) of the cut in
// lexicographic order, d2 the exact FP64 squared distance the search
// computes and id the observation's index.  {+inf, INT_MAX}: no cut.
struct CutKey {
    double d2;
    int id;
    int pad;
};

__host__ __device__ __forceinline__ bool cut_keeps(double d2, int id, const CutKey& c)
{
    return d2 < c.d2 || (d2 == c.d2 && id <= c.id);
}

struct enkfg_ctx {
    int device;
    cudaStream_t stream;        // stream all work goes to
    cudaStream_t own_stream;    // the context's own stream while a caller stream is bound
    cudaStream_t cstream[2];    // host-buffer update: copies in, copies out (created on first use)
    cudaEvent_t uev[9];         // host-buffer update: per buffer, copy-in / update / copy-out done
    int field_buffer;           // host-buffer update: field-layers per group (0: automatic)
    int field_rows;             // host-buffer update: model rows per block (0: automatic)
    int solve_batch;            // batched solves: points per batch (0: automatic)
    char err[1024];
    long long launches;
    unsigned long long wait_ns; // bound on a device wait (enkfg_set_wait_limit)
    int wait_drill;             // enkfg_set_wait_drill
    float stage_ms[4];
    cudaEvent_t ev[10];         // [8, 9]: the transform kernel alone (first batch)

    // observation types
    int ntypes;
    int geographic;
    int nlocrad[ENKFG_MAXTYPES];
    double locrad[ENKFG_MAXTYPES][ENKFG_MAXLOCRAD];
    double locweight[ENKFG_MAXTYPES][ENKFG_MAXLOCRAD];
    double rfactor[ENKFG_MAXTYPES];
    int nlobsmax[ENKFG_MAXTYPES];   // enkfg_set_obstype_nlobsmax (0: no limit)
    int hidden[ENKFG_MAXTYPES];     // enkfg_set_obstype_visible (1: hidden from the search)
    bool types_set;

    // observations (original order)
    int nobs;
    float* d_lon;
    float* d_lat;
    short* d_type;
    short* d_status;
    float* d_estd;
    float* d_value;
    double* d_rfac;             // [ntypes] scratch
    double* d_rfac_sqrt;        // [ntypes] sqrt(rfactor), uploaded with the obs types
    bool obs_set;

    // ensemble observations
    int nmem, nmem_dyn;
    float* d_S;                 // [nmem][nobs]
    double* d_s;                // [nobs]
    double* d_std;              // [nobs]
    int s_mode;                 // 0 none, 1 HE, 2 HA (innovations done), 3 S (standardised)

    // spatial index (rebuilt when obs or S change)
    bool index_valid;
    bool gather_valid;
    int nsorted;                // obs with status OK
    TypeIndex h_types[ENKFG_MAXTYPES];
    TypeIndex h_types_up[ENKFG_MAXTYPES];   // the copy uploaded (hidden types emptied)
    TypeIndex* d_types;
    long long nbuckets;
    long long* d_bstart;        // [nbuckets + 1]
    int* d_bfill;               // [nbuckets] scratch
    int* d_key;                 // [nobs] scratch
    int* d_sid;                 // [nsorted] obs id at sorted position
    float* d_sxf;               // [nsorted] FP32 copies of d_sx, d_sy (2-D only; exact for float inputs)
    float* d_syf;
    double* d_sx;               // [nsorted] kd coordinates in sorted order
    double* d_sy;
    double* d_sz;
    short* d_stype;             // [nsorted]
    int mpad;                   // member stride of d_St (multiple of 4)
    float* d_St;                // [nsorted][mpad] standardised S, sorted, member-contiguous
    double* d_ss;               // [nsorted] standardised innovation, sorted
    float* d_ssf;               // [nsorted] the same rounded to float (mixed path)
    // host outputs of the transform call being run, copied out batch by
    // batch when the queue segments match the batches (out_seg > 0)
    float* out_T;
    float* out_w;
    double* out_T64;
    double* out_w64;
    int out_seg;
    cudaEvent_t out_ev;
    float* d_gtmp;              // [nobs][mpad] transpose scratch of the gather
    unsigned int* d_smax;       // [ENKFG_MAXMEM] max |St| per member (float bits), mixed-path quantum
    float* d_qscale;            // [2][ENKFG_MAXMEM] per-member quantum q and 1/q (powers of two)
    // grow-only capacities: rebuilding the index or the gather keeps the
    // device addresses when the sizes do not grow (CUDA graphs captured on
    // the cycle keep pointing at valid buffers)
    size_t bstart_cap, bfill_cap, key_cap, sid_cap, sx_cap, sy_cap, sz_cap, sxf_cap, syf_cap, stype_cap;
    size_t St_cap, ss_cap, ssf_cap, gtmp_cap;
    // NLOBSMAX cuts of the current grid: [ntypes][nj*ni] (valid while
    // cut_valid; computed only when a type has a limit)
    CutKey* d_cut;
    size_t cut_cap;
    bool cut_valid;
    double* d_ox;               // [nobs] kd coordinates (original order)
    double* d_oy;
    double* d_oz;

    // grid
    bool grid_set;
    int mni, mnj, stride, periodic_i, ni, nj;
    double* d_qx;               // [nj*ni] query coordinates of the strided points
    double* d_qy;
    double* d_qz;

    // transforms (resident)
    int t_mode, t_nmem, t_ndyn;
    bool want64;                // the next calc also writes the FP64 T and w
    bool t_valid;
    float* d_T;                 // [nj*ni][ndyn][nmem]
    float* d_w;                 // [nj*ni][nmem]
    double* d_T64;
    double* d_w64;
    size_t T_cap, w_cap, T64_cap, w64_cap;
    int* d_nlobs;
    float* d_dfs;
    float* d_srf;
    int* d_pnlobs;
    float* d_pdfs;
    float* d_psrf;
    size_t nlobs_cap, dfs_cap, srf_cap, pnlobs_cap, pdfs_cap, psrf_cap;

    // batched ETKF eigensolver scratch (per slot of a batch of points)
    double* d_eq;               // [slots][m][m]
    double* d_ed;               // [slots][m]
    double* d_ee;               // [slots][m]
    double* d_eb;               // [slots][m]
    double* d_eaux;             // [slots][2]
    double* d_eval;             // [slots][m]
    double2* d_erot;            // [slots][rcap]
    int2* d_ehdr;               // [slots][hcap]
    int* d_enh;                 // [slots]
    size_t eq_cap, ed_cap, ee_cap, eb_cap, eaux_cap, eval_cap, erot_cap, ehdr_cap, enh_cap;

    // refined mixed-precision ETKF solve scratch (per slot; etkf_mixed.cu)
    float* d_emq;               // [slots][m][m]
    float2* d_emmhl;            // [slots][m][m]
    float* d_emd;               // [slots][m]
    float* d_eme;               // [slots][m]
    float2* d_emrot;            // [slots][rcap]
    int2* d_emhdr;              // [slots][hcap]
    int* d_emnh;                // [slots]
    float* d_emz0;              // [slots][MP][MP]
    float2* d_emp;              // [slots][MP][MP]
    size_t emq_cap, emmhl_cap, emd_cap, eme_cap, emrot_cap, emhdr_cap, emnh_cap, emz0_cap, emp_cap;
    // per-batch timing of the last transform stage: events before the
    // transform kernel, after it and after the batch's solve kernels
#define ENKFG_TIMED_BATCHES 256
    cudaEvent_t bev[3 * ENKFG_TIMED_BATCHES];
    int nbev;                   // events created so far
    int nbatch;                 // batches marked in the last transform stage

    // work queue / scratch
    int* d_counts;              // [npoints]
    int* d_order;               // [npoints]
    int* d_qhead;               // queue head + error flag
    int* d_status_pt;           // [npoints] per-point status
    bool kc_tuned;              // d_qhead[2+16 ..] holds an autotuned chunk-size table
    int kc_tuned_prec;          // precision the table was tuned for
    int kc_table[16];           // host copy of the tuned table
    int kc_loaded;              // table now on the device: 0 none, 1 FP64 default, 2 mixed default, 3 tuned
    void* d_scratch;
    size_t scratch_cap;
    size_t counts_cap, order_cap, status_cap;

    // update scratch
    int h_levels[448];          // levels last uploaded for the update (d_qhead + 64)
    int n_levels;               // their count (0: none)
    int* d_numlevels;
    size_t numlevels_cap;
    float* d_fields;
    size_t fields_cap;
    float* d_infl;
    size_t infl_cap;

    // RANDOMISE of the next update call (enkfg_set_field_noise): d_noise
    // holds [noise_nlayer] deflations, then [noise_nlayer][noise_nmem]
    // member terms; noise_nfield = noise_nlayer until an update call takes
    // the noise (0: none pending)
    int noise_nfield, noise_nmem, noise_nlayer;
    double* d_noise;
    size_t noise_cap;

    // forward-operator (HE) stage
    double* d_fi;               // [nobs] observation.fij[0]
    double* d_fj;               // [nobs] observation.fij[1]
    float* d_fk;                // [nobs] observation.fk (NULL until given)
    float* d_Hx;                // [nobs] EnOI background row
    unsigned long long* d_hflag;// [4] first bad forecast (obs << 32 | value bits), first position off the grid, BADFC count
    int* d_hids;
    size_t hids_cap;
    float* d_hsrc;              // host fields staged on the device
    size_t hsrc_cap;
    int* d_hlev;
    size_t hlev_cap;
    float* d_hoff;
    size_t hoff_cap;
    int he_nmem, he_nmem_dyn;   // ensemble of the open HE stage (0: none open)
    bool he_bg;                 // the open stage has a background row
    bool pos_set;               // observation positions uploaded
    bool pos_3d;                // with fk
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
void set_err(enkfg_ctx* c, const char* fmt, ...);
enkfg_status cuda_fail(enkfg_ctx* c, cudaError_t e, const char* what, int line);

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call, __LINE__); \
    } while (0)

#define CKL()                                                           \
    do {                                                                \
        ctx->launches++;                                                \
        cudaError_t e_ = cudaGetLastError();                            \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, "kernel launch", __LINE__); \
    } while (0)

#define NEED(cond, code, ...)                \
    do {                                     \
        if (!(cond)) {                       \
            set_err(ctx, __VA_ARGS__);       \
            return code;                     \
        }                                    \
    } while (0)

#define SETDEV() CK(cudaSetDevice(ctx->device))

template <typename T>
static inline enkfg_status ensure(enkfg_ctx* ctx, T** p, size_t* cap, size_t n)
{
    if (n == 0) n = 1;
    if (*p != nullptr && *cap >= n) return ENKFG_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_err(ctx, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
        return ENKFG_ENOMEM;
    }
    *cap = n;
    return ENKFG_OK;
}

static inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// exclusive scan of int counts into long long offsets (device), n entries;
// offsets[n] = total.  Uses ctx scratch.
enkfg_status scan_counts(enkfg_ctx* ctx, const int* d_in, long long* d_out, long long n, cudaStream_t st);

// stages implemented in the .cu files
enkfg_status build_index(enkfg_ctx* ctx, cudaStream_t st);
// the index (built if stale) and, when a type has an NLOBSMAX, the cuts of
// the current grid's points: what every local search needs first
enkfg_status prepare_search(enkfg_ctx* ctx, cudaStream_t st);
// device copy of the type table: types hidden by enkfg_set_obstype_visible
// get an empty position range, so that no search visits them
enkfg_status upload_types(enkfg_ctx* ctx, cudaStream_t st);
// true when some type has an NLOBSMAX (the cut table is in use)
bool any_nlobsmax(const enkfg_ctx* ctx);
enkfg_status build_gather(enkfg_ctx* ctx, cudaStream_t st);
enkfg_status count_local(enkfg_ctx* ctx, int* d_counts, int* d_pcounts, cudaStream_t st);
enkfg_status count_candidates(enkfg_ctx* ctx, int* d_counts, cudaStream_t st);
enkfg_status list_local(enkfg_ctx* ctx, const long long* d_offsets, int* d_ids, double* d_coeffs, cudaStream_t st);
enkfg_status run_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, cudaStream_t st);
// per-batch timing (calc.cu): k = 0 before a batch's transform kernel, 1
// after it, 2 after the batch's solve kernels
void batch_mark(enkfg_ctx* ctx, int k, cudaStream_t st);
// points per batch of a batched solve: budget / per-slot bytes (or the
// context's setting, enkfg_set_solve_batch), at least 256, a multiple of
// 1024 from 1024 on, at most nitems
size_t batch_points(const enkfg_ctx* ctx, size_t per_slot, size_t budget, int nitems);
size_t etkf_mixed_slot_bytes(int m);
// after the last kernel of the batch of queue items [i0, i0 + nb): the
// host outputs of those points (a contiguous range when the queue is
// sorted within batch-sized segments) start to copy out
void batch_out(enkfg_ctx* ctx, int i0, int nb, cudaStream_t st);
// the transform stage's FP32 eigendecomposition + refined solve for ETKF on
// the mixed path (etkf_mixed.cu); false if nmem is beyond its register tiles
bool etkf_mixed_supported(int m);
enkfg_status run_etkf_mixed(enkfg_ctx* ctx, const CalcArgs& a0, cudaStream_t st);
enkfg_status launch_mixed(enkfg_ctx* ctx, CalcArgs& a, cudaStream_t st);
// CTAs of `fn` (nt threads, dsmem bytes of dynamic shared memory) that fit on
// one SM at once, from the shared memory (with the per-block reserve),
// register and thread limits of the device; and the shared-memory carveout
// (percent of the maximum) that holds that many, so that the rest of the
// unified L1 / shared array stays L1.
enkfg_status resident_ctas(enkfg_ctx* ctx, const void* fn, int nt, size_t dsmem, int* per_sm, int* carveout);
enkfg_status run_update(enkfg_ctx* ctx, const enkfg_update_params* p, const int* d_numlevels, int nfield,
                        const int* levels, float* d_fields, float* d_infl, cudaStream_t st);
enkfg_status run_innovations(enkfg_ctx* ctx, cudaStream_t st);
// RANDOMISE on nf field-layers (layers f0.. of the set the noise was given
// for) at d_v: [nf][nmem] planes of ncell floats
enkfg_status run_noise(enkfg_ctx* ctx, float* d_v, int f0, int nf, int nmem, long long ncell, cudaStream_t st);
// (re)allocate S, s and std_f for nmem members of the current observations
extern "C" enkfg_status alloc_S(enkfg_ctx* ctx, int nmem, int nmem_dynamic);
enkfg_status run_standardise(enkfg_ctx* ctx, cudaStream_t st);
enkfg_status run_hybrid(enkfg_ctx* ctx, int nmem, int nmem_d, double gamma, int nij, float* d_v, cudaStream_t st);
