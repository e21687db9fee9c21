/*
 * libdymgpu -- C ABI of the GB300 discrete-group Symanzik Metropolis engine.
 *
 * The reference (hlammiv/dym_symanzik_action) has no library API: its hot path
 * is the `dym-mod-metro` process, whose C-linkage internals are the globals
 * and functions of group.h:8-16 and lattice.h:7-16, driven by update() and the
 * measurement block of dym-mod-metro.cpp:146-337.  Each entry point below
 * names the reference piece it replaces.
 *
 * Conventions
 *   - Every function returns an int status: DYM_OK (0) or a negative DYM_E*.
 *     The library never aborts or exits; dym_last_error() gives the message.
 *   - Opaque handles are created and freed by the library.  Host buffers
 *     belong to the caller.  No torch or CUDA types cross this boundary.
 *   - A chain owns one CUDA stream; calls on one chain are serialised by the
 *     caller.  Entry points that return results synchronise that stream.
 *   - Link layout of host buffers: uint16 element ids, direction-major,
 *     links[d*V + site], site = t + Nt*(x1 + Nx*(x2 + ...)) (lattice.c
 *     getidx, lattice.c:119-125 of the reference).
 */
#ifndef DYMGPU_H
#define DYMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DYM_OK 0
#define DYM_EINVAL -1     /* bad argument */
#define DYM_EIO -2        /* file cannot be opened or read */
#define DYM_EFORMAT -3    /* group file malformed: truncated, out of range, no identity/inverse */
#define DYM_ENOMEM -4     /* host or device allocation failed */
#define DYM_ECUDA -5      /* CUDA runtime error (no device, launch failure) */
#define DYM_ENOTSUP -6    /* combination not supported (e.g. D out of range) */
#define DYM_ETIMEDOUT -7  /* reserved for a bounded device wait that expired; no kernel of this
                                  library waits on another, so no entry point returns it */
#define DYM_ERANGE -8     /* size limit exceeded (group order > DYM_PMAX, ...) */

/* Largest group order accepted; same limit as the reference's PMAX (group.h:4). */
#define DYM_PMAX 5040

#define DYM_START_HOT 0   /* every link a uniform random element (dym-mod-metro.cpp:255) */
#define DYM_START_COLD 1  /* every link the identity */

#define DYM_POOL_NEAREST 0 /* elements of the 2nd-smallest ReTr (dym-mod-metro.cpp:239-245) */
#define DYM_POOL_ALL 1     /* uniform over the whole group */

#define DYM_PREC_FP64 0    /* every accept test in FP64, as the reference */
#define DYM_PREC_MIXED 1   /* dS from exact int32 sums of fixed-point class values,
                              scaled and tested against -log(u2) in FP32; FP64
                              re-evaluation within a proven bound of the threshold.
                              Decisions identical to DYM_PREC_FP64 (four dimensions,
                              tables with <= 32 ReTr classes whose packed sub-table
                              fits shared memory: 16-bit entries for P <= 2048,
                              32-bit above; else as DYM_PREC_SHARED) */
#define DYM_PREC_SHARED 2  /* FP64 decisions, hit loop served from the shared
                              sub-table (four dimensions, class-constant tables) */

typedef struct dym_group dym_group;
typedef struct dym_chain dym_chain;

/* Message of the last failed call on this thread ("" if none). */
const char* dym_last_error(void);
/* Library version string. */
const char* dym_version(void);

/* ---------------------------------------------------------------- group --- */

/* Parse a group file (format of groups/README.md:7-21; replaces load_group,
 * group.c:13-81).  Finds the identity and inverses as the reference does;
 * returns DYM_EFORMAT where the reference would abort, DYM_ERANGE for P >
 * DYM_PMAX, DYM_EIO if the file cannot be read.  Trailing tokens are ignored. */
int dym_group_load(const char* path, dym_group** out);
int dym_group_free(dym_group* g);

typedef struct {
  uint32_t order;          /* P */
  uint32_t identity;       /* id */
  uint32_t pool_nearest;   /* size of the nearest-to-identity proposal pool */
  double min_retr;         /* reference min_retr (dym-mod-metro.cpp:239-241) */
  double nn_retr;          /* reference nn_retr (dym-mod-metro.cpp:242) */
  int32_t n_classes;       /* distinct ReTr values (tolerance 1e-9) */
  int32_t classes_exact;   /* 1 if each ReTr value class is one bit pattern */
  int32_t fast_path;       /* 1 if the shared-memory sub-table path applies */
  double class_spread;     /* largest ReTr deviation inside a class */
} dym_group_info;

int dym_group_get_info(const dym_group* g, dym_group_info* out);
/* Copy the tables out (any pointer may be NULL): mult[P*P] row-major,
 * inv[P], retr[P], imtr[P], pool[pool_nearest]. */
int dym_group_get_tables(const dym_group* g, int32_t* mult, int32_t* inv,
                         double* retr, double* imtr, int32_t* pool);

/* ---------------------------------------------------------------- chain --- */

typedef struct {
  int32_t D, Nt, Nx;             /* lattice.h:7 (D, Nt, Nx); V = Nt*Nx^(D-1) */
  double beta0, beta1, beta2;    /* lattice.h:8 */
  uint64_t seed;                 /* Philox key (reference: per-site minstd seeds) */
  int32_t start;                 /* DYM_START_HOT / DYM_START_COLD */
  int32_t pool;                  /* DYM_POOL_NEAREST / DYM_POOL_ALL */
  int32_t precision;             /* DYM_PREC_FP64 / DYM_PREC_MIXED / DYM_PREC_SHARED */
  int32_t device;                /* CUDA device ordinal */
} dym_chain_params;

/* Create a chain on the device with its start configuration (replaces
 * dym-mod-metro.cpp:221-268: V, rnd[], hot/cold start, parity table). */
int dym_chain_create(const dym_group* g, const dym_chain_params* p, dym_chain** out);
int dym_chain_free(dym_chain* c);
/* Change the couplings of an existing chain (beta scans). */
int dym_chain_set_beta(dym_chain* c, double beta0, double beta1, double beta2);

/* Pin the group's Cayley table in L2 for this chain's kernels (on != 0), or
 * stop (on == 0).  Sets an access-policy window over the table on the chain's
 * stream (hits persisting, misses streaming) and raises the device's
 * persisting-L2 set-aside to the window size while any chain of the process
 * holds a window; the previous set-aside is restored when the last one stops
 * or is freed.  Opt-in: no gain was measured with it, even beside a lattice
 * (96^3 x 24, 170 MB of links) larger than L2: sweeps took the same time
 * with and without the window.  Configurations do not depend on it.  DYM_ENOTSUP when the device has
 * no persisting L2.  (No reference counterpart: group.c keeps the table in
 * host memory.) */
int dym_chain_set_l2_window(dym_chain* c, int32_t on);

/* Checkpoint / resume (no reference counterpart for dym-mod-metro, which
 * keeps no state between runs; llr2d.cpp:262-271 saves raw int32 links).  A
 * checkpoint holds the links and everything else that, with the group table,
 * fixes the rest of the run: shape, proposal pool, seed, sweeps done and
 * couplings.  Hits draw from Philox keyed by (seed, sweep, link, hit), so a
 * chain loaded from a checkpoint continues bit for bit as the chain that
 * wrote it, in any precision mode.  File layout: csrc/checkpoint.cpp. */
typedef struct {
  int32_t D, Nt, Nx;
  uint32_t order;        /* P of the group whose ids the links hold */
  int32_t pool;          /* DYM_POOL_* */
  uint64_t table_hash;   /* FNV-1a 64 of the Cayley table, row-major uint16 little-endian */
  uint64_t seed;
  uint32_t sweep;        /* sweeps done: the key component of the next sweep */
  double beta0, beta1, beta2;
} dym_checkpoint_info;

/* Write the chain's checkpoint to `path` (through `path`.tmp, renamed over
 * it, so an interrupted save keeps the previous file).  DYM_EIO on a file
 * error. */
int dym_chain_checkpoint_save(dym_chain* c, const char* path);
/* Load a checkpoint into a chain of the same shape, pool and group table
 * (else DYM_EINVAL, chain unchanged): links (ids checked on the device as
 * dym_links_set), seed, sweeps done and couplings.  DYM_EFORMAT for a file
 * that is not a valid checkpoint (magic, version, size, link checksum),
 * DYM_EIO when it cannot be read. */
int dym_chain_checkpoint_load(dym_chain* c, const char* path);
/* Header of a checkpoint file (validated as by the load; host only, no
 * device needed). */
int dym_checkpoint_read_info(const char* path, dym_checkpoint_info* out);
/* FNV-1a 64 of the group's Cayley table, as stored in checkpoints. */
int dym_group_table_hash(const dym_group* g, uint64_t* out);

typedef struct {
  uint64_t hits;        /* Metropolis hits (reference `hit`) */
  uint64_t accepts;     /* accepted hits (reference `acc`) */
  uint64_t rechecks;    /* mixed precision: hits re-evaluated in FP64 */
  double max_ds_err;    /* mixed precision: max |dS_fp32 - dS_fp64| seen on rechecks */
  uint32_t sweep;       /* sweeps done by the chain so far */
  uint32_t launches;    /* sweep kernels launched by this call */
  float device_ms;      /* device time of those launches (CUDA events on the chain's stream) */
  int32_t kernel;       /* sweep kernel of this call: DYM_KERNEL_* (batches: 0) */
} dym_stats;

#define DYM_KERNEL_DIRECT 1   /* FP64, table gathers for every hit (DYM_PREC_FP64) */
#define DYM_KERNEL_SHARED 2   /* FP64, hits from the shared sub-table (DYM_PREC_SHARED) */
#define DYM_KERNEL_MIXED 3    /* DYM_PREC_MIXED, shared (element | class) table */
#define DYM_KERNEL_MIXED_VALUES 4  /* DYM_PREC_MIXED, shared table of fixed-point values: chosen for a
                                      call when the chain's previous call accepted under 1% of its hits
                                      (accepted moves then fetch their elements from the Cayley table) */

/* nsweeps full sweeps with nhit hits per link (replaces update(),
 * dym-mod-metro.cpp:146-197, called nsweeps times).  Counters in `out`
 * (may be NULL) are for this call only. */
int dym_sweep(dym_chain* c, int32_t nsweeps, int32_t nhit, dym_stats* out);

typedef struct {
  int32_t wl_nx;   /* Wilson grid spatial extent 1..wl_nx (0: Nx, as the reference) */
  int32_t wl_nt;   /* temporal extent 1..wl_nt (0: Nt) */
} dym_meas_opts;

typedef struct {
  double poly_re, poly_im;   /* getpoly (lattice.c:179-194) */
  double plaq;               /* mean plaquette ReTr (dym-mod-metro.cpp:285-291) */
  double rect;               /* mean rectangle ReTr (dym-mod-metro.cpp:297-303) */
  int32_t wl_nx, wl_nt;      /* grid actually measured */
} dym_obs;

/* Observables of the current configuration (dym-mod-metro.cpp:282-318).
 * wloop (may be NULL) receives wl_nx*wl_nt doubles, spatial extent outer:
 * wloop[k*wl_nt + l] for a (k+1) x (l+1) loop.  Sums are exact integer
 * histograms over group elements followed by one FP64 dot product. */
int dym_measure(dym_chain* c, const dym_meas_opts* opts, dym_obs* out, double* wloop);

/* Same observables as dym_measure, with no memory allocation (no reference
 * counterpart: the reference measures on the host).  For callers that must not
 * allocate while they run, e.g. a server whose device-memory budget is all
 * given to resident chains, or a caller whose other streams cudaMalloc and
 * cudaFree would stall by synchronising the device.  dym_measure allocates
 * per-chain histogram buffers (device and pinned host) on first use; this call
 * uses instead one fixed device array of DYM_NOALLOC_HIST_BINS 64-bit bins
 * (1 MiB) plus room for DYM_NOALLOC_MAX_LOOPS Wilson loops, built into the
 * library's device code, walks Wilson loops link by link instead of building
 * lattice-sized line-product tables, takes the dot products on the device and
 * copies only the results, into *out and wloop.  Results are identical to
 * dym_measure's, bit for bit (the same exact histograms, and the same
 * correctly rounded multiplies, adds and division in the same order).
 * Cost: a walked (k+1) x (l+1) loop takes 2(k+l+2) table products against
 * dym_measure's 3 (line products), so a Wilson grid costs about (k+l)/1.5
 * times dym_measure's Wilson-loop work (8x8 grid: up to ~11x).
 * Limits: (3 + wl_nx*wl_nt) * P <= DYM_NOALLOC_HIST_BINS and
 * wl_nx*wl_nt <= DYM_NOALLOC_MAX_LOOPS (S(1080): up to 118 loops, e.g. the 8x8
 * grid); larger requests return DYM_ERANGE before any device work.
 * The array is per device and shared by all chains on it; every call clears
 * the bins it uses (they must start at zero), so calls whose device work
 * overlaps -- from several host threads, or on chains of one device -- race
 * and must be serialised by the caller.  The first call on each device looks
 * up the array's device address (which may load the library's device code).
 * The call synchronises the chain's stream and copies into pageable host
 * memory, so it must not be made while any stream of the device is being
 * captured into a CUDA graph.  On success nothing is allocated, host or
 * device; an error records its message as every call. */
#define DYM_NOALLOC_HIST_BINS 131072
#define DYM_NOALLOC_MAX_LOOPS 1024
int dym_measure_noalloc(dym_chain* c, const dym_meas_opts* opts, dym_obs* out, double* wloop);

/* Host <-> device copies of the configuration (layout in the header comment). */
int dym_links_get(dym_chain* c, uint16_t* host_out);
int dym_links_set(dym_chain* c, const uint16_t* host_in);

/* nsweeps sweeps of a configuration held in host memory, in one call: the
 * drop-in for the reference's update() (dym-mod-metro.cpp:146-197) applied to
 * its host-resident link array `a` (malloc at dym-mod-metro.cpp:253).
 * host_in (may be NULL: keep the chain's configuration) is uploaded and
 * checked as by dym_links_set, the sweeps run as by dym_sweep, and the
 * result is written into host_out (may be NULL; may equal host_in), with one
 * synchronisation at the end instead of one per step.  Page-locked host
 * buffers are read by the checking kernel directly, and a page-locked
 * host_out is written by the final sweep itself (every link as it is
 * visited), so no copy of the configuration follows the sweeps; other
 * buffers go through copies.  A host_in with an id >=
 * the group order returns DYM_EINVAL with the chain unchanged (the sweeps do
 * nothing, the chain's sweep counter is not advanced) and host_out, if
 * given, holding the chain's unchanged configuration. */
int dym_sweep_host(dym_chain* c, const uint16_t* host_in, uint16_t* host_out, int32_t nsweeps, int32_t nhit,
                   dym_stats* out);

/* nsweeps sweeps applied in place to an array in the reference's own layout:
 * a[i*D + d] holds the element id (int32, group_t of group.h:6) of link
 * (site i, direction d), site i = getidx(pos) (lattice.c), the array that
 * update() (dym-mod-metro.cpp:146-197) reads and writes, malloc'd at
 * dym-mod-metro.cpp:253.  So the reference's `for (k < K) update();` becomes
 * one call on its own array.  The array is uploaded and checked (every id in
 * [0, P)), the sweeps run, and the result is written back into it.  A
 * page-locked array (cudaHostAlloc / cudaHostRegister) is read and written by
 * the kernels through its device mapping; any other is copied through a
 * device array of V*D int32 (allocated on first use, kept with the chain).
 * An id outside [0, P) returns DYM_EINVAL with the chain, its sweep counter
 * and `a` unchanged. */
int dym_sweep_refarray(dym_chain* c, int32_t* a, int32_t nsweeps, int32_t nhit, dym_stats* out);

/* Lattice and schedule facts: V, number of colour phases per sweep, and the
 * phase layout (arrays may be NULL; sizes nphase, nphase, V*D). */
int dym_chain_get_schedule(const dym_chain* c, uint32_t* V, int32_t* nphase,
                           int32_t* phase_dir, uint32_t* phase_len, uint32_t* sites);

/* Staple elements of links (site[k], dir) built on the device: out[k*ns + j],
 * ns = 8*(D-1): the 2(D-1) plaquette staples (get_staples,
 * dym-mod-metro.cpp:63-78) then the 6(D-1) rectangle staples (get_rect_loops,
 * dym-mod-metro.cpp:83-142), in the reference's order. */
int dym_chain_staples(dym_chain* c, int32_t dir, const uint32_t* sites, int32_t n, uint16_t* out);

/* Same-phase read conflicts of a lattice shape's schedule (0 = race-free);
 * host-only, no device needed. */
int dym_schedule_check(int32_t D, int32_t Nt, int32_t Nx, int32_t* nphase, uint64_t* conflicts);
/* The colour schedule of a lattice shape without a device: call once with
 * NULL arrays to get V and nphase, then with arrays of nphase, nphase and V*D
 * entries.  Phases are ordered by direction (as the reference's d-major loop,
 * dym-mod-metro.cpp:152-153), sites ascending inside a phase. */
int dym_schedule_get(int32_t D, int32_t Nt, int32_t Nx, uint32_t* V, int32_t* nphase, int32_t* phase_dir,
                     uint32_t* phase_len, uint32_t* sites);

/* ----------------------------------------------------------------- batch --- */

/* An ensemble of independent chains updated together (no reference
 * counterpart: the reference runs one process per chain, evermore.sh and
 * jobs2run).  One kernel per colour-phase slot updates the slot's phase of
 * every chain; each chain's configurations are bit-identical to running it
 * alone with dym_sweep.  Chains stay owned by the caller and must outlive
 * the batch; they must share D and the device, use DYM_POOL_NEAREST and
 * DYM_PREC_MIXED or DYM_PREC_SHARED with a table eligible for the shared-table path
 * (dym_group_info.fast_path), at most 4 distinct groups. */
typedef struct dym_batch dym_batch;

typedef struct {
  int32_t tile;         /* links per work tile (multiple of 32) */
  int32_t threads;      /* threads per block (128, 256; 512 when every chain is DYM_PREC_MIXED) */
  int32_t grid_per_sm;  /* blocks launched per SM per slot (>= 1) */
  int32_t use_graph;    /* 1: replay each sweep as a captured CUDA graph */
  int32_t hit_unroll;   /* mixed-precision batches: hits whose random draws are computed ahead as a group
                           (1, 2, 5 or 10; 0 means 1); configurations do not depend on it */
} dym_batch_tuning;

int dym_batch_create(int32_t device, dym_batch** out);
int dym_batch_add(dym_batch* b, dym_chain* c);
int dym_batch_size(const dym_batch* b, int32_t* nchains, uint64_t* nlinks, int32_t* nslots);
int dym_batch_set_tuning(dym_batch* b, const dym_batch_tuning* t);
int dym_batch_get_tuning(const dym_batch* b, dym_batch_tuning* t);
/* nsweeps sweeps of every chain (nhit hits per link); totals in `total`. */
int dym_batch_sweep(dym_batch* b, int32_t nsweeps, int32_t nhit, dym_stats* total);
/* Counters of chain `idx` (order of dym_batch_add) for the last dym_batch_sweep. */
int dym_batch_chain_counters(const dym_batch* b, int32_t idx, uint64_t* hits, uint64_t* accepts);
/* Time candidate tunings on the batch's own chains (their configurations,
 * sweep counters and counters are restored afterwards) and keep the fastest:
 * tile 128..1024, threads 128/256/512, 1 or 2 blocks per SM, hit_unroll 1 or
 * 2 (the last two choices for mixed-precision batches only). */
int dym_batch_autotune(dym_batch* b, int32_t nhit, int32_t nsweeps_per_trial, dym_batch_tuning* best);
int dym_batch_free(dym_batch* b);

/* ------------------------------------------------------------------- LLR --- */

#define DYM_LLR_MAX_NRM 1024

#define DYM_LLR_DRIVE 0      /* energy outside the window, greedy drive-in */
#define DYM_LLR_SETTLE 1     /* entered the window during the current sweep */
#define DYM_LLR_RM 2         /* Robbins-Monro iterations */
#define DYM_LLR_DONE 3       /* all NRM iterations done */
#define DYM_LLR_UNREACHED 4  /* drive-in cap reached outside the window */
#define DYM_LLR_CANCELLED 5  /* server only: withdrawn by dym_server_cancel */
#define DYM_LLR_REJECTED 6   /* server only: the request's window or parameters are invalid, or its
                                chain could not be created with no other chain resident */

typedef struct {
  int32_t axis;      /* 1: window on S1 (plaquettes), background bg on S2; 2: the reverse (llr.cpp:42-43, 286) */
  double bg;         /* fixed background coupling BG (llr.cpp:43, 287) */
  double ewin;       /* window centre */
  double hw;         /* half-width: window [ewin-hw, ewin+hw], W = 2 hw (llr.cpp:236) */
  double a0;         /* initial a (also the drive-in tilt, seed_window's a_guess, llr.cpp:223) */
  int32_t K;         /* sweeps per Robbins-Monro iteration (llr.cpp:294, default 50) */
  int32_t NRM;       /* Robbins-Monro iterations (llr.cpp:295, default 80), <= DYM_LLR_MAX_NRM;
                        0: drive into the window only (seed_window) */
  int32_t nhit;      /* hits per link per visit (llr.cpp:32, NHIT 20) */
  int32_t drive_cap; /* max drive-in sweeps (llr.cpp:225, CAP 20000) */
} dym_llr_req;

typedef struct {
  double a;            /* final a_n */
  double S1, S2;       /* energies at the end (exact 2^-32 fixed-point class sums) */
  int32_t status;      /* DYM_LLR_DONE or DYM_LLR_UNREACHED */
  int32_t drive_sweeps;
  int32_t sweeps;      /* sweeps run by this call */
  uint64_t hits, accepts;
  uint64_t phase_accepts, phase_rejects;  /* changed links kept / reverted by the window scan */
} dym_llr_result;

/* Exact S1 = sum over plaquettes of ReTr and S2 = sum over 1x2 rectangles of
 * ReTr of the current configuration (recompute_S1, recompute_S2 with
 * RECT_MULT = 6: llr.cpp:46-55, 139-151). */
int dym_llr_energy(dym_chain* c, double* S1, double* S2);

/* One LLR window on the device: drive the windowed energy into
 * [ewin-hw, ewin+hw] (seed_window, llr.cpp:223-231), then NRM Robbins-Monro
 * iterations of K constrained sweeps, a += 12/(W^2 (m+1)) (<E> - ewin)
 * (rm_solve, llr.cpp:234-250).  Sweeps are colour-parallel: every link of a
 * colour class does nhit Metropolis hits of weight exp(-a dE_w - bg dE_bg)
 * (llr.cpp:208-212), then the class's changed links are scanned in site-list
 * order and a link's move is kept iff the running windowed energy stays in
 * the window, else reverted (outside the window: kept iff it moves the energy
 * towards the centre) -- the reference's per-hit window test at the
 * granularity of one link's hits.  a_hist (may be NULL) receives a after each
 * of the NRM iterations. */
int dym_llr_run(dym_chain* c, const dym_llr_req* req, dym_llr_result* out, double* a_hist);

/* Two-dimensional LLR cell (replaces update_constrained2d, seed_cell and
 * rm_solve2d, llr2d.cpp:178-259): both actions windowed, S1 in [E1-hw1, E1+hw1]
 * and S2 in [E2-hw2, E2+hw2], weight exp(-a1 dS1 - a2 dS2) inside the cell;
 * drive-in moves closer to the cell centre in normalised distance; two
 * Robbins-Monro recursions a_i += 12/(W_i^2 (m+1)) (<S_i> - E_i).  Same
 * colour-parallel rule as dym_llr_run.  Every extent must be >= 3. */
typedef struct {
  double E1, hw1;    /* S1 window */
  double E2, hw2;    /* S2 window */
  double a1, a2;     /* initial (a1, a2): drive-in tilt and Robbins-Monro start */
  int32_t K, NRM;    /* sweeps per iteration, iterations (<= DYM_LLR_MAX_NRM) */
  int32_t nhit, drive_cap;
} dym_llr2d_req;

typedef struct {
  double a1, a2;
  double S1, S2;
  int32_t status;    /* DYM_LLR_DONE or DYM_LLR_UNREACHED */
  int32_t drive_sweeps, sweeps;
  uint64_t hits, accepts;
  uint64_t phase_accepts, phase_rejects;
} dym_llr2d_result;

/* a_hist (may be NULL) receives 2*NRM doubles: (a1, a2) after each iteration. */
int dym_llr2d_run(dym_chain* c, const dym_llr2d_req* req, dym_llr2d_result* out, double* a_hist);

/* ---------------------------------------------------------------- server --- */

/* A request loop for LLR windows (no reference counterpart: the reference
 * runs one llr process per window range, scripts/llr2d_parallel.sh).  Requests
 * queue on submit; dym_server_step admits queued requests while the resident
 * chain count and the device-memory budget allow, runs nsweeps LLR sweeps of
 * every resident chain together (one kernel per colour-phase slot), and
 * retires finished chains, whose responses dym_server_poll returns.  A
 * request's result depends only on the request: it is the same alone or in
 * any mix.  Chains of a finished request are reused for later requests of the
 * same shape. */
#define DYM_SERVE_MAX_NRM 64

typedef struct dym_server dym_server;

typedef struct {
  int32_t max_chains;   /* resident chains at most */
  uint64_t hbm_budget;  /* device bytes of resident chains at most */
  int32_t nhit;         /* hits per link per visit */
  int32_t device;
  uint64_t max_links;   /* links of resident chains at most (0: no limit).  All resident chains
                           advance together, so a smaller limit lets the oldest requests finish
                           sooner; a larger one keeps more work per kernel. */
} dym_server_params;

typedef struct {
  uint64_t id;
  int32_t D, Nt, Nx;
  int32_t start;        /* DYM_START_HOT / DYM_START_COLD */
  uint64_t seed;
  int32_t axis;
  double bg, ewin, hw, a0;
  int32_t K, NRM, drive_cap;  /* NRM <= DYM_SERVE_MAX_NRM */
} dym_llr_request;

typedef struct {
  uint64_t id;
  double a, S1, S2;
  int32_t status;       /* DYM_LLR_DONE, DYM_LLR_UNREACHED, DYM_LLR_CANCELLED or DYM_LLR_REJECTED */
  int32_t sweeps, drive_sweeps, NRM;
  uint64_t hits, accepts;
  double a_hist[DYM_SERVE_MAX_NRM];
} dym_llr_response;

int dym_server_create(const dym_group* g, const dym_server_params* p, dym_server** out);
/* Queue a request.  DYM_ERANGE when its chain alone needs more device memory
 * than the server's budget; DYM_EINVAL for a malformed shape or NRM.  Every
 * accepted request gets exactly one response. */
int dym_server_submit(dym_server* s, const dym_llr_request* r);
/* Withdraw a queued or resident request: its response (status
 * DYM_LLR_CANCELLED, with the state reached so far for a resident one) is
 * queued for dym_server_poll at once and its chain and budget are freed.
 * DYM_EINVAL when no queued or resident request has this id. */
int dym_server_cancel(dym_server* s, uint64_t id);
int dym_server_step(dym_server* s, int32_t nsweeps);
/* Up to `max` finished responses (in completion order); *n receives the count. */
int dym_server_poll(dym_server* s, dym_llr_response* out, int32_t max, int32_t* n);
int dym_server_status(const dym_server* s, int32_t* active, int32_t* queued, uint64_t* hbm_used,
                      uint64_t* link_hits);
int dym_server_free(dym_server* s);

/* Roofline probe (no reference counterpart): random 2-byte gathers from an
 * L2-resident table of table_bytes bytes on `device`, as the sweep kernels
 * issue them; returns the sustained gather rate in 32-byte sectors per second
 * (one gather touches one sector). */
int dym_probe_l2_gather(int32_t device, uint32_t table_bytes, double* sectors_per_s);

#ifdef __cplusplus
}
#endif
#endif /* DYMGPU_H */
