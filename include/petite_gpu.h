/*
 * petite_gpu.h -- C ABI of the GB300 electromagnetic-shower engine.
 *
 * PETITE (kjkellyphys/PETITE) is pure Python and has no FFI; these entry
 * points replace the Python functions named in each comment (paths are
 * inside PETITE's src/PETITE/).  The ctypes layer in petite_gb300/_lib.py
 * binds exactly these symbols.
 *
 * Conventions
 *  - Every pointer inside a struct below is a DEVICE pointer (cudaMalloc'd or
 *    a torch tensor's data_ptr()); the caller owns all memory and the library
 *    never frees it.  Handles own only a small device copy of the scalar
 *    table description.
 *  - Functions return a pt_status; no exception or C++ type crosses the ABI.
 *  - Work is enqueued on the given stream (0 = legacy default stream); calls
 *    that must report a count or an error synchronise that stream.
 *  - Handles are not thread-safe; use one per host thread.
 */
#ifndef PETITE_GPU_H
#define PETITE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pt_status {
  PT_OK = 0,
  PT_NO_SAMPLE = 1,   /* rejection sampler exhausted max_n_integrators*neval proposals
                         ("No Sample Found", shower.py:460-461) */
  PT_TIMEOUT = 2,     /* a bounded device loop or wait hit its limit; pt_last_error_info's process is
                         -1 for a loop bound (substep loop, waves of a run, the persistent kernel's
                         grid barrier) and -2 for a table-staging copy into shared memory that did
                         not land in time: that copy may still be in flight, so later results on
                         the device are suspect and the handle should be discarded */
  PT_BAD_TABLE = 3,   /* inconsistent table description */
  PT_OOM = 4,         /* output/queue capacity too small: retry with more rows */
  PT_CUDA_ERR = 5,    /* a CUDA runtime call failed */
  PT_BAD_ARG = 6      /* invalid argument (null pointer, unsupported PID, ...) */
} pt_status;

enum { PT_N_PROCESSES = 8, PT_N_NSIGMA = 8, PT_MAX_DIM = 4 };

/* Process codes follow shower.py:36. */
enum { PT_BREM = 0, PT_ANN = 1, PT_PAIRPROD = 2, PT_COMP = 3, PT_MOLLER = 4,
       PT_BHABHA = 5, PT_MUONE = 6, PT_MUONBREM = 7 };

/* Tables for one target material: the content of sm_maps.pkl/sm_xsec.pkl
 * after Shower.__init__ (shower.py:100-142,210-320).  Map rows of all
 * processes are concatenated; process p owns rows [map_base[p], map_base[p]+map_rows[p]). */
typedef struct pt_tables {
  int32_t map_base[PT_N_PROCESSES];
  int32_t map_rows[PT_N_PROCESSES];
  int32_t n_rows;                 /* total map rows */
  const double* map_energy;       /* [n_rows] incoming energy of each trained map */
  const double* map_maxF;         /* [n_rows] max_F[target] * maxF_fudge_global */
  const double* map_neval;        /* [n_rows] neval of each map */
  const int64_t* grid_offset;     /* [n_rows*4] first node of dimension d of row r */
  const int32_t* grid_ninc;       /* [n_rows*4] increments (nodes - 1) */
  const double* grid_nodes;       /* [n_nodes] all grid nodes, float64 */
  const float* grid_f32x4;        /* [n_nodes][4] float32 (node, increment to next node, 1-node, 1+node),
                                     each rounded once from float64 (mixed-precision form) */
  int64_t n_nodes;
  /* n*sigma(E) interpolation tables in 1/cm, slots: Brem, PairProd, Ann, Comp,
   * Moller, Bhabha, MuonE, MuonBrem (shower.py:280-295) */
  int32_t ns_base[PT_N_NSIGMA];
  int32_t ns_len[PT_N_NSIGMA];
  const double* ns_x;
  const double* ns_y;
  /* float32 forms for the mixed-precision engine: nodes, values and slopes
   * (y[j+1]-y[j])/(x[j+1]-x[j]) computed in float64; first-guess index
   * j ~ (ln E - ns_lnx0) * ns_invdlog (exact for the geometric grids PETITE
   * uses, corrected by one step otherwise) */
  const float* ns_x32;
  const float* ns_y32;
  const float* ns_s32;
  float ns_lnx0[PT_N_NSIGMA];
  float ns_invdlog[PT_N_NSIGMA];
  const float* map_energy32;      /* [n_rows] */
  const float* map_cnorm32;       /* [n_rows] K_process / (max_F * neval) for the float32 acceptance ratio;
                                     K_process: 8 alpha^3 Z^2 a0^4 (Brem, MuonBrem, PairProd), pi alpha^2
                                     (Comp, MuonE), 2 pi alpha^2 (Ann, Moller), pi alpha^2 / 2 (Bhabha) */
  float map_lnE0[PT_N_PROCESSES];
  float map_invdlog[PT_N_PROCESSES];
  /* target and thresholds */
  double Z, A, rho;               /* physical_constants.py:49-55 */
  double dEdx_GeV_per_m;          /* 0.1 * dEdx[MeV/cm] (shower.py:649) */
  double Eg_min, Ee_min;          /* shower.py:214-215 */
  double min_calc_electron, min_calc_positron, min_calc_muon, min_calc_photon; /* shower.py:242-246 */
  /* form-factor and multiple-scattering constants, evaluated on the host with
   * the reference's expressions: a0 = aa(Z, m_e) (all_processes.py:92-94) */
  double a0sq;                    /* a0**2 */
  double Z2a04;                   /* Z**2 * a0**4  (g2_elastic, all_processes.py:99-103) */
  double Z23;                     /* Z**(2/3)      (moliere.py:219) */
  double Z13;                     /* Z**(1/3)      (moliere.py:152) */
} pt_tables;

typedef struct pt_handle pt_handle;

/* Shower.__init__ (shower.py:100-142): validates and keeps the table description. */
pt_status pt_create(const pt_tables* tables, pt_handle** out);
/* Releases the handle (not the caller's device buffers). */
void pt_destroy(pt_handle* h);
/* Text for a status code. */
const char* pt_strerror(int status);
/* Details of the last PT_NO_SAMPLE/PT_TIMEOUT: process code, energy, LU_Key. */
pt_status pt_last_error_info(pt_handle* h, int32_t* process, double* energy, int32_t* lu_key);

/* Particle list in structure-of-arrays form; one row per Particle
 * (particle.py:50-131).  Vectors are component-major: p0[c*capacity + row]. */
typedef struct pt_particles {
  double* p0;        /* [4][capacity] initial four-momentum (E, px, py, pz) */
  double* r0;        /* [3][capacity] initial position (m) */
  double* pf;        /* [4][capacity] four-momentum after propagation */
  double* rf;        /* [3][capacity] position after propagation */
  double* weight;    /* [capacity] */
  double* mass;      /* [capacity] */
  int32_t* pid;      /* [capacity] PDG id */
  int32_t* gen;      /* [capacity] generation_number */
  int32_t* proc;     /* [capacity] generation_process code, -1 = "Input" */
  int32_t* bit;      /* [capacity] 0/1: first or second daughter (ID = 2*parent_ID + bit) */
  int32_t* primary;  /* [capacity] index of the primary the row belongs to */
  int32_t* draws;    /* [capacity] uniforms consumed by this particle (diagnostic) */
  int64_t* parent;   /* [capacity] parent row, -1 for a primary */
  uint64_t* pkey;    /* [capacity] random-stream key of the particle */
  int64_t capacity;
} pt_particles;

typedef struct pt_opts {
  double min_energy;             /* Shower(min_energy) */
  int64_t max_n_integrators;     /* Shower(max_n_integrators): proposals <= this * neval */
  double rescale_MCS;            /* Shower(rescale_MCS) */
  int32_t multiple_scattering;   /* generate_shower(GlobalMS) */
  int32_t precision;             /* 0 = float64 throughout, 1 = float32 sampling + float64 kinematics */
  uint64_t seed;                 /* Philox key */
  int64_t primary_offset;        /* primary i draws from the stream of index primary_offset + i */
  int32_t mcs_mode;              /* 0 = Shower(fast_MCS_mode=True): Lynch-Dahl Gaussian (moliere.py:350-400);
                                    1 = fast_MCS_mode=False: Bethe-Moliere (moliere.py:403-453) */
  int32_t loop_limit;            /* 0 = the library's bounds (2^22 substeps per particle in pt_run_sm,
                                    2^20 waves per pt_run_batch).  > 0: pt_run_sm ends a particle's
                                    substep loop after this many iterations and pt_run_batch ends after
                                    this many waves, with PT_TIMEOUT; for tests of the bounded paths */
} pt_opts;

/* Shower.generate_shower (shower.py:603-708) for n_primaries independent
 * primaries at once.  Rows [0, n_primaries) of `out` must hold the primaries
 * (p0, r0, pid, mass, weight; the remaining fields are filled here).  The
 * call transports every particle, appends daughters with E > min_energy,
 * and returns the number of rows used in *n_rows.  Row order is not the
 * reference's list order; parent/bit give the tree (the Python layer
 * restores list order).  Returns PT_OOM if capacity is too small. */
pt_status pt_run_sm(pt_handle* h, pt_particles* out, int64_t n_primaries,
                    const pt_opts* opts, int64_t* n_rows, void* stream);

/* pt_run_sm without any allocation.  No counterpart in the reference: it is
 * for callers that cannot allocate device memory during a run (a host whose
 * free device memory belongs to its own caching pool or a fixed budget, where
 * cudaMalloc may fail, or that cannot accept the device-wide synchronisation
 * of cudaFree).  Same kernels, streams and results as pt_run_sm; the scratch
 * (live lists, counters, status, error record) is one static device array of
 * 8 MB per device instead of handle memory grown with cudaMalloc.
 *  - out->capacity must not exceed 2^19 rows (524288); larger stores are
 *    rejected with PT_BAD_ARG and a message on stderr.
 *  - The first call on each device looks up the array's address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.  A failed lookup returns PT_CUDA_ERR and is
 *    tried again by the next call; only a successful one is kept.
 *  - The status word, error record and counters are zeroed (cudaMemsetAsync)
 *    at the start of every call.
 *  - All calls on a device share the one array: calls that overlap in time
 *    (other streams, other host threads, other handles) race on it. */
pt_status pt_run_sm_noalloc(pt_handle* h, pt_particles* out, int64_t n_primaries,
                            const pt_opts* opts, int64_t* n_rows, void* stream);

/* Tallies of a batched run (all device pointers; accumulated, never cleared
 * by the library).  Histograms: [kind][species][PT_HIST_BINS] with kinds
 * 0 = log10(E0/GeV) at creation in [-2, 2], 1 = log10(polar angle of p0 / rad)
 * in [-6, 0.5], 2 = depth z of the interaction point in [0, z_max] m;
 * species 0 = photon, 1 = electron, 2 = positron, 3 = muon. */
enum { PT_HIST_BINS = 100, PT_N_COUNTS = 16, PT_N_ESUM = 8 };
enum { PT_C_STEPS = 0, PT_C_PROPOSALS = 1, PT_C_SUBSTEPS = 2, PT_C_ENDED = 3, PT_C_PUSHED = 4,
       PT_C_BELOW_CUT = 5, PT_C_WAVES = 6, PT_C_SAMPLED = 7, PT_C_SPECIES = 8 /* ..11 */ };
enum { PT_E_CONTINUOUS = 0, PT_E_BELOW_CUT = 1, PT_E_ENDED = 2, PT_E_PRIMARY = 3 };
typedef struct pt_tally {
  unsigned long long* counts;   /* [PT_N_COUNTS] */
  double* energy;               /* [PT_N_ESUM] GeV: continuous dE/dx loss, daughters below the cut,
                                   particles that end without an interaction, primaries */
  unsigned int* hist;           /* [3][4][PT_HIST_BINS] */
  unsigned int* primary_count;  /* [n_primaries] particles per shower (rows of its list) */
  double* primary_edep;         /* [n_primaries] deposited energy per shower */
  double z_max;                 /* depth histogram range (m) */
} pt_tally;

/* Shower.generate_shower (shower.py:603-708) for many primaries without
 * materialising the particle list: every particle-step is tallied instead.
 * Primaries: p0 [4][n] and r0 [3][n] component-major, pid/mass [n].  Uses
 * the same per-particle random streams as pt_run_sm, so opts->precision = 0
 * reproduces pt_run_sm's showers exactly.  queue_capacity bounds the live
 * particles per wave (0 = library default); primaries are fed in chunks. */
pt_status pt_run_batch(pt_handle* h, const double* p0, const double* r0, const int32_t* pid, const double* mass,
                       int64_t n_primaries, const pt_opts* opts, pt_tally* tally, int64_t queue_capacity,
                       void* stream);

/* Counters of the last pt_run_sm on this handle: kernel launches and waves
 * (transport iterations).  Diagnostic; no reference counterpart. */
pt_status pt_last_run_stats(pt_handle* h, int64_t* kernel_launches, int64_t* waves);

/* Work-distribution settings of pt_run_batch (0 = library default).  No
 * counterpart in the reference: chosen by petite_gb300.autotune.
 *  refill_min[k]: idle lanes a warp gathers before refilling them, 1..32
 *                 (k = 0 propagation kernel, 1 sampler kernel; default 8)
 *  chunk[k]:      entries a warp claims from the wave's pool per atomic,
 *                 32..4096 (defaults 128 and 64)
 *  loop:          who runs the waves: PT_LOOP_HOST (0, default) launches the
 *                 two kernels per wave and reads its counters back;
 *                 PT_LOOP_GRAPH a CUDA graph whose conditional WHILE node
 *                 repeats the wave with its plan made on the GPU;
 *                 PT_LOOP_PERSISTENT one cooperative kernel runs every wave
 *                 between grid barriers.  Results are identical.
 *  staging:       where the mixed engine's propagation kernel reads the
 *                 float32 n*sigma tables: PT_STAGE_SHARED each block's
 *                 shared memory, filled by TMA bulk copies at block start
 *                 (used with PT_LOOP_HOST and PT_LOOP_GRAPH when the tables
 *                 fit PT_STAGE_MAX_NODES entries and are 16-byte aligned;
 *                 otherwise the cached path runs); PT_STAGE_CACHED through
 *                 the read-only data cache; PT_STAGE_DEFAULT (0) the shared
 *                 form.  Results are identical.
 *  threads:       threads per block of the mixed engine's two kernels with
 *                 PT_LOOP_HOST and PT_LOOP_GRAPH: 64, 128 or 256 (0: 128).
 *                 The FP64 kernels and the persistent kernel run 128.
 *                 Results are identical. */
enum { PT_LOOP_HOST = 0, PT_LOOP_GRAPH = 1, PT_LOOP_PERSISTENT = 2 };
enum { PT_STAGE_DEFAULT = 0, PT_STAGE_CACHED = 1, PT_STAGE_SHARED = 2, PT_STAGE_MAX_NODES = 2048 };
typedef struct pt_batch_tuning {
  int32_t refill_min[2];
  int32_t chunk[2];
  int32_t loop;
  int32_t staging;
  int32_t threads;
  int32_t barrier_ns;             /* the persistent kernel's bound on one grid-barrier wait, ns (0 = 20 s);
                                     a wait that runs out returns PT_TIMEOUT.  For tests of that path. */
  int32_t lanes;                  /* 0 or 1: one wave at a time.  2..8 (host loop only): the primaries
                                     split into that many contiguous groups, each with its own ring,
                                     task pools and CUDA stream, whose waves the host interleaves, so
                                     that one group's kernels use the SMs another group's wave tail
                                     leaves idle.  Every primary keeps its stream, so the showers and
                                     integer tallies are those of one lane; each extra lane holds a ring
                                     of queue_capacity entries. */
} pt_batch_tuning;
/* Stores the settings on the handle (NULL restores the defaults);
 * PT_BAD_ARG for a value out of range. */
pt_status pt_set_batch_tuning(pt_handle* h, const pt_batch_tuning* t);

/* Device time of the last pt_run_batch on this handle, summed over its waves
 * and measured with CUDA events on the run's stream: the propagation kernel
 * and the sampler kernel, in milliseconds (with PT_LOOP_GRAPH or
 * PT_LOOP_PERSISTENT: the whole run, and 0).  Diagnostic; no reference
 * counterpart. */
pt_status pt_last_kernel_times(pt_handle* h, double* propagate_ms, double* sample_ms);

/* Measured arithmetic peaks of the current GPU, for the rooflines of the
 * issue-bound kernels: float32 and float64 fused multiply-add throughput in
 * flop/s (chains of independent FMAs on every SM, timed with CUDA events on
 * `stream`; about 10 ms).  Diagnostic; no reference counterpart. */
pt_status pt_alu_peaks(double* fp32_flops, double* fp64_flops, void* stream);

/* Shower.draw_sample (shower.py:401-465) for a batch: for each i, draws the
 * final-state variables of `process` at energy energy[i] from stream key
 * pkey[i] starting at draw 0.  Writes x[i*4 + d], proposals[i], lu_key[i]. */
pt_status pt_sample_only(pt_handle* h, int32_t process, const double* energy,
                         const uint64_t* pkey, int64_t n, const pt_opts* opts,
                         double* x, int64_t* proposals, int32_t* lu_key, void* stream);

/* Differential cross section of `process` (all_processes.py, the dsigma_*
 * classes) at n points x[i*4 + d] and energies energy[i]: value[i]. */
pt_status pt_dsigma(pt_handle* h, int32_t process, const double* x, const double* energy,
                    int64_t n, int32_t precision, double* value, void* stream);

/* inverse_moliere_cdf(u, B) (moliere.py:84-120), the sampler of
 * fast_MCS_mode=False, for n device pairs: x[i] with Moliere's
 * x = theta^2 / (chi_c^2 B).  precision 0 = float64 (the engines' form),
 * 1 = float32 (the mixed engine's).  Needs no handle. */
pt_status pt_moliere_inverse_cdf(const double* u, const double* B, int64_t n, int32_t precision, double* x,
                                 void* stream);

/* ------------------------------------------------------------------------
 * Map training (utilities/generate_integrators.py, utilities/find_maxes.py):
 * VEGAS adaptive maps for every energy row of one SM process at once, and
 * the scan of each map for max_F and the cross section.  All pointers are
 * device pointers except `target`/`targets` and `ninc` (host; increments
 * per dimension, 1..1000).  Grids: nodes[row][d][k], k = 0..ninc[d], rows
 * padded to max_nodes; acc/cnt: [row][d][1000].
 * ------------------------------------------------------------------------ */
typedef struct pt_train_target {   /* what the cross sections read of a target */
  double Eg_min, Ee_min;           /* shower.py:214-215 */
  double a0sq, Z2a04;              /* aa(Z, m_e)^2 and Z^2 aa^4 (all_processes.py:92-103) */
  double mV;                       /* dark processes: the vector's mass (GeV) */
  double MT, Z, A;                 /* dark processes: event_info mT, Z_T, A_T (all_processes.py:208-372) */
} pt_train_target;
/* Process codes of the table builder: the SM codes (PT_BREM ...), and
 * PT_TRAIN_DARK + a dark code (PT_DARKBREM ...) for the dark processes. */
enum { PT_TRAIN_DARK = 16 };
/* One training iteration's samples: points_per_row map points per row
 * (iteration 0..63 selects the draws); accumulates (jac f)^2 and counts per
 * increment into acc/cnt and (sum w, sum w^2) into sums[row][2]. */
pt_status pt_vegas_accumulate(int32_t process, const pt_train_target* target, const double* energy,
                              int32_t n_rows, int32_t dims, const int32_t* ninc, const double* nodes,
                              int32_t max_nodes, int64_t points_per_row, uint64_t seed, int32_t iteration,
                              double* acc, uint32_t* cnt, double* sums, void* stream);
/* The VEGAS adaptation of every row's grid from acc/cnt (damping alpha). */
pt_status pt_vegas_adapt(int32_t n_rows, int32_t dims, const int32_t* ninc, double* nodes, int32_t max_nodes,
                         const double* acc, const uint32_t* cnt, double alpha, void* stream);
/* find_maxes (find_maxes.py:56-115): per row and target, n_trials batches of
 * neval points weighted jac/neval: max_F[row][t] = the largest weight*f,
 * xsec[row][t] = the sum of weight*f divided by n_trials. */
pt_status pt_find_maxes(int32_t process, const pt_train_target* targets, int32_t n_targets, const double* energy,
                        int32_t n_rows, int32_t dims, const int32_t* ninc, const double* nodes, int32_t max_nodes,
                        int32_t neval, int32_t n_trials, uint64_t seed, double* max_F, double* xsec, void* stream);

/* ------------------------------------------------------------------------
 * Dark-vector production on an SM shower (DarkShower, dark_shower.py).
 * ------------------------------------------------------------------------ */
enum { PT_N_DARK = 4, PT_DARK_MAX_MASSES = 8 };
/* Dark process codes (dark_shower.py:49); PT_DARK_BOUND is added to the
 * output process code when the bound-electron form produced the vector
 * ("DarkAnn_bound", "DarkComp_bound", dark_shower.py:799-802). */
enum { PT_DARKBREM = 0, PT_DARKANN = 1, PT_DARKCOMP = 2, PT_DARKMUONBREM = 3, PT_DARK_BOUND = 4 };
/* TwoBody_BSMDecay (dark_shower.py:633-638,836-844; Particle.two_body_decay,
 * particle.py:209-256): a pi0 row decays to gamma + V.  PT_TWOBODY is its bit
 * in pt_dark_params.active and its yield slot; its vectors carry process
 * code PT_TWOBODY_CODE. */
enum { PT_TWOBODY = 4, PT_TWOBODY_CODE = 8 };

/* VEGAS maps of the dark processes for one target, for up to
 * PT_DARK_MAX_MASSES vector masses (dark_maps.pkl, dark_shower.py:148-201):
 * rows of (mass m, process p) are [map_base[m*PT_N_DARK+p], +map_rows[...]). */
typedef struct pt_dark_maps {
  int32_t n_masses;
  double mass[PT_DARK_MAX_MASSES];
  int32_t map_base[PT_DARK_MAX_MASSES * PT_N_DARK];
  int32_t map_rows[PT_DARK_MAX_MASSES * PT_N_DARK];
  int32_t n_rows;
  const double* map_energy;       /* [n_rows] */
  const double* map_maxF;         /* [n_rows] max_F[target] * maxF_fudge_global */
  const double* map_neval;        /* [n_rows] */
  const int64_t* grid_offset;     /* [n_rows*4] */
  const int32_t* grid_ninc;       /* [n_rows*4] */
  const double* grid_nodes;
  int64_t n_nodes;
  double Z, A;                    /* target Z_T and A_T (A_T is also the target mass
                                     draw_dark_sample passes, dark_shower.py:673) */
  const float* grid_f32x2;        /* [n_nodes][2] float32 (node, increment to the next node), each rounded
                                     once from float64: the proposals of pt_dark_params.precision = 1
                                     (NULL: float64 proposals only) */
} pt_dark_maps;

/* One DarkShower's per-mass tables (dark_shower.py:69-130, 219-593), all
 * device pointers.  Index k of the four weight and dR/dE tables:
 * 0 = electron DarkBrem, 1 = positron DarkBrem, 2 = positron DarkAnn,
 * 3 = muon DarkMuonBrem. */
typedef struct pt_dark_params {
  int32_t mass_index;             /* map block sampled (the mV estimator) */
  int32_t bound_electron;         /* 1: bound-electron DarkAnn/DarkComp (the reference default); 0: free */
  int32_t active;                 /* bit p: dark process p active; bit PT_TWOBODY: TwoBody_BSMDecay */
  double mV;                      /* vector mass used in the cross sections and kinematics */
  double coupling;                /* g_e^2 / (4 pi alpha_em) */
  double Zeff;
  double E_res, E_compth;         /* resonant annihilation and Compton threshold energies */
  double min_dark[5];             /* e- DarkBrem, e+ DarkBrem, e+ DarkAnn, gamma DarkComp, mu DarkMuonBrem */
  double min_calc_photon;         /* the SM photon minimum (GetBSMWeights, dark_shower.py:612) */
  const double* w_x[4];           /* track-length weights, interp1d(fill 0) tables */
  const double* w_y[4];
  int32_t w_n[4];
  const double* dr_Ei[4];         /* dR/dE: saved energies [dr_n] */
  const double* dr_bins[4];       /* [dr_n][dr_nbmax][2] (bin energy, weight) */
  const int32_t* dr_nbins[4];     /* [dr_n] bins used */
  int32_t dr_n[4];
  int32_t dr_nbmax[4];
  const double* nsc_lx;           /* DarkComp n*sigma, log10 energies and log10 values */
  const double* nsc_ly;
  int32_t nsc_n;
  double kinetic_mixing;          /* DarkShower(kinetic_mixing): the TwoBody_BSMDecay weight */
  /* bound_electron = 0 (free electrons): the DarkAnn weight adds a closed-form
   * resonant part (dark_shower.py:619-630) */
  double ann_E0;                  /* first energy of the free DarkAnn cross section (get_DarkAnnXSec()[0][0]) */
  double ann_K;                   /* (1/dEdx[GeV/cm]) (2 pi^2 alpha/m_e) n_e GeVsqcm2, the reference's order */
  const double* ii_x[3];          /* interaction integrals of Brem, Ann, Bhabha (shower.py:296-314): */
  const double* ii_y[3];          /*   interp1d(fill 0) tables behind _positron_exponential_factor */
  int32_t ii_n[3];
  int32_t precision;              /* draw_dark_sample's proposals: 0 = float64 throughout; 1 = float32
                                     uniforms, map transform and dark-brem screen, with the float64
                                     cross section deciding wherever the float32 estimate cannot (near
                                     the acceptance boundary or a kinematic edge); the vector's
                                     kinematics stay float64 (needs pt_dark_maps.grid_f32x2) */
} pt_dark_params;

/* Vectors produced by pt_run_dark (device pointers; SoA like pt_particles). */
/* A histogram of dark-vector energies: counts[p * bins + b] += weight for
 * process p and b = floor(bins * (log10(E_V/GeV) - log10_lo) / (log10_hi -
 * log10_lo)), clamped to [0, bins): the bins of a process sum to its yield.
 * No reference counterpart (PETITE returns the vectors). */
typedef struct pt_dark_hist {
  double* counts;      /* [PT_N_DARK + 1][bins] (accumulated); NULL: none */
  int32_t bins;
  int32_t reserved0;
  double log10_lo, log10_hi;
} pt_dark_hist;

typedef struct pt_dark_out {
  double* p4;          /* [4][capacity] lab four-momentum */
  double* r;           /* [3][capacity] production point (the parent's final position) */
  double* weight;      /* [capacity] */
  int64_t* parent;     /* [capacity] SM row */
  int32_t* process;    /* [capacity] dark process code (+PT_DARK_BOUND), or PT_TWOBODY_CODE */
  int32_t* draws;      /* [capacity] uniforms used (diagnostic) */
  int64_t capacity;
  double* yield;       /* [PT_N_DARK + 1] summed weights per process, PT_TWOBODY last (accumulated) */
  double* yield_E;     /* [PT_N_DARK + 1] summed weight * E_V per process (accumulated) */
  pt_dark_hist hist;   /* energy histogram of the vectors (counts NULL: none) */
} pt_dark_out;

typedef struct pt_dark pt_dark;

/* DarkShower.__init__ (dark_shower.py:69-130): binds the dark maps of one
 * target to an SM handle (whose tables give the photon n*sigma of
 * GetBSMWeights and the multiple-scattering constants). */
pt_status pt_dark_create(pt_handle* sm, const pt_dark_maps* maps, pt_dark** out);
void pt_dark_destroy(pt_dark* d);

/* The dark differential cross sections draw_dark_sample evaluates
 * (dark_shower.py:673-684): dsig_dx_dcostheta_dark_brem_exact_tree_level
 * (all_processes.py:208-372; DarkBrem with m_e, DarkMuonBrem with m_mu),
 * dsigma_compton_dCT with mV (:624-742) and dsigma_radiative_return_du
 * (:400-466), at x[i*4 + d], energy[i] and mass mV. */
pt_status pt_dark_dsigma(pt_dark* d, int32_t process, const double* x, const double* energy, int64_t n, double mV,
                         double* value, void* stream);

/* The float32 estimate of the DarkBrem / DarkMuonBrem integrand, or of the
 * DarkAnn (radiative-return) one, that screens the map's accept/reject
 * decisions (no reference counterpart; diagnostic): code[i] = 0 estimate not
 * trusted (near a kinematic edge or a cancellation), 1 value[i] holds it,
 * 2 the point lies outside the allowed region (dark bremsstrahlung only). */
pt_status pt_dark_screen32(pt_dark* d, int32_t process, const double* x, const double* energy, int64_t n, double mV,
                           float* value, int32_t* code, void* stream);

/* DarkShower.draw_dark_sample (dark_shower.py:649-704) for a batch, stream
 * key[i] from draw 0: x[i*4 + d], proposals[i] (-1 when no sample was found:
 * the reference returns None), lu_key[i]. */
pt_status pt_dark_sample_only(pt_dark* d, const pt_dark_params* prm, int32_t process, const double* energy,
                              const uint64_t* key, int64_t n, const pt_opts* opts, double* x, int64_t* proposals,
                              int32_t* lu_key, void* stream);

/* DarkShower.generate_dark_shower (dark_shower.py:806-849) over the rows of
 * an SM particle store: for every row and active process, GetBSMWeights
 * (:595-647) and, when positive, produce_bsm_particle (:721-804).  Row k,
 * process p draws from the stream mix64(pkey[k] + 0x9E3779B97F4A7C15*(3+p)).
 * Vectors are appended to `out` (any order; parent/process identify them);
 * *n_out returns the count.  PT_OOM if out->capacity is too small.  With
 * out->p4 == NULL only the yields and the count are accumulated. */
/* pt_run_batch with dark-vector production on every wave: each particle's
 * row (the record engine's row of that particle: p0 at the start of its
 * propagation, pf/rf at its end, its stream key) goes through pt_run_dark's
 * GetBSMWeights and produce_bsm_particle for each of n_params parameter
 * sets (dark masses, 1..16) on the same showers, so precision 0 gives
 * pt_run_sm + pt_run_dark's vectors.  Only the yields are kept:
 * yield/yield_E (device, [n_params][PT_N_DARK + 1], accumulated), the
 * energy histogram when hist is not NULL (hist->counts: [n_params][PT_N_DARK
 * + 1][bins], accumulated) and *n_vectors (all sets).  d must be bound to h.  The waves run on the host
 * loop; TwoBody_BSMDecay is not applied (SM showers hold no mesons).  No
 * reference counterpart as one call: PETITE runs generate_shower and then
 * generate_dark_shower over its list, once per mass. */
pt_status pt_run_batch_dark(pt_handle* h, pt_dark* d, const pt_dark_params* prm, int32_t n_params, const double* p0,
                            const double* r0, const int32_t* pid, const double* mass, int64_t n_primaries,
                            const pt_opts* opts, pt_tally* tally, int64_t queue_capacity, double* yield,
                            double* yield_E, const pt_dark_hist* hist, int64_t* n_vectors, void* stream);

pt_status pt_run_dark(pt_dark* d, const pt_dark_params* prm, const pt_particles* sm, int64_t n_rows,
                      const pt_opts* opts, pt_dark_out* out, int64_t* n_out, void* stream);

/* Dark-vector yield at fixed uniforms: for pair i, the map block
 * mass_index[i] of `process` at LU_Key(energy[i]) and n_samples points whose
 * uniforms are draws 4j..4j+3 of stream (seed, mix64(4*i + process + 1)):
 * yield[i] = mean(jac * dsigma(x; energy[i], mV[i])) (the map's cross-section
 * estimate, find_maxes.py:143-147) and moment[i] = mean(jac * dsigma * E_V).
 * mV_anchor (may be NULL): for DarkBrem/DarkMuonBrem, each sample's log10 t~
 * is carried along the momentum-transfer range from mass mV_anchor[i] to
 * mV[i] (a change of variables; equal to the plain estimate at
 * mV = mV_anchor), which makes the estimate smooth in mV around the anchor.
 * No counterpart in the reference as one function. */
pt_status pt_dark_yield(pt_dark* d, int32_t process, const double* energy, const double* mV,
                        const double* mV_anchor, const int32_t* mass_index, int64_t n_pairs, int64_t n_samples,
                        uint64_t seed, double* yield, double* moment, void* stream);

/* Adjoint of pt_dark_yield with respect to mV: recomputes every sample and
 * writes g_mV[i] = g_yield[i] * d yield[i]/d mV + g_moment[i] * d moment[i]/d mV,
 * including the motion of the DarkBrem momentum-transfer range with mV (the
 * derivative of the anchored estimate at its anchor). */
pt_status pt_dark_yield_adjoint(pt_dark* d, int32_t process, const double* energy, const double* mV,
                                const int32_t* mass_index, int64_t n_pairs, int64_t n_samples, uint64_t seed,
                                const double* g_yield, const double* g_moment, double* g_mV, void* stream);

/* ------------------------------------------------------------------------
 * Detector acceptance: detector_cut (shower.py:825-865) with
 * transverse_position (shower.py:815-823) over n device rows in SoA form,
 * E/px/py/pz at p4 + {0,1,2,3} * p4_stride and x0/y0/z0 at
 * r + {0,1,2} * r_stride (a pt_particles store's p0/r0 with the store's
 * capacity as stride, or pt_dark_out's p4/r), weight[n] (null: weights 1).
 * Row i passes disk detector d at z_det[d] (device, [n_det]) when its initial
 * straight line crosses z_det[d] at a transverse radius in the open interval
 * (r_inner, r_outer) and, with use_window, e_min < E < e_max; each operation
 * rounded on its own as numpy evaluates the reference's expressions.
 * Outputs (device, each may be null): pass[n_det][n], 1 where row i passes
 * detector d; sums[n_det + 1], the weight passing each detector, then the
 * weight of the rows in the energy window (all rows without one).  The sums
 * add block totals atomically, so their last bits may vary from run to run.
 * Needs no handle.  Replaces the reference's detector_cut over a Python list
 * of Particle objects (methods "SampleW", "Sample", "Efficiency" and
 * "TotalWeight" are read from these outputs). */
pt_status pt_detector_cut(const double* p4, int64_t p4_stride, const double* r, int64_t r_stride,
                          const double* weight, int64_t n, const double* z_det, int32_t n_det,
                          double r_inner, double r_outer, int32_t use_window, double e_min, double e_max,
                          uint8_t* pass, double* sums, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PETITE_GPU_H */
