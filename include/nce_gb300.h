/* nce_gb300.h -- C ABI of libnce_gb300.so, the GB300 (sm_103a) engine for neuralce's parallel-tempering
 * Monte Carlo hot path.
 *
 * Plain C types only: pointers, sizes, status codes.  Device pointers are CUDA global-memory addresses
 * (a caller typically takes them from torch tensors); "stream" is a cudaStream_t passed as void*
 * (NULL = legacy default stream).  Every function returns 0 (NCE_OK) or a negative NCE_ERR_* code;
 * nce_last_error() gives the message of the calling thread's last failure.
 *
 * Threading: a handle may be used from one host thread at a time; calls are asynchronous on the given
 * stream unless stated otherwise.  A NeuralCE model handle keeps one set of step scratch (slot map, site
 * lists, new rows) for all states that use it, so its chunks must be ordered on one stream; full caches and
 * energies take per-call scratch and may overlap on several streams.  Table inputs are host pointers and are
 * copied during *_create; the caller keeps ownership.
 *
 * Reference interfaces replaced (paths inside the neuralce project):
 *   nce_ce_create        GPUClusterExpansion(..., table_mode='implicit')      neuralce/ce/classical_ce_gpu.py:496-535
 *                        build_ce_gpu_implicit tables                         neuralce/ce/ce_gpu_implicit.py:50-126
 *   nce_ce_energy        GPUClusterExpansion.energy_a / energy               neuralce/ce/ce_gpu_implicit.py:147-163
 *   nce_ce_delta         GPUClusterExpansion.delta_energy_a                  neuralce/ce/ce_gpu_implicit.py:181-191
 *   nce_ce_run_chunk     run_chunk = scan(micro) + exchange_slots            neuralce/ce/pt_mcmc_ce.py:748-818
 *                        (mc_step delta branch                               neuralce/ce/pt_mcmc_ce.py:558-566,
 *                         make_fast_swap_implicit proposal                   neuralce/ce/ce_gpu_implicit.py:194-211)
 *   nce_ce_run_batch     vmap over independent jobs of run_chunk             neuralce/ce/pt_mcmc_ce.py:733,765-818
 *   nce_ce_run_chunk_host  same as nce_ce_run_chunk with host buffers (the e2e call of a host-side driver)
 *   nce_philox4x32       counter-based RNG used on the device (replaces jax.random keys in micro, pt_mcmc_ce.py:773-774)
 */
#ifndef NCE_GB300_H
#define NCE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NCE_OK                 0
#define NCE_ERR_INVALID       -1   /* bad argument (size, pointer, range) */
#define NCE_ERR_CUDA          -2   /* a CUDA call failed */
#define NCE_ERR_UNSUPPORTED   -3   /* valid but not supported by this library (e.g. cluster order > 8) */
#define NCE_ERR_TIMEOUT       -4   /* a bounded device wait gave up */
#define NCE_ERR_NOMEM         -5   /* device allocation failed / admission refused */

int nce_version(void);
/* Copies the calling thread's last error message into buf (NUL-terminated); returns its full length. */
int nce_last_error(char *buf, size_t len);

/* ── cluster expansion (orthonormal, template-only tables) ──────────────────────────────────────── */

typedef struct {
    int32_t nB;            /* basis sites of the primitive */
    int32_t J;             /* reverse rows per basis site (padded) */
    int32_t mo;            /* maximum cluster order (members per row), 1..8 */
    int32_t n_nbr;         /* neighbourhood entries per basis site (entry 0 = the site itself) */
    int32_t n_pfc;         /* point-function columns = n_sublattices * (max_bf + 1) */
    int32_t max_sp;        /* species per site, maximum over sublattices */
    int64_t d[3];          /* Smith-normal-form diagonal of the supercell */
    int64_t n_cells;       /* primitive cells in the supercell = d0*d1*d2 */
    double zerolet;        /* constant term (already multiplied by energy_scale) */
    const int32_t *Rv_len; /* (nB) valid reverse rows per basis site */
    const uint16_t *Rv_loc;/* (nB, J, mo) neighbourhood index of each row member */
    const uint8_t *Rv_pfc; /* (nB, J, mo) point-function column of each row member */
    const double *Rv_eci;  /* (nB, J) eci per row = eci * scale / (instances * n_cells); padded rows 0 */
    const int32_t *nb_b;   /* (nB, n_nbr) basis of each neighbourhood entry */
    const int32_t *nb_uo;  /* (nB, n_nbr, 3) U*offset mod d of each neighbourhood entry */
    int32_t Rt;            /* template rows (full energy) */
    const int32_t *T_b;    /* (Rt, mo) */
    const int32_t *T_uo;   /* (Rt, mo, 3) */
    const uint8_t *T_pfc;  /* (Rt, mo) */
    const double *T_eci;   /* (Rt) */
    const double *pf;      /* (n_pfc, max_sp) point-function values */
    int32_t n_groups;      /* active sublattices (swap groups) */
    int32_t max_gb;        /* basis sites per group, maximum */
    const int32_t *act_b;  /* (n_groups, max_gb) basis sites of each group */
    const int32_t *act_nb; /* (n_groups) */
    const uint64_t *grp_cum; /* (n_groups) cumulative choice thresholds in units of 2^-32 (last = 2^32) */
    const int32_t *Rv_col; /* (nB, J) cluster-vector column of each reverse row (non-decreasing within a site), or NULL */
    int32_t n_cols;        /* columns (<= 255 for the sign-parity kernel) */
    const int8_t *Rv_slot; /* (nB, J) slot of the site in the template row (0 = the row's anchor), or NULL */
} nce_ce_tables;

typedef struct nce_ce_model *nce_ce_handle;

/* Copy the tables to the current device.  Replaces GPUClusterExpansion(table_mode='implicit'). */
int nce_ce_create(const nce_ce_tables *tables, nce_ce_handle *out);
int nce_ce_destroy(nce_ce_handle h);

/* Full energy of R configurations sigma (R, N) int8 (device) -> E (R) float64 (device).
 * precision: 64 = float64 tables and products, 32 = float32 products with float64 accumulation. */
int nce_ce_energy(nce_ce_handle h, const int8_t *sigma, int32_t R, int32_t precision, double *E, void *stream);

/* Same result as nce_ce_energy, for callers that cannot allocate device memory while they run (their device
 * memory is reserved up front by their own pool, or they cannot afford the device synchronisation that
 * cudaMalloc/cudaFree imply).  It allocates nothing: its scratch is a fixed array of 65,536 float64 partials
 * built into this library, one per device, kept until the process exits; R may be at most 65,535 (one grid row
 * per configuration).  The first call on a device looks up that array's address; make this first call before any
 * stream capture.  Calls that overlap on the GPU share the array and race.  This entry point has no counterpart
 * in the reference. */
int nce_ce_energy_noalloc(nce_ce_handle h, const int8_t *sigma, int32_t R, int32_t precision, double *E, void *stream);

/* n independent swap energy differences on device data: for query q, configuration rep[q] of sigma (R,N),
 * E(after sigma[ia]=sa_new, sigma[ib]=sb_new) - E(before) -> out[q] (float64).  Replaces delta_energy_a. */
int nce_ce_delta(nce_ce_handle h, const int8_t *sigma, int32_t R, int32_t n, const int32_t *rep,
                 const int64_t *ia, const int64_t *ib, const int8_t *sa_new, const int8_t *sb_new,
                 int32_t precision, int32_t warps, double *out, void *stream);

/* Cluster-vector sums of R configurations (sign-parity tables only): cv[r, c] = sum over the cluster instances
 * of column c of the product of the point functions (+-1), exact integers.  cv is (R, n_cols) int64 on the device.
 * E = zerolet + sum_c eci_c * cv[r, c] (the orbit's eci per instance).  No counterpart in the reference, whose
 * float64 re-anchor recomputes the energy from scratch (ce_gpu_implicit.py energy_a). */
int nce_ce_cluster_counts(nce_ce_handle h, const int8_t *sigma, int32_t R, int64_t *cv, void *stream);

/* E[r] = zerolet + sum_c eci_c * cv[r, c] in float64, columns in order (the exact re-anchor of the carried
 * energies from tracked cluster-vector sums). */
int nce_ce_energy_from_counts(nce_ce_handle h, const int64_t *cv, int32_t R, double *E, void *stream);

/* Local fields of R configurations sigma (R, N) (device) -> field (R, N) int64 (device): G(i) = sum over the cluster
 * instances containing site i of 2 eci Pi, fixed point.  A swap of a and b then changes the energy by
 * -G(a) - G(b) + 2 C(a, b) (C: the instances containing both), so the chunk kernel decides a proposal in O(1) and
 * pays for the rows only when a swap is accepted.  Needs +-1 point functions and a cell without aliasing
 * (nce_ce_has_local_field).  No counterpart in the reference, whose delta_energy_a re-evaluates the rows of both
 * sites at every step (neuralce/ce/ce_gpu_implicit.py:181-191). */
int nce_ce_field_init(nce_ce_handle h, const int8_t *sigma, int32_t R, int64_t *field, void *stream);
/* ok = 1 when the local-field path can run on this cell; scale (may be NULL) = eV per fixed-point unit (2^-S). */
int nce_ce_has_local_field(nce_ce_handle h, int32_t *ok, double *scale);

/* Parallel-tempering state of one job, all device pointers. */
typedef struct {
    int32_t R;             /* replicas = temperature slots */
    int64_t N;             /* sites per replica */
    int8_t *sigma;         /* (R, N) species index, canonical site order; replica r's row */
    double *E;             /* (R) carried energy per replica */
    const float *beta_slot;/* (R) 1/(kB T) of each temperature slot (float32, as the reference) */
    int32_t *rep_of_slot;  /* (R) replica holding slot t */
    int32_t *slot_of_rep;  /* (R) inverse; a shard of a larger ladder may hold that ladder's slots here (beta_slot then
                              has the ladder's length; proposals are keyed by these slots; no in-kernel exchange or
                              E_samples in that use) */
    const int32_t *ladder_id; /* (R) ladder of each slot (exchange only within a ladder) */
    double *E_min_rep;     /* (R) running minimum of E per replica */
    int64_t *n_acc;        /* (R) accepted swaps per replica (accumulated) */
    int64_t *n_ex;         /* (1) accepted exchanges (accumulated) */
    int64_t *cv;           /* (R, n_cols) or NULL: per replica, the sums over all cluster instances of each
                              cluster-vector column of the product of point functions (exact integers on the
                              sign-parity path), kept current by the chunk kernel; the float64 energy follows
                              from them exactly (nce_ce_energy_from_counts) */
    int64_t *n_near;       /* (R) or NULL: near-threshold steps per replica (accumulated).  A swap with dE is accepted
                              when log u < -beta dE (neuralce/ce/pt_mcmc_ce.py:563); a step is near its threshold when
                              |dE + ln(u) / beta| < the chunk's near_eV, the stated per-swap dE error bound of the
                              precision form: only there can a decision differ from a float64 reference's */
    int64_t *field;        /* (R, N) or NULL: every site's local field G(i) = sum over the reverse rows of i of
                              2 eci Pi, in the float64 kernels' fixed point (exact integers).  When set (and the cell
                              supports it, nce_ce_has_local_field), precision-64 chunks run the local-field kernel and
                              keep the fields current; fill it with nce_ce_field_init after (re)setting sigma. */
    int32_t *ex_sync;      /* (1) or NULL: a counter, 0 between chunks.  When every job of a launch has one, the chunk-
                              end exchange (and the step_dev advance) runs inside the chunk kernel: the last replica
                              of a job to finish performs it and resets the counter; otherwise a second kernel does. */
} nce_pt_state;

/* One chunk of steps.  Proposals: host-supplied stream (prop_a/prop_b/prop_u device arrays indexed
 * [step][slot]) or, when prop_a is NULL, Philox4x32-10 keyed by seed with counter (global step, slot). */
typedef struct {
    int64_t n_steps;       /* steps in this chunk */
    int64_t step0;         /* global index of the chunk's first step */
    const int32_t *prop_a; /* (n_steps, R) or NULL */
    const int32_t *prop_b;
    const double *prop_u;  /* (n_steps, R) uniforms in (0,1] */
    uint64_t seed;
    int64_t sample_interval;   /* record E every sample_interval steps (slot order) */
    double *E_samples;         /* (n_steps/sample_interval, R) device, or NULL */
    int32_t do_exchange;       /* chunk ends on an exchange step */
    int32_t ex_parity;         /* used when ex_u != NULL */
    const double *ex_u;        /* (ceil((R-1)/2)) device uniforms, or NULL -> Philox */
    int32_t precision;         /* 64 or 32 */
    int32_t warps;             /* warps per replica (0 = default) */
    int32_t path;              /* 0 auto (local field when the state has a field, else sign parity when the point
                                  functions are in {-1,+1}, else general), 1 general point-function products, 2 sign
                                  parity, 3 local field (precision 64, state.field set) */
    int32_t cluster;           /* sign parity: CTAs per replica (1, 2, 4, 8; thread-block cluster); the cell must fit in
                                  shared memory, otherwise one CTA is used */
    int64_t *step_dev;         /* device counter or NULL: when set, the chunk's first global step is read from it
                                  (step0 is ignored) and it advances by n_steps when the chunk ends, so that a
                                  captured CUDA graph of chunks continues the Philox stream on every replay */
    double near_eV;            /* near-threshold band of n_near; 0 = the form's stated dE error bound: 1e-9 eV at
                                  precision 64 (its fixed-point sums are within 2e-13 eV of float64), 1e-6 eV at 32 */
} nce_pt_chunk;

int nce_ce_run_chunk(nce_ce_handle h, const nce_pt_state *st, const nce_pt_chunk *ck, void *stream);

/* Independent jobs (different cells, ladders, tables) in one launch; n_jobs <= 64 per call.
 * Every chunk in the batch must use the same precision and warps. */
int nce_ce_run_batch(int32_t n_jobs, const nce_ce_handle *h, const nce_pt_state *st, const nce_pt_chunk *ck,
                     void *stream);

/* e2e form: the same chunk with HOST buffers.  sigma_host (R,N), E_host (R) and the permutations are read
 * and written back; prop_* are host arrays (or NULL for Philox); E_samples_host (n_steps/si, R) receives
 * the samples.  Synchronous.  Replaces a host driver's call of run_chunk on host arrays. */
int nce_ce_run_chunk_host(nce_ce_handle h, int32_t R, int8_t *sigma_host, double *E_host, const float *beta_slot_host,
                          int32_t *rep_of_slot_host, int32_t *slot_of_rep_host, const int32_t *ladder_id_host,
                          double *E_min_rep_host, int64_t *n_acc_host, int64_t *n_ex_host,
                          const nce_pt_chunk *ck_host_pointers, double *E_samples_host);

/* chunk epilogue: global running minimum and the replica index of the lowest current energy.
 * out (device): out_min[0] = min_r E_min_rep[r], out_arg[0] = argmin_r E[r] (first on ties). */
int nce_pt_minimum(const nce_pt_state *st, double *out_min, int32_t *out_arg, void *stream);

/* Reads and clears the handle's device error word (synchronous).  Bit 0: a proposal index was outside
 * [0, N) (that step was rejected instead of read). */
int nce_ce_errors(nce_ce_handle h, int32_t *flags);

/* ── NeuralCE receptive-field update ─────────────────────────────────────────────────────────────
 * Reference interfaces replaced:
 *   nce_nce_create      setup / setup_implicit geometry + expand_params      neuralce/nce/mc_model.py:60-111,175-228
 *                       (build_geometry                                      neuralce/nce/gpu_layer0_implicit.py:17-118)
 *   nce_nce_full_cache  full_cache + energy_of (h0 cache mode)               neuralce/nce/local_update_implicit.py:89-112
 *   nce_nce_run_chunk   scan(step): propose, local_delta, accept, commit    neuralce/nce/mcmc.py:130-199,
 *                                                                            neuralce/nce/local_update_implicit.py:117-194
 *                       + neighbour exchange rounds at the chunk end         neuralce/nce/mcmc.py:370-384
 *   nce_nce_local_delta setup()['local_delta'](cache, sig, flips)            neuralce/nce/mc_model.py:221-226,
 *                                                                            neuralce/nce/local_update_implicit.py:117-183
 *   nce_nce_commit      setup()['commit'](cache, patch, accept)             neuralce/nce/local_update_implicit.py:185-194
 *   nce_nce_accept      the driver's Metropolis rule on dE (mean over an     neuralce/nce/mcmc.py:167-185,
 *                       ensemble of models, seed_idx < 0)                    neuralce/nce/mc_model.py:181-188
 */
typedef struct {
    int32_t nB, J, mo, P, W, depth, C0, D, maxM, maxP, wL;
    int64_t d[3];
    int64_t n_cells;
    const int32_t *Rv_b;   /* (nB, J, mo) member basis of the reverse rows */
    const int32_t *Rv_uo;  /* (nB, J, mo, 3) */
    const int32_t *Rv_p;   /* (nB, J, mo) point-function index */
    const int32_t *Rv_col; /* (nB, J) cluster-vector column (channel = col + 1) */
    const uint8_t *Rv_m;   /* (nB, J, mo) member mask */
    const double *Rv_w;    /* (nB, J) nA / (order * count * n_cells * sd[col+1]); 0 for padded rows */
    const int32_t *Mb;     /* (nB) species per basis site */
    const double *theta;   /* (maxM+1, maxP, maxM) point functions */
    const int32_t *Sh_b;   /* (nB, P, W) shell partners */
    const int32_t *Sh_uo;  /* (nB, P, W, 3) */
    const uint8_t *Sh_m;   /* (nB, P, W) */
    const float *Sh_inv;   /* (nB, P) 1 / max(partners, 1) */
    const int32_t *ball_b; /* (nB, wL) receptive-field offsets, ordered by the level where they first appear */
    const int32_t *ball_uo;/* (nB, wL, 3) */
    const int32_t *ball_end; /* (nB, depth+1) end of each level in the ball lists */
    const float *lin;      /* (C0) layer-0 linear readout */
    const float *head_w;   /* (D) */
    double head_b;
    const float *W_cat[4]; /* per layer ((1+P)*Cin, D): [W_self; W_shell[0]; ...] */
    const float *bias[4];  /* (D) */
    const float *G_cat[4]; /* per layer (P*Cin, D) sigmoid-gate weights, or NULL */
    const float *gate_b[4];
    const float *mu, *sd;  /* (C0) standardisation of layer 0 */
    int32_t act;           /* 0 tanh (reference model), 1 SiLU */
    int32_t gate;          /* layers carry a sigmoid gate */
    double norm;           /* energy = sum(e) / norm + head_b: nA (site mean) or 1 (sum) */
    double scale_eV;       /* dE in eV = dE * scale_eV (ys * N for model.pkl, 1 for eV-valued models) */
    int32_t n_groups, max_gb;
    const int32_t *act_b, *act_nb; const uint64_t *grp_cum;   /* swap groups, as in nce_ce_tables */
    const uint16_t *Rv_loc;/* (nB, J, mo) index of each masked row member in its site's ball-0 list (ball_b/ball_uo order) */
    int32_t mma;           /* layer contractions: 0 float32 on CUDA cores; 1 bf16 operands on tensor cores (mma.sync,
                              float32 accumulation); 3 the same with each operand split into two bf16 terms
                              (hi*hi + hi*lo + lo*hi, near-float32 accuracy); 2 and 4 the bf16 and split forms on
                              the fifth-generation tensor cores (tcgen05: 128-site tiles, accumulator in tensor
                              memory).  Tensor-core forms need an ungated model.  Full caches and steps use the same
                              form, so a run samples one consistent energy. */
} nce_nce_desc;

typedef struct nce_nce_model *nce_nce_handle;

typedef struct {
    int32_t R; int64_t N;
    int8_t *sigma;         /* (R, N) */
    float *h0;             /* (R, N, C0) standardised layer 0 */
    float *hmid;           /* (depth-1, R, N, D) hidden layers 1..depth-1, or NULL for depth < 2 */
    float *e;              /* (R, N) per-site energy */
    double *E;             /* (R) energy: sum(e)/norm + head_b */
    const float *beta_slot; int32_t *rep_of_slot, *slot_of_rep; const int32_t *ladder_id;
    int64_t *n_acc, *n_ex;
    int64_t *n_near;       /* (R) or NULL: Metropolis steps whose margin |dE_eV + ln(u) / beta| was below the chunk's
                              near_eV (accept rule dE_eV <= 0 or u < exp(-beta dE_eV), neuralce/nce/mcmc.py:179) */
} nce_nce_state;

typedef struct {
    int64_t n_steps, step0;
    const int32_t *prop_a, *prop_b; const double *prop_u; /* (n_steps, R) or NULL -> Philox */
    uint64_t seed;
    int64_t sample_interval; double *E_samples;           /* (n_steps/si, R) or NULL */
    double *dE_out;        /* (n_steps, R) dE of every step (0 for same-species draws), or NULL */
    int32_t force;         /* 0 Metropolis, 1 accept every move, -1 reject every move */
    int32_t exchange_rounds; /* neighbour-slot exchange rounds at the chunk end (0 = none) */
    int32_t ex_parity; const double *ex_u; /* host-supplied exchange randoms: (rounds) parities packed in bits,
                                              ex_u (rounds, ceil((R-1)/2)); NULL -> Philox */
    int32_t cluster;       /* CTAs (SMs) per replica: 1, 2, 4 or 8 (thread-block cluster) */
    int32_t ctas_per_sm;   /* 0 or 1: one CTA per SM; 2: two CTAs per SM (at most 128 registers a thread, layer
                              weights read through L1; the CTA's shared memory must fit half an SM) */
    double near_eV;        /* near-threshold band of n_near; 0 = the form's stated dE error bound: 1e-4 eV (float32
                              and split-bf16 contractions), 1e-2 eV (bf16 contractions) */
} nce_nce_chunk;

int nce_nce_create(const nce_nce_desc *desc, nce_nce_handle *out);
int nce_nce_destroy(nce_nce_handle h);
int nce_nce_full_cache(nce_nce_handle h, const nce_nce_state *st, void *stream);
int nce_nce_run_chunk(nce_nce_handle h, const nce_nce_state *st, const nce_nce_chunk *ck, void *stream);
int nce_nce_errors(nce_nce_handle h, int32_t *flags);

/* Makes a tensor-core completion wait run out on purpose (one CTA: tensor memory and an mbarrier set up as in the
 * layer tiles, no MMA issued, the wait gives up after `limit` polls) and takes the layer tiles' way out of it: flag 32
 * in the handle's device error word (read with nce_nce_errors), abandoned work drained with a bounded wait, tensor
 * memory freed.  Tests the timeout path without faulting or hanging the GPU.  No counterpart in the reference. */
int nce_nce_tc_wait_selftest(nce_nce_handle h, int32_t limit, void *stream);

/* The reference's local_delta / commit pair on device data, one swap per replica.  nce_nce_local_delta evaluates,
 * for every replica r, the swap of sites prop_a[r] and prop_b[r] (device int32, indexed by replica) on the state's
 * caches without changing them: dE_out[r] (device float64, model units as in nce_nce_chunk.dE_out; 0 for two sites of
 * one species, NaN for a site outside the cell).  The evaluated rows are kept in the model's step scratch.
 * nce_nce_commit then applies the kept swap of every replica with accept[r] != 0 (device int32): caches, occupancy,
 * E += dE, n_acc += 1 (two sites of one species: only n_acc).  Each kept swap is consumed by the next commit; any
 * other call that runs steps on the same model handle (a chunk, another local_delta) replaces it. */
int nce_nce_local_delta(nce_nce_handle h, const nce_nce_state *st, const int32_t *prop_a, const int32_t *prop_b, double *dE_out,
                        void *stream);
int nce_nce_commit(nce_nce_handle h, const nce_nce_state *st, const int32_t *accept, void *stream);

/* Metropolis decisions from dE of n_models models (device float64 (n_models, R), model units, indexed by replica):
 * accept[r] = mean dE_eV <= 0 or u[r] < exp(-beta dE_eV), dE_eV = mean over models of dE * scale_eV, beta of the
 * replica's slot (beta_slot[slot_of_rep[r]]).  n_models > 1 is the reference's ensemble energy (mean over trained
 * seeds).  A NaN dE (a refused proposal) is rejected.  u (device, (R)) in (0, 1]; accept (device int32, (R)). */
int nce_nce_accept(const double *dE, int32_t n_models, int32_t R, double scale_eV, const float *beta_slot,
                   const int32_t *slot_of_rep, const double *u, int32_t *accept, void *stream);

/* Tensor-core tile GEMM of the NeuralCE layers (tcgen05, tensor-memory accumulator), exposed for testing:
 * C[M x N] = A[M x K] B[K x N], float32 row-major device arrays, operands rounded to bf16 (split != 0: bf16 hi/lo
 * pairs, hi*hi + hi*lo + lo*hi).  M a multiple of 128, N a multiple of 16 in [16, 256], K in [1, 256].
 * No counterpart in the reference (its layers are XLA matmuls, local_update_implicit.py:43-80). */
int nce_tc_gemm(const float *A, const float *B, float *C, int32_t M, int32_t N, int32_t K, int32_t split, void *stream);

/* ── Job server (serving form) ──────────────────────────────────────────────────────────────────────────────
 * A resident server that runs many parallel-tempering jobs at once.  Jobs are admitted in submission order as
 * device memory within the server's budget frees up (a later job that fits may start before an earlier one
 * that does not, unless the earlier one has waited longer than starve_s); their state stays on the device until
 * they finish.  Two host worker threads drive the GPU: one advances the running CE jobs with persistent batch
 * launches on eight lanes (streams), a job joining the next launch on an idle lane as soon as its previous one has
 * completed (continuous batching without a global round), the other each NeuralCE job's next chunk as soon as its
 * previous one has completed (a few streams), so the two kinds overlap on the device.  A job's chunks depend only on its own parameters,
 * so its result is the same alone and in any mix.  No call below waits for the device.
 * The reference has no serving mode; these entry points are new (they replace running neuralce-mc per job). */
typedef struct nce_server *nce_server_handle;

typedef struct {
    int64_t hbm_budget;    /* bytes of device memory for job state; 0 = 90% of the free memory at creation */
    int32_t max_batch;     /* CE jobs per persistent launch (1..64; 0 = 64) */
    int32_t precision;     /* CE dE precision, 32 (carried energies re-anchored exactly every chunk) or 64 */
    int32_t warps;         /* CE warps per replica (0 = 8) */
    int32_t nce_cluster;   /* NeuralCE CTAs per replica (0 = 1) */
    int32_t nce_streams;   /* NeuralCE streams (0 = 4) */
    double starve_s;       /* no job overtakes one that has waited this long (0 = 5 s) */
    int32_t ce_kernel;     /* 0 or 2: every CE job on the sign-parity kernel at `precision`; 3: jobs whose cell allows it
                              on the local-field kernel (exact fixed-point dE, fields of 8 bytes per site and replica
                              counted in the job's memory), the others on the sign-parity kernel */
    int32_t ce_lf_warps;   /* warps per replica of the local-field launches (0 = `warps`) */
} nce_server_config;

#define NCE_JOB_CE   0
#define NCE_JOB_NCE  1

typedef struct {
    int32_t kind;          /* NCE_JOB_CE (model = nce_ce_handle) or NCE_JOB_NCE (model = nce_nce_handle) */
    void *model;           /* must stay valid until the job has finished or been cancelled */
    int32_t R;
    const int8_t *sigma;   /* host (R, N) initial occupancies (copied at submission unless flags borrow them) */
    const float *beta_slot;/* host (R) */
    const int32_t *ladder_id; /* host (R) or NULL (one ladder) */
    int64_t n_steps;       /* MC steps per replica */
    int64_t exchange_every;/* steps between slot exchanges = chunk length (> 0) */
    uint64_t seed;         /* Philox key of the job's proposals and exchanges */
    int32_t reanchor_chunks; /* NeuralCE: full cache rebuild every this many chunks (0 = ceil(N / exchange_every)) */
    /* host outputs, written before the job is reported done (any may be NULL) */
    int8_t *sigma_out;     /* (R, N) */
    double *E_out;         /* (R) */
    int64_t *n_acc_out;    /* (R) */
    int32_t *rep_of_slot_out; /* (R) */
    int64_t *n_ex_out;     /* (1) */
    int32_t flags;         /* NCE_JOB_BORROW_SIGMA: `sigma` is read in place when the job is admitted instead of being
                              copied at submission; the caller keeps it unchanged until the job has finished, failed or
                              been cancelled (in page-locked memory the upload is one direct copy) */
} nce_job_desc;

#define NCE_JOB_BORROW_SIGMA 1

#define NCE_JOB_QUEUED     0
#define NCE_JOB_RUNNING    1
#define NCE_JOB_DONE       2
#define NCE_JOB_CANCELLED  3
#define NCE_JOB_FAILED     4

typedef struct {
    int32_t status;        /* NCE_JOB_* */
    int32_t error;         /* NCE_ERR_* of a failed job */
    int64_t steps_done, n_steps;
    int64_t device_bytes;  /* device memory the job holds while it runs */
    double t_submit, t_start, t_end;   /* seconds on the server's clock (steady, from creation); -1 if not yet */
} nce_job_info;

typedef struct {
    int64_t queued, running, done, cancelled, failed;
    int64_t bytes_used, hbm_budget;
    int64_t rounds_ce, rounds_nce;     /* CE batch launches completed; NeuralCE chunks completed */
    int64_t attempts;      /* swap attempts completed (replicas x steps) */
    double now;            /* server clock */
} nce_server_stats;

int nce_server_create(const nce_server_config *cfg, nce_server_handle *out);
int nce_server_destroy(nce_server_handle s);         /* cancels what is left and joins the workers */
/* NCE_ERR_NOMEM when the job can never fit the budget; NCE_ERR_INVALID for bad descriptors. */
int nce_job_submit(nce_server_handle s, const nce_job_desc *job, int64_t *job_id);
int nce_job_poll(nce_server_handle s, int64_t job_id, nce_job_info *info);
int nce_job_cancel(nce_server_handle s, int64_t job_id);
int nce_server_query(nce_server_handle s, nce_server_stats *stats);
/* text of the error that failed a job */
int nce_job_error(nce_server_handle s, int64_t job_id, char *buf, size_t n);

/* Philox4x32-10 on the host (same function the kernels use), for tests and host drivers. */
void nce_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif /* NCE_GB300_H */
