// Cluster-expansion parallel-tempering engine for GB300 (sm_103a).
//
// Kernels
//   ce_pt_chunk_kernel  one CTA per replica (of one or many jobs): for every step of a chunk it draws or
//                       reads the swap proposal, gathers the occupancy of the two sites' neighbourhoods
//                       (n_nbr entries each, integer lattice arithmetic on the SNF coordinates), evaluates
//                       every reverse row of both sites with warp-parallel products of point functions,
//                       reduces dE with warp shuffles, applies the Metropolis rule and writes the two sites.
//                       Row tables are staged in shared memory once per chunk.
//   ce_exchange_kernel  chunk-end replica exchange of temperature slots (one CTA per job).
//   ce_energy_kernel    full energy: cells x template rows, per-block float64 partials, fixed-order sum.
//   ce_delta_kernel     batched swap dE queries through the same block routine as the chunk kernel.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cooperative_groups.h>
#include <type_traits>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace nce {

constexpr int kMaxJobs = 64;

struct CEJob {
    // tables (device)
    const uint16_t *loc;   // (nB, J, mo)
    const uint8_t *pfc;    // (nB, J, mo)
    const void *eci;       // (nB, J) double or float
    const int32_t *rv_len; // (nB)
    const int32_t *nb_b;   // (nB, n_nbr)
    const int32_t *nb_uo;  // (nB, n_nbr, 3)
    const void *pf;        // (n_pfc, max_sp) double or float
    const int32_t *act_b;  // (n_groups, max_gb)
    const int32_t *act_nb; // (n_groups)
    const uint64_t *grp_cum;
    int32_t nB, J, n_nbr, n_pfc, max_sp, n_groups, max_gb;
    int32_t d0, d1, d2;
    int64_t n_cells, N;
    // state
    int8_t *sigma; double *E; const float *beta_slot; int32_t *slot_of_rep;
    double *E_min_rep; int64_t *n_acc;
    int32_t R;
    // chunk
    int64_t n_steps, step0;
    const int64_t *step_dev;   // device step counter (overrides step0) or null
    const int32_t *prop_a, *prop_b; const double *prop_u;
    uint64_t seed;
    int64_t sample_interval; double *E_samples;
    int32_t cta_base;      // first CTA of this job
    int32_t *err;          // device error word
    const uint8_t *sbits;  // (n_pfc, 4) sign bit of each point-function value (sign-parity kernel)
    const uint16_t *bix;   // (nB, J, mo) pfc * n_nbr + loc of each member (sign-parity kernel)
    const uint8_t *rcol;   // (nB, J) cluster-vector column of each reverse row
    const void *ecol2;     // (n_cols) 2 * eci of each column, double or float
    int32_t n_cols;
    const uint32_t *chunks;// (nB, max_chunks) column-aligned row chunks: col | start << 8 | len << 24
    const int32_t *n_chunks; // (nB)
    int32_t max_chunks;
    int32_t sig_smem;      // this job's occupancy is copied into shared memory for the chunk
    int64_t *cv;           // (R, n_cols) tracked cluster-vector sums or null
    const int64_t *ecol_fix; // (n_cols) 2 eci of each column in fixed point (x 2^fix_shift), float64 kernels
    int32_t fix_shift;
    int64_t *n_near;       // (R) near-threshold step counts or null
    double near_eV;        // near-threshold band (eV)
    int64_t near_fix;      // the band in fixed point, rounded up, plus one unit (threshold rounding), fixed-point kernels
    // local-field kernel
    int64_t *field;        // (R, N) G of every site (fixed point, x 2^fix_shift)
    const int32_t *lf_off; // (nB, n_nbr + 1) start of each neighbour's row list
    const uint16_t *lf_idx;// rows of the site containing that neighbour as a member
    const int16_t *lf_box; // (nB, 2e0+1, 2e1+1, 2e2+1, nB) neighbour index of a displacement, or -1
    int32_t lf_e0, lf_e1, lf_e2, lf_nidx;
    int32_t gf_smem;       // this job's occupancy and field are copied into shared memory for the chunk
    // chunk-end exchange inside the chunk kernel (fused_chunk_end), when ex_sync is set
    int32_t *rep_of_slot; const int32_t *ladder_id; int64_t *n_ex; const double *ex_u;
    int32_t *ex_sync;      // replicas of the job done with the chunk (0 between chunks)
    int32_t ex_flags;      // bit 0: the chunk ends on an exchange; bit 1: host parity (with ex_u)
};

struct CEBatch {
    int32_t n_jobs;
    int32_t tables_in_smem;
    CEJob job[kMaxJobs];
};
static_assert(sizeof(CEBatch) <= 32764, "the batch descriptor is passed by value: kernel parameters hold 32,764 bytes");

struct CEShared {          // per-step control block (shared memory)
    int64_t ia, ib;
    double u;
    int32_t valid, near, b_a, b_b;
    int32_t ka[3], kb[3];
    int32_t sa, sb;
};

template <typename Real>
struct Layout {            // offsets of the dynamic shared-memory regions
    size_t loc, pfc, eci, vals, hit, red, total;
    __host__ __device__ static Layout make(int nB, int J, int mo, int n_nbr, int n_pfc, int nwarps, bool tables) {
        Layout L; size_t o = 0;
        auto al = [](size_t x, size_t a) { return (x + a - 1) / a * a; };
        if (tables) {
            L.loc = o; o = al(o + sizeof(uint16_t) * (size_t)nB * J * mo, 16);
            L.pfc = o; o = al(o + (size_t)nB * J * mo, 16);
            L.eci = o; o = al(o + sizeof(Real) * (size_t)nB * J, 16);
        } else {
            L.loc = L.pfc = L.eci = 0;
        }
        L.vals = o; o = al(o + sizeof(Real) * 4 * (size_t)n_pfc * n_nbr, 16);
        L.hit = o; o = al(o + (size_t)n_nbr, 16);
        L.red = o; o = al(o + sizeof(Real) * 32, 16);
        L.total = o;
        return L;
    }
};

__device__ __forceinline__ int32_t wrap_add(int32_t k, int32_t u, int32_t d) {
    int32_t q = k + u;
    return q >= d ? q - d : q;
}

__device__ __forceinline__ void site_coords(const CEJob &jb, int64_t i, int32_t &b, int32_t k[3]) {
    b = (int32_t)(i % jb.nB);
    int64_t c = i / jb.nB;
    int64_t d12 = (int64_t)jb.d1 * jb.d2;
    k[0] = (int32_t)(c / d12);
    k[1] = (int32_t)((c / jb.d2) % jb.d1);
    k[2] = (int32_t)(c % jb.d2);
}

template <typename Real>
__device__ __forceinline__ Real warp_sum(Real v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Gathers both neighbourhoods into shared value tables, then sums the reverse rows of both sites.
// Must be called by all threads of the block with cs (ia, ib, sa, sb, b_a, b_b, ka, kb, valid) set.
// Returns dE in thread 0 (other threads: undefined).  Contains three __syncthreads.
template <typename Real, int MO>
__device__ Real block_delta(const CEJob &jb, const int8_t *__restrict__ sig, CEShared &cs, unsigned char *smem,
                            const Layout<Real> &L, const uint16_t *tloc, const uint8_t *tpfc, const Real *teci) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n_nbr = jb.n_nbr, n_pfc = jb.n_pfc, max_sp = jb.max_sp;
    Real *vals = reinterpret_cast<Real *>(smem + L.vals);     // [side][old/new][pfc][n_nbr]
    uint8_t *hit = smem + L.hit;
    Real *red = reinterpret_cast<Real *>(smem + L.red);
    const Real *pf = reinterpret_cast<const Real *>(jb.pf);
    const int64_t ia = cs.ia, ib = cs.ib;
    const int sa_new = cs.sb, sb_new = cs.sa;
    // 1. neighbourhood gather
    int near_local = 0;
    for (int t = tid; t < 2 * n_nbr; t += nt) {
        const int side = t >= n_nbr, n = side ? t - n_nbr : t;
        const int b0 = side ? cs.b_b : cs.b_a;
        const int32_t *k = side ? cs.kb : cs.ka;
        const int e = b0 * n_nbr + n;
        const int32_t *uo = jb.nb_uo + 3 * e;
        int32_t q0 = wrap_add(k[0], __ldg(uo + 0), jb.d0);
        int32_t q1 = wrap_add(k[1], __ldg(uo + 1), jb.d1);
        int32_t q2 = wrap_add(k[2], __ldg(uo + 2), jb.d2);
        int64_t s = (((int64_t)q0 * jb.d1 + q1) * jb.d2 + q2) * jb.nB + __ldg(jb.nb_b + e);
        int so = sig[s];
        int sn = (s == ia) ? sa_new : ((s == ib) ? sb_new : so);
        Real *vo = vals + (size_t)(2 * side) * n_pfc * n_nbr;
        Real *vn = vo + (size_t)n_pfc * n_nbr;
        for (int c = 0; c < n_pfc; ++c) {
            vo[c * n_nbr + n] = pf[c * max_sp + so];
            vn[c * n_nbr + n] = pf[c * max_sp + sn];
        }
        if (side) { hit[n] = (s == ia); near_local |= (s == ia); }
    }
    const int near = __syncthreads_or(near_local);
    // 2. rows
    Real acc = Real(0);
    const int Ja = __ldg(jb.rv_len + cs.b_a), Jb = __ldg(jb.rv_len + cs.b_b);
    for (int side = 0; side < 2; ++side) {
        const int b0 = side ? cs.b_b : cs.b_a;
        const int Jn = side ? Jb : Ja;
        const uint16_t *loc = tloc + (size_t)b0 * jb.J * MO;
        const uint8_t *pfc = tpfc + (size_t)b0 * jb.J * MO;
        const Real *eci = teci + (size_t)b0 * jb.J;
        const Real *vo = vals + (size_t)(2 * side) * n_pfc * n_nbr;
        const Real *vn = vo + (size_t)n_pfc * n_nbr;
        const bool check = side && near;
        for (int r = tid; r < Jn; r += nt) {
            Real po = Real(1), pn = Real(1);
            bool skip = false;
#pragma unroll
            for (int m = 0; m < MO; ++m) {
                const int l = loc[(size_t)r * MO + m];
                const int c = pfc[(size_t)r * MO + m];
                po *= vo[c * n_nbr + l];
                pn *= vn[c * n_nbr + l];
                if (check) skip |= hit[l] != 0;
            }
            if (!skip) acc += eci[r] * (pn - po);
        }
    }
    acc = warp_sum(acc);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    Real dE = Real(0);
    if (tid == 0) {
        const int nw = (nt + 31) >> 5;
        for (int w = 0; w < nw; ++w) dE += red[w];
    }
    return dE;
}

// Stage (or point at) the job's row tables.
template <typename Real>
__device__ void stage_tables(const CEJob &jb, bool in_smem, unsigned char *smem, const Layout<Real> &L, int MO,
                             const uint16_t *&tloc, const uint8_t *&tpfc, const Real *&teci) {
    const size_t nl = (size_t)jb.nB * jb.J * MO, ne = (size_t)jb.nB * jb.J;
    if (!in_smem) {
        tloc = jb.loc; tpfc = jb.pfc; teci = reinterpret_cast<const Real *>(jb.eci);
        return;
    }
    uint16_t *sl = reinterpret_cast<uint16_t *>(smem + L.loc);
    uint8_t *sp = smem + L.pfc;
    Real *se = reinterpret_cast<Real *>(smem + L.eci);
    for (size_t i = threadIdx.x; i < nl; i += blockDim.x) { sl[i] = __ldg(jb.loc + i); sp[i] = __ldg(jb.pfc + i); }
    const Real *ge = reinterpret_cast<const Real *>(jb.eci);
    for (size_t i = threadIdx.x; i < ne; i += blockDim.x) se[i] = ge[i];
    tloc = sl; tpfc = sp; teci = se;
    __syncthreads();
}

__device__ __forceinline__ int find_job(const CEBatch &bt, int cta) {
    int j = 0;
    while (j + 1 < bt.n_jobs && cta >= bt.job[j + 1].cta_base) ++j;
    return j;
}

// job j's descriptor into shared memory (all threads of the CTA; synchronises)
__device__ __forceinline__ void copy_job(const CEBatch &bt, int j, CEJob &dst) {
    static_assert(sizeof(CEJob) % 4 == 0, "the descriptor is copied in 4-byte words");
    const int *src = reinterpret_cast<const int *>(&bt.job[j]);
    int *d = reinterpret_cast<int *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(CEJob) / 4); i += blockDim.x) d[i] = src[i];
    __syncthreads();
}

// proposal of slot t at global step g (same layout as the C oracle)
__device__ __forceinline__ void propose(const CEJob &jb, int64_t g, int32_t t, int64_t &ia, int64_t &ib, double &u) {
    const uint32_t k0 = (uint32_t)jb.seed, k1 = (uint32_t)(jb.seed >> 32);
    const uint32_t c0 = (uint32_t)g, c1 = (uint32_t)((uint64_t)g >> 32);
    u32x4 x = philox4x32(c0, c1, (uint32_t)t, 0u, k0, k1);
    int grp = 0; uint32_t ba = 0, bb = 0;
    if (jb.n_groups > 1 || __ldg(jb.act_nb) > 1) {
        u32x4 y = philox4x32(c0, c1, (uint32_t)t, 1u, k0, k1);
        if (jb.n_groups > 1)
            while (grp < jb.n_groups - 1 && (uint64_t)y.x >= __ldg(jb.grp_cum + grp)) ++grp;
        const uint32_t nb = (uint32_t)__ldg(jb.act_nb + grp);
        ba = draw_index(y.y, nb); bb = draw_index(y.z, nb);
    }
    const uint32_t nc = (uint32_t)jb.n_cells;
    ia = (int64_t)draw_index(x.x, nc) * jb.nB + __ldg(jb.act_b + grp * jb.max_gb + ba);
    ib = (int64_t)draw_index(x.y, nc) * jb.nB + __ldg(jb.act_b + grp * jb.max_gb + bb);
    u = draw_u01(x.z, x.w);
}

// Chunk end, called by one thread of each replica (the cluster's first CTA) once its outputs are written: the last
// replica of the job to arrive performs the job's slot exchange -- the rule, random counters and sample rewrite of
// ce_exchange_kernel, with the pairs swapped in place -- advances the device step counter and re-arms the counter.
// No thread waits for another, so the chunk kernel never depends on its CTAs running at the same time.
__device__ void fused_chunk_end(const CEJob &jb, int64_t g0) {
    __threadfence();                                      // this replica's energy is visible before it is counted
    if (atomicAdd(jb.ex_sync, 1) != jb.R - 1) return;
    __threadfence();
    const int R = jb.R;
    const int64_t g_end = g0 + jb.n_steps;
    if (jb.step_dev) *const_cast<int64_t *>(jb.step_dev) = g_end;   // every CTA of the job has read it by now
    if ((jb.ex_flags & 1) && R > 1) {
        const uint32_t k0 = (uint32_t)jb.seed, k1 = (uint32_t)(jb.seed >> 32);
        const uint32_t c0 = (uint32_t)g_end, c1 = (uint32_t)((uint64_t)g_end >> 32);
        const uint32_t cq = 0xFFFFFFFFu;                   // round 0 of the exchange counters
        const int parity = jb.ex_u ? ((jb.ex_flags >> 1) & 1) : (int)(philox4x32(c0, c1, cq, 0u, k0, k1).x & 1u);
        int32_t *ros = jb.rep_of_slot;
        int64_t nswap = 0;
        for (int k = 0; 2 * k < R - 1; ++k) {
            const int a = 2 * k + parity, b = a + 1;
            if (b >= R || jb.ladder_id[a] != jb.ladder_id[b]) continue;
            const double Ea = __ldcg(jb.E + __ldcg(ros + a)), Eb = __ldcg(jb.E + __ldcg(ros + b));
            const double log_acc = ((double)jb.beta_slot[b] - (double)jb.beta_slot[a]) * (Eb - Ea);
            double u;
            if (jb.ex_u) u = jb.ex_u[k];
            else { const u32x4 w = philox4x32(c0, c1, cq - 1u, (uint32_t)k, k0, k1); u = draw_u01(w.x, w.y); }
            if (log(u) < log_acc) { const int32_t x = ros[a]; ros[a] = ros[b]; ros[b] = x; ++nswap; }
        }
        for (int q = 0; q < R; ++q) jb.slot_of_rep[ros[q]] = q;
        *jb.n_ex += nswap;
        if (jb.E_samples && jb.n_steps > 0 && jb.n_steps % jb.sample_interval == 0) {
            const int64_t row = jb.n_steps / jb.sample_interval - 1;
            for (int q = 0; q < R; ++q) jb.E_samples[row * R + q] = __ldcg(jb.E + ros[q]);
        }
    }
    *jb.ex_sync = 0;
}

template <typename Real, int MO>
__global__ void __launch_bounds__(1024) ce_pt_chunk_kernel(const __grid_constant__ CEBatch bt) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CEShared cs;
    const int j = find_job(bt, blockIdx.x);
    const CEJob &jb = bt.job[j];
    const int r = blockIdx.x - jb.cta_base;
    if (r >= jb.R) return;
    const Layout<Real> L = Layout<Real>::make(jb.nB, jb.J, MO, jb.n_nbr, jb.n_pfc, blockDim.x >> 5, bt.tables_in_smem);
    const uint16_t *tloc; const uint8_t *tpfc; const Real *teci;
    stage_tables<Real>(jb, bt.tables_in_smem, smem, L, MO, tloc, tpfc, teci);
    int8_t *sig = jb.sigma + (int64_t)r * jb.N;
    const int32_t t = jb.slot_of_rep[r];
    const double beta = (double)jb.beta_slot[t];
    double E = jb.E[r], Emin = jb.E_min_rep[r];
    int64_t nacc = 0, nnear = 0;
    const int R = jb.R;
    const int64_t g0 = jb.step_dev ? *jb.step_dev : jb.step0;
    for (int64_t s = 0; s < jb.n_steps; ++s) {
        if (threadIdx.x == 0) {
            int64_t ia, ib; double u;
            if (jb.prop_a) {
                ia = jb.prop_a[s * R + t]; ib = jb.prop_b[s * R + t]; u = jb.prop_u[s * R + t];
            } else {
                propose(jb, g0 + s, t, ia, ib, u);
            }
            int valid = 0;
            if (ia < 0 || ib < 0 || ia >= jb.N || ib >= jb.N) {
                atomicOr(jb.err, 1);                 // out-of-range proposal: rejected, flagged
            } else {
                cs.sa = sig[ia]; cs.sb = sig[ib];
                valid = cs.sa != cs.sb;
            }
            cs.ia = ia; cs.ib = ib; cs.u = u; cs.valid = valid;
            if (valid) { site_coords(jb, ia, cs.b_a, cs.ka); site_coords(jb, ib, cs.b_b, cs.kb); }
        }
        __syncthreads();
        if (cs.valid) {
            Real dE = block_delta<Real, MO>(jb, sig, cs, smem, L, tloc, tpfc, teci);
            if (threadIdx.x == 0) {
                const double dEd = (double)dE;
                if (beta > 0.0 && fabs(dEd + log(cs.u) / beta) < jb.near_eV) ++nnear;
                if (log(cs.u) < -beta * dEd) {
                    sig[cs.ia] = (int8_t)cs.sb; sig[cs.ib] = (int8_t)cs.sa;
                    E += dEd; ++nacc;
                }
            }
        }
        if (threadIdx.x == 0) {
            Emin = fmin(Emin, E);
            if (jb.E_samples && (s + 1) % jb.sample_interval == 0)
                jb.E_samples[((s + 1) / jb.sample_interval - 1) * R + t] = E;
        }
    }
    if (threadIdx.x == 0) {
        jb.E[r] = E; jb.E_min_rep[r] = Emin; jb.n_acc[r] += nacc;
        if (jb.n_near) jb.n_near[r] += nnear;
        if (jb.ex_sync) fused_chunk_end(jb, g0);
    }
}

// ── sign-parity kernel for point functions in {-1, +1} ───────────────────────────────────────────────
// Binary orthonormal point functions take the values -1 / +1 (and 1 for padded members), so every row product
// is a sign: Pi = (-1)^p with p the XOR of one bit per member.  Per neighbourhood entry the kernel keeps, for each
// point-function column, the bit of the old species (bit 0), of the new species (bit 1) and, for the second
// site, whether the entry is the first site (bit 2).  A row's member bytes are XOR-ed (parities) and OR-ed
// (contains the first site); dPi = (-1)^p_new - (-1)^p_old is 0 or +-2 exactly.  All rows of one cluster-vector
// column share one eci, so dE = sum over columns of 2 eci_c * n_c with n_c the exact integer sum of the rows'
// +-1 parity changes; the reverse rows of a site are ordered by column, so each warp folds its 32 consecutive
// rows with a segmented scan and adds one integer per column run.  Products and the column sum run in the
// kernel's precision (float64 or float32); the counts are exact.
struct BinProp {
    int64_t ia, ib; double logu;
    int64_t thr;                  // fixed-point acceptance threshold: accept iff dE * 2^S < thr (float64 kernels)
    int32_t ka[3], kb[3], ba, bb;
};

constexpr int kBinNchTab = 64;                          // bases up to which the chunk counts are kept on chip
struct BinLayout {
    size_t bix, chunk, nb, ecol, sig, bits, cnt, dcv, total;
    __host__ __device__ static BinLayout make(int nB, int J, int mo, int n_nbr, int n_pfc, int n_cols, int max_chunks, size_t acc_bytes,
                                                int64_t N, bool tables, bool sig_smem) {
        BinLayout L; size_t o = 0;
        auto al = [](size_t x, size_t a) { return (x + a - 1) / a * a; };
        if (tables) {
            L.bix = o; o = al(o + sizeof(uint16_t) * (size_t)nB * J * mo, 16);
        } else {
            L.bix = 0;
        }
        L.chunk = o; o = al(o + sizeof(uint32_t) * (size_t)nB * max_chunks, 16);
        L.nb = o; o = al(o + sizeof(int32_t) * 4 * (size_t)nB * n_nbr, 16);
        L.ecol = o; o = al(o + acc_bytes * (size_t)n_cols, 16);
        if (sig_smem) { L.sig = o; o = al(o + (size_t)N, 16); } else { L.sig = 0; }
        L.bits = o; o = al(o + (size_t)2 * n_pfc * n_nbr, 16);             // [side][pfc][n_nbr]
        L.cnt = o; o = al(o + sizeof(int32_t) * 2 * (size_t)n_cols, 16);   // [buffer parity][n_cols]
        L.dcv = o; o = al(o + sizeof(int32_t) * (size_t)n_cols, 16);       // chunk change of the cluster-vector sums
        L.total = o;
        return L;
    }
};

__device__ __forceinline__ void site_coords32(const CEJob &jb, int64_t i, int32_t &b, int32_t k[3]) {
    const uint32_t ii = (uint32_t)i, nB = (uint32_t)jb.nB, d1 = (uint32_t)jb.d1, d2 = (uint32_t)jb.d2;
    const uint32_t c = ii / nB;
    b = (int32_t)(ii - c * nB);
    const uint32_t c12 = c / d2;
    k[2] = (int32_t)(c - c12 * d2);
    k[0] = (int32_t)(c12 / d1);
    k[1] = (int32_t)(c12 - (uint32_t)k[0] * d1);
}

__device__ __forceinline__ void bin_propose(const CEJob &jb, int64_t g0, int64_t s, int32_t t, BinProp &P) {
    int64_t ia, ib; double u;
    if (jb.prop_a) {
        ia = jb.prop_a[s * jb.R + t]; ib = jb.prop_b[s * jb.R + t]; u = jb.prop_u[s * jb.R + t];
    } else {
        propose(jb, g0 + s, t, ia, ib, u);
    }
    if (ia < 0 || ib < 0 || ia >= jb.N || ib >= jb.N) {
        atomicOr(jb.err, 1);
        ia = ib = 0;                                   // same site -> same species -> rejected step
    }
    P.ia = ia; P.ib = ib; P.logu = log(u);
    if (jb.fix_shift > 0) {
        // logu < -beta dE  <=>  dE < -logu / beta (beta > 0)  <=>  dE 2^S < ceil(-logu / beta 2^S)
        const double beta = (double)jb.beta_slot[t];
        if (beta > 0.0) {
            const double xs = -P.logu / beta * ldexp(1.0, jb.fix_shift);
            P.thr = xs >= 4.611686018427388e18 ? (int64_t)4611686018427387904ll : (int64_t)ceil(xs);
        } else {
            P.thr = P.logu < 0.0 ? (int64_t)4611686018427387904ll : -(int64_t)4611686018427387904ll;
        }
    } else {
        P.thr = 0;
    }
    site_coords32(jb, ia, P.ba, P.ka); site_coords32(jb, ib, P.bb, P.kb);
}

template <typename Acc, int MO, bool CLUSTER, bool SMT>
__global__ void __launch_bounds__(1024) ce_bin_chunk_kernel(const __grid_constant__ CEBatch bt, int32_t sig_budget) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ BinProp prop[64];                      // ring of two batches of 32 proposals
    __shared__ int32_t near_flag[2];                  // per evaluated-swap parity
    // CLUSTER: one replica per thread-block cluster; every CTA keeps its own copy of the replica's occupancy and draws
    // the same proposals, and the row chunks are split over the CTAs.  With a cluster in fixed point (float64):
    // every warp adds its chunks' exact partial dE into the evaluated swap's accumulator of every CTA of the
    // cluster, and after the cluster barrier every warp of every CTA reads the total and reaches the same decision;
    // the accumulators alternate between evaluated swaps and each CTA clears its previous one after the next step's
    // first barrier.  The accepted swap is written to the occupancy by one thread; until the next barrier every
    // thread reads the two sites through the swap it holds in registers, so no barrier follows the decision.
    // Otherwise (one CTA per replica, or float32): each CTA counts its chunks per column, after the barrier the
    // decision warp sums the columns in a fixed order (reading every CTA's counts through distributed shared memory
    // with a cluster), and a barrier ends the evaluated step; a count buffer is cleared by its owner only after the
    // next cluster barrier.
    int CL = 1, rank = 0;
    if (CLUSTER) { cg::cluster_group cl = cg::this_cluster(); CL = (int)cl.num_blocks(); rank = (int)cl.block_rank(); }
    const int rep_idx = blockIdx.x / CL;
    const int j = find_job(bt, rep_idx);
    // the job's descriptor in shared memory: kernel-parameter reads at a computed job index go through the constant
    // cache, which the batch descriptor (up to 31 KB) overflows, and the step loop reads the descriptor throughout
    __shared__ CEJob sjob;
    copy_job(bt, j, sjob);
    const CEJob &jb = sjob;
    const int r = rep_idx - jb.cta_base;
    if (r >= jb.R) return;
    const int tid = threadIdx.x, nt = blockDim.x, nw = nt >> 5, lane = tid & 31, warp = tid >> 5;
    const int ncons = nw > 1 ? nw - 1 : 1;            // consumer warps; the last warp (when there are two or more) draws proposals
    const bool producer = nw > 1 ? (warp == nw - 1) : (tid == 0);
    const int n_nbr = jb.n_nbr, n_pfc = jb.n_pfc, n_cols = jb.n_cols;
    const int32_t sig_smem = jb.sig_smem;
    const BinLayout L = BinLayout::make(jb.nB, jb.J, MO, n_nbr, n_pfc, n_cols, jb.max_chunks, sizeof(Acc), sig_budget, SMT,
                                        sig_budget > 0);
    // SMT (the launch's tables fit in shared memory): the member table is staged there, and the compiler sees a
    // shared-memory pointer (32-bit addresses, shared loads); otherwise it is read from global memory
    const uint16_t *tbix;
    const size_t nl = (size_t)jb.nB * jb.J * MO;
    if (SMT) {
        uint16_t *sb = reinterpret_cast<uint16_t *>(smem + L.bix);
        for (size_t i = tid; i < nl; i += nt) sb[i] = __ldg(jb.bix + i);
        tbix = sb;
    } else {
        tbix = jb.bix;
    }
    uint32_t *chunks = reinterpret_cast<uint32_t *>(smem + L.chunk);        // [basis][k]: col | start << 8 | len << 24
    for (int i = tid; i < jb.nB * jb.max_chunks; i += nt) chunks[i] = __ldg(jb.chunks + i);
    // chunks per basis site, read by every evaluated swap: from shared memory, not a global load on the step's path
    __shared__ uint16_t nch[kBinNchTab];
    for (int i = tid; i < jb.nB && i < kBinNchTab; i += nt) nch[i] = (uint16_t)__ldg(jb.n_chunks + i);
    int4 *nbt = reinterpret_cast<int4 *>(smem + L.nb);                          // [basis][n]: (uo0, uo1, uo2, basis)
    for (int i = tid; i < jb.nB * n_nbr; i += nt) nbt[i] = make_int4(__ldg(jb.nb_uo + 3 * i), __ldg(jb.nb_uo + 3 * i + 1),
                                                                      __ldg(jb.nb_uo + 3 * i + 2), __ldg(jb.nb_b + i));
    Acc *ecol = reinterpret_cast<Acc *>(smem + L.ecol);
    const Acc *gecol = reinterpret_cast<const Acc *>(jb.ecol2);
    int32_t *cnt = reinterpret_cast<int32_t *>(smem + L.cnt);      // [parity][n_cols]
    int32_t *dcv = reinterpret_cast<int32_t *>(smem + L.dcv);
    const bool track = jb.cv != nullptr;
    for (int c = tid; c < n_cols; c += nt) { ecol[c] = gecol[c]; cnt[c] = 0; cnt[n_cols + c] = 0; dcv[c] = 0; }
    __shared__ long long pslot[2];                    // fixed-point dE accumulator of the evaluated swap [parity]
    int8_t *gsig = jb.sigma + (int64_t)r * jb.N;
    int8_t *sig = sig_smem ? reinterpret_cast<int8_t *>(smem + L.sig) : gsig;
    if (sig_smem)
        for (int64_t i = tid; i < jb.N; i += nt) sig[i] = gsig[i];
    uint8_t *bits = smem + L.bits;                         // [side][pfc][n_nbr]
    uint32_t smask = 0;                                    // sign bit of (point-function column c, species q) at c*4+q
    for (int c = 0; c < n_pfc; ++c)
        for (int q = 0; q < 4; ++q) smask |= (uint32_t)(__ldg(jb.sbits + c * 4 + q) & 1u) << (c * 4 + q);
    const int32_t t = jb.slot_of_rep[r];
    const double beta = (double)jb.beta_slot[t];
    // float64: the step's dE is an exact fixed-point integer sum (x 2^S); the chunk's energy change and its running
    // minimum are kept in it and turned into float64 at the samples and at the end (from the chunk's first energy,
    // which no one writes before the end of the chunk); float32 carries the energy
    constexpr bool FIX = std::is_same<Acc, double>::value;
    constexpr bool fix = FIX;                            // float64 launches need fixed point (checked on the host)
    // fixed point over a cluster: per-warp partial dE into every CTA's accumulator, the decision in every thread
    constexpr bool wsum = CLUSTER && fix;
    double E = fix ? 0.0 : jb.E[r], Emin = fix ? 0.0 : jb.E_min_rep[r];
    auto fixed_energy = [&](long long d) -> double { return jb.E[r] + (double)d * ldexp(1.0, -jb.fix_shift); };
    long long dsum = 0, dmin = 0;
    long long *efix = reinterpret_cast<long long *>(ecol);
    if (fix) {
        __syncthreads();                                   // ecol (float64) was just written; the same bytes take the fixed-point values
        for (int c = tid; c < n_cols; c += nt) efix[c] = (long long)__ldg(jb.ecol_fix + c);
    }
    int32_t nacc = 0, nnear = 0;                           // a chunk has fewer than 2^31 steps (checked on the host)
    int32_t scd = (int32_t)min(jb.sample_interval, jb.n_steps + 1), srow = 0;   // steps to the next sample, rows written
    const int R = jb.R;
    // proposals are drawn 32 at a time (one per lane of the producer warp), one batch ahead of their use
    const int64_t g0 = jb.step_dev ? *jb.step_dev : jb.step0;
    if (tid < 2) { near_flag[tid] = 0; pslot[tid] = 0; }
    if (warp == 0 && lane < jb.n_steps) bin_propose(jb, g0, lane, t, prop[lane]);
    __syncthreads();
    if (CLUSTER) cg::this_cluster().sync();              // every CTA's counters are zero before any remote add
    // counter buffer of the current evaluated swap: alternates between swaps that reach the row phase, so that a
    // cluster barrier always separates a CTA's clearing of a buffer from the next remote add into it
    int par = 0;
    // the last accepted swap, not yet covered by a barrier (fixed-point form): sites and their new species
    uint32_t pnd_a = 0xffffffffu, pnd_b = 0xffffffffu; int pnd_sa = 0, pnd_sb = 0;
    auto occ = [&](uint32_t i) -> int {
        return i == pnd_a ? pnd_sa : (i == pnd_b ? pnd_sb : (int)sig[i]);
    };
    const int32_t n_steps = (int32_t)jb.n_steps;
    for (int32_t s = 0; s < n_steps; ++s) {
        // a step whose two sites hold the same species changes nothing and passes no barrier; every 32 steps one
        // barrier lets the producer refill the half of the ring that the last 32 steps used
        if ((s & 31) == 0) {
            __syncthreads();
            pnd_a = pnd_b = 0xffffffffu;                   // the occupancy holds every accepted swap
            if (nw == 1 ? true : warp == nw - 1) {         // draw the next batch (steps s+32 .. s+63)
                const int32_t q = s + 32 + lane;
                if (q < n_steps) bin_propose(jb, g0, q, t, prop[q & 63]);
            }
        }
        const BinProp &P = prop[s & 63];
        int32_t *cntp = cnt + par * n_cols;
        const uint32_t ia = (uint32_t)P.ia, ib = (uint32_t)P.ib;        // sites are below 2^32
        const int64_t thr = P.thr;
        if (!sig_smem && s + 1 < n_steps && ((s + 1) & 31) != 0) {
            // occupancy in global memory (cells beyond the shared-memory budget): the next step's two
            // neighbourhoods are fetched into L2 while this step runs, one site a consumer thread (a step's first
            // reads would otherwise wait on DRAM).  Only within a batch of 32 steps: the next batch's slots are
            // visible after the barrier that opens it, and the slot of step s + 1 is not refilled before step s + 33
            const BinProp &Q = prop[(s + 1) & 63];
            for (int q = tid; q < 2 * n_nbr && tid < ncons * 32; q += ncons * 32) {
                const int side = q >= n_nbr, n = side ? q - n_nbr : q;
                const int32_t *k = side ? Q.kb : Q.ka;
                const int4 nbe = nbt[(side ? Q.bb : Q.ba) * n_nbr + n];
                const uint32_t st = ((((uint32_t)wrap_add(k[0], nbe.x, jb.d0) * (uint32_t)jb.d1 + (uint32_t)wrap_add(k[1], nbe.y, jb.d1)) *
                                      (uint32_t)jb.d2 + (uint32_t)wrap_add(k[2], nbe.z, jb.d2)) * (uint32_t)jb.nB + (uint32_t)nbe.w);
                asm volatile("prefetch.global.L2 [%0];" :: "l"(gsig + st));
            }
        }
        const int sa = occ(ia), sb = occ(ib);
        if (sa != sb) {
            const int sa_new = sb, sb_new = sa;
            // 1. neighbourhood bits (consumer threads); near_flag[par] was cleared two evaluated swaps ago
            const int ct = ncons * 32;
            for (int q = tid; q < 2 * n_nbr && tid < ct; q += ct) {
                const int side = q >= n_nbr, n = side ? q - n_nbr : q;
                const int b0 = side ? P.bb : P.ba;
                const int32_t *k = side ? P.kb : P.ka;
                const int4 nbe = nbt[b0 * n_nbr + n];
                const uint32_t st = ((((uint32_t)wrap_add(k[0], nbe.x, jb.d0) * (uint32_t)jb.d1 + (uint32_t)wrap_add(k[1], nbe.y, jb.d1)) *
                                      (uint32_t)jb.d2 + (uint32_t)wrap_add(k[2], nbe.z, jb.d2)) * (uint32_t)jb.nB + (uint32_t)nbe.w);
                const int so = occ(st);
                const int sn = (st == (uint32_t)ia) ? sa_new : ((st == (uint32_t)ib) ? sb_new : so);
                const int isa = side && (st == (uint32_t)ia);
                if (isa) near_flag[par] = 1;
                uint8_t *bs = bits + (size_t)side * n_pfc * n_nbr;
                for (int c = 0; c < n_pfc; ++c)
                    bs[c * n_nbr + n] = (uint8_t)(((smask >> (c * 4 + so)) & 1u) | (((smask >> (c * 4 + sn)) & 1u) << 1) | (isa << 2));
            }
        }
        if (sa != sb) {
            __syncthreads();
            pnd_a = pnd_b = 0xffffffffu;                   // the occupancy now holds every accepted swap
            const int sa_new = sb, sb_new = sa;
            if (wsum && tid == 0) pslot[par ^ 1] = 0;      // every warp of the cluster has read it (before this barrier)
            long long pw = 0;                              // this warp's exact partial dE (fixed point)
            if (!producer || nw == 1) {
                // 2. rows: column-aligned chunks of <= 32 rows (one lane per row); one integer reduction per chunk
                // per-side bases held in registers for the loop (shared-memory atomics below could alias the
                // descriptor and proposal, which would otherwise be re-read every chunk)
                const int ba = P.ba, bb = P.bb;
                const int nca = jb.nB <= kBinNchTab ? (int)nch[ba] : __ldg(jb.n_chunks + ba);
                const int ncb = jb.nB <= kBinNchTab ? (int)nch[bb] : __ldg(jb.n_chunks + bb);
                const bool near = near_flag[par] != 0;
                const int cw = nw > 1 ? warp : 0;
                const int maxc = jb.max_chunks, J = jb.J;
                const int offa = ba * maxc, offb = bb * maxc;            // chunk k of side a / side b
                const uint16_t *rwa = tbix + (size_t)ba * J * MO, *rwb = tbix + (size_t)bb * J * MO;
                const uint8_t *bsb = bits + (size_t)n_pfc * n_nbr;
                // a rows loop per kind of step: with the other site in the neighbourhood (near) the rows of b that
                // contain a were counted with a and are skipped; otherwise no row needs that test
                auto rows = [&](auto near_c) {
                    constexpr bool NEAR = decltype(near_c)::value;
                    // chunk k of one side: the sign of each row's change, one lane per row
                    auto chunk_count = [&](auto side_c, int k, int &col) -> int {
                        constexpr bool SIDE = decltype(side_c)::value;
                        const uint32_t d = chunks[(SIDE ? offb : offa) + k];
                        col = (int)(d & 0xffu);
                        const int start = (int)((d >> 8) & 0xffffu), len = (int)(d >> 24);
                        int sgn = 0;
                        if (lane < len) {
                            const uint16_t *bx = (SIDE ? rwb : rwa) + (start + lane) * MO;
                            const uint8_t *bs = SIDE ? bsb : bits;
                            unsigned x = 0, y = 0;
                            if (MO == 4) {
                                const uint2 w = *reinterpret_cast<const uint2 *>(bx);
                                const unsigned v0 = bs[w.x & 0xffffu], v1 = bs[w.x >> 16], v2 = bs[w.y & 0xffffu], v3 = bs[w.y >> 16];
                                x = v0 ^ v1 ^ v2 ^ v3;
                                if (NEAR && SIDE) y = v0 | v1 | v2 | v3;
                            } else {
#pragma unroll
                                for (int m = 0; m < MO; ++m) { const unsigned vv = bs[bx[m]]; x ^= vv; if (NEAR && SIDE) y |= vv; }
                            }
                            const bool skip = NEAR && SIDE && (y & 4u);
                            if (!skip && ((x ^ (x >> 1)) & 1u)) sgn = (x & 1u) ? 1 : -1;   // odd old parity: Pi -1 -> +1
                        }
                        return sgn;
                    };
                    // the consumer warps of the whole cluster are split between the two sides in proportion to their
                    // chunks; a warp takes its side's chunks round-robin, two at a time
                    const int gw = rank * ncons + cw, gstr = ncons * CL;
                    auto side_loop = [&](auto side_c, int n, int k0, int stride) {
                        for (int k = k0; k < n; k += 2 * stride) {
                            const int k2 = k + stride;
                            int c1 = 0, c2 = 0;
                            const int s1 = chunk_count(side_c, k, c1);
                            const int s2 = k2 < n ? chunk_count(side_c, k2, c2) : 0;
                            const int n1 = (int)__reduce_add_sync(0xffffffffu, (unsigned)s1);
                            const int n2 = (int)__reduce_add_sync(0xffffffffu, (unsigned)s2);
                            if (wsum) pw += (long long)n1 * efix[c1] + (long long)n2 * efix[c2];
                            if (lane == 0 && (!wsum || track)) {
                                if (n1) atomicAdd(&cntp[c1], n1);
                                if (n2) atomicAdd(&cntp[c2], n2);
                            }
                        }
                    };
                    if (gstr >= 2) {
                        // (equal sides, as in every swap of a one-site basis: half the warps, without a division)
                        const int wa = nca == ncb ? (gstr + 1) >> 1
                                                  : min(gstr - 1, max(1, (gstr * nca + (nca + ncb) / 2) / max(1, nca + ncb)));
                        if (gw < wa) side_loop(std::false_type{}, nca, gw, wa);
                        else side_loop(std::true_type{}, ncb, gw - wa, gstr - wa);
                    } else {
                        side_loop(std::false_type{}, nca, 0, 1);
                        side_loop(std::true_type{}, ncb, 0, 1);
                    }
                };
                if (near) rows(std::true_type{}); else rows(std::false_type{});
                if (wsum && pw != 0 && lane < CL)           // lane q adds into CTA q's accumulator
                    atomicAdd(reinterpret_cast<unsigned long long *>(cg::this_cluster().map_shared_rank(pslot + par, lane)),
                              (unsigned long long)pw);
            }
            if (CLUSTER) cg::this_cluster().sync(); else __syncthreads();
            // 3. dE = sum_c 2 eci_c n_c, accept, write
            if (wsum) {
                // every thread takes the decision; one thread writes the occupancy and the statistics
                const long long part = pslot[par];
                const bool accept = part < thr;
                if (accept) { pnd_a = ia; pnd_b = ib; pnd_sa = sa_new; pnd_sb = sb_new; }
                if (tid == 0) {
                    const long long dd = part - thr;       // near the threshold: |dE 2^S - (-ln u / beta) 2^S| below the band
                    nnear += (dd < 0 ? -dd : dd) < (long long)jb.near_fix;
                    near_flag[par] = 0;
                    if (accept) { sig[ia] = (int8_t)sa_new; sig[ib] = (int8_t)sb_new; dsum += part; ++nacc; }
                }
                if (track && warp == 0)                    // each changed row moves its column's sum by +-2
                    for (int c = lane; c < n_cols; c += 32) {
                        const int n = cntp[c];
                        if (n) { if (accept) dcv[c] += 2 * n; cntp[c] = 0; }
                    }
            } else if (warp == 0) {
                // this swap's count of column c, summed over the cluster's CTAs
                auto count = [&](int c) -> int {
                    if (!CLUSTER) return cntp[c];
                    int n = 0;
                    for (int q = 0; q < CL; ++q) n += *cg::this_cluster().map_shared_rank(cntp + c, q);
                    return n;
                };
                if (CLUSTER)                            // every CTA has read the other buffer (previous swap) by now
                    for (int c = lane; c < n_cols; c += 32) cnt[(par ^ 1) * n_cols + c] = 0;
                bool accept;
                if (fix) {
                    long long part = 0;
                    for (int c = lane; c < n_cols; c += 32) {
                        const int n = count(c);
                        if (n) { part += (long long)n * efix[c]; if (!track) cntp[c] = 0; }
                    }
                    // exact warp sum of |part| < 2^61 in three 21-bit slices (hardware 32-bit reductions, no carries lost)
                    const unsigned l0 = (unsigned)(part & 0x1fffff), l1 = (unsigned)((part >> 21) & 0x1fffff);
                    const int l2 = (int)(part >> 42);
                    const unsigned s0 = __reduce_add_sync(0xffffffffu, l0), s1 = __reduce_add_sync(0xffffffffu, l1);
                    const int s2 = __reduce_add_sync(0xffffffffu, l2);
                    part = (long long)s0 + ((long long)s1 << 21) + ((long long)s2 << 42);
                    accept = part < thr;
                    if (lane == 0) {                    // near the threshold: |dE 2^S - (-ln u / beta) 2^S| below the band
                        const long long dd = part - thr;
                        nnear += (dd < 0 ? -dd : dd) < (long long)jb.near_fix;
                        near_flag[par] = 0;
                    }
                    if (lane == 0 && accept) {
                        sig[ia] = (int8_t)sa_new; sig[ib] = (int8_t)sb_new;
                        dsum += part; ++nacc;
                    }
                } else {
                    Acc part = Acc(0);
                    for (int c = lane; c < n_cols; c += 32) {
                        const int n = count(c);
                        if (n) { part += ecol[c] * (Acc)n; if (!track && !CLUSTER) cntp[c] = 0; }
                    }
                    part = warp_sum(part);              // butterfly: every lane holds the same sum
                    const double dEd = (double)part;
                    accept = P.logu < -beta * dEd;     // the float form's barrier at the step end keeps P intact
                    if (lane == 0 && beta > 0.0) nnear += fabs(dEd + P.logu / beta) < jb.near_eV;
                    if (lane == 0) near_flag[par] = 0;
                    if (lane == 0 && accept) {
                        sig[ia] = (int8_t)sa_new; sig[ib] = (int8_t)sb_new;
                        E += dEd; ++nacc;
                    }
                }
                if (track)                              // each changed row moves its column's sum by +-2
                    for (int c = lane; c < n_cols; c += 32) {
                        const int n = count(c);
                        if (n) { if (accept) dcv[c] += 2 * n; if (!CLUSTER) cntp[c] = 0; }
                    }
            }
            if (!wsum) __syncthreads();                    // the decision warp has written the occupancy
            par ^= 1;
        }
        if (tid == 0) {
            if (fix) dmin = dsum < dmin ? dsum : dmin;
            else Emin = fmin(Emin, E);
            if (--scd == 0) {                              // a sample every sample_interval steps
                scd = (int32_t)jb.sample_interval;
                if (rank == 0 && jb.E_samples) jb.E_samples[(int64_t)srow * R + t] = fix ? fixed_energy(dsum) : E;
                ++srow;
            }
        }
    }
    __syncthreads();                                       // every accepted swap is in the occupancy
    if (fix && tid == 0) {
        E = fixed_energy(dsum);
        Emin = jb.n_steps > 0 ? fmin(jb.E_min_rep[r], fixed_energy(dmin)) : jb.E_min_rep[r];
    }
    if (track && wsum)                                   // every CTA adds the changes its own rows counted
        for (int c = tid; c < n_cols; c += nt)
            if (dcv[c]) atomicAdd(reinterpret_cast<unsigned long long *>(jb.cv + (int64_t)r * n_cols + c),
                                  (unsigned long long)(long long)dcv[c]);
    if (rank == 0) {
        if (sig_smem)
            for (int64_t i = tid; i < jb.N; i += nt) gsig[i] = sig[i];
        if (track && !wsum)
            for (int c = tid; c < n_cols; c += nt) jb.cv[(int64_t)r * n_cols + c] += dcv[c];
        if (sig_smem || track) __syncthreads();          // the replica's outputs are written before it is counted
        if (tid == 0) {
            jb.E[r] = E; jb.E_min_rep[r] = Emin; jb.n_acc[r] += nacc;
            if (jb.n_near) jb.n_near[r] += nnear;
            if (jb.ex_sync) fused_chunk_end(jb, g0);
        }
    }
    if (CLUSTER) cg::this_cluster().sync();              // no CTA leaves while others may still add into its counters
}

// ── local-field kernel ───────────────────────────────────────────────────────────────────────────────
// Every site i of a replica carries its field G(i) = sum over the reverse rows r of i of 2 eci_r Pi_r, in the
// float64 kernels' fixed point (x 2^S, exact integers).  Flipping one site negates every product it is a member of,
// so a swap of a and b (different species) changes the energy by
//     dE = -G(a) - G(b) + 2 C(a, b),   C(a, b) = sum over the rows of a that also contain b of 2 eci Pi,
// which is exactly the sum the sign-parity kernel forms (-2 eci Pi_old over the rows containing one of the two
// sites), as the same integers.  C is non-zero only when b lies in a's neighbourhood: an O(1) lookup of the
// displacement (a box of k-space offsets) names b's neighbourhood entry, and the rows of a that contain that entry
// are listed per entry (lf_off / lf_idx).  A rejected swap changes nothing, so warp 0 evaluates the next 32 steps
// at once, one per lane, on the same state: every step before the first accepted one is rejected as evaluated, and
// the first accepted one is exact too; steps after it are evaluated again in the next round.  Near pairs (C to
// compute) are resolved in step order by the whole warp.  Only an accepted swap costs the block: both sites' rows
// are evaluated once (parity change per row, as the sign-parity kernel), and each neighbour's field moves by the
// sum of its changed rows' 2 eci dPi; the two sites' own fields become -G + 2C.
struct LfLayout {
    size_t bix, rcol, chunk, nb, efix, off, idx, box, v, bits, nbits, dcv, fld, sig, total;
    __host__ __device__ static LfLayout make(int nB, int J, int mo, int n_nbr, int n_pfc, int n_cols, int max_chunks, int nidx,
                                             int boxsz, int64_t budget_sites, bool tables) {
        LfLayout L; size_t o = 0;
        auto al = [](size_t x, size_t a) { return (x + a - 1) / a * a; };
        if (tables) {
            L.bix = o; o = al(o + sizeof(uint16_t) * (size_t)nB * J * mo, 16);
            L.rcol = o; o = al(o + (size_t)nB * J, 16);
        } else {
            L.bix = L.rcol = 0;
        }
        L.chunk = o; o = al(o + sizeof(uint32_t) * (size_t)nB * max_chunks, 16);
        L.nb = o; o = al(o + sizeof(int4) * (size_t)nB * n_nbr, 16);
        L.efix = o; o = al(o + sizeof(long long) * (size_t)n_cols, 16);
        L.off = o; o = al(o + sizeof(int32_t) * (size_t)nB * (n_nbr + 1), 16);
        L.idx = o; o = al(o + sizeof(uint16_t) * (size_t)nidx, 16);
        L.box = o; o = al(o + sizeof(int16_t) * (size_t)nB * boxsz * nB, 16);
        L.v = o; o = al(o + sizeof(long long) * 2 * (size_t)J, 16);                 // [side][row] 2 eci dPi (fixed point)
        L.bits = o; o = al(o + (size_t)2 * n_pfc * n_nbr, 16);                      // [side][pfc][n_nbr] old | new << 1
        L.nbits = o; o = al(o + (size_t)n_pfc * n_nbr, 16);                         // decider: old bits of one neighbourhood
        L.dcv = o; o = al(o + sizeof(int32_t) * (size_t)n_cols, 16);
        if (budget_sites > 0) {
            L.fld = o; o = al(o + sizeof(long long) * (size_t)budget_sites, 16);
            L.sig = o; o = al(o + (size_t)budget_sites, 16);
        } else {
            L.fld = L.sig = 0;
        }
        L.total = o;
        return L;
    }
};

struct LfStep {                          // the accepted swap, published by the decider warp to the block
    int64_t ia, ib;
    long long C;
    int32_t ka[3], kb[3], ba, bb, sa, sb, go;
};

// neighbourhood entry of site (bb, kb) in the neighbourhood of (ba, ka), or -1 (not a neighbour)
__device__ __forceinline__ int lf_lookup(const CEJob &jb, const int16_t *box, int ba, const int32_t ka[3], int bb,
                                         const int32_t kb[3]) {
    int x0 = kb[0] - ka[0], x1 = kb[1] - ka[1], x2 = kb[2] - ka[2];
    x0 += x0 < 0 ? jb.d0 : 0; x1 += x1 < 0 ? jb.d1 : 0; x2 += x2 < 0 ? jb.d2 : 0;
    x0 -= x0 > jb.d0 / 2 ? jb.d0 : 0; x1 -= x1 > jb.d1 / 2 ? jb.d1 : 0; x2 -= x2 > jb.d2 / 2 ? jb.d2 : 0;
    if (x0 < -jb.lf_e0 || x0 > jb.lf_e0 || x1 < -jb.lf_e1 || x1 > jb.lf_e1 || x2 < -jb.lf_e2 || x2 > jb.lf_e2) return -1;
    const int w1 = 2 * jb.lf_e1 + 1, w2 = 2 * jb.lf_e2 + 1, bsz = (2 * jb.lf_e0 + 1) * w1 * w2;
    const int cell = ((x0 + jb.lf_e0) * w1 + (x1 + jb.lf_e1)) * w2 + (x2 + jb.lf_e2);
    return box[((size_t)ba * bsz + cell) * jb.nB + bb];
}

__device__ __forceinline__ uint32_t lf_site(const CEJob &jb, const int32_t k[3], const int4 nbe) {
    return (((uint32_t)wrap_add(k[0], nbe.x, jb.d0) * (uint32_t)jb.d1 + (uint32_t)wrap_add(k[1], nbe.y, jb.d1)) *
            (uint32_t)jb.d2 + (uint32_t)wrap_add(k[2], nbe.z, jb.d2)) * (uint32_t)jb.nB + (uint32_t)nbe.w;
}

// exact warp sum of int64 terms whose total stays below 2^61 in magnitude (three 21-bit slices)
__device__ __forceinline__ long long warp_sum_i64(long long part) {
    const unsigned l0 = (unsigned)(part & 0x1fffff), l1 = (unsigned)((part >> 21) & 0x1fffff);
    const int l2 = (int)(part >> 42);
    const unsigned s0 = __reduce_add_sync(0xffffffffu, l0), s1 = __reduce_add_sync(0xffffffffu, l1);
    const int s2 = __reduce_add_sync(0xffffffffu, l2);
    return (long long)s0 + ((long long)s1 << 21) + ((long long)s2 << 42);
}

// proposal of a local-field step: the sites and their coordinates as the other kernels draw them, and the uniform
// kept as its 53 random bits (u = (m + 1) 2^-53) with ln u in float32 for the filter of the Metropolis test
struct LfProp {
    int64_t ia, ib;
    uint64_t um;                     // Philox: the uniform's 53 bits
    double uh;                       // host stream: the uniform itself (-1 for Philox)
    float lnu;
    int32_t ka[3], kb[3], ba, bb;
};

__device__ __forceinline__ void lf_propose(const CEJob &jb, int64_t g0, int64_t s, int32_t t, LfProp &P) {
    int64_t ia, ib;
    uint64_t m = 0;
    double uh = -1.0;
    if (jb.prop_a) {
        ia = jb.prop_a[s * jb.R + t]; ib = jb.prop_b[s * jb.R + t];
        uh = jb.prop_u[s * jb.R + t];
    } else {
        const uint32_t k0 = (uint32_t)jb.seed, k1 = (uint32_t)(jb.seed >> 32);
        const uint32_t c0 = (uint32_t)(g0 + s), c1 = (uint32_t)((uint64_t)(g0 + s) >> 32);
        const u32x4 x = philox4x32(c0, c1, (uint32_t)t, 0u, k0, k1);
        int grp = 0; uint32_t ba = 0, bb = 0;
        if (jb.n_groups > 1 || __ldg(jb.act_nb) > 1) {
            const u32x4 y = philox4x32(c0, c1, (uint32_t)t, 1u, k0, k1);
            if (jb.n_groups > 1)
                while (grp < jb.n_groups - 1 && (uint64_t)y.x >= __ldg(jb.grp_cum + grp)) ++grp;
            const uint32_t nb = (uint32_t)__ldg(jb.act_nb + grp);
            ba = draw_index(y.y, nb); bb = draw_index(y.z, nb);
        }
        const uint32_t nc = (uint32_t)jb.n_cells;
        ia = (int64_t)draw_index(x.x, nc) * jb.nB + __ldg(jb.act_b + grp * jb.max_gb + ba);
        ib = (int64_t)draw_index(x.y, nc) * jb.nB + __ldg(jb.act_b + grp * jb.max_gb + bb);
        m = ((uint64_t)x.z << 21) | (uint64_t)(x.w >> 11);  // draw_u01's 53 bits
    }
    if (ia < 0 || ib < 0 || ia >= jb.N || ib >= jb.N) { atomicOr(jb.err, 1); ia = ib = 0; }   // rejected no-op
    P.ia = ia; P.ib = ib; P.um = m; P.uh = uh;
    P.lnu = __logf(uh >= 0.0 ? (float)uh : (float)(m + 1ull) * 1.1102230246251565e-16f);
    site_coords32(jb, ia, P.ba, P.ka); site_coords32(jb, ib, P.bb, P.kb);
}

// Metropolis decision of dE = part 2^-S: accept iff ln u < -beta dE (the reference's rule) with the fixed-point
// threshold ceil(-ln u / beta 2^S) of the other float64 kernels.  float32 settles it when |beta dE + ln u| exceeds
// 1e-6 + 1e-6 (|beta dE| + |ln u|), far above float32's error on these terms and above beta times any near-threshold
// band; otherwise the threshold is formed in float64 (rare).  near: |part - threshold| below the band.
__device__ __forceinline__ bool lf_accept(const CEJob &jb, long long part, const LfProp &P, float beta_f, double beta,
                                          float scale_f, bool &near) {
    const float bd = beta_f * ((float)part * scale_f);
    const float y = bd + P.lnu;
    const float tol = 1e-6f + 1e-6f * (fabsf(bd) + fabsf(P.lnu));
    near = false;
    if (y < -tol) return true;
    if (y > tol) return false;
    const double logu = log(P.uh >= 0.0 ? P.uh : (double)(P.um + 1ull) * 1.1102230246251565404236316680908203125e-16);
    long long thr;
    if (beta > 0.0) {
        const double xs = -logu / beta * ldexp(1.0, jb.fix_shift);
        thr = xs >= 4.611686018427388e18 ? 4611686018427387904ll : (long long)ceil(xs);
    } else {
        thr = logu < 0.0 ? 4611686018427387904ll : -4611686018427387904ll;
    }
    const long long dd = part - thr;
    near = (dd < 0 ? -dd : dd) < (long long)jb.near_fix;
    return part < thr;
}

constexpr int kLfMaxWarps = 16;                            // the decider's registers: at most 512 threads a CTA

template <int MO>
__global__ void __launch_bounds__(32 * kLfMaxWarps) ce_lf_chunk_kernel(const __grid_constant__ CEBatch bt, int32_t budget) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ LfStep X;
    const int j = find_job(bt, blockIdx.x);
    __shared__ CEJob sjob;                            // the descriptor in shared memory (see ce_bin_chunk_kernel)
    copy_job(bt, j, sjob);
    const CEJob &jb = sjob;
    const int r = blockIdx.x - jb.cta_base;
    if (r >= jb.R) return;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int n_nbr = jb.n_nbr, n_pfc = jb.n_pfc, n_cols = jb.n_cols, J = jb.J;
    const int bsz = (2 * jb.lf_e0 + 1) * (2 * jb.lf_e1 + 1) * (2 * jb.lf_e2 + 1);
    const LfLayout L = LfLayout::make(jb.nB, J, MO, n_nbr, n_pfc, n_cols, jb.max_chunks, jb.lf_nidx, bsz, budget,
                                      bt.tables_in_smem);
    const uint16_t *tbix; const uint8_t *trcol;
    const size_t nl = (size_t)jb.nB * J * MO, ne = (size_t)jb.nB * J;
    if (bt.tables_in_smem) {
        uint16_t *sb = reinterpret_cast<uint16_t *>(smem + L.bix); uint8_t *sc = smem + L.rcol;
        for (size_t i = tid; i < nl; i += nt) sb[i] = __ldg(jb.bix + i);
        for (size_t i = tid; i < ne; i += nt) sc[i] = __ldg(jb.rcol + i);
        tbix = sb; trcol = sc;
    } else {
        tbix = jb.bix; trcol = jb.rcol;
    }
    int4 *nbt = reinterpret_cast<int4 *>(smem + L.nb);
    for (int i = tid; i < jb.nB * n_nbr; i += nt) nbt[i] = make_int4(__ldg(jb.nb_uo + 3 * i), __ldg(jb.nb_uo + 3 * i + 1),
                                                                      __ldg(jb.nb_uo + 3 * i + 2), __ldg(jb.nb_b + i));
    long long *efix = reinterpret_cast<long long *>(smem + L.efix);
    for (int c = tid; c < n_cols; c += nt) efix[c] = (long long)__ldg(jb.ecol_fix + c);
    int32_t *loff = reinterpret_cast<int32_t *>(smem + L.off);
    for (int i = tid; i < jb.nB * (n_nbr + 1); i += nt) loff[i] = __ldg(jb.lf_off + i);
    uint16_t *lidx = reinterpret_cast<uint16_t *>(smem + L.idx);
    for (int i = tid; i < jb.lf_nidx; i += nt) lidx[i] = __ldg(jb.lf_idx + i);
    int16_t *box = reinterpret_cast<int16_t *>(smem + L.box);
    for (int i = tid; i < jb.nB * bsz * jb.nB; i += nt) box[i] = __ldg(jb.lf_box + i);
    long long *v = reinterpret_cast<long long *>(smem + L.v);
    uint8_t *bits = smem + L.bits, *nbits = smem + L.nbits;
    int32_t *dcv = reinterpret_cast<int32_t *>(smem + L.dcv);
    for (int c = tid; c < n_cols; c += nt) dcv[c] = 0;
    const bool track = jb.cv != nullptr;
    int8_t *gsig = jb.sigma + (int64_t)r * jb.N;
    long long *gfld = reinterpret_cast<long long *>(jb.field) + (int64_t)r * jb.N;
    int8_t *sig = jb.gf_smem ? reinterpret_cast<int8_t *>(smem + L.sig) : gsig;
    long long *G = jb.gf_smem ? reinterpret_cast<long long *>(smem + L.fld) : gfld;
    if (jb.gf_smem)
        for (int64_t i = tid; i < jb.N; i += nt) { sig[i] = gsig[i]; G[i] = gfld[i]; }
    uint32_t smask = 0;
    for (int c = 0; c < n_pfc; ++c)
        for (int q = 0; q < 4; ++q) smask |= (uint32_t)(__ldg(jb.sbits + c * 4 + q) & 1u) << (c * 4 + q);
    const int32_t t = jb.slot_of_rep[r];
    const float beta_f = jb.beta_slot[t];
    const double beta = (double)beta_f;
    const double E0c = jb.E[r];
    double Emin = jb.E_min_rep[r];
    const double fscale = ldexp(1.0, -jb.fix_shift);
    const float scale_f = ldexpf(1.0f, -jb.fix_shift);
    const int64_t g0 = jb.step_dev ? *jb.step_dev : jb.step0;
    const int64_t T = jb.n_steps;
    const int64_t si = jb.sample_interval;
    long long dsum = 0, dmin = 0;                          // warp 0: the chunk's energy change and its running minimum
    int64_t nacc = 0, s_cur = 0;
    unsigned nnear = 0;                                    // warp 0, per lane: near-threshold steps it decided
    const int nrow_a_max = 2 * J;
    __syncthreads();
    for (;;) {
        if (warp == 0) {
            if (lane == 0) X.go = 0;
            __syncwarp();
            while (s_cur < T) {
                const int64_t s = s_cur + lane;
                const bool live = s < T;
                LfProp P;
                int sa = 0, sb = 0, nbi = -1, valid = 0;
                long long part = 0;
                if (live) {
                    lf_propose(jb, g0, s, t, P);
                    sa = sig[P.ia]; sb = sig[P.ib];
                    valid = sa != sb;
                    if (valid) {
                        nbi = lf_lookup(jb, box, P.ba, P.ka, P.bb, P.kb);
                        part = -(G[P.ia] + G[P.ib]);
                    }
                }
                bool near = false;
                bool acc = valid && nbi < 0 && lf_accept(jb, part, P, beta_f, beta, scale_f, near);
                const unsigned farm = __ballot_sync(0xffffffffu, acc);
                const unsigned nearm = __ballot_sync(0xffffffffu, valid && nbi >= 0);
                int first = farm ? __ffs(farm) - 1 : 32;
                unsigned pend = nearm & (first < 32 ? ((1u << first) - 1u) : 0xffffffffu);
                long long Cq = 0;
                while (pend) {                             // near pairs before the first far acceptance, in step order
                    const int q = __ffs(pend) - 1;
                    const int qba = __shfl_sync(0xffffffffu, P.ba, q), qnb = __shfl_sync(0xffffffffu, nbi, q);
                    int32_t qk[3];
                    for (int c = 0; c < 3; ++c) qk[c] = __shfl_sync(0xffffffffu, P.ka[c], q);
                    for (int n = lane; n < n_nbr; n += 32) {  // old bits of a's neighbourhood
                        const int so = sig[lf_site(jb, qk, nbt[qba * n_nbr + n])];
                        for (int c = 0; c < n_pfc; ++c) nbits[c * n_nbr + n] = (uint8_t)((smask >> (c * 4 + so)) & 1u);
                    }
                    __syncwarp();
                    long long cp = 0;
                    const int o0 = loff[qba * (n_nbr + 1) + qnb], o1 = loff[qba * (n_nbr + 1) + qnb + 1];
                    for (int k = o0 + lane; k < o1; k += 32) {
                        const int rr = lidx[k];
                        const uint16_t *bx = tbix + ((size_t)qba * J + rr) * MO;
                        unsigned x = 0;
#pragma unroll
                        for (int m = 0; m < MO; ++m) x ^= nbits[bx[m]];
                        const long long e = efix[trcol[(size_t)qba * J + rr]];
                        cp += (x & 1u) ? -e : e;
                    }
                    const long long C = warp_sum_i64(cp);
                    __syncwarp();
                    if (lane == q) { Cq = C; part += 2 * C; acc = lf_accept(jb, part, P, beta_f, beta, scale_f, near); }
                    if (__shfl_sync(0xffffffffu, (int)acc, q)) { first = q; break; }
                    pend &= pend - 1;
                }
                const int avail = (int)(T - s_cur < 32 ? T - s_cur : 32);
                const bool accepted = first < avail;
                const int n_adv = accepted ? first + 1 : avail;
                const long long dfirst = __shfl_sync(0xffffffffu, part, first & 31);
                if (lane < n_adv && valid) nnear += near;
                if (jb.E_samples && lane < n_adv && (s + 1) % si == 0) {
                    const long long da = dsum + ((accepted && lane == first) ? dfirst : 0);
                    jb.E_samples[((s + 1) / si - 1) * jb.R + t] = E0c + (double)da * fscale;
                }
                s_cur += n_adv;
                if (accepted) {
                    dsum += dfirst; dmin = dsum < dmin ? dsum : dmin; ++nacc;
                    if (lane == first) {
                        X.ia = P.ia; X.ib = P.ib; X.C = Cq; X.ba = P.ba; X.bb = P.bb; X.sa = sa; X.sb = sb;
                        for (int c = 0; c < 3; ++c) { X.ka[c] = P.ka[c]; X.kb[c] = P.kb[c]; }
                        X.go = 1;
                    }
                    break;
                }
            }
        }
        __syncthreads();
        if (!X.go) break;
        // ── accepted swap: the rows of both sites, then the neighbours' fields ──
        const int64_t ia = X.ia, ib = X.ib;
        for (int q = tid; q < 2 * n_nbr; q += nt) {
            const int side = q >= n_nbr, n = side ? q - n_nbr : q;
            const uint32_t st = lf_site(jb, side ? X.kb : X.ka, nbt[(side ? X.bb : X.ba) * n_nbr + n]);
            const int so = sig[st];
            const int sn = (st == (uint32_t)ia) ? X.sb : ((st == (uint32_t)ib) ? X.sa : so);
            uint8_t *bs = bits + (size_t)side * n_pfc * n_nbr;
            for (int c = 0; c < n_pfc; ++c)
                bs[c * n_nbr + n] = (uint8_t)(((smask >> (c * 4 + so)) & 1u) | (((smask >> (c * 4 + sn)) & 1u) << 1));
        }
        __syncthreads();
        {
            // every row of both sites, four per thread in flight: 2 eci dPi (dPi = 2 sgn), column sums when tracked
            const int Ja = __ldg(jb.rv_len + X.ba), Jb = __ldg(jb.rv_len + X.bb), nrow = Ja + Jb;
            for (int q0 = tid; q0 < nrow; q0 += 4 * nt) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int q = q0 + u * nt;
                    if (q >= nrow) break;
                    const int side = q >= Ja, rr = side ? q - Ja : q;
                    const int b0 = side ? X.bb : X.ba;
                    const uint16_t *bx = tbix + ((size_t)b0 * J + rr) * MO;
                    const uint8_t *bs = bits + (size_t)side * n_pfc * n_nbr;
                    unsigned x = 0;
#pragma unroll
                    for (int m = 0; m < MO; ++m) x ^= bs[bx[m]];
                    int sgn = 0;
                    if ((x ^ (x >> 1)) & 1u) sgn = (x & 1u) ? 1 : -1;
                    const int col = trcol[(size_t)b0 * J + rr];
                    v[side * J + rr] = sgn ? 2 * sgn * efix[col] : 0;
                    if (track && sgn) atomicAdd(&dcv[col], 2 * sgn);
                }
            }
        }
        __syncthreads();
        {
            // each neighbour's field: the sum of its changed rows, four lanes per neighbour entry
            const int grp = tid >> 2, gl = tid & 3, ngrp = nt >> 2, ntask = 2 * (n_nbr - 1);
            for (int task0 = 0; task0 < ntask; task0 += ngrp) {
                const int task = task0 + grp;
                long long sum = 0;
                int side = 0, n = 1;
                if (task < ntask) {
                    side = task >= n_nbr - 1; n = 1 + (side ? task - (n_nbr - 1) : task);
                    const int b0 = side ? X.bb : X.ba;
                    const int o0 = loff[b0 * (n_nbr + 1) + n], o1 = loff[b0 * (n_nbr + 1) + n + 1];
                    const long long *vs = v + side * J;
                    long long s0 = 0, s1 = 0;
                    int k = o0 + gl;
                    for (; k + 4 < o1; k += 8) { s0 += vs[lidx[k]]; s1 += vs[lidx[k + 4]]; }
                    if (k < o1) s0 += vs[lidx[k]];
                    sum = s0 + s1;
                }
                sum += __shfl_xor_sync(0xffffffffu, sum, 1, 4);
                sum += __shfl_xor_sync(0xffffffffu, sum, 2, 4);
                if (task < ntask && gl == 0 && sum) {
                    const uint32_t st = lf_site(jb, side ? X.kb : X.ka, nbt[(side ? X.bb : X.ba) * n_nbr + n]);
                    atomicAdd(reinterpret_cast<unsigned long long *>(G + st), (unsigned long long)sum);
                }
            }
            if (tid == 0) {                                // the two sites: every row flips except those with both
                G[ia] = -G[ia] + 2 * X.C; G[ib] = -G[ib] + 2 * X.C;
                sig[ia] = (int8_t)X.sb; sig[ib] = (int8_t)X.sa;
            }
        }
        __syncthreads();
    }
    (void)nrow_a_max;
    if (warp == 0) nnear = __reduce_add_sync(0xffffffffu, nnear);   // each lane counted the steps it decided
    if (jb.gf_smem)
        for (int64_t i = tid; i < jb.N; i += nt) { gsig[i] = sig[i]; gfld[i] = G[i]; }
    if (track)
        for (int c = tid; c < n_cols; c += nt) jb.cv[(int64_t)r * n_cols + c] += dcv[c];
    __syncthreads();                                       // the replica's outputs are written before it is counted
    if (tid == 0) {
        jb.E[r] = E0c + (double)dsum * fscale;
        jb.E_min_rep[r] = fmin(Emin, E0c + (double)dmin * fscale);
        jb.n_acc[r] += nacc;
        if (jb.n_near) jb.n_near[r] += nnear;
        if (jb.ex_sync) fused_chunk_end(jb, g0);
    }
}

// Full energy on the sign-parity tables, bit-sliced.  The occupancies become bit planes: per replica, point-
// function column with sign changes and basis site, one row of 2 * d2 bits per (k0, k1) holding the sign bit of
// every k2 twice over, so that any offset in [0, d2) reads 32 consecutive bits with one funnel shift.  A thread
// then takes 32 consecutive anchors along k2 and, for every cluster instance anchored at a site (the reverse rows
// of slot 0: each instance of the cell exactly once), XORs the members' shifted plane words: bit j is the parity
// of anchor j's product and the column's sum gains (valid anchors) - 2 popcount(parity).  Counts are exact
// integers; E = zerolet + sum_c eci_c * count_c follows in float64.
__global__ void ce_bitplane_kernel(const int8_t *__restrict__ sigma, int32_t R, int64_t N, int32_t nB, int64_t d0d1, int32_t d2,
                                   int32_t W2, const int32_t *__restrict__ plane_pfc, int32_t n_pl,
                                   const uint8_t *__restrict__ sbits, uint32_t *__restrict__ planes) {
    // one warp per plane row (replica, plane, basis, k0 * d1 + k1)
    const int64_t rows = (int64_t)R * n_pl * nB * d0d1;
    const int lane = threadIdx.x & 31;
    const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < rows; w += wstride) {
        const int64_t kk = w % d0d1;
        int64_t t = w / d0d1;
        const int b = (int)(t % nB); t /= nB;
        const int pl = (int)(t % n_pl);
        const int64_t r = t / n_pl;
        const uint8_t *sb = sbits + 4 * plane_pfc[pl];
        const int8_t *sg = sigma + r * N + kk * d2 * nB + b;
        uint32_t *out = planes + w * W2;
        for (int q = 0; q < W2; ++q) {
            const int pos = q * 32 + lane;
            uint32_t bit = 0;
            if (pos < 2 * d2) {
                const int k2 = pos < d2 ? pos : pos - d2;
                bit = sb[sg[(int64_t)k2 * nB] & 3];
            }
            const uint32_t word = __ballot_sync(0xffffffffu, bit != 0u);
            if (lane == 0) out[q] = word;
        }
    }
}

// grid (item blocks x row slices, nB, R): threads over the (k0, k1, 32-anchor word) items of anchor basis
// blockIdx.y, replica blockIdx.z; a small cell's rows are split into slices over more blocks.  Every lane of a
// warp walks the same rows (lanes past the last item count nothing).
__global__ void __launch_bounds__(256) ce_energy_bits_kernel(const uint32_t *__restrict__ planes, int32_t P, int32_t d0, int32_t d1,
                                                              int32_t d2, int32_t W2, const uint32_t *__restrict__ brows,
                                                              const int4 *__restrict__ bmem, const int32_t *__restrict__ brow_off,
                                                              const int32_t *__restrict__ brow_n, int32_t n_cols, int32_t slices,
                                                              unsigned long long *__restrict__ cv) {
    extern __shared__ unsigned long long ccnt[];
    const int b = blockIdx.y, r = blockIdx.z, lane = threadIdx.x & 31;
    const int slice = (int)(blockIdx.x % (unsigned)slices), iblk = (int)(blockIdx.x / (unsigned)slices);
    const int iblocks = (int)(gridDim.x / (unsigned)slices);
    for (int c = threadIdx.x; c < n_cols; c += blockDim.x) ccnt[c] = 0ull;
    __syncthreads();
    const int Wn = (d2 + 31) >> 5;
    const int64_t items = (int64_t)d0 * d1 * Wn;
    const uint32_t *pr = planes + (int64_t)r * P * d0 * d1 * W2;
    const int nall = brow_n[b];
    const int q0 = (int)((int64_t)nall * slice / slices), q1 = (int)((int64_t)nall * (slice + 1) / slices);
    const uint32_t *rows = brows + brow_off[b];
    auto flush = [&](int col, int acc) {
        const int sum = (int)__reduce_add_sync(0xffffffffu, (unsigned)acc);
        if (lane == 0 && sum) atomicAdd(&ccnt[col], (unsigned long long)(long long)sum);
    };
    for (int64_t base = (int64_t)iblk * blockDim.x; base < items; base += (int64_t)iblocks * blockDim.x) {
        const int64_t it = base + threadIdx.x;
        const bool live = it < items;
        const int64_t itc = live ? it : 0;
        const int w = (int)(itc % Wn);
        const int64_t kk = itc / Wn;
        const int k1 = (int)(kk % d1), k0 = (int)(kk / d1);
        const int nv = live ? min(32, d2 - 32 * w) : 0;
        const uint32_t mask = nv >= 32 ? 0xffffffffu : ((1u << nv) - 1u);
        int col = -1, acc = 0;
        for (int q = q0; q < q1; ++q) {
            const uint32_t rd = __ldg(rows + q);
            const int c = (int)(rd & 0xffu), nm = (int)((rd >> 8) & 0xfu), st = (int)(rd >> 12);
            if (c != col) {
                if (col >= 0) flush(col, acc);
                col = c; acc = 0;
            }
            uint32_t par = 0;
            for (int m = 0; m < nm; ++m) {
                const int4 e = __ldg(bmem + st + m);           // (plane, uo0, uo1, uo2)
                int a0 = k0 + e.y; a0 -= a0 >= d0 ? d0 : 0;
                int a1 = k1 + e.z; a1 -= a1 >= d1 ? d1 : 0;
                const int pos = 32 * w + e.w;
                const uint32_t *row = pr + (((int64_t)e.x * d0 + a0) * d1 + a1) * W2 + (pos >> 5);
                par ^= __funnelshift_r(__ldg(row), __ldg(row + 1), (unsigned)(pos & 31));
            }
            acc += nv - 2 * __popc(par & mask);
        }
        if (col >= 0) flush(col, acc);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < n_cols; c += blockDim.x)
        if (ccnt[c]) atomicAdd(cv + (int64_t)r * n_cols + c, ccnt[c]);
}

// Local fields of every site of R configurations, bit-sliced like the full energy: a thread takes 32 consecutive
// sites along k2 of one basis and, for every reverse row of that basis (every cluster instance containing the
// site), XORs the members' shifted plane words (bit j: the parity of site j's product); odd parities are counted
// per site in a vertical counter while the rows of one column go by, and the column adds 2 eci (rows - 2 odd) to
// each site's field (fixed point, exact).
__global__ void __launch_bounds__(128) ce_field_bits_kernel(const uint32_t *__restrict__ planes, int32_t P, int32_t d0, int32_t d1,
                                                             int32_t d2, int32_t W2, int32_t nB, int64_t N,
                                                             const uint32_t *__restrict__ frows, const int4 *__restrict__ fmem,
                                                             const int32_t *__restrict__ frow_off, const int32_t *__restrict__ frow_n,
                                                             const int64_t *__restrict__ efix, long long *__restrict__ field) {
    const int b = blockIdx.y, r = blockIdx.z;
    const int Wn = (d2 + 31) >> 5;
    const int64_t items = (int64_t)d0 * d1 * Wn;
    const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= items) return;
    const int w = (int)(it % Wn);
    const int64_t kk = it / Wn;
    const int k1 = (int)(kk % d1), k0 = (int)(kk / d1);
    const int nv = min(32, d2 - 32 * w);
    const uint32_t mask = nv >= 32 ? 0xffffffffu : ((1u << nv) - 1u);
    const uint32_t *pr = planes + (int64_t)r * P * d0 * d1 * W2;
    constexpr int NQ = 13;                                  // up to 8191 rows per column
    uint32_t cnt[NQ];
    long long acc[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[j] = 0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) cnt[q] = 0u;
    int col = -1, nrows = 0;
    auto flush = [&]() {
        if (col < 0 || nrows == 0) return;
        const long long e = (long long)__ldg(efix + col);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            int odd = 0;
#pragma unroll
            for (int q = 0; q < NQ; ++q) odd |= (int)((cnt[q] >> j) & 1u) << q;
            acc[j] += e * (long long)(nrows - 2 * odd);
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) cnt[q] = 0u;
        nrows = 0;
    };
    const uint32_t *rows = frows + frow_off[b];
    const int nr = frow_n[b];
    for (int q = 0; q < nr; ++q) {
        const uint32_t rd = __ldg(rows + q);
        const int c = (int)(rd & 0xffu), nm = (int)((rd >> 8) & 0xfu), st = (int)(rd >> 12);
        if (c != col) { flush(); col = c; }
        uint32_t par = 0;
        for (int m = 0; m < nm; ++m) {
            const int4 e = __ldg(fmem + st + m);                  // (plane, uo0, uo1, uo2)
            int a0 = k0 + e.y; a0 -= a0 >= d0 ? d0 : 0;
            int a1 = k1 + e.z; a1 -= a1 >= d1 ? d1 : 0;
            const int pos = 32 * w + e.w;
            const uint32_t *row = pr + (((int64_t)e.x * d0 + a0) * d1 + a1) * W2 + (pos >> 5);
            par ^= __funnelshift_r(__ldg(row), __ldg(row + 1), (unsigned)(pos & 31));
        }
        uint32_t carry = par & mask;
#pragma unroll
        for (int k = 0; k < NQ; ++k) { const uint32_t tq = cnt[k] & carry; cnt[k] ^= carry; carry = tq; }
        ++nrows;
    }
    flush();
    long long *out = field + (int64_t)r * N + ((int64_t)(k0 * d1 + k1) * d2 + 32 * w) * nB + b;
#pragma unroll
    for (int j = 0; j < 32; ++j)
        if (j < nv) out[(int64_t)j * nB] = acc[j];
}

// E[r] = zerolet + sum_c eci_c * cv[r, c], columns in order (one thread per configuration)
__global__ void ce_energy_counts_kernel(const int64_t *__restrict__ cv, int32_t R, int32_t n_cols, const double *__restrict__ ecol,
                                        double zerolet, double *E) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double e = 0.0;
    for (int c = 0; c < n_cols; ++c) e += ecol[c] * (double)cv[(int64_t)r * n_cols + c];
    E[r] = zerolet + e;
}

// chunk-end exchange of temperature slots, one CTA (thread 0) per job
struct CEExJob {
    int32_t R; double *E; const float *beta_slot; int32_t *rep_of_slot, *slot_of_rep; const int32_t *ladder_id;
    int64_t *n_ex; uint64_t seed; int64_t g_end; int32_t parity; const double *ex_u;
    double *E_samples; int64_t last_row; int32_t do_exchange;
    double E_scale; int32_t rounds;          // energies in eV = E * E_scale; exchange rounds back to back
    int64_t *step_dev; int64_t n_steps;      // device step counter advanced by the chunk (or null)
};
struct CEExBatch { int32_t n_jobs; CEExJob job[kMaxJobs]; };

__global__ void ce_exchange_kernel(const __grid_constant__ CEExBatch bt) {
    extern __shared__ int32_t xsm[];
    const int j = blockIdx.x;
    if (j >= bt.n_jobs || threadIdx.x != 0) return;
    const CEExJob &x = bt.job[j];
    const int64_t g_end = x.step_dev ? *x.step_dev + x.n_steps : x.g_end;
    if (x.step_dev) *x.step_dev = g_end;      // the chunk kernel has finished reading it (stream order)
    if (!x.do_exchange || x.R < 2) return;
    int32_t *perm = xsm;
    int32_t *ros = perm + x.R;
    const int R = x.R;
    const uint32_t k0 = (uint32_t)x.seed, k1 = (uint32_t)(x.seed >> 32);
    const uint32_t c0 = (uint32_t)g_end, c1 = (uint32_t)((uint64_t)g_end >> 32);
    const int npair = R / 2;                 // ceil((R-1)/2)
    int64_t nswap = 0;
    for (int q = 0; q < max(x.rounds, 1); ++q) {
        const uint32_t cq = 0xFFFFFFFFu - 2u * (uint32_t)q;
        const int parity = x.ex_u ? ((x.parity >> q) & 1) : (int)(philox4x32(c0, c1, cq, 0u, k0, k1).x & 1u);
        for (int i = 0; i < R; ++i) perm[i] = i;
        for (int k = 0; 2 * k < R - 1; ++k) {
            const int a = 2 * k + parity, b = a + 1;
            if (b >= R) continue;
            if (x.ladder_id[a] != x.ladder_id[b]) continue;
            const double Ea = x.E[x.rep_of_slot[a]] * x.E_scale, Eb = x.E[x.rep_of_slot[b]] * x.E_scale;
            const double log_acc = ((double)x.beta_slot[b] - (double)x.beta_slot[a]) * (Eb - Ea);
            double u;
            if (x.ex_u) u = x.ex_u[(size_t)q * npair + k];
            else { u32x4 w = philox4x32(c0, c1, cq - 1u, (uint32_t)k, k0, k1); u = draw_u01(w.x, w.y); }
            if (log(u) < log_acc) { perm[a] = b; perm[b] = a; ++nswap; }
        }
        for (int t = 0; t < R; ++t) ros[t] = x.rep_of_slot[perm[t]];
        for (int t = 0; t < R; ++t) { x.rep_of_slot[t] = ros[t]; x.slot_of_rep[ros[t]] = t; }
    }
    *x.n_ex += nswap;
    if (x.E_samples && x.last_row >= 0)
        for (int t = 0; t < R; ++t) x.E_samples[x.last_row * R + t] = x.E[x.rep_of_slot[t]];
}

// full energy: grid (blocks_per_rep, R); per-block float64 partial -> partial[r * nblk + bx]
template <typename Real>
__global__ void __launch_bounds__(256) ce_energy_kernel(const int8_t *__restrict__ sigma, int64_t N, int64_t n_cells,
                                                        int32_t nB, int32_t d0, int32_t d1, int32_t d2, int32_t Rt, int32_t mo,
                                                        const int32_t *__restrict__ T_b, const int32_t *__restrict__ T_uo,
                                                        const uint8_t *__restrict__ T_pfc, const Real *__restrict__ T_eci,
                                                        const Real *__restrict__ pf, int32_t max_sp, double *partial) {
    __shared__ double red[32];
    const int r = blockIdx.y;
    const int8_t *sig = sigma + (int64_t)r * N;
    double acc = 0.0;
    const int64_t d12 = (int64_t)d1 * d2;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k0 = (int32_t)(c / d12), k1 = (int32_t)((c / d2) % d1), k2 = (int32_t)(c % d2);
        Real cell_sum = Real(0);
        for (int row = 0; row < Rt; ++row) {
            Real pr = Real(1);
            for (int m = 0; m < mo; ++m) {
                const int e = row * mo + m;
                const int32_t q0 = wrap_add(k0, __ldg(T_uo + 3 * e), d0);
                const int32_t q1 = wrap_add(k1, __ldg(T_uo + 3 * e + 1), d1);
                const int32_t q2 = wrap_add(k2, __ldg(T_uo + 3 * e + 2), d2);
                const int64_t s = (((int64_t)q0 * d1 + q1) * d2 + q2) * nB + __ldg(T_b + e);
                pr *= pf[(int)__ldg(T_pfc + e) * max_sp + sig[s]];
            }
            cell_sum += __ldg(T_eci + row) * pr;
        }
        acc += (double)cell_sum;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        partial[(int64_t)r * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void ce_energy_finish(const double *partial, int32_t nblk, int32_t R, double zerolet, double *E) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += partial[(int64_t)r * nblk + b];
    E[r] = zerolet + s;
}

// batched dE queries: one CTA per query
template <typename Real, int MO>
__global__ void __launch_bounds__(1024) ce_delta_kernel(const __grid_constant__ CEJob jb, int32_t n, const int32_t *rep,
                                                        const int64_t *qa, const int64_t *qb, const int8_t *qsa,
                                                        const int8_t *qsb, double *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CEShared cs;
    const int q = blockIdx.x;
    if (q >= n) return;
    // uniform per block: every thread reads the same query, so an invalid one returns the whole block
    if (rep[q] < 0 || rep[q] >= jb.R || qa[q] < 0 || qa[q] >= jb.N || qb[q] < 0 || qb[q] >= jb.N ||
        qsa[q] < 0 || qsa[q] >= jb.max_sp || qsb[q] < 0 || qsb[q] >= jb.max_sp) {
        if (threadIdx.x == 0) { out[q] = __longlong_as_double(0x7ff8000000000000ll); atomicOr(jb.err, 2); }
        return;
    }
    const Layout<Real> L = Layout<Real>::make(jb.nB, jb.J, MO, jb.n_nbr, jb.n_pfc, blockDim.x >> 5, false);
    const int8_t *sig = jb.sigma + (int64_t)rep[q] * jb.N;
    if (threadIdx.x == 0) {
        cs.ia = qa[q]; cs.ib = qb[q];
        // the swap writes sa_new at ia and sb_new at ib: block_delta takes the new species as (cs.sb, cs.sa)
        cs.sb = qsa[q]; cs.sa = qsb[q];
        site_coords(jb, cs.ia, cs.b_a, cs.ka); site_coords(jb, cs.ib, cs.b_b, cs.kb);
    }
    __syncthreads();
    Real dE = block_delta<Real, MO>(jb, sig, cs, smem, L, jb.loc, jb.pfc, reinterpret_cast<const Real *>(jb.eci));
    if (threadIdx.x == 0) out[q] = (double)dE;
}

// chunk-end minimum: out_min = min_r E_min_rep, out_arg = argmin_r E (first)
__global__ void pt_minimum_kernel(const double *E, const double *Emin, int32_t R, double *out_min, int32_t *out_arg) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = Emin[0]; int a = 0; double be = E[0];
    for (int r = 1; r < R; ++r) {
        m = fmin(m, Emin[r]);
        if (E[r] < be) { be = E[r]; a = r; }
    }
    *out_min = m; *out_arg = a;
}

}  // namespace nce

// ───────────────────────────── host side ──────────────────────────────────────────────────────

struct nce_ce_model {
    int32_t nB, J, mo, n_nbr, n_pfc, max_sp, n_groups, max_gb, Rt;
    int64_t d[3], n_cells, N;
    double zerolet;
    uint16_t *loc = nullptr; uint8_t *pfc = nullptr; double *eci64 = nullptr; float *eci32 = nullptr;
    int32_t *rv_len = nullptr, *nb_b = nullptr, *nb_uo = nullptr;
    double *pf64 = nullptr; float *pf32 = nullptr;
    int32_t *act_b = nullptr, *act_nb = nullptr; uint64_t *grp_cum = nullptr;
    int32_t *T_b = nullptr, *T_uo = nullptr; uint8_t *T_pfc = nullptr; double *T_eci64 = nullptr; float *T_eci32 = nullptr;
    int32_t *err = nullptr;                  // device error word
    bool binary = false;                     // every point-function value is -1 or +1 (sign-parity kernel applies)
    uint8_t *sbits = nullptr; uint16_t *bix = nullptr; uint8_t *rcol = nullptr; double *ecol2_64 = nullptr; float *ecol2_32 = nullptr;
    int64_t *ecol_fix = nullptr; int32_t fix_shift = 0;   // 2 eci per column x 2^fix_shift (exact dE sums, float64 path)
    int32_t n_cols = 0;
    uint32_t *chunks = nullptr; int32_t *n_chunks = nullptr; int32_t max_chunks = 0;
    // bit-sliced full energy: rows anchored at a site (col | members << 8 | first member << 12) per anchor basis,
    // members (plane, uo0, uo1, uo2), the point-function column of each plane
    uint32_t *brows = nullptr; int4 *bmem = nullptr; int32_t *brow_off = nullptr, *brow_n = nullptr;
    int32_t *plane_pfc = nullptr; int32_t n_planes = 0;
    double *ecol1 = nullptr;                 // eci of each column (full-energy kernel)
    // local-field kernel: per basis the rows containing each neighbourhood entry, the displacement box, and every
    // reverse row as (col | members << 8 | first member << 12) with its members (plane, uo0, uo1, uo2) for the fields
    bool lf_ok = false;
    int32_t *lf_off = nullptr; uint16_t *lf_idx = nullptr; int16_t *lf_box = nullptr;
    int32_t lf_e[3] = {0, 0, 0}, lf_nidx = 0;
    uint32_t *frows = nullptr; int4 *fmem = nullptr; int32_t *frow_off = nullptr, *frow_n = nullptr;

    int device = 0;
    std::mutex mu;
    // staging for the host-buffer entry point
    std::vector<void *> staging; size_t staging_bytes = 0; void *staging_base = nullptr;
};

namespace nce {

template <typename T>
static int upload(T *&dst, const T *src, size_t n) {
    if (n == 0) { dst = nullptr; return NCE_OK; }
    NCE_CUDA(cudaMalloc((void **)&dst, sizeof(T) * n));
    NCE_CUDA(cudaMemcpy(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    return NCE_OK;
}

static int free_model(nce_ce_model *m) {
    void *ptrs[] = {m->loc, m->pfc, m->eci64, m->eci32, m->rv_len, m->nb_b, m->nb_uo, m->pf64, m->pf32, m->act_b,
                    m->act_nb, m->grp_cum, m->T_b, m->T_uo, m->T_pfc, m->T_eci64, m->T_eci32, m->err, m->sbits, m->bix, m->rcol, m->ecol2_64, m->ecol2_32, m->ecol_fix, m->chunks, m->n_chunks, m->brows, m->bmem, m->brow_off, m->brow_n, m->plane_pfc, m->ecol1,
                    m->staging_base, m->lf_off, m->lf_idx, m->lf_box, m->frows, m->fmem, m->frow_off, m->frow_n};
    for (void *p : ptrs) if (p) cudaFree(p);
    delete m;
    return NCE_OK;
}

template <typename Real>
static bool tables_fit(const nce_ce_model *m, int warps, size_t *bytes_out) {
    const Layout<Real> L1 = Layout<Real>::make(m->nB, m->J, m->mo, m->n_nbr, m->n_pfc, warps, true);
    const Layout<Real> L0 = Layout<Real>::make(m->nB, m->J, m->mo, m->n_nbr, m->n_pfc, warps, false);
    const size_t limit = 200 * 1024;
    if (L1.total <= limit) { *bytes_out = L1.total; return true; }
    *bytes_out = L0.total;
    return false;
}

static CEJob make_job(const nce_ce_model *m, const nce_pt_state *st, const nce_pt_chunk *ck, int cta_base, bool bin = false) {
    CEJob j;
    std::memset(&j, 0, sizeof(j));
    const bool p64 = ck ? ck->precision != 32 : true;
    j.loc = m->loc; j.pfc = m->pfc; j.eci = p64 ? (const void *)m->eci64 : (const void *)m->eci32;
    j.sbits = m->sbits; j.bix = m->bix; j.rcol = m->rcol; j.n_cols = m->n_cols;
    j.ecol2 = p64 ? (const void *)m->ecol2_64 : (const void *)m->ecol2_32;
    j.ecol_fix = m->ecol_fix; j.fix_shift = p64 ? m->fix_shift : 0;
    j.chunks = m->chunks; j.n_chunks = m->n_chunks; j.max_chunks = m->max_chunks;
    (void)bin;
    j.rv_len = m->rv_len; j.nb_b = m->nb_b; j.nb_uo = m->nb_uo; j.pf = p64 ? (const void *)m->pf64 : (const void *)m->pf32;
    j.act_b = m->act_b; j.act_nb = m->act_nb; j.grp_cum = m->grp_cum;
    j.nB = m->nB; j.J = m->J; j.n_nbr = m->n_nbr; j.n_pfc = m->n_pfc; j.max_sp = m->max_sp;
    j.n_groups = m->n_groups; j.max_gb = m->max_gb;
    j.d0 = (int32_t)m->d[0]; j.d1 = (int32_t)m->d[1]; j.d2 = (int32_t)m->d[2];
    j.n_cells = m->n_cells; j.N = m->N; j.err = m->err;
    if (st) {
        j.sigma = st->sigma; j.E = st->E; j.beta_slot = st->beta_slot; j.slot_of_rep = st->slot_of_rep;
        j.E_min_rep = st->E_min_rep; j.n_acc = st->n_acc; j.R = st->R; j.cv = st->cv; j.n_near = st->n_near;
        j.field = st->field;
        j.rep_of_slot = st->rep_of_slot; j.ladder_id = st->ladder_id; j.n_ex = st->n_ex; j.ex_sync = st->ex_sync;
    }
    if (ck) {
        j.n_steps = ck->n_steps; j.step0 = ck->step0; j.step_dev = ck->step_dev; j.prop_a = ck->prop_a; j.prop_b = ck->prop_b; j.prop_u = ck->prop_u;
        j.seed = ck->seed; j.sample_interval = ck->sample_interval > 0 ? ck->sample_interval : 1;
        j.E_samples = ck->E_samples;
        j.ex_u = ck->ex_u; j.ex_flags = (ck->do_exchange ? 1 : 0) | ((ck->ex_parity & 1) << 1);
        j.lf_off = m->lf_off; j.lf_idx = m->lf_idx; j.lf_box = m->lf_box;
        j.lf_e0 = m->lf_e[0]; j.lf_e1 = m->lf_e[1]; j.lf_e2 = m->lf_e[2]; j.lf_nidx = m->lf_nidx;
        j.near_eV = ck->near_eV > 0.0 ? ck->near_eV : (p64 ? 1e-9 : 1e-6);
        if (j.fix_shift > 0) {
            const double nf = std::ldexp(j.near_eV, j.fix_shift);
            j.near_fix = nf >= 4.0e18 ? (int64_t)4000000000000000000ll : (int64_t)std::ceil(nf) + 1;
        }
    }
    j.cta_base = cta_base;
    return j;
}

template <typename Real, int MO>
static int launch_chunk_mo(const CEBatch &bt, int total, int warps, size_t smem, cudaStream_t s) {
    auto kern = ce_pt_chunk_kernel<Real, MO>;
    NCE_CUDA(::nce::raise_smem_limit((const void *)kern, smem));
    kern<<<total, warps * 32, smem, s>>>(bt);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

template <typename Acc, int MO, bool SMT>
static int launch_bin_smt(const CEBatch &bt, int total, int warps, size_t smem, int sig_smem, cudaStream_t s, int CL) {
    if (CL <= 1) {
        auto kern = ce_bin_chunk_kernel<Acc, MO, false, SMT>;
        NCE_CUDA(::nce::raise_smem_limit((const void *)kern, smem));
        kern<<<total, warps * 32, smem, s>>>(bt, sig_smem);
    } else {
        auto kern = ce_bin_chunk_kernel<Acc, MO, true, SMT>;
        NCE_CUDA(::nce::raise_smem_limit((const void *)kern, smem));
        // 16 CTAs per cluster is beyond the portable size of 8 (allowed on this GPU)
        if (CL > 8) NCE_CUDA(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cudaLaunchConfig_t cfg; std::memset(&cfg, 0, sizeof(cfg));
        cfg.gridDim = dim3((unsigned)(total * CL)); cfg.blockDim = dim3(warps * 32); cfg.dynamicSmemBytes = smem; cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)CL; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr; cfg.numAttrs = 1;
        NCE_CUDA(cudaLaunchKernelEx(&cfg, kern, bt, sig_smem));
    }
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

template <typename Acc, int MO>
static int launch_bin_mo(const CEBatch &bt, int total, int warps, size_t smem, int sig_smem, cudaStream_t s, int CL) {
    return bt.tables_in_smem ? launch_bin_smt<Acc, MO, true>(bt, total, warps, smem, sig_smem, s, CL)
                             : launch_bin_smt<Acc, MO, false>(bt, total, warps, smem, sig_smem, s, CL);
}

template <typename Acc>
static int launch_bin(const CEBatch &bt, int mo, int total, int warps, size_t smem, int sig_smem, cudaStream_t s, int CL) {
    switch (mo) {
#define NCE_BIN_CASE(M) case M: return launch_bin_mo<Acc, M>(bt, total, warps, smem, sig_smem, s, CL);
        NCE_BIN_CASE(1) NCE_BIN_CASE(2) NCE_BIN_CASE(3) NCE_BIN_CASE(4) NCE_BIN_CASE(5) NCE_BIN_CASE(6) NCE_BIN_CASE(7) NCE_BIN_CASE(8)
#undef NCE_BIN_CASE
        default: return fail(NCE_ERR_UNSUPPORTED, "cluster order %d > 8", mo);
    }
}

static int launch_lf(const CEBatch &bt, int mo, int total, int warps, size_t smem, int32_t budget, cudaStream_t s) {
    void (*kern)(CEBatch, int32_t) = nullptr;
    switch (mo) {
        case 1: kern = ce_lf_chunk_kernel<1>; break;
        case 2: kern = ce_lf_chunk_kernel<2>; break;
        case 3: kern = ce_lf_chunk_kernel<3>; break;
        case 4: kern = ce_lf_chunk_kernel<4>; break;
        case 5: kern = ce_lf_chunk_kernel<5>; break;
        case 6: kern = ce_lf_chunk_kernel<6>; break;
        case 7: kern = ce_lf_chunk_kernel<7>; break;
        case 8: kern = ce_lf_chunk_kernel<8>; break;
        default: return fail(NCE_ERR_UNSUPPORTED, "cluster order %d > 8", mo);
    }
    NCE_CUDA(::nce::raise_smem_limit((const void *)kern, smem));
    kern<<<total, std::min(warps, kLfMaxWarps) * 32, smem, s>>>(bt, budget);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

template <typename Real>
static int launch_chunk(const CEBatch &bt, int mo, int total, int warps, size_t smem, cudaStream_t s) {
    switch (mo) {
        case 1: return launch_chunk_mo<Real, 1>(bt, total, warps, smem, s);
        case 2: return launch_chunk_mo<Real, 2>(bt, total, warps, smem, s);
        case 3: return launch_chunk_mo<Real, 3>(bt, total, warps, smem, s);
        case 4: return launch_chunk_mo<Real, 4>(bt, total, warps, smem, s);
        case 5: return launch_chunk_mo<Real, 5>(bt, total, warps, smem, s);
        case 6: return launch_chunk_mo<Real, 6>(bt, total, warps, smem, s);
        case 7: return launch_chunk_mo<Real, 7>(bt, total, warps, smem, s);
        case 8: return launch_chunk_mo<Real, 8>(bt, total, warps, smem, s);
        default: return fail(NCE_ERR_UNSUPPORTED, "cluster order %d > 8", mo);
    }
}

static int check_state(const nce_ce_model *m, const nce_pt_state *st) {
    NCE_CHECK(st && st->R >= 1, "state: R must be >= 1");
    NCE_CHECK(st->N == m->N, "state: N=%lld but the tables are for %lld sites", (long long)st->N, (long long)m->N);
    NCE_CHECK(st->sigma && st->E && st->beta_slot && st->rep_of_slot && st->slot_of_rep && st->ladder_id &&
              st->E_min_rep && st->n_acc && st->n_ex, "state: null device pointer");
    return NCE_OK;
}

static int check_chunk(const nce_pt_state *st, const nce_pt_chunk *ck) {
    NCE_CHECK(ck, "chunk: null");
    NCE_CHECK(ck->n_steps >= 0 && ck->n_steps < 2147483647ll, "chunk: n_steps must be in [0, 2^31 - 1)");
    NCE_CHECK(ck->precision == 64 || ck->precision == 32, "chunk: precision must be 64 or 32");
    NCE_CHECK((ck->prop_a == nullptr) == (ck->prop_b == nullptr) && (ck->prop_a == nullptr) == (ck->prop_u == nullptr),
              "chunk: prop_a/prop_b/prop_u must be all set or all NULL");
    NCE_CHECK(!ck->E_samples || ck->sample_interval > 0, "chunk: sample_interval must be > 0 with E_samples");
    NCE_CHECK(ck->warps >= 0 && ck->warps <= 32, "chunk: warps must be 0..32");
    NCE_CHECK(ck->cluster == 0 || ck->cluster == 1 || ck->cluster == 2 || ck->cluster == 4 || ck->cluster == 8 ||
              ck->cluster == 16, "chunk: cluster must be 0, 1, 2, 4, 8 or 16");
    NCE_CHECK(!ck->do_exchange || !ck->ex_u || (ck->ex_parity == 0 || ck->ex_parity == 1), "chunk: ex_parity must be 0/1");
    NCE_CHECK(ck->near_eV >= 0.0 && ck->near_eV <= 1e3, "chunk: near_eV must be in [0, 1e3]");
    (void)st;
    return NCE_OK;
}

static int run_batch(int n_jobs, const nce_ce_handle *hs, const nce_pt_state *sts, const nce_pt_chunk *cks, cudaStream_t s) {
    NCE_CHECK(n_jobs >= 1 && n_jobs <= kMaxJobs, "batch: n_jobs must be 1..%d", kMaxJobs);
    const int precision = cks[0].precision;
    const int warps = cks[0].warps > 0 ? cks[0].warps : 8;
    int mo = 0, total = 0, max_R = 0;
    for (int j = 0; j < n_jobs; ++j) {
        NCE_CHECK(hs[j], "batch: null handle");
        int rc = check_state(hs[j], &sts[j]); if (rc) return rc;
        rc = check_chunk(&sts[j], &cks[j]); if (rc) return rc;
        NCE_CHECK(cks[j].precision == precision, "batch: all chunks must use the same precision");
        NCE_CHECK((cks[j].warps > 0 ? cks[j].warps : 8) == warps, "batch: all chunks must use the same warps");
        mo = std::max(mo, hs[j]->mo);
        total += sts[j].R; max_R = std::max(max_R, sts[j].R);
    }
    for (int j = 0; j < n_jobs; ++j)
        NCE_CHECK(hs[j]->mo == mo, "batch: all jobs must have the same maximum cluster order");
    const int path = cks[0].path;
    bool all_bin = true;
    for (int j = 0; j < n_jobs; ++j) {
        NCE_CHECK(cks[j].path == path, "batch: all chunks must use the same path");
        all_bin = all_bin && hs[j]->binary;
    }
    NCE_CHECK(path >= 0 && path <= 3, "chunk: path must be 0 (auto), 1 (general), 2 (sign parity) or 3 (local field)");
    NCE_CHECK(path < 2 || all_bin, "chunk: the sign-parity and local-field paths need point functions in {-1, +1}");
    // local field: every job has its tables and a field buffer, float64 (fixed-point) arithmetic
    bool all_lf = precision == 64;
    for (int j = 0; j < n_jobs; ++j) all_lf = all_lf && hs[j]->lf_ok && sts[j].field != nullptr;
    if (path == 3) {
        for (int j = 0; j < n_jobs; ++j) {
            NCE_CHECK(hs[j]->lf_ok, "chunk: the local-field path is not available for this cell (aliasing neighbourhood "
                                    "or tables too large)");
            NCE_CHECK(sts[j].field, "chunk: the local-field path needs the state's field buffer (nce_ce_field_init)");
        }
        NCE_CHECK(precision == 64, "chunk: the local-field path computes in fixed point (precision 64)");
    }
    const bool use_lf = path == 3 || (path == 0 && all_lf);
    // the float64 sign-parity kernel sums in fixed point: a table whose column eci allow no exact fixed point (never
    // for eci of physical size) runs the general kernel
    bool all_fix = true;
    for (int j = 0; j < n_jobs; ++j) all_fix = all_fix && hs[j]->fix_shift > 0;
    NCE_CHECK(!(path == 2 && precision == 64 && !all_fix),
              "chunk: the float64 sign-parity path needs fixed-point column eci (2 J max|eci| below 2^41)");
    const bool use_bin = !use_lf && ((path == 2) || (path == 0 && all_bin && (precision == 32 || all_fix)));
    for (int j = 0; j < n_jobs; ++j)
        NCE_CHECK(!sts[j].cv || use_bin || use_lf, "chunk: tracked cluster-vector sums need the sign-parity or local-field path");
    CEBatch bt; std::memset(&bt, 0, sizeof(bt));
    bt.n_jobs = n_jobs;
    size_t smem = 0; bool all_fit = true;
    int sig_smem = 0;
    int64_t lf_budget = 0;
    if (use_lf) {
        size_t t_on = 0, t_off = 0; int64_t maxN = 0;
        for (int j = 0; j < n_jobs; ++j) {
            const nce_ce_model *m = hs[j];
            const int bsz = (2 * m->lf_e[0] + 1) * (2 * m->lf_e[1] + 1) * (2 * m->lf_e[2] + 1);
            t_on = std::max(t_on, LfLayout::make(m->nB, m->J, mo, m->n_nbr, m->n_pfc, m->n_cols, m->max_chunks, m->lf_nidx, bsz, 0, true).total);
            t_off = std::max(t_off, LfLayout::make(m->nB, m->J, mo, m->n_nbr, m->n_pfc, m->n_cols, m->max_chunks, m->lf_nidx, bsz, 0, false).total);
            maxN = std::max(maxN, m->N);
        }
        const size_t limit = 200 * 1024;
        all_fit = t_on <= limit;
        const size_t base = all_fit ? t_on : t_off;
        // occupancy and field (9 bytes a site) in shared memory: the whole cell of one job when it fits, else a per-CTA
        // budget that the jobs with small cells use
        int64_t sites = n_jobs == 1 ? maxN : (int64_t)(48 * 1024) / 9;
        sites = (sites + 15) / 16 * 16;
        if (base + 9 * (size_t)sites + 64 > limit) sites = n_jobs == 1 ? 0 : (int64_t)((limit > base + 64 ? (limit - base - 64) / 9 : 0) / 16 * 16);
        lf_budget = sites;
        smem = sites > 0 ? LfLayout::make(0, 0, 0, 0, 0, 0, 0, 0, 0, sites, false).total + base : base;
    } else if (use_bin) {
        const size_t accb = precision == 64 ? 8 : 4;
        size_t t_on = 0, t_off = 0; int64_t maxN = 0;
        for (int j = 0; j < n_jobs; ++j) {
            const nce_ce_model *m = hs[j];
            t_on = std::max(t_on, BinLayout::make(m->nB, m->J, mo, m->n_nbr, m->n_pfc, m->n_cols, m->max_chunks, accb, 0, true, false).total);
            t_off = std::max(t_off, BinLayout::make(m->nB, m->J, mo, m->n_nbr, m->n_pfc, m->n_cols, m->max_chunks, accb, 0, false, false).total);
            maxN = std::max(maxN, m->N);
        }
        const size_t limit = 200 * 1024;
        all_fit = t_on <= limit;
        const size_t base = all_fit ? t_on : t_off;
        // occupancy in shared memory: the whole cell for one job when it fits, else a per-CTA budget that the
        // jobs with small cells use (larger cells stay in global memory)
        size_t budget = n_jobs == 1 ? (size_t)((maxN + 15) / 16 * 16) : (size_t)48 * 1024;
        if (base + budget > limit) budget = n_jobs == 1 ? 0 : (limit > base ? (limit - base) / 16 * 16 : 0);
        if (n_jobs == 1 && budget > 0 && cks[0].cluster <= 1) {
            // one job: its occupancy goes on chip only while that costs no resident replicas; a cell that would
            // push replicas into a second wave of CTAs stays in global memory (the kernel prefetches each next
            // step's neighbourhoods into L2)
            int dev = 0, smem_sm = 0, n_sm = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
            cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
            const int threads = warps * 32;
            auto resident = [&](size_t dyn) -> int64_t {
                const size_t per_cta = dyn + 5 * 1024 + 1024;          // + static shared memory and the reserve
                int64_t b = (int64_t)(smem_sm / per_cta);
                b = std::min<int64_t>(b, 65536 / (64 * threads));        // 64 registers a thread
                b = std::min<int64_t>(b, 2048 / threads);
                return b * n_sm;
            };
            if (smem_sm > 0 && n_sm > 0 && resident(base + budget) < total && resident(base) > resident(base + budget))
                budget = 0;
        }
        sig_smem = (int)budget;
        smem = base + budget;
    } else {
        for (int j = 0; j < n_jobs; ++j) {
            size_t b; bool fit = precision == 64 ? tables_fit<double>(hs[j], warps, &b) : tables_fit<float>(hs[j], warps, &b);
            all_fit = all_fit && fit;
        }
        for (int j = 0; j < n_jobs; ++j) {
            size_t b;
            if (precision == 64) {
                b = Layout<double>::make(hs[j]->nB, hs[j]->J, mo, hs[j]->n_nbr, hs[j]->n_pfc, warps, all_fit).total;
            } else {
                b = Layout<float>::make(hs[j]->nB, hs[j]->J, mo, hs[j]->n_nbr, hs[j]->n_pfc, warps, all_fit).total;
            }
            smem = std::max(smem, b);
        }
    }
    bt.tables_in_smem = all_fit ? 1 : 0;
    // the chunk-end exchange runs inside the chunk kernel when every job has a counter and steps to run; otherwise
    // no job counts and the exchange kernel follows the launch
    bool fused = true;
    for (int j = 0; j < n_jobs; ++j) fused = fused && sts[j].ex_sync != nullptr && cks[j].n_steps > 0;
    int base = 0;
    for (int j = 0; j < n_jobs; ++j) {
        bt.job[j] = make_job(hs[j], &sts[j], &cks[j], base, use_bin);
        if (!fused) bt.job[j].ex_sync = nullptr;
        bt.job[j].sig_smem = (use_bin && sig_smem > 0 && hs[j]->N <= sig_smem) ? 1 : 0;
        bt.job[j].gf_smem = (use_lf && lf_budget > 0 && hs[j]->N <= lf_budget) ? 1 : 0;
        base += sts[j].R;
    }
    int64_t max_steps = 0;
    for (int j = 0; j < n_jobs; ++j) max_steps = std::max(max_steps, cks[j].n_steps);
    if (max_steps > 0) {
        int rc;
        int CL = cks[0].cluster > 1 ? cks[0].cluster : 1;
        for (int j = 0; j < n_jobs; ++j)
            NCE_CHECK((cks[j].cluster > 1 ? cks[j].cluster : 1) == CL, "batch: all chunks must use the same cluster");
        if (!use_bin) CL = 1;
        if (CL > 1) {
            // every CTA of a cluster keeps its own copy of the occupancy: all jobs must fit the shared-memory budget
            for (int j = 0; j < n_jobs; ++j) if (!bt.job[j].sig_smem) CL = 1;
        }
        if (use_lf)
            rc = launch_lf(bt, mo, total, warps, smem, (int32_t)lf_budget, s);
        else if (use_bin)
            rc = precision == 64 ? launch_bin<double>(bt, mo, total, warps, smem, sig_smem, s, CL)
                                 : launch_bin<float>(bt, mo, total, warps, smem, sig_smem, s, CL);
        else
            rc = precision == 64 ? launch_chunk<double>(bt, mo, total, warps, smem, s)
                                 : launch_chunk<float>(bt, mo, total, warps, smem, s);
        if (rc) return rc;
    }
    if (fused) return NCE_OK;                            // the chunk kernel exchanged
    CEExBatch ex; std::memset(&ex, 0, sizeof(ex));
    ex.n_jobs = n_jobs;
    bool any = false;
    for (int j = 0; j < n_jobs; ++j) {
        const nce_pt_state &st = sts[j]; const nce_pt_chunk &ck = cks[j];
        CEExJob &x = ex.job[j];
        x.R = st.R; x.E = st.E; x.beta_slot = st.beta_slot; x.rep_of_slot = st.rep_of_slot; x.slot_of_rep = st.slot_of_rep;
        x.ladder_id = st.ladder_id; x.n_ex = st.n_ex; x.seed = ck.seed; x.g_end = ck.step0 + ck.n_steps;
        x.parity = ck.ex_parity; x.ex_u = ck.ex_u; x.E_samples = ck.E_samples;
        x.last_row = (ck.E_samples && ck.n_steps > 0 && ck.n_steps % ck.sample_interval == 0) ? ck.n_steps / ck.sample_interval - 1 : -1;
        x.do_exchange = ck.do_exchange && st.R > 1;
        x.E_scale = 1.0; x.rounds = 1;
        x.step_dev = ck.step_dev; x.n_steps = ck.n_steps;
        any = any || x.do_exchange || x.step_dev;
    }
    if (any) {
        const size_t xs = sizeof(int32_t) * 2 * (size_t)max_R;
        NCE_CHECK(xs <= 200 * 1024, "batch: %d replicas per job exceed the exchange kernel's shared memory", max_R);
        NCE_CUDA(::nce::raise_smem_limit((const void *)ce_exchange_kernel, xs));
        ce_exchange_kernel<<<n_jobs, 32, xs, s>>>(ex);
        NCE_CUDA(cudaGetLastError());
    }
    return NCE_OK;
}

// chunk-end slot exchange of one job (used by the NCE engine)
int launch_exchange(int32_t R, double *E, double E_scale, const float *beta_slot, int32_t *ros, int32_t *sor, const int32_t *lid,
                    int64_t *n_ex, uint64_t seed, int64_t g_end, int32_t parity_bits, const double *ex_u, int32_t rounds,
                    cudaStream_t s) {
    if (R < 2 || rounds < 1) return NCE_OK;
    CEExBatch ex; std::memset(&ex, 0, sizeof(ex));
    ex.n_jobs = 1;
    CEExJob &x = ex.job[0];
    x.R = R; x.E = E; x.beta_slot = beta_slot; x.rep_of_slot = ros; x.slot_of_rep = sor; x.ladder_id = lid; x.n_ex = n_ex;
    x.seed = seed; x.g_end = g_end; x.parity = parity_bits; x.ex_u = ex_u; x.E_samples = nullptr; x.last_row = -1;
    x.do_exchange = 1; x.E_scale = E_scale; x.rounds = rounds;
    const size_t xs = sizeof(int32_t) * 2 * (size_t)R;
    NCE_CHECK(xs <= 200 * 1024, "exchange: %d replicas exceed the exchange kernel's shared memory", R);
    NCE_CUDA(::nce::raise_smem_limit((const void *)ce_exchange_kernel, xs));
    ce_exchange_kernel<<<1, 32, xs, s>>>(ex);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

template <typename Real, int MO>
static int launch_delta_mo(const CEJob &jb, int n, const int32_t *rep, const int64_t *ia, const int64_t *ib,
                           const int8_t *sa, const int8_t *sb, double *out, int warps, cudaStream_t s) {
    const size_t smem = Layout<Real>::make(jb.nB, jb.J, MO, jb.n_nbr, jb.n_pfc, warps, false).total;
    auto kern = ce_delta_kernel<Real, MO>;
    NCE_CUDA(::nce::raise_smem_limit((const void *)kern, smem));
    kern<<<n, warps * 32, smem, s>>>(jb, n, rep, ia, ib, sa, sb, out);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

template <typename Real>
static int launch_delta(const CEJob &jb, int mo, int n, const int32_t *rep, const int64_t *ia, const int64_t *ib,
                        const int8_t *sa, const int8_t *sb, double *out, int warps, cudaStream_t s) {
    switch (mo) {
#define NCE_MO_CASE(M) case M: return launch_delta_mo<Real, M>(jb, n, rep, ia, ib, sa, sb, out, warps, s);
        NCE_MO_CASE(1) NCE_MO_CASE(2) NCE_MO_CASE(3) NCE_MO_CASE(4) NCE_MO_CASE(5) NCE_MO_CASE(6) NCE_MO_CASE(7) NCE_MO_CASE(8)
#undef NCE_MO_CASE
        default: return fail(NCE_ERR_UNSUPPORTED, "cluster order %d > 8", mo);
    }
}

}  // namespace nce

namespace nce {
int ce_model_dims(nce_ce_handle h, int64_t *N, int32_t *n_cols, int32_t *mo, int32_t *binary) {
    NCE_CHECK(h, "null CE handle");
    *N = h->N; *n_cols = h->n_cols; *mo = h->mo; *binary = (h->binary && h->brows) ? 1 : 0;
    return NCE_OK;
}
}  // namespace nce

using namespace nce;

static int energy_impl(nce_ce_model *h, const int8_t *sigma, int32_t R, int32_t precision, double *E, int64_t *cv_out,
                       cudaStream_t s);
static int field_init_impl(nce_ce_model *h, const int8_t *sigma, int32_t R, int64_t *field, cudaStream_t s);

// Tables of the local-field kernel (see ce_lf_chunk_kernel).  The path is enabled when the cell has no aliasing
// (every neighbourhood entry of a site is a different site: their k-space displacements, taken as representatives in
// (-d/2, d/2], differ), the lists fit 16-bit indices and the displacement box stays small; otherwise lf_ok stays
// false and the sign-parity kernel runs.  sb: sign bit of (point-function column, species), 4 species per column.
static int build_local_field_tables(nce_ce_model *m, const nce_ce_tables *t, const std::vector<uint8_t> &sb) {
    const int nB = t->nB, J = t->J, mo = t->mo, n_nbr = t->n_nbr;
    std::vector<char> real((size_t)t->n_pfc, 0);           // point-function columns that change sign
    for (int c = 0; c < t->n_pfc; ++c)
        for (int q = 0; q < 4; ++q) real[c] = real[c] || sb[(size_t)c * 4 + q] != 0;
    // signed k-space offsets of the neighbourhood entries, extents of the box
    const int64_t d[3] = {t->d[0], t->d[1], t->d[2]};
    std::vector<int32_t> so((size_t)nB * n_nbr * 3);
    int e[3] = {0, 0, 0};
    for (size_t i = 0; i < (size_t)nB * n_nbr; ++i)
        for (int c = 0; c < 3; ++c) {
            int64_t x = t->nb_uo[3 * i + c];
            if (x > d[c] / 2) x -= d[c];
            so[3 * i + c] = (int32_t)x;
            e[c] = std::max(e[c], (int)std::llabs(x));
        }
    // (the representatives lie in (-d/2, d/2]: a displacement names one neighbourhood entry at most, unless two
    // entries are one site, which the table construction below refuses)
    const int w0 = 2 * e[0] + 1, w1 = 2 * e[1] + 1, w2 = 2 * e[2] + 1;
    const int64_t bsz = (int64_t)w0 * w1 * w2;
    if ((int64_t)nB * bsz * nB > 65536) return NCE_OK;
    std::vector<int16_t> box((size_t)(nB * bsz * nB), (int16_t)-1);
    for (int a = 0; a < nB; ++a)
        for (int n = 0; n < n_nbr; ++n) {
            const int32_t *x = &so[((size_t)a * n_nbr + n) * 3];
            const int64_t cell = ((int64_t)(x[0] + e[0]) * w1 + (x[1] + e[1])) * w2 + (x[2] + e[2]);
            int16_t &slot = box[((size_t)a * bsz + cell) * nB + t->nb_b[(size_t)a * n_nbr + n]];
            if (slot >= 0) return NCE_OK;                    // two entries at one site: aliasing
            slot = (int16_t)n;
        }
    // per basis and neighbourhood entry n >= 1: the rows with n as a (sign-changing) member
    std::vector<int32_t> off((size_t)nB * (n_nbr + 1), 0);
    std::vector<uint16_t> idx;
    for (int a = 0; a < nB; ++a) {
        std::vector<std::vector<uint16_t>> lists((size_t)n_nbr);
        for (int q = 0; q < t->Rv_len[a]; ++q) {
            int seen = 0;
            for (int k = 0; k < mo; ++k) {
                const size_t i = ((size_t)a * J + q) * mo + k;
                if (!real[t->Rv_pfc[i]]) continue;
                const int n = t->Rv_loc[i];
                for (int k2 = 0; k2 < k; ++k2) {                 // a member listed twice: not a plain cluster instance
                    const size_t i2 = ((size_t)a * J + q) * mo + k2;
                    if (real[t->Rv_pfc[i2]] && t->Rv_loc[i2] == n) return NCE_OK;
                }
                if (n > 0) lists[n].push_back((uint16_t)q);
                seen += n == 0;
            }
            if (seen != 1) return NCE_OK;                        // the row must contain its site exactly once
        }
        for (int n = 0; n < n_nbr; ++n) {
            off[(size_t)a * (n_nbr + 1) + n] = (int32_t)idx.size();
            idx.insert(idx.end(), lists[n].begin(), lists[n].end());
        }
        off[(size_t)a * (n_nbr + 1) + n_nbr] = (int32_t)idx.size();
    }
    if (idx.size() >= 65536 || idx.empty()) return NCE_OK;
    // every reverse row with its sign-changing members, for the field initialisation
    std::vector<int32_t> pmap((size_t)t->n_pfc, -1); int np = 0;
    for (int c = 0; c < t->n_pfc; ++c) if (real[c]) pmap[c] = np++;
    std::vector<uint32_t> rows; std::vector<int4> mem; std::vector<int32_t> roff(nB), rn(nB);
    for (int a = 0; a < nB; ++a) {
        roff[a] = (int32_t)rows.size();
        int last = -1, run = 0;
        for (int q = 0; q < t->Rv_len[a]; ++q) {
            const uint32_t start = (uint32_t)mem.size();
            int nm = 0;
            for (int k = 0; k < mo; ++k) {
                const size_t i = ((size_t)a * J + q) * mo + k;
                const int pl = pmap[t->Rv_pfc[i]];
                if (pl < 0) continue;
                const size_t nb = (size_t)a * n_nbr + t->Rv_loc[i];
                mem.push_back(make_int4(pl * nB + t->nb_b[nb], t->nb_uo[3 * nb], t->nb_uo[3 * nb + 1], t->nb_uo[3 * nb + 2]));
                ++nm;
            }
            const int col = t->Rv_col[(size_t)a * J + q];
            run = col == last ? run + 1 : 1; last = col;
            if (nm > 15 || start >= (1u << 20) || run > 8191) return NCE_OK;
            rows.push_back((uint32_t)col | ((uint32_t)nm << 8) | (start << 12));
        }
        rn[a] = (int32_t)rows.size() - roff[a];
    }
    if (np != m->n_planes) return NCE_OK;                      // same planes as the full-energy kernel
    int rc = upload(m->lf_off, off.data(), off.size());
    if (!rc) rc = upload(m->lf_idx, idx.data(), idx.size());
    if (!rc) rc = upload(m->lf_box, box.data(), box.size());
    if (!rc) rc = upload(m->frows, rows.data(), rows.size());
    if (!rc) rc = upload(m->fmem, mem.data(), mem.size());
    if (!rc) rc = upload(m->frow_off, roff.data(), roff.size());
    if (!rc) rc = upload(m->frow_n, rn.data(), rn.size());
    if (rc) return rc;
    for (int c = 0; c < 3; ++c) m->lf_e[c] = e[c];
    m->lf_nidx = (int32_t)idx.size();
    m->lf_ok = true;
    return NCE_OK;
}

extern "C" {

int nce_ce_create(const nce_ce_tables *t, nce_ce_handle *out) {
    NCE_CHECK(t && out, "nce_ce_create: null argument");
    NCE_CHECK(t->nB >= 1 && t->J >= 1 && t->mo >= 1 && t->mo <= 8, "nce_ce_create: nB/J/mo out of range (mo 1..8)");
    NCE_CHECK(t->n_nbr >= 1 && t->n_nbr <= 65535, "nce_ce_create: n_nbr out of range");
    NCE_CHECK(t->n_pfc >= 1 && t->n_pfc <= 255 && t->max_sp >= 1 && t->max_sp <= 127, "nce_ce_create: n_pfc/max_sp out of range");
    NCE_CHECK(t->d[0] >= 1 && t->d[1] >= 1 && t->d[2] >= 1 && t->d[0] < (1 << 30) && t->d[1] < (1 << 30) && t->d[2] < (1 << 30),
              "nce_ce_create: bad SNF diagonal");
    NCE_CHECK(t->n_cells == t->d[0] * t->d[1] * t->d[2], "nce_ce_create: n_cells != d0*d1*d2");
    NCE_CHECK(t->n_cells <= 0xFFFFFFFFll, "nce_ce_create: more than 2^32 cells");
    NCE_CHECK(t->n_groups >= 1 && t->max_gb >= 1, "nce_ce_create: no active sublattice");
    NCE_CHECK(t->Rv_len && t->Rv_loc && t->Rv_pfc && t->Rv_eci && t->nb_b && t->nb_uo && t->pf && t->act_b && t->act_nb &&
              t->grp_cum && t->T_b && t->T_uo && t->T_pfc && t->T_eci, "nce_ce_create: null table pointer");
    const size_t nl = (size_t)t->nB * t->J * t->mo;
    for (size_t i = 0; i < nl; ++i) {
        NCE_CHECK(t->Rv_loc[i] < t->n_nbr, "nce_ce_create: Rv_loc[%zu]=%d >= n_nbr", i, (int)t->Rv_loc[i]);
        NCE_CHECK(t->Rv_pfc[i] < t->n_pfc, "nce_ce_create: Rv_pfc[%zu] >= n_pfc", i);
    }
    for (int b = 0; b < t->nB; ++b) NCE_CHECK(t->Rv_len[b] >= 0 && t->Rv_len[b] <= t->J, "nce_ce_create: Rv_len out of range");
    for (size_t i = 0; i < (size_t)t->nB * t->n_nbr; ++i) {
        NCE_CHECK(t->nb_b[i] >= 0 && t->nb_b[i] < t->nB, "nce_ce_create: nb_b out of range");
        for (int c = 0; c < 3; ++c)
            NCE_CHECK(t->nb_uo[3 * i + c] >= 0 && t->nb_uo[3 * i + c] < t->d[c], "nce_ce_create: nb_uo out of [0,d)");
    }
    for (size_t i = 0; i < (size_t)t->Rt * t->mo; ++i) {
        NCE_CHECK(t->T_b[i] >= 0 && t->T_b[i] < t->nB && t->T_pfc[i] < t->n_pfc, "nce_ce_create: template row out of range");
        for (int c = 0; c < 3; ++c) NCE_CHECK(t->T_uo[3 * i + c] >= 0 && t->T_uo[3 * i + c] < t->d[c], "nce_ce_create: T_uo out of [0,d)");
    }
    for (int g = 0; g < t->n_groups; ++g) {
        NCE_CHECK(t->act_nb[g] >= 1 && t->act_nb[g] <= t->max_gb, "nce_ce_create: act_nb out of range");
        for (int q = 0; q < t->act_nb[g]; ++q)
            NCE_CHECK(t->act_b[g * t->max_gb + q] >= 0 && t->act_b[g * t->max_gb + q] < t->nB, "nce_ce_create: act_b out of range");
    }
    nce_ce_model *m = new nce_ce_model();
    m->nB = t->nB; m->J = t->J; m->mo = t->mo; m->n_nbr = t->n_nbr; m->n_pfc = t->n_pfc; m->max_sp = t->max_sp;
    m->n_groups = t->n_groups; m->max_gb = t->max_gb; m->Rt = t->Rt;
    for (int c = 0; c < 3; ++c) m->d[c] = t->d[c];
    m->n_cells = t->n_cells; m->N = t->n_cells * t->nB; m->zerolet = t->zerolet;
    cudaGetDevice(&m->device);
    std::vector<float> e32((size_t)t->nB * t->J), p32((size_t)t->n_pfc * t->max_sp), te32(t->Rt);
    for (size_t i = 0; i < e32.size(); ++i) e32[i] = (float)t->Rv_eci[i];
    for (size_t i = 0; i < p32.size(); ++i) p32[i] = (float)t->pf[i];
    for (int i = 0; i < t->Rt; ++i) te32[i] = (float)t->T_eci[i];
    int rc = NCE_OK;
    if (!rc) rc = upload(m->loc, t->Rv_loc, nl);
    if (!rc) rc = upload(m->pfc, t->Rv_pfc, nl);
    if (!rc) rc = upload(m->eci64, t->Rv_eci, e32.size());
    if (!rc) rc = upload(m->eci32, e32.data(), e32.size());
    if (!rc) rc = upload(m->rv_len, t->Rv_len, (size_t)t->nB);
    if (!rc) rc = upload(m->nb_b, t->nb_b, (size_t)t->nB * t->n_nbr);
    if (!rc) rc = upload(m->nb_uo, t->nb_uo, (size_t)t->nB * t->n_nbr * 3);
    if (!rc) rc = upload(m->pf64, t->pf, p32.size());
    if (!rc) rc = upload(m->pf32, p32.data(), p32.size());
    if (!rc) rc = upload(m->act_b, t->act_b, (size_t)t->n_groups * t->max_gb);
    if (!rc) rc = upload(m->act_nb, t->act_nb, (size_t)t->n_groups);
    if (!rc) rc = upload(m->grp_cum, t->grp_cum, (size_t)t->n_groups);
    if (!rc) rc = upload(m->T_b, t->T_b, (size_t)t->Rt * t->mo);
    if (!rc) rc = upload(m->T_uo, t->T_uo, (size_t)t->Rt * t->mo * 3);
    if (!rc) rc = upload(m->T_pfc, t->T_pfc, (size_t)t->Rt * t->mo);
    if (!rc) rc = upload(m->T_eci64, t->T_eci, (size_t)t->Rt);
    if (!rc) rc = upload(m->T_eci32, te32.data(), (size_t)t->Rt);
    if (!rc) {
        cudaError_t e = cudaMalloc((void **)&m->err, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int32_t));
        if (e != cudaSuccess) rc = fail(NCE_ERR_CUDA, "nce_ce_create: %s", cudaGetErrorString(e));
    }
    // sign-parity eligibility: every point-function value is exactly -1 or +1, at most 4 species
    bool bin = t->max_sp <= 4 && t->n_pfc <= 8;          // sign bits of (column, species) fit one 32-bit mask
    // point-function columns the rows use (an inert sublattice's unused columns, and species a sublattice does not
    // allow, carry 0 in the table and do not matter)
    std::vector<char> used((size_t)t->n_pfc, 0);
    for (int b = 0; b < t->nB; ++b)
        for (int q = 0; q < t->Rv_len[b]; ++q)
            for (int k = 0; k < t->mo; ++k) {
                const int c = t->Rv_pfc[((size_t)b * t->J + q) * t->mo + k];
                if (c >= 0 && c < t->n_pfc) used[c] = 1;
            }
    std::vector<uint8_t> sb((size_t)t->n_pfc * 4, 0);
    for (int c = 0; c < t->n_pfc && bin; ++c)
        for (int q = 0; q < t->max_sp && used[c]; ++q) {
            const double v = t->pf[(size_t)c * t->max_sp + q];
            if (v == 1.0 || v == 0.0) sb[(size_t)c * 4 + q] = 0;
            else if (v == -1.0) sb[(size_t)c * 4 + q] = 1;
            else bin = false;
        }
    // column eci: every reverse row of one cluster-vector column must carry the same eci
    if (bin && t->Rv_col && t->n_cols >= 1 && t->n_cols <= 255 && (int64_t)t->n_pfc * t->n_nbr <= 65535 && t->J <= 65535) {
        std::vector<double> colv((size_t)t->n_cols, 0.0); std::vector<char> seen((size_t)t->n_cols, 0);
        for (int b = 0; b < t->nB && bin; ++b)
            for (int q = 0; q < t->Rv_len[b]; ++q) {
                const int c = t->Rv_col[(size_t)b * t->J + q];
                const double v = t->Rv_eci[(size_t)b * t->J + q];
                if (c < 0 || c >= t->n_cols) { bin = false; break; }
                if (!seen[c]) { seen[c] = 1; colv[c] = v; }
                else if (colv[c] != v) { bin = false; break; }
                if (q > 0 && c < t->Rv_col[(size_t)b * t->J + q - 1]) { bin = false; break; }   // rows sorted by column
            }
        if (bin && !rc) {
            std::vector<double> e2(colv.size()); std::vector<float> f2(colv.size());
            for (size_t i = 0; i < colv.size(); ++i) { e2[i] = 2.0 * colv[i]; f2[i] = 2.0f * (float)colv[i]; }
            std::vector<uint16_t> bx(nl); std::vector<uint8_t> rc8((size_t)t->nB * t->J);
            for (size_t i = 0; i < nl; ++i) bx[i] = (uint16_t)(t->Rv_pfc[i] * t->n_nbr + t->Rv_loc[i]);
            for (size_t i = 0; i < rc8.size(); ++i) rc8[i] = (uint8_t)std::max(0, std::min(254, t->Rv_col[i]));
            rc = upload(m->sbits, sb.data(), sb.size());
            if (!rc) rc = upload(m->bix, bx.data(), bx.size());
            if (!rc) rc = upload(m->rcol, rc8.data(), rc8.size());
            if (!rc) rc = upload(m->ecol2_64, e2.data(), e2.size());
            {
                // fixed point for exact dE sums: |sum_c n_c e_c| <= 2 J max|e| 2^S < 2^61
                double emax = 0.0;
                for (double v : e2) emax = std::max(emax, std::fabs(v));
                int S = 60;
                if (emax > 0.0) S = std::min(60, (int)std::floor(61.0 - std::log2(2.0 * t->J * emax)));
                if (S >= 20) {
                    std::vector<int64_t> ef(e2.size());
                    for (size_t i = 0; i < e2.size(); ++i) ef[i] = (int64_t)std::llround(std::ldexp(e2[i], S));
                    if (!rc) rc = upload(m->ecol_fix, ef.data(), ef.size());
                    m->fix_shift = S;
                }
            }
            if (!rc) rc = upload(m->ecol2_32, f2.data(), f2.size());
            // column-aligned chunks of at most 32 consecutive rows
            std::vector<std::vector<uint32_t>> ch(t->nB);
            for (int b = 0; b < t->nB; ++b) {
                int q = 0;
                const int Jb = t->Rv_len[b];
                while (q < Jb) {
                    const int c = t->Rv_col[(size_t)b * t->J + q];
                    int e = q;
                    while (e < Jb && e - q < 32 && t->Rv_col[(size_t)b * t->J + e] == c) ++e;
                    ch[b].push_back((uint32_t)c | ((uint32_t)q << 8) | ((uint32_t)(e - q) << 24));
                    q = e;
                }
            }
            size_t mx = 1;
            for (auto &v : ch) mx = std::max(mx, v.size());
            std::vector<uint32_t> flat((size_t)t->nB * mx, 0u); std::vector<int32_t> nch(t->nB);
            for (int b = 0; b < t->nB; ++b) { nch[b] = (int32_t)ch[b].size(); std::copy(ch[b].begin(), ch[b].end(), flat.begin() + (size_t)b * mx); }
            if (!rc) rc = upload(m->chunks, flat.data(), flat.size());
            if (!rc) rc = upload(m->n_chunks, nch.data(), nch.size());
            m->max_chunks = (int32_t)mx;
            m->n_cols = t->n_cols;
            // rows anchored at the site (slot 0): every cluster instance of the cell exactly once, for the full energy
            if (t->Rv_slot && !rc) {
                std::vector<int32_t> pmap((size_t)t->n_pfc, -1), ppfc;
                for (int c = 0; c < t->n_pfc; ++c) {
                    bool any = false;
                    for (int q = 0; q < 4; ++q) any = any || (sb[(size_t)c * 4 + q] != 0);
                    if (any) { pmap[c] = (int32_t)ppfc.size(); ppfc.push_back(c); }
                }
                std::vector<uint32_t> rows; std::vector<int4> mem; std::vector<int32_t> roff(t->nB), rn(t->nB);
                for (int b = 0; b < t->nB; ++b) {
                    roff[b] = (int32_t)rows.size();
                    for (int q = 0; q < t->Rv_len[b]; ++q) {
                        if (t->Rv_slot[(size_t)b * t->J + q] != 0) continue;
                        const uint32_t start = (uint32_t)mem.size();
                        int nm = 0;
                        for (int k = 0; k < t->mo; ++k) {
                            const size_t e = ((size_t)b * t->J + q) * t->mo + k;
                            const int pl = pmap[t->Rv_pfc[e]];
                            if (pl < 0) continue;                          // constant point function (padded member)
                            const int loc = t->Rv_loc[e];
                            const size_t nb = (size_t)b * t->n_nbr + loc;
                            mem.push_back(make_int4(pl * t->nB + t->nb_b[nb], t->nb_uo[3 * nb], t->nb_uo[3 * nb + 1], t->nb_uo[3 * nb + 2]));
                            ++nm;
                        }
                        if (nm > 15 || start >= (1u << 20)) { bin = false; break; }
                        rows.push_back((uint32_t)t->Rv_col[(size_t)b * t->J + q] | ((uint32_t)nm << 8) | (start << 12));
                    }
                    rn[b] = (int32_t)rows.size() - roff[b];
                }
                if (bin && !ppfc.empty()) {
                    if (!rc) rc = upload(m->brows, rows.data(), rows.size());
                    if (!rc) rc = upload(m->bmem, mem.data(), mem.size());
                    if (!rc) rc = upload(m->brow_off, roff.data(), roff.size());
                    if (!rc) rc = upload(m->brow_n, rn.data(), rn.size());
                    if (!rc) rc = upload(m->plane_pfc, ppfc.data(), ppfc.size());
                    if (!rc) rc = upload(m->ecol1, colv.data(), colv.size());
                    m->n_planes = (int32_t)ppfc.size();
                }
            }
            if (!rc && bin && m->brows && m->fix_shift > 0) rc = build_local_field_tables(m, t, sb);
            m->binary = !rc;
        }
    }
    if (rc) { free_model(m); return rc; }
    *out = m;
    return NCE_OK;
}

int nce_ce_destroy(nce_ce_handle h) {
    if (!h) return NCE_OK;
    cudaDeviceSynchronize();
    return free_model(h);
}

int nce_ce_energy(nce_ce_handle h, const int8_t *sigma, int32_t R, int32_t precision, double *E, void *stream) {
    NCE_CHECK(h && sigma && E && R >= 1, "nce_ce_energy: bad argument");
    NCE_CHECK(precision == 64 || precision == 32, "nce_ce_energy: precision must be 64 or 32");
    std::lock_guard<std::mutex> lk(h->mu);
    return energy_impl(h, sigma, R, precision, E, nullptr, (cudaStream_t)stream);
}

int nce_ce_cluster_counts(nce_ce_handle h, const int8_t *sigma, int32_t R, int64_t *cv, void *stream) {
    NCE_CHECK(h && sigma && cv && R >= 1, "nce_ce_cluster_counts: bad argument");
    NCE_CHECK(h->binary && h->brows, "nce_ce_cluster_counts: needs point functions in {-1, +1}");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaStream_t s = (cudaStream_t)stream;
    NCE_CUDA(cudaMemsetAsync(cv, 0, sizeof(int64_t) * (size_t)R * h->n_cols, s));
    return energy_impl(h, sigma, R, 64, nullptr, cv, s);
}

int nce_ce_energy_from_counts(nce_ce_handle h, const int64_t *cv, int32_t R, double *E, void *stream) {
    NCE_CHECK(h && cv && E && R >= 1, "nce_ce_energy_from_counts: bad argument");
    NCE_CHECK(h->binary && h->ecol1, "nce_ce_energy_from_counts: needs point functions in {-1, +1}");
    ce_energy_counts_kernel<<<(R + 127) / 128, 128, 0, (cudaStream_t)stream>>>(cv, R, h->n_cols, h->ecol1, h->zerolet, E);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

}  // extern "C"

// full energy of R configurations; cv_out (R, n_cols) additionally receives the cluster-vector sums (sign-parity
// kernel only, zeroed by the caller); E may be null when only the sums are wanted
static int energy_impl(nce_ce_model *h, const int8_t *sigma, int32_t R, int32_t precision, double *E, int64_t *cv_out,
                       cudaStream_t s) {
    if (h->binary && h->brows) {
        // sign-parity full energy, bit-sliced: planes of the configurations, exact column sums, float64 energy
        NCE_CHECK(R <= 65535, "energy: at most 65535 configurations per call");
        const int64_t d0 = h->d[0], d1 = h->d[1], d2 = h->d[2];
        NCE_CHECK(d2 < (1 << 28) && d0 * d1 < (1ll << 40), "energy: lattice too large");
        const int32_t W2 = (int32_t)((2 * d2 + 31) / 32 + 1);
        const int32_t P = h->n_planes * h->nB;
        StreamScratch planes, cvs;
        NCE_CUDA(planes.alloc(sizeof(uint32_t) * (size_t)R * P * d0 * d1 * W2, s));
        int64_t *cv = cv_out;
        if (!cv) {
            const size_t need_c = (size_t)R * h->n_cols;
            NCE_CUDA(cvs.alloc(sizeof(int64_t) * need_c, s));
            cv = (int64_t *)cvs.p;
            NCE_CUDA(cudaMemsetAsync(cv, 0, sizeof(int64_t) * need_c, s));
        }
        const int64_t prow = (int64_t)R * P * d0 * d1;
        const int pb = (int)std::min<int64_t>((prow + 7) / 8, 1 << 20);
        ce_bitplane_kernel<<<pb, 256, 0, s>>>(sigma, R, h->N, h->nB, d0 * d1, (int32_t)d2, W2, h->plane_pfc, h->n_planes, h->sbits,
                                              (uint32_t *)planes.p);
        NCE_CUDA(cudaGetLastError());
        const int64_t items = d0 * d1 * ((d2 + 31) / 32);
        const int64_t ib = std::min<int64_t>((items + 255) / 256, 8192);
        // small cells: split the rows so that the launch still covers the SMs (about 4 blocks per SM)
        int nsm = 152;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device);
        const int64_t have = ib * h->nB * R;
        const int slices = (int)std::max<int64_t>(1, std::min<int64_t>(32, (4ll * nsm + have - 1) / have));
        ce_energy_bits_kernel<<<dim3((unsigned)(ib * slices), h->nB, R), 256, sizeof(unsigned long long) * h->n_cols, s>>>(
            (const uint32_t *)planes.p, P, (int32_t)d0, (int32_t)d1, (int32_t)d2, W2, h->brows, h->bmem, h->brow_off, h->brow_n, h->n_cols, slices,
            (unsigned long long *)cv);
        NCE_CUDA(cudaGetLastError());
        if (E) {
            ce_energy_counts_kernel<<<(R + 127) / 128, 128, 0, s>>>(cv, R, h->n_cols, h->ecol1, h->zerolet, E);
            NCE_CUDA(cudaGetLastError());
        }
        return NCE_OK;
    }
    NCE_CHECK(E && !cv_out, "energy: cluster-vector sums need the sign-parity tables");
    NCE_CHECK(R <= 65535, "energy: at most 65535 configurations per call");   // one grid row per configuration
    const int threads = 256;
    int nblk = (int)std::min<int64_t>((h->n_cells + threads - 1) / threads, 1184);
    nblk = std::max(nblk, 1);
    StreamScratch partial;
    NCE_CUDA(partial.alloc(sizeof(double) * (size_t)nblk * R, s));
    double *energy_partial = (double *)partial.p;
    dim3 grid(nblk, R);
    if (precision == 64)
        ce_energy_kernel<double><<<grid, threads, 0, s>>>(sigma, h->N, h->n_cells, h->nB, (int)h->d[0], (int)h->d[1], (int)h->d[2],
                                                          h->Rt, h->mo, h->T_b, h->T_uo, h->T_pfc, h->T_eci64, h->pf64, h->max_sp,
                                                          energy_partial);
    else
        ce_energy_kernel<float><<<grid, threads, 0, s>>>(sigma, h->N, h->n_cells, h->nB, (int)h->d[0], (int)h->d[1], (int)h->d[2],
                                                         h->Rt, h->mo, h->T_b, h->T_uo, h->T_pfc, h->T_eci32, h->pf32, h->max_sp,
                                                         energy_partial);
    NCE_CUDA(cudaGetLastError());
    ce_energy_finish<<<(R + 127) / 128, 128, 0, s>>>(energy_partial, nblk, R, h->zerolet, E);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

extern "C" {

int nce_ce_delta(nce_ce_handle h, const int8_t *sigma, int32_t R, int32_t n, const int32_t *rep, const int64_t *ia,
                 const int64_t *ib, const int8_t *sa_new, const int8_t *sb_new, int32_t precision, int32_t warps,
                 double *out, void *stream) {
    NCE_CHECK(h && sigma && R >= 1 && n >= 0, "nce_ce_delta: bad argument");
    if (n == 0) return NCE_OK;
    NCE_CHECK(rep && ia && ib && sa_new && sb_new && out, "nce_ce_delta: null pointer");
    NCE_CHECK(precision == 64 || precision == 32, "nce_ce_delta: precision must be 64 or 32");
    if (warps <= 0) warps = 8;
    NCE_CHECK(warps <= 32, "nce_ce_delta: warps must be <= 32");
    nce_pt_state st; std::memset(&st, 0, sizeof(st));
    st.R = R; st.N = h->N; st.sigma = const_cast<int8_t *>(sigma);
    nce_pt_chunk ck; std::memset(&ck, 0, sizeof(ck)); ck.precision = precision;
    CEJob jb = make_job(h, &st, &ck, 0);
    cudaStream_t s = (cudaStream_t)stream;
    return precision == 64 ? launch_delta<double>(jb, h->mo, n, rep, ia, ib, sa_new, sb_new, out, warps, s)
                           : launch_delta<float>(jb, h->mo, n, rep, ia, ib, sa_new, sb_new, out, warps, s);
}

int nce_ce_run_chunk(nce_ce_handle h, const nce_pt_state *st, const nce_pt_chunk *ck, void *stream) {
    NCE_CHECK(h && st && ck, "nce_ce_run_chunk: null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    return run_batch(1, &h, st, ck, (cudaStream_t)stream);
}

int nce_ce_run_batch(int32_t n_jobs, const nce_ce_handle *hs, const nce_pt_state *st, const nce_pt_chunk *ck, void *stream) {
    NCE_CHECK(hs && st && ck, "nce_ce_run_batch: null argument");
    return run_batch(n_jobs, hs, st, ck, (cudaStream_t)stream);
}

int nce_pt_minimum(const nce_pt_state *st, double *out_min, int32_t *out_arg, void *stream) {
    NCE_CHECK(st && st->E && st->E_min_rep && out_min && out_arg && st->R >= 1, "nce_pt_minimum: bad argument");
    pt_minimum_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(st->E, st->E_min_rep, st->R, out_min, out_arg);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

int nce_ce_run_chunk_host(nce_ce_handle h, int32_t R, int8_t *sigma_host, double *E_host, const float *beta_slot_host,
                          int32_t *rep_of_slot_host, int32_t *slot_of_rep_host, const int32_t *ladder_id_host,
                          double *E_min_rep_host, int64_t *n_acc_host, int64_t *n_ex_host, const nce_pt_chunk *ckh,
                          double *E_samples_host) {
    NCE_CHECK(h && R >= 1 && sigma_host && E_host && beta_slot_host && rep_of_slot_host && slot_of_rep_host && ladder_id_host &&
              E_min_rep_host && n_acc_host && n_ex_host && ckh, "nce_ce_run_chunk_host: null argument");
    int rc = check_chunk(nullptr, ckh); if (rc) return rc;
    std::lock_guard<std::mutex> lk(h->mu);
    const int64_t N = h->N, T = ckh->n_steps;
    const bool props = ckh->prop_a != nullptr;
    const int64_t nsamp = (E_samples_host && ckh->sample_interval > 0) ? T / ckh->sample_interval : 0;
    const int64_t nexu = ckh->ex_u ? (R - 1 + 1) / 2 : 0;
    // the local-field path keeps per-site fields on the device; here they are rebuilt from the uploaded occupancies
    const bool lf = h->lf_ok && ckh->precision == 64 && (ckh->path == 3 || ckh->path == 0);
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    size_t off[16]; size_t o = 0; int k = 0;
    const size_t sizes[] = {(size_t)R * N, sizeof(double) * R, sizeof(float) * R, sizeof(int32_t) * R, sizeof(int32_t) * R,
                            sizeof(int32_t) * R, sizeof(double) * R, sizeof(int64_t) * R, sizeof(int64_t),
                            props ? sizeof(int32_t) * T * R : 0, props ? sizeof(int32_t) * T * R : 0,
                            props ? sizeof(double) * T * R : 0, sizeof(double) * nsamp * R, sizeof(double) * nexu,
                            lf ? sizeof(int64_t) * R * N : 0};
    for (size_t sz : sizes) { off[k++] = o; o = al(o + sz); }
    if (o > h->staging_bytes) {
        if (h->staging_base) cudaFree(h->staging_base);
        h->staging_base = nullptr; h->staging_bytes = 0;
        NCE_CUDA(cudaMalloc(&h->staging_base, o));
        h->staging_bytes = o;
    }
    char *b = (char *)h->staging_base;
    nce_pt_state st; std::memset(&st, 0, sizeof(st));
    st.R = R; st.N = N; st.sigma = (int8_t *)(b + off[0]); st.E = (double *)(b + off[1]); st.beta_slot = (float *)(b + off[2]);
    st.rep_of_slot = (int32_t *)(b + off[3]); st.slot_of_rep = (int32_t *)(b + off[4]); st.ladder_id = (int32_t *)(b + off[5]);
    st.E_min_rep = (double *)(b + off[6]); st.n_acc = (int64_t *)(b + off[7]); st.n_ex = (int64_t *)(b + off[8]);
    nce_pt_chunk ck = *ckh;
    cudaStream_t s = 0;
    NCE_CUDA(cudaMemcpyAsync(st.sigma, sigma_host, (size_t)R * N, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.E, E_host, sizeof(double) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync((void *)st.beta_slot, beta_slot_host, sizeof(float) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.rep_of_slot, rep_of_slot_host, sizeof(int32_t) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.slot_of_rep, slot_of_rep_host, sizeof(int32_t) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync((void *)st.ladder_id, ladder_id_host, sizeof(int32_t) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.E_min_rep, E_min_rep_host, sizeof(double) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.n_acc, n_acc_host, sizeof(int64_t) * R, cudaMemcpyHostToDevice, s));
    NCE_CUDA(cudaMemcpyAsync(st.n_ex, n_ex_host, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    if (props) {
        ck.prop_a = (int32_t *)(b + off[9]); ck.prop_b = (int32_t *)(b + off[10]); ck.prop_u = (double *)(b + off[11]);
        NCE_CUDA(cudaMemcpyAsync((void *)ck.prop_a, ckh->prop_a, sizeof(int32_t) * T * R, cudaMemcpyHostToDevice, s));
        NCE_CUDA(cudaMemcpyAsync((void *)ck.prop_b, ckh->prop_b, sizeof(int32_t) * T * R, cudaMemcpyHostToDevice, s));
        NCE_CUDA(cudaMemcpyAsync((void *)ck.prop_u, ckh->prop_u, sizeof(double) * T * R, cudaMemcpyHostToDevice, s));
    }
    ck.E_samples = nsamp ? (double *)(b + off[12]) : nullptr;
    if (nexu) {
        ck.ex_u = (double *)(b + off[13]);
        NCE_CUDA(cudaMemcpyAsync((void *)ck.ex_u, ckh->ex_u, sizeof(double) * nexu, cudaMemcpyHostToDevice, s));
    }
    if (lf) {
        st.field = (int64_t *)(b + off[14]);
        if (R > 65535) return fail(NCE_ERR_INVALID, "nce_ce_run_chunk_host: at most 65535 replicas on the local-field path");
        rc = field_init_impl(h, st.sigma, R, st.field, s);
        if (rc) return rc;
    }
    rc = run_batch(1, &h, &st, &ck, s);
    if (rc) return rc;
    NCE_CUDA(cudaMemcpyAsync(sigma_host, st.sigma, (size_t)R * N, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaMemcpyAsync(E_host, st.E, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaMemcpyAsync(rep_of_slot_host, st.rep_of_slot, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaMemcpyAsync(slot_of_rep_host, st.slot_of_rep, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaMemcpyAsync(E_min_rep_host, st.E_min_rep, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaMemcpyAsync(n_acc_host, st.n_acc, sizeof(int64_t) * R, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaMemcpyAsync(n_ex_host, st.n_ex, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    if (nsamp) NCE_CUDA(cudaMemcpyAsync(E_samples_host, ck.E_samples, sizeof(double) * nsamp * R, cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaStreamSynchronize(s));
    return NCE_OK;
}

}  // extern "C"

// ── full energy without any allocation ─────────────────────────────────────────────────────────────
// Some callers cannot allocate device memory once they are running: a process whose device memory is all
// reserved up front by its own pool (nce_ce_energy takes its scratch from the device's default stream-ordered
// pool, which would fail or fragment it), or a loop that must not touch any allocator.  nce_ce_energy_noalloc serves
// them: the per-block float64 partials of ce_energy_kernel live in the fixed array below, which the CUDA driver
// places in device memory with the rest of this library's image on each device the library is used on, and
// which stays there until the process exits.  Every call on a device shares this one array; calls that overlap
// on the GPU (two streams at once) race on it.  Each launch writes every partial it later reads, so nothing
// has to be cleared between calls.
namespace nce {
constexpr int64_t kNoAllocPartials = 65536;                                    // 512 KiB of float64 partials
// configurations per call: one grid row (gridDim.y) per configuration, and gridDim.y is at most 65,535
constexpr int32_t kNoAllocMaxConfigs = 65535;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];
static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[256];                                             // per device ordinal

// Device address of the array on the current device (host code must not use the symbol itself as a pointer).
static int noalloc_partials(double **out) {
    int dev = 0;
    NCE_CUDA(cudaGetDevice(&dev));
    NCE_CHECK(dev >= 0 && dev < 256, "nce_ce_energy_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        NCE_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partials));
        g_noalloc_ptr[dev] = (double *)p;
    }
    *out = g_noalloc_ptr[dev];
    return NCE_OK;
}
}  // namespace nce

namespace nce {
int ce_error_peek(nce_ce_handle h, int32_t *flags) {
    NCE_CHECK(h && flags, "ce_error_peek: null argument");
    NCE_CUDA(cudaMemcpy(flags, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return NCE_OK;
}
const char *ce_error_text(int32_t f) {
    if (f & 2) return "a delta query was out of range (NaN returned)";
    if (f & 1) return "a proposal index was out of range (the move was rejected)";
    return "no error";
}
}  // namespace nce

extern "C" {

int nce_ce_energy_noalloc(nce_ce_handle h, const int8_t *sigma, int32_t R, int32_t precision, double *E, void *stream) {
    NCE_CHECK(h && sigma && E && R >= 1, "nce_ce_energy_noalloc: bad argument");
    NCE_CHECK(precision == 64 || precision == 32, "nce_ce_energy_noalloc: precision must be 64 or 32");
    NCE_CHECK(R <= kNoAllocMaxConfigs, "nce_ce_energy_noalloc: %d configurations exceed the limit of %d per call", R,
              kNoAllocMaxConfigs);
    double *partial = nullptr;
    int rc = noalloc_partials(&partial);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int threads = 256;
    // same blocks per configuration as nce_ce_energy, reduced so that R x blocks fits the fixed array
    int64_t nblk = std::min<int64_t>((h->n_cells + threads - 1) / threads, 1184);
    nblk = std::max<int64_t>(1, std::min<int64_t>(nblk, kNoAllocPartials / R));
    dim3 grid((unsigned)nblk, R);
    if (precision == 64)
        ce_energy_kernel<double><<<grid, threads, 0, s>>>(sigma, h->N, h->n_cells, h->nB, (int)h->d[0], (int)h->d[1], (int)h->d[2],
                                                          h->Rt, h->mo, h->T_b, h->T_uo, h->T_pfc, h->T_eci64, h->pf64, h->max_sp,
                                                          partial);
    else
        ce_energy_kernel<float><<<grid, threads, 0, s>>>(sigma, h->N, h->n_cells, h->nB, (int)h->d[0], (int)h->d[1], (int)h->d[2],
                                                         h->Rt, h->mo, h->T_b, h->T_uo, h->T_pfc, h->T_eci32, h->pf32, h->max_sp,
                                                         partial);
    NCE_CUDA(cudaGetLastError());
    ce_energy_finish<<<(R + 127) / 128, 128, 0, s>>>(partial, (int32_t)nblk, R, h->zerolet, E);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

int nce_ce_has_local_field(nce_ce_handle h, int32_t *ok, double *scale) {
    NCE_CHECK(h && ok, "nce_ce_has_local_field: null argument");
    *ok = h->lf_ok ? 1 : 0;
    if (scale) *scale = h->fix_shift > 0 ? std::ldexp(1.0, -h->fix_shift) : 0.0;
    return NCE_OK;
}

int nce_ce_field_init(nce_ce_handle h, const int8_t *sigma, int32_t R, int64_t *field, void *stream) {
    NCE_CHECK(h && sigma && field && R >= 1, "nce_ce_field_init: bad argument");
    std::lock_guard<std::mutex> lk(h->mu);
    return field_init_impl(h, sigma, R, field, (cudaStream_t)stream);
}

}  // extern "C"

static int field_init_impl(nce_ce_model *h, const int8_t *sigma, int32_t R, int64_t *field, cudaStream_t s) {
    NCE_CHECK(h->lf_ok, "nce_ce_field_init: the local-field path is not available for this cell");
    NCE_CHECK(R <= 65535, "nce_ce_field_init: at most 65535 configurations per call");
    const int64_t d0 = h->d[0], d1 = h->d[1], d2 = h->d[2];
    NCE_CHECK(d2 < (1 << 28) && d0 * d1 < (1ll << 40), "nce_ce_field_init: lattice too large");
    const int32_t W2 = (int32_t)((2 * d2 + 31) / 32 + 1);
    const int32_t P = h->n_planes * h->nB;
    StreamScratch planes;
    NCE_CUDA(planes.alloc(sizeof(uint32_t) * (size_t)R * P * d0 * d1 * W2, s));
    const int64_t prow = (int64_t)R * P * d0 * d1;
    const int pb = (int)std::min<int64_t>((prow + 7) / 8, 1 << 20);
    ce_bitplane_kernel<<<pb, 256, 0, s>>>(sigma, R, h->N, h->nB, d0 * d1, (int32_t)d2, W2, h->plane_pfc, h->n_planes, h->sbits,
                                          (uint32_t *)planes.p);
    NCE_CUDA(cudaGetLastError());
    const int64_t items = d0 * d1 * ((d2 + 31) / 32);
    ce_field_bits_kernel<<<dim3((unsigned)((items + 127) / 128), h->nB, R), 128, 0, s>>>(
        (const uint32_t *)planes.p, P, (int32_t)d0, (int32_t)d1, (int32_t)d2, W2, h->nB, h->N, h->frows, h->fmem, h->frow_off,
        h->frow_n, h->ecol_fix, (long long *)field);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

extern "C" {

int nce_ce_errors(nce_ce_handle h, int32_t *flags) {
    NCE_CHECK(h && flags, "nce_ce_errors: null argument");
    NCE_CUDA(cudaMemcpy(flags, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    NCE_CUDA(cudaMemset(h->err, 0, sizeof(int32_t)));
    return NCE_OK;
}

}  // extern "C"
