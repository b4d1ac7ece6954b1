/* CPU oracle of the cluster-expansion parallel-tempering path -- TEST INFRASTRUCTURE ONLY.
 *
 * Used by the tests, the smoke check and the CPU-baseline legs of bench.py to check the product path;
 * the product never links or calls it.  float64 throughout, sequential sums in the reference's order.
 *
 * Restates, on the reference's own table layout (Rv_b / Rv_uo / Rv_st / Rv_bf / Rv_eci per basis site):
 *   delta_energy_a          neuralce/ce/ce_gpu_implicit.py:181-191  (rows of i_a, plus rows of i_b not containing i_a)
 *   energy_a                neuralce/ce/ce_gpu_implicit.py:147-163
 *   mc_step (delta branch)  neuralce/ce/pt_mcmc_ce.py:558-566      (accept = valid && log u < -beta*dE, E += dE)
 *   micro / run_chunk       neuralce/ce/pt_mcmc_ce.py:765-818      (per-slot proposals, slot-ordered samples,
 *                                                                   running minimum, chunk-end exchange)
 *   exchange_slots          neuralce/ce/pt_mcmc_ce.py:748-760
 * Proposals and uniforms come either from host arrays indexed [step][slot] or from Philox4x32-10
 * (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), with the same
 * counter layout as the CUDA kernels.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int32_t nB, J, mo, Rt, n_bf, max_sp;
    int64_t d[3];
    int64_t n_cells;
    double zerolet;
    const int32_t *Rv_b, *Rv_uo, *Rv_st, *Rv_bf; const double *Rv_eci;     /* (nB,J,mo[,3]), (nB,J) */
    const int32_t *T_b, *T_uo, *T_st, *T_bf; const double *T_eci;          /* (Rt,mo[,3]), (Rt,)   */
    const double *pf;                                                       /* (n_sl, n_bf, max_sp) */
    /* proposal groups (active sublattices) */
    int32_t n_groups, max_gb;
    const int32_t *act_b, *act_nb;                                          /* (n_groups,max_gb), (n_groups,) */
    const uint64_t *grp_cum;                                                /* (n_groups,) thresholds in 2^32 units */
} orc_tables;

typedef struct {
    int32_t R; int64_t N;
    int8_t *sigma; double *E; const float *beta_slot;
    int32_t *rep_of_slot, *slot_of_rep; const int32_t *ladder_id;
    double *E_min_rep; int64_t *n_acc; int64_t *n_ex;
    int64_t *n_near;                                          /* (R) near-threshold steps per replica, or NULL */
} orc_state;

typedef struct {
    int64_t n_steps, step0;
    const int32_t *prop_a, *prop_b; const double *prop_u;   /* [step][slot]; NULL -> Philox */
    uint64_t seed;
    int64_t sample_interval; double *E_samples;            /* [(n_steps/si)][slot] or NULL */
    int32_t do_exchange; int32_t ex_parity; const double *ex_u; /* ex_u NULL -> Philox; ex_parity: bit q = round q */
    int32_t n_threads;
    int32_t rounds;          /* exchange rounds back to back (0 or 1: one round) */
    double near_eV;          /* a step is near its threshold when |dE - (-ln u / beta)| < near_eV */
} orc_chunk;

/* ── Philox4x32-10 ─────────────────────────────────────────────────────────────────────────────── */
void orc_philox4x32(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline uint32_t mulhi_idx(uint32_t x, uint32_t n) { return (uint32_t)(((uint64_t)x * n) >> 32); }
static inline double u01_open0(uint32_t hi, uint32_t lo) {   /* (0, 1] with 53 random bits */
    uint64_t m = ((uint64_t)hi << 21) | (lo >> 11);
    return (double)(m + 1) * 0x1.0p-53;
}

/* proposal of replica-slot t at global step g: (i_a, i_b, u) */
void orc_propose(const orc_tables *tb, uint64_t seed, int64_t g, int32_t t, int64_t *ia, int64_t *ib, double *u) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)g, (uint32_t)((uint64_t)g >> 32), (uint32_t)t, 0u}, x[4];
    orc_philox4x32(ctr, key, x);
    uint32_t n_cells = (uint32_t)tb->n_cells;
    int32_t grp = 0; uint32_t ba = 0, bb = 0;
    if (tb->n_groups > 1 || tb->act_nb[0] > 1) {
        uint32_t y[4]; ctr[3] = 1u; orc_philox4x32(ctr, key, y);
        if (tb->n_groups > 1) { while (grp < tb->n_groups - 1 && (uint64_t)y[0] >= tb->grp_cum[grp]) ++grp; }
        ba = mulhi_idx(y[1], (uint32_t)tb->act_nb[grp]); bb = mulhi_idx(y[2], (uint32_t)tb->act_nb[grp]);
    }
    *ia = (int64_t)mulhi_idx(x[0], n_cells) * tb->nB + tb->act_b[grp * tb->max_gb + ba];
    *ib = (int64_t)mulhi_idx(x[1], n_cells) * tb->nB + tb->act_b[grp * tb->max_gb + bb];
    *u = u01_open0(x[2], x[3]);
}

/* exchange randoms of round q of the chunk ending at global step g (after the step): parity and pair uniforms,
 * counter word 2 = 0xFFFFFFFF - 2q (parity) and 0xFFFFFFFE - 2q (uniform of pair k, word 3 = k) */
int32_t orc_ex_parity(uint64_t seed, int64_t g, int32_t q) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)g, (uint32_t)((uint64_t)g >> 32), 0xFFFFFFFFu - 2u * (uint32_t)q, 0u}, x[4];
    orc_philox4x32(ctr, key, x);
    return (int32_t)(x[0] & 1u);
}
double orc_ex_uniform(uint64_t seed, int64_t g, int32_t q, int32_t k) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)g, (uint32_t)((uint64_t)g >> 32), 0xFFFFFFFEu - 2u * (uint32_t)q, (uint32_t)k}, x[4];
    orc_philox4x32(ctr, key, x);
    return u01_open0(x[0], x[1]);
}

/* ── energy ────────────────────────────────────────────────────────────────────────────────────── */
static inline int64_t site_of(const orc_tables *tb, int32_t b, int64_t k0, int64_t k1, int64_t k2) {
    return ((k0 * tb->d[1] + k1) * tb->d[2] + k2) * tb->nB + b;
}

double orc_ce_energy(const orc_tables *tb, const int8_t *sigma) {
    double tot = 0.0;
    const int64_t *d = tb->d;
    for (int64_t c = 0; c < tb->n_cells; ++c) {
        int64_t k0 = c / (d[1] * d[2]), k1 = (c / d[2]) % d[1], k2 = c % d[2];
        for (int32_t r = 0; r < tb->Rt; ++r) {
            double pr = 1.0;
            for (int32_t m = 0; m < tb->mo; ++m) {
                const int32_t *uo = tb->T_uo + ((int64_t)r * tb->mo + m) * 3;
                int64_t s = site_of(tb, tb->T_b[r * tb->mo + m], (k0 + uo[0]) % d[0], (k1 + uo[1]) % d[1], (k2 + uo[2]) % d[2]);
                int32_t st = tb->T_st[r * tb->mo + m], bf = tb->T_bf[r * tb->mo + m];
                pr *= tb->pf[((int64_t)st * tb->n_bf + bf) * tb->max_sp + sigma[s]];
            }
            tot += tb->T_eci[r] * pr;
        }
    }
    return tb->zerolet + tot;
}

/* ── delta energy of the swap (i_a -> s_a_new, i_b -> s_b_new) ──────────────────────────────────── */
double orc_ce_delta(const orc_tables *tb, const int8_t *sigma, int64_t ia, int64_t ib, int32_t sa_new, int32_t sb_new) {
    const int64_t *d = tb->d;
    double sum_a = 0.0, sum_b = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        int64_t i = pass ? ib : ia;
        int32_t b = (int32_t)(i % tb->nB); int64_t c = i / tb->nB;
        int64_t k0 = c / (d[1] * d[2]), k1 = (c / d[2]) % d[1], k2 = c % d[2];
        for (int32_t j = 0; j < tb->J; ++j) {
            double pn = 1.0, po = 1.0; int hits_a = 0;
            for (int32_t m = 0; m < tb->mo; ++m) {
                int64_t e = ((int64_t)b * tb->J + j) * tb->mo + m;
                const int32_t *uo = tb->Rv_uo + e * 3;
                int64_t s = site_of(tb, tb->Rv_b[e], (k0 + uo[0]) % d[0], (k1 + uo[1]) % d[1], (k2 + uo[2]) % d[2]);
                int32_t so = sigma[s], sn = so;
                if (s == ia) { sn = sa_new; hits_a = 1; }
                if (s == ib) sn = sb_new;
                const double *col = tb->pf + ((int64_t)tb->Rv_st[e] * tb->n_bf + tb->Rv_bf[e]) * tb->max_sp;
                pn *= col[sn]; po *= col[so];
            }
            double v = tb->Rv_eci[(int64_t)b * tb->J + j] * (pn - po);
            if (pass == 0) sum_a += v; else if (!hits_a) sum_b += v;
        }
    }
    return sum_a + sum_b;
}

/* ── chunk of PT steps + optional chunk-end exchange ────────────────────────────────────────────── */
static void run_replica(const orc_tables *tb, orc_state *st, const orc_chunk *ck, int32_t r) {
    int8_t *sig = st->sigma + (int64_t)r * st->N;
    int32_t t = st->slot_of_rep[r];
    double beta = (double)st->beta_slot[t];
    double E = st->E[r], Emin = st->E_min_rep[r];
    int64_t nacc = 0, nnear = 0;
    for (int64_t s = 0; s < ck->n_steps; ++s) {
        int64_t ia, ib; double u;
        if (ck->prop_a) {
            ia = ck->prop_a[s * st->R + t]; ib = ck->prop_b[s * st->R + t]; u = ck->prop_u[s * st->R + t];
        } else {
            orc_propose(tb, ck->seed, ck->step0 + s, t, &ia, &ib, &u);
        }
        int32_t sa = sig[ia], sb = sig[ib];
        if (sa != sb) {
            double dE = orc_ce_delta(tb, sig, ia, ib, sb, sa);
            if (beta > 0.0 && fabs(dE + log(u) / beta) < ck->near_eV) ++nnear;
            if (log(u) < -beta * dE) { sig[ia] = (int8_t)sb; sig[ib] = (int8_t)sa; E += dE; ++nacc; }
        }
        if (E < Emin) Emin = E;
        if (ck->E_samples && (s + 1) % ck->sample_interval == 0)
            ck->E_samples[((s + 1) / ck->sample_interval - 1) * st->R + t] = E;
    }
    st->E[r] = E; st->E_min_rep[r] = Emin; st->n_acc[r] += nacc;
    if (st->n_near) st->n_near[r] += nnear;
}

void orc_exchange(orc_state *st, const orc_chunk *ck) {
    int32_t R = st->R;
    int64_t g = ck->step0 + ck->n_steps;            /* global step count after the chunk */
    int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * R), *ros = (int32_t *)malloc(sizeof(int32_t) * R);
    const int32_t npair = R / 2;                    /* ceil((R - 1) / 2) */
    int32_t nswap = 0;
    for (int32_t q = 0; q < (ck->rounds > 1 ? ck->rounds : 1); ++q) {
        int32_t parity = ck->ex_u ? ((ck->ex_parity >> q) & 1) : orc_ex_parity(ck->seed, g, q);
        for (int32_t i = 0; i < R; ++i) perm[i] = i;
        for (int32_t k = 0; 2 * k < R - 1; ++k) {
            int32_t i = 2 * k + parity, j = i + 1;
            if (j >= R) continue;
            if (st->ladder_id[i] != st->ladder_id[j]) continue;
            double Ei = st->E[st->rep_of_slot[i]], Ej = st->E[st->rep_of_slot[j]];
            double log_acc = ((double)st->beta_slot[j] - (double)st->beta_slot[i]) * (Ej - Ei);
            double u = ck->ex_u ? ck->ex_u[(int64_t)q * npair + k] : orc_ex_uniform(ck->seed, g, q, k);
            if (log(u) < log_acc) { perm[i] = j; perm[j] = i; ++nswap; }
        }
        for (int32_t t = 0; t < R; ++t) ros[t] = st->rep_of_slot[perm[t]];
        for (int32_t t = 0; t < R; ++t) { st->rep_of_slot[t] = ros[t]; st->slot_of_rep[ros[t]] = t; }
    }
    *st->n_ex += nswap;
    if (ck->E_samples && ck->n_steps % ck->sample_interval == 0) {       /* last sample: post-exchange slot order */
        int64_t row = ck->n_steps / ck->sample_interval - 1;
        for (int32_t t = 0; t < R; ++t) ck->E_samples[row * R + t] = st->E[st->rep_of_slot[t]];
    }
    free(perm); free(ros);
}

int orc_ce_run(const orc_tables *tb, orc_state *st, const orc_chunk *ck) {
    int32_t R = st->R;
#pragma omp parallel for schedule(dynamic, 1) num_threads(ck->n_threads > 0 ? ck->n_threads : 1)
    for (int32_t r = 0; r < R; ++r) run_replica(tb, st, ck, r);
    if (ck->do_exchange && R > 1) orc_exchange(st, ck);
    return 0;
}
