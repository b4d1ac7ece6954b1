// NeuralCE receptive-field local update on GB300 (sm_103a).
//
// One CTA per replica runs every step of a chunk:
//   1. proposal (i, j) from Philox or a host stream; same species -> accepted no-op (reference rule dE = 0 <= 0)
//   2. nested unique receptive field: the ball offsets of i and j are enumerated level by level and claimed in
//      a per-replica slot map, so positions [0, n_l) of the site list are exactly ball_l(i) U ball_l(j)
//   3. layer-0 change: the reverse rows of both flips (the second with the first applied) push
//      dPi * nA / (order * norm * sd) onto every member; sums are int64 fixed point (2^-40) in shared memory,
//      so the result does not depend on the order of the atomic adds
//   4. layer l+1 on positions [0, n_{l+1}): gather [h, masked shell means] of the patched level-l values into a
//      shared tile, FP32 FMA against [W_self; W_shell] (+ sigmoid gate), tanh or SiLU
//   5. dE = sum over the last level of (e_new - e) (fixed point), Metropolis rule of the reference's NCE driver
//      (dE_eV <= 0 or u < exp(-beta dE_eV)), commit of h0 / hidden / e rows on accept, slot map cleared.
// Full cache (h0 pull over reverse rows, layers on all sites, per-site e) and the energy are separate kernels.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <climits>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "umma.cuh"

namespace cg = cooperative_groups;

namespace nce {

int launch_exchange(int32_t R, double *E, double E_scale, const float *beta_slot, int32_t *ros, int32_t *sor, const int32_t *lid,
                    int64_t *n_ex, uint64_t seed, int64_t g_end, int32_t parity_bits, const double *ex_u, int32_t rounds,
                    cudaStream_t s);

constexpr int kMaxLayers = 4;
constexpr int kZeroRow = 256;                 // >= every layer's input width
constexpr double kFix = 1099511627776.0;      // 2^40
constexpr double kInvFix = 1.0 / 1099511627776.0;

struct NceDev {
    int32_t nB, J, mo, P, W, depth, C0, D, maxM, maxP;
    int32_t d0, d1, d2;
    int64_t N, n_cells;
    int32_t wL;                           // ball offsets per basis (last level)
    const int32_t *Rv_b, *Rv_uo, *Rv_p, *Rv_col; const uint8_t *Rv_m; const double *Rv_w;   // (nB,J,mo[,3]), (nB,J)
    const int32_t *Mb; const double *theta;                                                  // (nB), (maxM+1,maxP,maxM)
    const int32_t *Sh_b, *Sh_uo; const uint8_t *Sh_m; const float *Sh_inv;                  // (nB,P,W[,3]), (nB,P)
    const int32_t *ball_b, *ball_uo, *ball_end;                                              // (nB,wL[,3]), (nB,depth+1)
    const float *lin, *head_w; float head_b;
    const float *Wc[kMaxLayers], *bias[kMaxLayers], *G[kMaxLayers], *gb[kMaxLayers];
    const float *mu, *sd;
    int32_t act, gate; double norm, scale_eV;
    int32_t n0max, nmax;
    int32_t n_groups, max_gb; const int32_t *act_b, *act_nb; const uint64_t *grp_cum;
    const uint16_t *Rv_loc;                   // (nB, J, mo) index of each row member in its site's ball-0 list
    int32_t w0max;                            // ball-0 entries per basis, maximum
    int32_t mma;                              // 0 float32 CUDA cores, 1 bf16 tensor cores, 3 split bf16 (3 products)
    // point functions +-1 (l0bin): the layer-0 change of a row is 0 or +-2 w exactly; Rv_wfix = llrint(2 w 2^40),
    // thsign[(M * maxP + p) * maxM + s] = 1 where theta < 0
    int32_t l0bin; const long long *Rv_wfix; const uint8_t *thsign;
    const int32_t *Rv_desc;                   // (nB, J, mo) l0bin member: loc | valid << 16 | sign bits of species 0..3 << 20
    const long long *col_wfix;                // (K + 1) l0bin: the (shared) 2 w 2^40 of each channel's rows
    // bit-sliced layer 0 (full caches; l0bin with every member on point function 0): per basis, the reverse rows'
    // members as (basis, uo0, uo1, uo2) or basis -1, each row's channel, and the channel weight (w, float64)
    int32_t h0bits; const int4 *h0mem; const double *col_w;
    int32_t h0_slices; const int2 *h0_slice;  // (nB, S + 1) slice starts (first row, first channel); last = (J, C0)
    // tcgen05 layer contractions (mma 2: bf16, mma 4: split bf16): per layer the weights as the B operand in bf16
    // core-matrix layout ([D][Kp], Kp = Kin rounded up to 16; hi, then lo when split)
    int32_t tc, tc_split; const uint8_t *Wt[kMaxLayers];
    int32_t tc_ks;                            // K columns the A tile holds (a layer with more is issued in K slices)
    const float *zrow;                        // kZeroRow zeros: the row a masked shell partner reads
};

// A swap evaluated and kept for a later commit (nce_nce_local_delta / nce_nce_commit): the new rows stay in the
// model's step scratch (site list, new rows, new site energies) until the next call on the handle.
struct NcePending {
    int64_t si, sj;
    double dE;
    int32_t ssi, ssj, same, valid;
    int32_t nl[kMaxLayers + 1];
};

struct NceJob {
    NceDev m;
    // state
    int8_t *sigma; float *h0; float *hmid; float *e; double *E;
    const float *beta_slot; const int32_t *slot_of_rep; int64_t *n_acc;
    int32_t R;
    // scratch (per replica stride)
    int32_t *slot; int32_t *list; float *newbuf; float *e_new; int64_t scratch_stride;   // floats per replica in newbuf
    // chunk
    int64_t n_steps, step0; const int32_t *prop_a, *prop_b; const double *prop_u; uint64_t seed;
    int64_t sample_interval; double *E_samples; double *dE_out; int32_t force;   // force: 0 Metropolis, 1 accept, -1 reject
    int32_t *err;
    int64_t *n_near; double near_eV;          // near-threshold step counts (or null) and their band in eV
    NcePending *pend;                         // (R) force = -2: the evaluated swap of each replica, kept for a commit
    int32_t rep_index;                        // proposals and dE_out indexed by replica instead of temperature slot
};

__device__ __forceinline__ int32_t wadd(int32_t k, int32_t u, int32_t d) { int32_t q = k + u; return q >= d ? q - d : q; }

__device__ __forceinline__ void coords(const NceDev &m, int64_t i, int32_t &b, int32_t k[3]) {
    const uint32_t ii = (uint32_t)i, nB = (uint32_t)m.nB, d1 = (uint32_t)m.d1, d2 = (uint32_t)m.d2;   // N < 2^31
    const uint32_t c = ii / nB;
    b = (int32_t)(ii - c * nB);
    const uint32_t c12 = c / d2;
    k[2] = (int32_t)(c - c12 * d2);
    k[0] = (int32_t)(c12 / d1);
    k[1] = (int32_t)(c12 - (uint32_t)k[0] * d1);
}

__device__ __forceinline__ int64_t site_at(const NceDev &m, const int32_t k[3], const int32_t *uo, int32_t b) {
    return (((int64_t)wadd(k[0], uo[0], m.d0) * m.d1 + wadd(k[1], uo[1], m.d1)) * m.d2 + wadd(k[2], uo[2], m.d2)) * m.nB + b;
}

__device__ __forceinline__ float act_fn(int act, float x) {
    return act == 0 ? tanhf(x) : x / (1.0f + expf(-x));
}

// the activation of the tensor-core epilogue: SiLU through the hardware exponential and division (a few ulp, far
// below the bf16 operands' rounding; full caches and steps share it)
__device__ __forceinline__ float act_fn_tc(int act, float x) {
    return act == 0 ? tanhf(x) : __fdividef(x, 1.0f + __expf(-x));
}

// newbuf layout per replica: level 0 block (n0max x C0, rounded up to 4 floats so that every later block and
// replica starts on 16 bytes for float4 rows), then level l (1..depth-1) blocks (nmax x D)
__host__ __device__ __forceinline__ size_t l0_floats(const NceDev &m) { return ((size_t)m.n0max * m.C0 + 3) & ~(size_t)3; }
__device__ __forceinline__ float *level_buf(const NceJob &jb, float *base, int lvl) {
    if (lvl == 0) return base;
    return base + l0_floats(jb.m) + (size_t)(lvl - 1) * jb.m.nmax * jb.m.D;
}

struct NceCtl {
    int64_t si, sj; double u; int32_t same, bi, bj, ki[3], kj[3], ssi, ssj;
    int32_t cnt; int32_t nl[kMaxLayers + 1];
    unsigned long long dacc;
    int32_t err, acc;
};

// value of level lvl at site q (patched by the step's new values), channel c
__device__ __forceinline__ float patched(const NceJob &jb, int lvl, const float *cache, const float *newl, const int32_t *slot,
                                         int32_t nlev, int64_t q, int c, int Cin) {
    const int32_t p = slot[q];
    if (p >= 0 && p < nlev) return newl[(size_t)p * Cin + c];
    return cache[(size_t)q * Cin + c];
}

// Tile geometry of the layer GEMM: D/4 column groups of 4 outputs, 256/(D/4) site groups, TM sites per tile,
// MS sites per thread (register micro-tile MS x 4).  D in {16, 32, 64, 128}.
// Tile rows: 128 on the tcgen05 path; otherwise MS sites per thread x SG = 256 / (D / 4) site groups, MS = 4
// (the mma.sync warp tiling needs it), on the float32 path at most 128 rows (D = 16: MS = 2)
__host__ __device__ __forceinline__ int tile_tm(int D, int tc = 0, int mma = 0) {
    const int SG = 256 / (D / 4);
    return tc ? 128 : (mma ? 4 : (SG >= 64 ? 2 : 4)) * SG;
}
__host__ __device__ __forceinline__ int kpad16(int k) { return (k + 15) & ~15; }
// float32 tile row stride: a multiple of 4 floats (16-byte rows for float4 reads along K) above Kin
__host__ __device__ __forceinline__ int x_stride(int kin) { return (kin + 4) & ~3; }

// tensor-memory accumulator, completion mbarrier and the staged B operand of the tcgen05 tile path; `phase` is the
// parity of the next completion (every thread of the CTA keeps the same count).  `failed`: a completion wait gave up
// (the whole CTA agrees on it); from then on the CTA issues no MMA, writes no operand tile and reads no accumulator
// for the rest of the kernel, and only drains the abandoned MMAs (bounded) before freeing tensor memory.
struct TcCtx {
    uint32_t tmem; uint64_t *mbar; uint32_t phase; uint8_t *W; int failed;
};

// allocation by warp 0 (D columns rounded up to a power of two >= 32) and the mbarrier, for the whole kernel
__device__ __forceinline__ void tc_begin(int D, TcCtx &tc, uint8_t *wsm, uint64_t *mbar, uint32_t *tslot) {
    if ((threadIdx.x >> 5) == 0) umma::tmem_alloc(tslot, umma::tmem_cols(D));
    if (threadIdx.x == 0) umma::mbar_init(mbar, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    tc.tmem = *tslot; tc.mbar = mbar; tc.phase = 0; tc.W = wsm; tc.failed = 0;
}

__device__ __forceinline__ void tc_end(int D, const TcCtx &tc, uint32_t limit = 1u << 20) {
    // after a wait that gave up, give the abandoned MMAs one more bounded wait before their tensor memory is freed
    if (tc.failed) umma::mbar_wait(tc.mbar, tc.phase ^ 1u, limit);
    umma::fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) umma::tmem_free(tc.tmem, umma::tmem_cols(D));
}

// the completion wait of one tile's MMAs, agreed on by the whole CTA: false when it gave up (error flag 32 set, the
// CTA's tensor-core work stops)
__device__ __forceinline__ bool tc_wait(TcCtx &tc, int32_t *err, uint32_t limit = 1u << 20) {
    const bool ok = umma::mbar_wait(tc.mbar, tc.phase, limit);
    tc.phase ^= 1u;
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(err, 32);
        tc.failed = 1;
        return false;
    }
    return true;
}
__host__ __device__ __forceinline__ int tile_kin(int P, int C0, int D) { return (1 + P) * (C0 > D ? C0 : D); }

// bf16 tensor-core helpers: mma.sync m16n8k16 (row-major A, column-major B, float32 accumulation).  Fragment
// layout (g = lane / 4, t = lane % 4): A regs {r g, k 2t..2t+1}, {r g+8, k 2t..}, {r g, k 2t+8..}, {r g+8, k 2t+8..};
// B regs {k 2t..2t+1, n g}, {k 2t+8..2t+9, n g}; C {r g, n 2t..2t+1}, {r g+8, n 2t..2t+1}.
__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

__device__ __forceinline__ void bf16_split(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    hi = bf16x2_bits(h);
    lo = bf16x2_bits(__floats2bfloat162_rn(x0 - hf.x, x1 - hf.y));
}

__device__ __forceinline__ void mma_bf16_16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct LayerW {            // weights of one layer as seen by the kernel (shared or global memory)
    const float *W, *b, *G, *gb;
};

// Evaluate one layer for the sites list[pos0 .. pos0+cnt) (or direct0 + 0..cnt-1).  Inputs come from level lvl
// (cache patched with the step's values, or unpatched when slot == nullptr).  For every site and group of 4
// consecutive output columns, `sink(pos, col0, v[4])` receives the activated outputs (pos < 0: padding lane).
template <typename Sink>
__device__ void layer_tiles(const NceJob &jb, int lvl, const LayerW &LW, const float *cache, const float *newl, const int32_t *slot,
                            int32_t nlev, const int32_t *list, int64_t pos0, int64_t cnt, const int64_t *direct0, float *X,
                            int32_t *src, Sink sink, int tile_begin = 0, int tile_stride = 1, TcCtx *tc = nullptr) {
    const NceDev &m = jb.m;
    const int Cin = lvl == 0 ? m.C0 : m.D, D = m.D, P = m.P, W = m.W;
    const int Kin = (1 + P) * Cin, XS = x_stride(Kin);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int ncg = D / 4, SG = 256 / ncg, TM = tile_tm(D, tc != nullptr, m.mma), MS = TM / SG;
    const int cg = tid % ncg, sg = tid / ncg;
    const int PW = 1 + P * W;
    // row of each site and shell partner: the step's new value, the cache, or a row of zeros (masked partner)
    const float **srcp = reinterpret_cast<const float **>(src);
    int32_t *tsite = reinterpret_cast<int32_t *>(srcp + TM * PW);   // the tile's sites
    float *tinv = reinterpret_cast<float *>(tsite + TM);     // 1 / |first-shell partners| of each
    int4 *tk = reinterpret_cast<int4 *>(tinv + TM);          // (basis, k0, k1, k2) of each
    int32_t *tslot = reinterpret_cast<int32_t *>(tk + TM);   // slot-map value of each (-1: not in the field)
    // tcgen05 path: the tile is the bf16 A operand [128][KS] (hi, then lo when split) in core-matrix layout, one K
    // slice [klo, klo + KS) of the layer's Kp input columns at a time (KS = Kp unless the whole A operand does not
    // fit shared memory: the split form at width 128 takes its self channels, then its shell means); every slice's
    // MMAs accumulate into the same tensor-memory tile
    const int Kp = kpad16(Kin);
    const int KS = (tc && Kp > m.tc_ks) ? m.tc_ks : Kp, nks = Kp / KS;
    int klo = 0, khi = Kp;                                   // the slice being gathered (all of K off the tcgen05 path)
    uint8_t *A0 = reinterpret_cast<uint8_t *>(X), *A1 = A0 + (size_t)128 * KS * 2;
    if (tc && tc->failed) return;                            // an earlier completion wait gave up: no more tensor work
    if (tc) {
        // this layer's B operand into shared memory (read by the tensor cores after the first tile barrier)
        const size_t n16 = (size_t)Kp * D * 2 * (m.tc_split ? 2 : 1) / 16;
        const uint4 *g = reinterpret_cast<const uint4 *>(m.Wt[lvl]);
        uint4 *d = reinterpret_cast<uint4 *>(tc->W);
        for (size_t i = tid; i < n16; i += nt) d[i] = __ldg(g + i);
        umma::fence_async_smem();
    }
    auto xput = [&](int ms, int k, float v) {
        if (tc) {
            if (k < klo || k >= khi) return;
            const uint32_t off = umma::core_off(ms, k - klo, KS);
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            *reinterpret_cast<__nv_bfloat16 *>(A0 + off) = h;
            if (m.tc_split) *reinterpret_cast<__nv_bfloat16 *>(A1 + off) = __float2bfloat16_rn(v - __bfloat162float(h));
        } else {
            X[(size_t)ms * XS + k] = v;
        }
    };
    // channels k, k + 1 (k even): one 4-byte bf16 pair on the tcgen05 path
    auto xput2 = [&](int ms, int k, float v0, float v1) {
        if (tc) {
            if (k < klo || k >= khi) return;                 // slices start on multiples of 16: a pair never straddles
            const uint32_t off = umma::core_off(ms, k - klo, KS);
            const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
            *reinterpret_cast<__nv_bfloat162 *>(A0 + off) = h;
            if (m.tc_split) {
                const float2 hf = __bfloat1622float2(h);
                *reinterpret_cast<__nv_bfloat162 *>(A1 + off) = __floats2bfloat162_rn(v0 - hf.x, v1 - hf.y);
            }
        } else {
            X[(size_t)ms * XS + k] = v0; X[(size_t)ms * XS + k + 1] = v1;
        }
    };
    for (int64_t t0 = (int64_t)tile_begin * TM; t0 < cnt; t0 += (int64_t)tile_stride * TM) {
        const int tm = (int)min((int64_t)TM, cnt - t0);
        // 1) the tile's sites and their first shell's 1/|partners| into shared memory, then the source row of each
        //    site and shell partner: patched rows >= 0, cache rows -(q+1), masked partner INT_MIN.  Four items per
        //    thread with their slot-map loads in flight together.
        for (int mm = tid; mm < tm; mm += nt) {
            const int64_t s = direct0 ? (*direct0 + pos0 + t0 + mm) : list[pos0 + t0 + mm];
            int32_t b, k[3]; coords(m, s, b, k);
            tsite[mm] = (int32_t)s;
            tinv[mm] = m.Sh_inv[b * P];
            tk[mm] = make_int4(b, k[0], k[1], k[2]);
        }
        __syncthreads();
        // item idx = mm PW + q, stepped by nt without divisions: (mm, q) advance by (nt / PW, nt % PW) with a carry
        const int dq = nt % PW, dm = nt / PW;
        int im = tid / PW, iq = tid % PW;
        for (int base = tid; base < tm * PW; base += 4 * nt) {
            int64_t site[4];
            int mmu[4], qu[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                mmu[u] = im; qu[u] = iq;
                site[u] = -1;
                if (base + u * nt < tm * PW) {
                    site[u] = tsite[im];
                    if (iq > 0) {
                        const int4 c = tk[im];
                        const int32_t k[3] = {c.y, c.z, c.w};
                        const int e0 = c.x * P * W + (iq - 1);
                        site[u] = m.Sh_m[e0] ? site_at(m, k, m.Sh_uo + 3 * e0, m.Sh_b[e0]) : -1;
                    }
                }
                iq += dq; im += dm;
                if (iq >= PW) { iq -= PW; ++im; }
            }
            int32_t pv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) pv[u] = (slot && site[u] >= 0) ? slot[site[u]] : -1;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int idx = base + u * nt;
                if (idx >= tm * PW) continue;
                if (qu[u] == 0) tslot[mmu[u]] = pv[u];
                srcp[idx] = site[u] < 0 ? m.zrow
                          : (pv[u] >= 0 && pv[u] < nlev) ? newl + (size_t)pv[u] * Cin : cache + (size_t)site[u] * Cin;
            }
        }
        __syncthreads();
        for (int ks = 0; ks < nks; ++ks) {
        klo = ks * KS; khi = tc ? klo + KS : Kp;
        // 2) X = [h | masked shell means] of the tile's sites: lanes over channels (coalesced rows); masked
        //    partners read the zero row, so every sum runs over all W slots in order
        const float *zr = m.zrow;
        if (P == 1 && W <= 12 && Cin <= 64 && (Cin & 1) == 0) {
            // one shell of at most 12 partners: two sites per warp with all 2 x 13 rows' loads in flight at once;
            // a lane takes the channel pair (2 lane, 2 lane + 1) as one 8-byte load
            const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
            const int c0 = 2 * lane;
            const bool ok = c0 < Cin;
            for (int mm = warp; mm < tm; mm += 2 * nwarp) {
                const int mb = mm + nwarp;
                const bool two = mb < tm;
                float2 v[2][13];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float *const *sr = srcp + (two ? (h ? mb : mm) : mm) * PW;
#pragma unroll
                    for (int u = 0; u < 13; ++u) {
                        const float *rr = u <= W ? sr[u] : zr;
                        v[h][u] = ok ? *reinterpret_cast<const float2 *>(rr + c0) : make_float2(0.f, 0.f);
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (h == 1 && !two) break;
                    const int ms = h ? mb : mm;
                    float s0 = 0.f, s1 = 0.f;
#pragma unroll
                    for (int u = 1; u < 13; ++u) { s0 += v[h][u].x; s1 += v[h][u].y; }
                    const float inv = tinv[ms];
                    if (ok) xput2(ms, c0, v[h][0].x, v[h][0].y), xput2(ms, Cin + c0, s0 * inv, s1 * inv);
                }
            }
        } else if (P == 1 && W <= 12 && Cin <= 128) {
            // one shell, up to 128 channels: one site per warp, four channels per lane, all 13 rows' loads in flight
            // (a K slice that holds only the self channels, or only the shell means, loads only those rows)
            const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
            const bool need_self = klo < Cin, need_shell = khi > Cin;
            for (int mm = warp; mm < tm; mm += nwarp) {
                const float *const *sr = srcp + mm * PW;
                float v[4][13];
#pragma unroll
                for (int u = 0; u < 13; ++u) {
                    const bool want = u == 0 ? need_self : (need_shell && u <= W);
                    const float *rr = want ? sr[u] : zr;
#pragma unroll
                    for (int j = 0; j < 4; ++j) v[j][u] = (want && lane + 32 * j < Cin) ? rr[lane + 32 * j] : 0.f;
                }
                const float inv = tinv[mm];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = lane + 32 * j;
                    if (c >= Cin) continue;
                    float a = 0.f;
#pragma unroll
                    for (int u = 1; u < 13; ++u) a += v[j][u];
                    if (need_self) xput(mm, c, v[j][0]);
                    if (need_shell) xput(mm, Cin + c, a * inv);
                }
            }
        } else if (Cin <= 20 && (Cin & 1) == 0 && W <= 32) {
            // narrow inputs and wide shells (the reference's shipped model: 18 channels, shells of 12 / 6 / 24): a lane
            // takes one channel pair of one of three sites per warp (Cin / 2 lanes a site, 8-byte loads), all partner
            // loads of one shell in flight; each channel's sum runs over the W slots in order, as below
            const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
            const int hc = Cin >> 1, sl = lane / hc, c0 = 2 * (lane - sl * hc);
            for (int m0 = warp * 3; m0 < tm; m0 += nwarp * 3) {
                const int mm = m0 + (sl < 3 ? sl : 0);
                const bool ok = sl < 3 && mm < tm;
                const float *const *sr = srcp + (ok ? mm : m0) * PW;
                if (ok) {
                    const float2 x = *reinterpret_cast<const float2 *>(sr[0] + c0);
                    xput2(mm, c0, x.x, x.y);
                }
                const int b = tk[ok ? mm : m0].x;
                for (int p = 0; p < P; ++p) {
                    float2 v[32];
#pragma unroll
                    for (int u = 0; u < 32; ++u)
                        v[u] = (ok && u < W) ? *reinterpret_cast<const float2 *>(sr[1 + p * W + u] + c0) : make_float2(0.f, 0.f);
                    float s0 = 0.f, s1 = 0.f;
#pragma unroll
                    for (int u = 0; u < 32; ++u) { s0 += v[u].x; s1 += v[u].y; }
                    if (ok) {
                        const float inv = m.Sh_inv[b * P + p];
                        xput2(mm, Cin + p * Cin + c0, s0 * inv, s1 * inv);
                    }
                }
            }
        } else if (Cin <= 32 && W <= 32) {
            // narrow inputs and wide shells (the reference's shipped model: 18 channels, shells of 12 / 6 / 24):
            // one lane per channel, two sites per warp, all partner loads of one shell of both sites in flight
            const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
            const bool cok = lane < Cin;
            const int cl = cok ? lane : 0;
            for (int mm = warp; mm < tm; mm += 2 * nwarp) {
                const int mb = mm + nwarp;
                const bool two = mb < tm;
                const float *const *sa = srcp + mm * PW, *const *sb = srcp + (two ? mb : mm) * PW;
                const float xa = sa[0][cl], xb = sb[0][cl];
                if (cok) { xput(mm, lane, xa); if (two) xput(mb, lane, xb); }
                const int ba = tk[mm].x, bb = tk[two ? mb : mm].x;
                for (int p = 0; p < P; ++p) {
                    float va[32], vb[32];
#pragma unroll
                    for (int u = 0; u < 32; ++u) {
                        va[u] = u < W ? sa[1 + p * W + u][cl] : 0.f;
                        vb[u] = u < W ? sb[1 + p * W + u][cl] : 0.f;
                    }
                    float s0 = 0.f, s1 = 0.f;
#pragma unroll
                    for (int u = 0; u < 32; ++u) { s0 += va[u]; s1 += vb[u]; }
                    if (cok) {
                        xput(mm, Cin + p * Cin + lane, s0 * m.Sh_inv[ba * P + p]);
                        if (two) xput(mb, Cin + p * Cin + lane, s1 * m.Sh_inv[bb * P + p]);
                    }
                }
            }
        } else {
            const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
            for (int mm = warp; mm < tm; mm += nwarp) {
                const float *const *sr = srcp + mm * PW;
                const int32_t b = tk[mm].x;
                // two channels per lane (c, c + 32), all partner loads of a group of 8 issued before summing
                const int c0 = lane, c1 = lane + 32;
                const bool h0ok = c0 < Cin, h1ok = c1 < Cin;
                if (h0ok) xput(mm, c0, sr[0][c0]);
                if (h1ok) xput(mm, c1, sr[0][c1]);
                for (int p = 0; p < P; ++p) {
                    const float *const *pc = sr + 1 + p * W;
                    float s0 = 0.f, s1 = 0.f;
                    for (int w0 = 0; w0 < W; w0 += 8) {
                        float va[8], vb[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const float *rr = w0 + u < W ? pc[w0 + u] : zr;
                            va[u] = h0ok ? rr[c0] : 0.f;
                            vb[u] = h1ok ? rr[c1] : 0.f;
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) { s0 += va[u]; s1 += vb[u]; }
                    }
                    const float inv = m.Sh_inv[b * P + p];
                    if (h0ok) xput(mm, Cin + p * Cin + c0, s0 * inv);
                    if (h1ok) xput(mm, Cin + p * Cin + c1, s1 * inv);
                }
                for (int c = lane + 64; c < Cin; c += 32) {        // widths above 64 channels
                    xput(mm, c, sr[0][c]);
                    for (int p = 0; p < P; ++p) {
                        float a0 = 0.f;
                        for (int w = 0; w < W; ++w) a0 += sr[1 + p * W + w][c];
                        xput(mm, Cin + p * Cin + c, a0 * m.Sh_inv[b * P + p]);
                    }
                }
            }
        }
        if (tc) {
            // zero K padding of the tile's rows (rows past tm only feed outputs that are dropped)
            const int kz0 = max(Kin, klo), kz = khi - kz0;
            for (int idx = tid; kz > 0 && idx < tm * kz; idx += nt) xput(idx / kz, kz0 + idx % kz, 0.f);
            umma::fence_async_smem();
        }
        __syncthreads();
        if (tc) {
            // 3'') tcgen05: one thread issues the slice's MMAs into tensor memory (the B operand's K-steps of this
            // slice, accumulating onto the previous slices); every thread waits for their completion before the
            // next slice overwrites the A tile
            if (tid == 0) {
                const size_t bo = (size_t)klo * 16;             // K-step klo / 16 of the B tile (256 bytes per step)
                umma::issue_tile_k(tc->tmem, A0, A1, (uint32_t)KS * 16u, tc->W + bo, tc->W + (size_t)Kp * D * 2 + bo,
                                   (uint32_t)Kp * 16u, D, KS / 16, m.tc_split ? 3 : 1, ks > 0, tc->mbar);
            }
            if (!tc_wait(*tc, jb.err)) return;                  // operands and accumulator left alone from here on
            umma::fence_after();
        }
        }   // K slices
        if (tc) {
            // every warp reads its lane quarter (rows 32 (warp % 4) ..) and half of the columns of the accumulator,
            // adds the bias, activates and stages the rows in Y (over the A operand) for the sink's CUDA-core mapping
            const int warp = tid >> 5, q = warp & 3, hh = warp >> 2;
            const int cw = D / 2 >= 16 ? D / 2 : 16;
            const int YS = D + 4;
            float *Y = X;
            const int rrow = q * 32 + (tid & 31);
            for (int c0 = hh * cw; c0 < min(D, (hh + 1) * cw); c0 += 16) {
                float v[16];
                umma::tmem_ld16(tc->tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    float4 o;
                    o.x = act_fn_tc(m.act, v[i] + LW.b[c0 + i]); o.y = act_fn_tc(m.act, v[i + 1] + LW.b[c0 + i + 1]);
                    o.z = act_fn_tc(m.act, v[i + 2] + LW.b[c0 + i + 2]); o.w = act_fn_tc(m.act, v[i + 3] + LW.b[c0 + i + 3]);
                    *reinterpret_cast<float4 *>(Y + (size_t)rrow * YS + c0 + i) = o;
                }
            }
            umma::fence_before();
            __syncthreads();
#pragma unroll 8
            for (int i = 0; i < MS; ++i) {
                const int mm = sg + i * SG;
                const float4 y = *reinterpret_cast<const float4 *>(Y + (size_t)mm * YS + cg * 4);
                float v[4] = {y.x, y.y, y.z, y.w};
                sink(mm < tm ? t0 + mm : -1, cg * 4, v, tsite[mm < tm ? mm : 0], tslot[mm < tm ? mm : 0]);
            }
            __syncthreads();
            continue;
        }
        if (m.mma == 1 || m.mma == 3) {
            // 3') tensor cores: the tile's [TM x Kin] x [Kin x D] on mma.sync bf16 (split operands when m.mma == 3);
            // warps tile the output in 16 x 8 blocks (mt x nt = 4 per warp), then bias + activation go through a
            // [TM x (D + 4)] staging tile (over X) to the sink in the CUDA-core mapping
            const int lane = tid & 31, warp = tid >> 5, g8 = lane >> 2, t4 = lane & 3;
            const int wn = D >= 32 ? D / 32 : 1, wm = 8 / wn, NB = D / wn, nt = NB / 8, MB = TM / wm, mt = MB / 16;
            const int row0 = (warp / wn) * MB, col0 = (warp % wn) * NB;
            const bool split = m.mma == 3;
            float acc[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int nj = q % nt;
                const int c = col0 + nj * 8 + 2 * t4;
                const float b0 = LW.b[c], b1 = LW.b[c + 1];
                acc[q][0] = b0; acc[q][1] = b1; acc[q][2] = b0; acc[q][3] = b1;
            }
            auto xv = [&](int r, int k) -> float { return k < Kin ? X[(size_t)r * XS + k] : 0.f; };
            auto wv = [&](int k, int n) -> float { return k < Kin ? LW.W[(size_t)k * D + n] : 0.f; };
            for (int k0 = 0; k0 < Kin; k0 += 16) {
                const int ka = k0 + 2 * t4;
                uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
                for (int mi = 0; mi < 2; ++mi) {
                    if (mi < mt) {
                        const int r = row0 + mi * 16 + g8;
                        const float x00 = xv(r, ka), x01 = xv(r, ka + 1), x10 = xv(r + 8, ka), x11 = xv(r + 8, ka + 1);
                        const float x02 = xv(r, ka + 8), x03 = xv(r, ka + 9), x12 = xv(r + 8, ka + 8), x13 = xv(r + 8, ka + 9);
                        if (split) {
                            bf16_split(x00, x01, ah[mi][0], al[mi][0]); bf16_split(x10, x11, ah[mi][1], al[mi][1]);
                            bf16_split(x02, x03, ah[mi][2], al[mi][2]); bf16_split(x12, x13, ah[mi][3], al[mi][3]);
                        } else {
                            ah[mi][0] = bf16x2_bits(__floats2bfloat162_rn(x00, x01)); ah[mi][1] = bf16x2_bits(__floats2bfloat162_rn(x10, x11));
                            ah[mi][2] = bf16x2_bits(__floats2bfloat162_rn(x02, x03)); ah[mi][3] = bf16x2_bits(__floats2bfloat162_rn(x12, x13));
                        }
                    }
                }
#pragma unroll
                for (int nj = 0; nj < 4; ++nj) {
                    if (nj < nt) {
                        const int n = col0 + nj * 8 + g8;
                        const float w0 = wv(ka, n), w1 = wv(ka + 1, n), w2 = wv(ka + 8, n), w3 = wv(ka + 9, n);
                        if (split) {
                            bf16_split(w0, w1, bh[nj][0], bl[nj][0]); bf16_split(w2, w3, bh[nj][1], bl[nj][1]);
                        } else {
                            bh[nj][0] = bf16x2_bits(__floats2bfloat162_rn(w0, w1)); bh[nj][1] = bf16x2_bits(__floats2bfloat162_rn(w2, w3));
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int mi = q / nt, nj = q % nt;
                    mma_bf16_16816(acc[q], ah[mi], bh[nj]);
                    if (split) { mma_bf16_16816(acc[q], ah[mi], bl[nj]); mma_bf16_16816(acc[q], al[mi], bh[nj]); }
                }
            }
            __syncthreads();                                   // every warp is done reading X
            const int YS = D + 4;
            float *Y = X;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int mi = q / nt, nj = q % nt;
                const int r = row0 + mi * 16 + g8, c = col0 + nj * 8 + 2 * t4;
                Y[(size_t)r * YS + c] = act_fn(m.act, acc[q][0]); Y[(size_t)r * YS + c + 1] = act_fn(m.act, acc[q][1]);
                Y[(size_t)(r + 8) * YS + c] = act_fn(m.act, acc[q][2]); Y[(size_t)(r + 8) * YS + c + 1] = act_fn(m.act, acc[q][3]);
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (i < MS) {
                    const int mm = sg + i * SG;
                    const float4 y = *reinterpret_cast<const float4 *>(Y + (size_t)mm * YS + cg * 4);
                    float v[4] = {y.x, y.y, y.z, y.w};
                    sink(mm < tm ? t0 + mm : -1, cg * 4, v, tsite[mm < tm ? mm : 0], tslot[mm < tm ? mm : 0]);
                }
            }
            __syncthreads();
            continue;
        }
        // 3) register micro-tile GEMM: MS sites x 4 columns per thread
        float o[4][4], g[4][4];
        const float4 b4 = *reinterpret_cast<const float4 *>(LW.b + cg * 4);
        const float4 gb4 = LW.G ? *reinterpret_cast<const float4 *>(LW.gb + cg * 4) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            o[i][0] = b4.x; o[i][1] = b4.y; o[i][2] = b4.z; o[i][3] = b4.w;
            g[i][0] = gb4.x; g[i][1] = gb4.y; g[i][2] = gb4.z; g[i][3] = gb4.w;
        }
        // rows sg + i SG, i < MS (MS = 2: the last two micro-tile rows repeat the first two and are not used)
        const float *x0 = X + (size_t)sg * XS, *x1 = x0 + (size_t)SG * XS;
        const float *x2 = MS > 2 ? x1 + (size_t)SG * XS : x0, *x3 = MS > 2 ? x2 + (size_t)SG * XS : x1;
        auto fma16 = [&](float v0, float v1, float v2, float v3, const float4 w4) {
            o[0][0] = fmaf(v0, w4.x, o[0][0]); o[0][1] = fmaf(v0, w4.y, o[0][1]); o[0][2] = fmaf(v0, w4.z, o[0][2]); o[0][3] = fmaf(v0, w4.w, o[0][3]);
            o[1][0] = fmaf(v1, w4.x, o[1][0]); o[1][1] = fmaf(v1, w4.y, o[1][1]); o[1][2] = fmaf(v1, w4.z, o[1][2]); o[1][3] = fmaf(v1, w4.w, o[1][3]);
            o[2][0] = fmaf(v2, w4.x, o[2][0]); o[2][1] = fmaf(v2, w4.y, o[2][1]); o[2][2] = fmaf(v2, w4.z, o[2][2]); o[2][3] = fmaf(v2, w4.w, o[2][3]);
            o[3][0] = fmaf(v3, w4.x, o[3][0]); o[3][1] = fmaf(v3, w4.y, o[3][1]); o[3][2] = fmaf(v3, w4.z, o[3][2]); o[3][3] = fmaf(v3, w4.w, o[3][3]);
        };
        // four K at a time: one 16-byte read of each site row, the same fma order as one K at a time
        int kk = 0;
        for (; kk + 4 <= Kin; kk += 4) {
            const float4 a0 = *reinterpret_cast<const float4 *>(x0 + kk), a1 = *reinterpret_cast<const float4 *>(x1 + kk);
            const float4 a2 = *reinterpret_cast<const float4 *>(x2 + kk), a3 = *reinterpret_cast<const float4 *>(x3 + kk);
            const float *wk = LW.W + (size_t)kk * D + cg * 4;
            fma16(a0.x, a1.x, a2.x, a3.x, *reinterpret_cast<const float4 *>(wk));
            fma16(a0.y, a1.y, a2.y, a3.y, *reinterpret_cast<const float4 *>(wk + D));
            fma16(a0.z, a1.z, a2.z, a3.z, *reinterpret_cast<const float4 *>(wk + 2 * D));
            fma16(a0.w, a1.w, a2.w, a3.w, *reinterpret_cast<const float4 *>(wk + 3 * D));
        }
        for (; kk < Kin; ++kk)
            fma16(x0[kk], x1[kk], x2[kk], x3[kk], *reinterpret_cast<const float4 *>(LW.W + (size_t)kk * D + cg * 4));
        if (LW.G) {
#pragma unroll 4
            for (int kk = Cin; kk < Kin; ++kk) {
                const float4 g4 = *reinterpret_cast<const float4 *>(LW.G + (size_t)(kk - Cin) * D + cg * 4);
                const float v0 = x0[kk], v1 = x1[kk], v2 = x2[kk], v3 = x3[kk];
                g[0][0] = fmaf(v0, g4.x, g[0][0]); g[0][1] = fmaf(v0, g4.y, g[0][1]); g[0][2] = fmaf(v0, g4.z, g[0][2]); g[0][3] = fmaf(v0, g4.w, g[0][3]);
                g[1][0] = fmaf(v1, g4.x, g[1][0]); g[1][1] = fmaf(v1, g4.y, g[1][1]); g[1][2] = fmaf(v1, g4.z, g[1][2]); g[1][3] = fmaf(v1, g4.w, g[1][3]);
                g[2][0] = fmaf(v2, g4.x, g[2][0]); g[2][1] = fmaf(v2, g4.y, g[2][1]); g[2][2] = fmaf(v2, g4.z, g[2][2]); g[2][3] = fmaf(v2, g4.w, g[2][3]);
                g[3][0] = fmaf(v3, g4.x, g[3][0]); g[3][1] = fmaf(v3, g4.y, g[3][1]); g[3][2] = fmaf(v3, g4.z, g[3][2]); g[3][3] = fmaf(v3, g4.w, g[3][3]);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (i < MS) {
                const int mm = sg + i * SG;
                float v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float a = act_fn(m.act, o[i][q]);
                    if (LW.G) a *= 1.0f / (1.0f + expf(-g[i][q]));
                    v[q] = a;
                }
                sink(mm < tm ? t0 + mm : -1, cg * 4, v, tsite[mm < tm ? mm : 0], tslot[mm < tm ? mm : 0]);
            }
        }
        __syncthreads();
    }
}

// sum over the D/4 lanes of one site (consecutive lanes of one warp)
__device__ __forceinline__ float group_sum(float v, int ncg) {
    for (int o = ncg >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, ncg);
    return v;
}

// energy of a site from its last-layer outputs (this lane's 4 columns at c0) and its layer-0 row hr: every lane of
// the site's group adds its head terms and its share of the linear layer-0 term (channels c0/4, c0/4 + ncg, ...),
// then one group sum.  The full caches and the local update both use it, so unchanged inputs give identical bits.
__device__ __forceinline__ float site_energy(const float *v, int c0, const float *hw, const float *hr, const float *lin, int C0,
                                             int ncg) {
    float part = 0.f;
    for (int q = 0; q < 4; ++q) part = fmaf(v[q], hw[c0 + q], part);
    if (hr)
        for (int c = c0 >> 2; c < C0; c += ncg) part = fmaf(hr[c], lin[c], part);
    return group_sum(part, ncg);
}

// One MC step of one replica, run by a cluster of CL CTAs (CL = 1: a single CTA).  The leader (rank 0) draws the
// proposal, builds the receptive field and the layer-0 change; every level's tiles are spread over the cluster;
// dE partials reach the leader through distributed shared memory; the leader decides and every CTA commits its
// share.  Every branch that changes the number of cluster barriers is taken from the leader's flags.
struct NceCtx {
    int rank, CL;
    NceCtl *lctl;                       // the leader's control block (own block on the leader)
};

template <bool CLUSTER>
__device__ __forceinline__ void csync() {
    if (CLUSTER) { __threadfence(); cg::this_cluster().sync(); } else { __syncthreads(); }
}

template <bool CLUSTER>
__device__ void nce_step(const NceJob &jb, int r, int t, int64_t s_idx, NceCtl &ctl, unsigned long long *dh, float *X,
                         int32_t *src, const LayerW *LWs, const float *lin, const float *hw, int32_t *ent_site, int32_t *ent_pos,
                         int8_t *ent_sig, double &E, int64_t &nacc, int64_t &nnear, const NceCtx &cx, TcCtx *tc) {
    const bool leader = cx.rank == 0;
    const int CL = cx.CL, rank = cx.rank;
    const NceDev &m = jb.m;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t N = m.N;
    int8_t *sig = jb.sigma + (int64_t)r * N;
    float *h0 = jb.h0 + (size_t)r * N * m.C0;
    float *e = jb.e + (size_t)r * N;
    int32_t *slot = jb.slot + (size_t)r * N;
    int32_t *list = jb.list + (size_t)r * m.nmax;
    float *nb = jb.newbuf + (size_t)r * jb.scratch_stride;
    float *en = jb.e_new + (size_t)r * m.nmax;
    const int L = m.depth;
    const int q_ix = jb.rep_index ? r : t;            // column of the host proposal stream and of dE_out
    if (leader) {
    if (tid == 0) {
        int64_t i, j; double u;
        if (jb.prop_a) {
            i = jb.prop_a[s_idx * jb.R + q_ix]; j = jb.prop_b[s_idx * jb.R + q_ix];
            u = jb.prop_u ? jb.prop_u[s_idx * jb.R + q_ix] : 1.0;
        }
        else {
            const uint32_t k0 = (uint32_t)jb.seed, k1 = (uint32_t)(jb.seed >> 32);
            const int64_t g = jb.step0 + s_idx;
            const uint32_t c0 = (uint32_t)g, c1 = (uint32_t)((uint64_t)g >> 32);
            u32x4 x = philox4x32(c0, c1, (uint32_t)t, 0u, k0, k1);
            int grp = 0; uint32_t ba = 0, bb = 0;
            if (m.n_groups > 1 || m.act_nb[0] > 1) {
                u32x4 y = philox4x32(c0, c1, (uint32_t)t, 1u, k0, k1);
                if (m.n_groups > 1)
                    while (grp < m.n_groups - 1 && (uint64_t)y.x >= m.grp_cum[grp]) ++grp;
                ba = draw_index(y.y, (uint32_t)m.act_nb[grp]); bb = draw_index(y.z, (uint32_t)m.act_nb[grp]);
            }
            const uint32_t nc = (uint32_t)m.n_cells;
            i = (int64_t)draw_index(x.x, nc) * m.nB + m.act_b[grp * m.max_gb + ba];
            j = (int64_t)draw_index(x.y, nc) * m.nB + m.act_b[grp * m.max_gb + bb];
            u = draw_u01(x.z, x.w);
        }
        int same = 1;
        if (i < 0 || j < 0 || i >= N || j >= N) { atomicOr(jb.err, 1); }
        else { ctl.ssi = sig[i]; ctl.ssj = sig[j]; same = ctl.ssi == ctl.ssj; }
        ctl.si = i; ctl.sj = j; ctl.u = u; ctl.same = same; ctl.cnt = 0; ctl.dacc = 0ull; ctl.err = 0; ctl.acc = 0;
        if (!same) { coords(m, i, ctl.bi, ctl.ki); coords(m, j, ctl.bj, ctl.kj); }
    }
    __syncthreads();
    if (!ctl.same) {
    // 2. nested unique receptive field
    for (int lvl = 0; lvl <= L; ++lvl) {
        for (int f = 0; f < 2; ++f) {
            const int b = f ? ctl.bj : ctl.bi;
            const int32_t *k = f ? ctl.kj : ctl.ki;
            const int q0 = lvl ? m.ball_end[b * (L + 1) + lvl - 1] : 0, q1 = m.ball_end[b * (L + 1) + lvl];
            // four offsets per thread with their claims (global compare-and-swap) in flight together
            for (int q = q0 + tid; q < q1; q += 4 * nt) {
                int32_t sq[4], won[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int qq = q + u * nt;
                    sq[u] = -1;
                    if (qq < q1) {
                        const int e0 = b * m.wL + qq;
                        sq[u] = (int32_t)site_at(m, k, m.ball_uo + 3 * e0, m.ball_b[e0]);
                        if (lvl == 0) ent_site[f * m.w0max + qq] = sq[u];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) won[u] = sq[u] >= 0 && atomicCAS(&slot[sq[u]], -1, -2) == -1;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (won[u]) {
                        const int p = atomicAdd(&ctl.cnt, 1);
                        list[p] = sq[u]; slot[sq[u]] = p;
                    }
            }
        }
        __syncthreads();
        if (tid == 0) ctl.nl[lvl] = ctl.cnt;
        __syncthreads();
    }
    if (ctl.nl[0] > m.n0max || ctl.nl[L] > m.nmax) {   // cannot happen for consistent tables; refuse instead of overflow
        if (tid == 0) { atomicOr(jb.err, 4); ctl.err = 1; }
        __syncthreads();
    }
    }   // !same
    }   // leader
    csync<CLUSTER>();
    if (CLUSTER && !leader) {                          // broadcast of the leader's control block
        if (tid == 0) ctl = *cx.lctl;
        __syncthreads();
    }
    if (ctl.same || ctl.err) {
        if (leader && tid == 0 && ctl.same) {
            if (jb.force != -2) ++nacc;               // an accepted no-op (kept for a commit when force = -2)
            if (jb.dE_out) jb.dE_out[s_idx * jb.R + q_ix] = 0.0;
        }
        if (leader && tid == 0 && jb.force == -2) {
            NcePending &pd = jb.pend[r];
            pd.si = ctl.si; pd.sj = ctl.sj; pd.dE = 0.0; pd.ssi = ctl.ssi; pd.ssj = ctl.ssj;
            pd.same = ctl.same; pd.valid = ctl.err ? 0 : 1;
            if (ctl.err && jb.dE_out) jb.dE_out[s_idx * jb.R + q_ix] = __longlong_as_double(0x7ff8000000000000ll);
        }
        if (ctl.err) for (int p = tid + rank * nt; p < min(ctl.nl[L], m.nmax); p += nt * CL) slot[list[p]] = -1;
        csync<CLUSTER>();
        return;
    }
    // 3. layer-0 change.  With +-1 point functions on a cluster, the rows are split over its CTAs (32-row chunks),
    //    each CTA counting into its own shared memory, and the new layer-0 rows sum the CTAs' counts through
    //    distributed shared memory; otherwise the leader does all of it.
    {
    const int n0 = ctl.nl[0];
    const bool spread = CLUSTER && m.l0bin;
    if (spread || leader) {
    // ball-0 entries of both flips: list position and occupancy (read once, reused by every row member); the
    // leader listed the sites while claiming them, the other CTAs of a cluster enumerate them again
    for (int f = 0; f < 2; ++f) {
        const int b = f ? ctl.bj : ctl.bi;
        const int32_t *k = f ? ctl.kj : ctl.ki;
        const int q1 = m.ball_end[b * (L + 1)];
        for (int q = tid; q < q1; q += nt) {
            int32_t st;
            if (leader) st = ent_site[f * m.w0max + q];
            else { st = (int32_t)site_at(m, k, m.ball_uo + 3 * (b * m.wL + q), m.ball_b[b * m.wL + q]); ent_site[f * m.w0max + q] = st; }
            ent_pos[f * m.w0max + q] = slot[st];
            ent_sig[f * m.w0max + q] = sig[st];
        }
    }
    // 3. layer-0 change (fixed point)
    if (m.l0bin) { for (int idx = tid; idx < n0 * m.C0; idx += nt) reinterpret_cast<int32_t *>(dh)[idx] = 0; }
    else { for (int idx = tid; idx < n0 * m.C0; idx += nt) dh[idx] = 0ull; }
    __syncthreads();
    const int Jt = 2 * m.J;
    if (m.l0bin) {
        // +-1 point functions: parities of the old and new products; each changed row moves its members' channel by
        // exactly +-2 w, and all rows of one channel share w, so the change is an integer count per (site, channel)
        // (32-bit atomics) times that channel's fixed-point 2 w.  Every row of a flip contains that flip's site, and
        // the rows of a channel are consecutive, so the site's own count is summed per warp and channel run.
        int32_t *dcount = reinterpret_cast<int32_t *>(dh);
        const int lane = tid & 31;
        for (int base = tid - lane + (spread ? rank * nt : 0); base < Jt; base += nt * (spread ? CL : 1)) {
            const int rr = base + lane;
            int f = 0, ch = 0, csign = 0, pc = 0;
            long long wf = 0;
            if (rr < Jt) {
                f = rr >= m.J;
                const int jr = f ? rr - m.J : rr;
                const int b = f ? ctl.bj : ctl.bi;
                const int e = b * m.J + jr;
                wf = m.Rv_wfix[e];
                if (wf != 0) {
                    unsigned po = 0, pn = 0;
                    int32_t pos[8], own[8];
                    const int32_t *es = ent_site + f * m.w0max;
                    const int32_t centre = f ? (int32_t)ctl.sj : (int32_t)ctl.si;
                    int n_own = 0;
                    int32_t dsc[8];
                    for (int mm = 0; mm < m.mo; ++mm) dsc[mm] = __ldg(m.Rv_desc + (size_t)e * m.mo + mm);   // loads in flight together
                    for (int mm = 0; mm < m.mo; ++mm) {
                        own[mm] = 0;
                        const int32_t d = dsc[mm];
                        if (!((d >> 16) & 1)) continue;
                        const int q = d & 0xffff;
                        const int32_t st = es[q];
                        pos[mm] = ent_pos[f * m.w0max + q];
                        own[mm] = st == centre;
                        n_own += own[mm];
                        int so = ent_sig[f * m.w0max + q], sn = so;
                        if (f == 0) { if (st == (int32_t)ctl.si) sn = ctl.ssj; }
                        else {
                            if (st == (int32_t)ctl.si) { so = ctl.ssj; sn = ctl.ssj; }
                            if (st == (int32_t)ctl.sj) sn = ctl.ssi;
                        }
                        po ^= (unsigned)(d >> (20 + so)) & 1u; pn ^= (unsigned)(d >> (20 + sn)) & 1u;
                    }
                    if (po != pn) {                                  // new product -1: (pn - po) w = -2 w
                        ch = m.Rv_col[e] + 1;
                        for (int mm = 0; mm < m.mo; ++mm) {
                            if (!((dsc[mm] >> 16) & 1)) continue;
                            const int p = pos[mm];
                            if (p < 0 || p >= n0) { atomicOr(jb.err, 8); continue; }
                            if (own[mm] && n_own == 1) { csign = pn ? -1 : 1; pc = p; continue; }
                            atomicAdd(&dcount[(size_t)p * m.C0 + ch], pn ? -1 : 1);
                        }
                    }
                }
            }
            const unsigned key = csign ? (((unsigned)f << 16) | (unsigned)ch) : 0xffffffffu;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            const unsigned plus = __ballot_sync(0xffffffffu, csign > 0), minus = __ballot_sync(0xffffffffu, csign < 0);
            if (csign && lane == __ffs(peers) - 1) {
                const int k = __popc(peers & plus) - __popc(peers & minus);
                if (k) atomicAdd(&dcount[(size_t)pc * m.C0 + ch], k);
            }
        }
    }
    for (int rr = tid; rr < Jt && !m.l0bin; rr += nt) {
        const int f = rr >= m.J, jr = f ? rr - m.J : rr;
        const int b = f ? ctl.bj : ctl.bi;
        const int e = b * m.J + jr;
        const double w = m.Rv_w[e];
        if (w == 0.0) continue;
        double po = 1.0, pn = 1.0;
        int32_t pos[8];
        const int32_t *es = ent_site + f * m.w0max;
        for (int mm = 0; mm < m.mo; ++mm) {
            const int em = e * m.mo + mm;
            if (!m.Rv_m[em]) continue;
            const int q = m.Rv_loc[em];
            const int32_t st = es[q];
            pos[mm] = ent_pos[f * m.w0max + q];
            int so = ent_sig[f * m.w0max + q], sn = so;
            // flip 0: i -> ssj ; flip 1 (f = 1) evaluated on the configuration after flip 0
            if (f == 0) { if (st == (int32_t)ctl.si) sn = ctl.ssj; }
            else {
                if (st == (int32_t)ctl.si) { so = ctl.ssj; sn = ctl.ssj; }
                if (st == (int32_t)ctl.sj) sn = ctl.ssi;
            }
            const int M = m.Mb[m.Rv_b[em]], pi = m.Rv_p[em];
            const double *th = m.theta + ((size_t)M * m.maxP + pi) * m.maxM;
            po *= th[so]; pn *= th[sn];
        }
        const double val = (pn - po) * w;
        if (val == 0.0) continue;
        const long long fx = llrint(val * kFix);
        const int ch = m.Rv_col[e] + 1;
        for (int mm = 0; mm < m.mo; ++mm) {
            if (!m.Rv_m[e * m.mo + mm]) continue;
            const int p = pos[mm];
            if (p < 0 || p >= n0) { atomicOr(jb.err, 8); continue; }
            atomicAdd(&dh[(size_t)p * m.C0 + ch], (unsigned long long)fx);
        }
    }
    __syncthreads();
    }
    if constexpr (CLUSTER) {
        if (spread) {
            csync<CLUSTER>();                              // every CTA's counts are complete
            cg::cluster_group cluster = cg::this_cluster();
            const int32_t *dcount = reinterpret_cast<const int32_t *>(dh);
            float *nb0w = level_buf(jb, nb, 0);
            const int lane = tid & 31, gw = (tid >> 5) + rank * (nt >> 5), nw = (nt >> 5) * CL;
            for (int p = gw; p < n0; p += nw) {
                const float *hrow = h0 + (size_t)list[p] * m.C0;
                for (int c = lane; c < m.C0; c += 32) {
                    const int idx = p * m.C0 + c;
                    long long cnt = 0;
                    for (int q = 0; q < CL; ++q) cnt += cluster.map_shared_rank(dcount, q)[idx];
                    nb0w[idx] = hrow[c] + (float)((double)(cnt * m.col_wfix[c]) * kInvFix);
                }
            }
        }
    }
    if (!spread && leader) {
    float *nb0w = level_buf(jb, nb, 0);
    if (m.l0bin) {
        const int32_t *dcount = reinterpret_cast<const int32_t *>(dh);
        for (int idx = tid; idx < n0 * m.C0; idx += nt) {
            const int p = idx / m.C0, c = idx % m.C0;
            const int64_t s = list[p];
            const long long fx = (long long)dcount[idx] * m.col_wfix[c];
            nb0w[idx] = h0[(size_t)s * m.C0 + c] + (float)((double)fx * kInvFix);
        }
    } else {
    for (int idx = tid; idx < n0 * m.C0; idx += nt) {
        const int p = idx / m.C0, c = idx % m.C0;
        const int64_t s = list[p];
        nb0w[idx] = h0[(size_t)s * m.C0 + c] + (float)((double)(long long)dh[idx] * kInvFix);
    }
    }
    }
    }
    csync<CLUSTER>();                                  // the new layer-0 rows are complete
    const int n0 = ctl.nl[0];
    float *nb0 = level_buf(jb, nb, 0);
    if (!leader && tid == 0) ctl.dacc = 0ull;
    __syncthreads();
    // 4. layers
    const int ncg = m.D / 4;
    unsigned long long dloc = 0ull;                  // this thread's share of dE (fixed point)
    for (int lvl = 0; lvl < L; ++lvl) {
        const float *cache = lvl == 0 ? h0 : jb.hmid + ((size_t)(lvl - 1) * jb.R + r) * N * m.D;
        const float *newl = level_buf(jb, nb, lvl);
        const int nout = ctl.nl[lvl + 1];
        if (lvl + 1 < L) {
            float *outb = level_buf(jb, nb, lvl + 1);
            const int D = m.D;
            layer_tiles(jb, lvl, LWs[lvl], cache, newl, slot, ctl.nl[lvl], list, 0, nout, nullptr, X, src,
                        [&](int64_t pos, int c0, const float *v, int32_t, int32_t) {
                            if (pos >= 0) *reinterpret_cast<float4 *>(outb + (size_t)pos * D + c0) = make_float4(v[0], v[1], v[2], v[3]);
                        }, rank, CL, tc);
            csync<CLUSTER>();
        } else {
            // the sink's reads and writes do not alias (caches, the step's new rows, the new site energies): the
            // loads of one tile site may run ahead of the stores of the previous one
            const float *__restrict__ e_r = e, *__restrict__ h0_r = h0, *__restrict__ nb0_r = nb0;
            float *__restrict__ en_r = en;
            layer_tiles(jb, lvl, LWs[lvl], cache, newl, slot, ctl.nl[lvl], list, 0, nout, nullptr, X, src,
                        [&](int64_t pos, int c0, const float *v, int32_t site, int32_t p0) {
                            // the tile passes the site and its slot value (read while building the tile)
                            const float *hr = nullptr;
                            const int64_t st = site;
                            if (pos >= 0) hr = (p0 >= 0 && p0 < n0) ? nb0_r + (size_t)p0 * m.C0 : h0_r + (size_t)st * m.C0;
                            const float tot = site_energy(v, c0, hw, hr, lin, m.C0, ncg);
                            if (pos >= 0 && c0 == 0) {
                                const bool active = m.Mb[site % m.nB] > 1;
                                const float ev = active ? tot : 0.f;
                                en_r[pos] = ev;
                                dloc += (unsigned long long)llrint(((double)ev - (double)e_r[st]) * kFix);
                            }
                        }, rank, CL, tc);
        }
    }
    if (L == 0) {
        for (int p = tid + rank * nt; p < n0; p += nt * CL) {
            const int64_t s = list[p];
            float l0 = 0.f;
            for (int c = 0; c < m.C0; ++c) l0 = fmaf(nb0[(size_t)p * m.C0 + c], lin[c], l0);
            const float ev = m.Mb[s % m.nB] > 1 ? l0 : 0.f;
            en[p] = ev;
            dloc += (unsigned long long)llrint(((double)ev - (double)e[s]) * kFix);
        }
    }
    // the fixed-point partials of this thread, then of its warp, into the CTA's sum (integer: order-free)
    for (int o = 16; o > 0; o >>= 1) dloc += __shfl_xor_sync(0xffffffffu, dloc, o);
    if ((tid & 31) == 0 && dloc) atomicAdd(&ctl.dacc, dloc);
    __syncthreads();
    if (CLUSTER && !leader && tid == 0 && ctl.dacc) atomicAdd(&cx.lctl->dacc, ctl.dacc);   // partial dE to the leader
    csync<CLUSTER>();
    // 5. accept (leader), broadcast, commit split over the cluster
    if (leader && tid == 0) {
        const double dE = (double)(long long)ctl.dacc * kInvFix / m.norm;
        const double dEeV = dE * m.scale_eV;
        const double beta = (double)jb.beta_slot[t];
        int a;
        if (jb.force > 0) a = 1;
        else if (jb.force < 0) a = 0;
        else a = (dEeV <= 0.0) || (ctl.u < exp(-beta * dEeV));
        if (jb.force == 0 && beta > 0.0 && fabs(dEeV + log(ctl.u) / beta) < jb.near_eV) ++nnear;
        ctl.acc = a;
        if (jb.dE_out) jb.dE_out[s_idx * jb.R + q_ix] = dE;
        if (jb.force == -2) {                          // keep the evaluated swap for nce_nce_commit
            NcePending &pd = jb.pend[r];
            pd.si = ctl.si; pd.sj = ctl.sj; pd.dE = dE; pd.ssi = ctl.ssi; pd.ssj = ctl.ssj; pd.same = 0; pd.valid = 1;
            for (int l = 0; l <= L; ++l) pd.nl[l] = ctl.nl[l];
        }
        if (a) { sig[ctl.si] = (int8_t)ctl.ssj; sig[ctl.sj] = (int8_t)ctl.ssi; E += dE; ++nacc; }
    }
    csync<CLUSTER>();
    __shared__ int acc_flag;
    if (tid == 0) acc_flag = CLUSTER ? cx.lctl->acc : ctl.acc;
    __syncthreads();
    const int nL = ctl.nl[L];
    const int ts = tid + rank * nt, tstr = nt * CL;
    if (acc_flag) {
        // a warp per row over the cluster's warps: the row's site read once, columns by lanes (float4 for D)
        const int lane = tid & 31, gw = (tid >> 5) + rank * (nt >> 5), nw = (nt >> 5) * CL;
        for (int p = gw; p < n0; p += nw) {
            float *dst = h0 + (size_t)list[p] * m.C0;
            const float *srow = nb0 + (size_t)p * m.C0;
            for (int c = lane; c < m.C0; c += 32) dst[c] = srow[c];
        }
        const int D4 = m.D / 4;
        for (int lvl = 1; lvl < L; ++lvl) {
            float *hm = jb.hmid + ((size_t)(lvl - 1) * jb.R + r) * N * m.D;
            const float *src = level_buf(jb, nb, lvl);
            const int nl = ctl.nl[lvl];
            for (int p = gw; p < nl; p += nw) {
                float4 *dst = reinterpret_cast<float4 *>(hm + (size_t)list[p] * m.D);
                const float4 *srow = reinterpret_cast<const float4 *>(src + (size_t)p * m.D);
                for (int c = lane; c < D4; c += 32) dst[c] = srow[c];
            }
        }
        for (int p = ts; p < nL; p += tstr) e[list[p]] = en[p];
    }
    for (int p = ts; p < nL; p += tstr) slot[list[p]] = -1;
    csync<CLUSTER>();
}

// weights of all layers staged in shared memory when they fit (w_smem), else read from global memory
__device__ void stage_weights(const NceDev &m, bool w_smem, float *wbuf, LayerW *LWs, const float *&lin, const float *&hw) {
    const int tid = threadIdx.x, nt = blockDim.x;
    size_t o = 0;
    auto put = [&](const float *g, size_t n) -> const float * {
        if (!g) return nullptr;
        if (!w_smem) return g;
        float *d = wbuf + o;
        for (size_t i = tid; i < n; i += nt) d[i] = __ldg(g + i);
        o += (n + 3) & ~(size_t)3;
        return d;
    };
    for (int l = 0; l < m.depth; ++l) {
        const int Cin = l == 0 ? m.C0 : m.D;
        LWs[l].W = put(m.Wc[l], (size_t)(1 + m.P) * Cin * m.D);
        LWs[l].b = put(m.bias[l], (size_t)m.D);
        LWs[l].G = m.gate ? put(m.G[l], (size_t)m.P * Cin * m.D) : nullptr;
        LWs[l].gb = m.gate ? put(m.gb[l], (size_t)m.D) : nullptr;
    }
    lin = put(m.lin, (size_t)m.C0);
    hw = put(m.head_w, (size_t)(m.depth ? m.D : 4));
    __syncthreads();
}

__host__ __device__ inline size_t weight_floats(int depth, int P, int C0, int D, int gate) {
    size_t o = 0;
    auto add = [&](size_t n) { o += (n + 3) & ~(size_t)3; };
    for (int l = 0; l < depth; ++l) {
        const int Cin = l == 0 ? C0 : D;
        add((size_t)(1 + P) * Cin * D); add((size_t)D);
        if (gate) { add((size_t)P * Cin * D); add((size_t)D); }
    }
    add((size_t)C0); add((size_t)(depth ? D : 4));
    return o;
}

// shared-memory plan of the step kernel (byte offsets, 16-byte aligned): X tile | partner codes | tcgen05 B operand,
// sharing its bytes with dh | ball-0 entries | weights.  dh (the layer-0 change) lives only between the receptive
// field's build and the first layer, and the B operand is copied in at the start of each layer, so the two share one
// region.  with_dh = false: the tile part alone (full-cache kernel).  On the tcgen05 path the X tile holds the bf16
// A operand(s) [128][tc_ks] or the float32 output rows [128][D + 4], whichever is larger.
struct SmemPlan {
    size_t dh, X, src, wt, ent, w, dh_bytes, tile_end, total_w;
    __host__ __device__ static SmemPlan make(const NceDev &m, bool with_dh = true) {
        auto al = [](size_t x) { return (x + 15) / 16 * 16; };
        auto al128 = [](size_t x) { return (x + 127) / 128 * 128; };
        SmemPlan p;
        const int TM = tile_tm(m.D, m.tc, m.mma), Kmax = tile_kin(m.P, m.C0, m.D);
        // layer-0 change per (site, channel): int32 counts for +-1 point functions, int64 fixed point otherwise
        p.dh_bytes = with_dh ? al((m.l0bin ? sizeof(int32_t) : sizeof(unsigned long long)) * (size_t)m.n0max * m.C0) : 0;
        p.X = 0;
        size_t xb = sizeof(float) * (size_t)TM * x_stride(Kmax);
        if (m.tc) {
            const size_t ab = (size_t)128 * m.tc_ks * 2 * (m.tc_split ? 2 : 1), yb = sizeof(float) * 128 * (size_t)(m.D + 4);
            xb = ab > yb ? ab : yb;
        }
        p.src = al(p.X + xb);
        p.wt = al128(p.src + sizeof(const float *) * (size_t)TM * (1 + m.P * m.W) + sizeof(int32_t) * (size_t)TM * 7);
        const size_t wtb = m.tc ? (size_t)kpad16(Kmax) * m.D * 2 * (m.tc_split ? 2 : 1) : 0;
        p.dh = p.wt;
        p.tile_end = p.wt + (with_dh ? (wtb > p.dh_bytes ? wtb : p.dh_bytes) : wtb);
        p.ent = al(p.tile_end);
        p.w = al(p.ent + (sizeof(int32_t) * 2 + 1) * 2 * (size_t)m.w0max);
        p.total_w = al(p.w + sizeof(float) * weight_floats(m.depth, m.P, m.C0, m.D, m.gate));
        return p;
    }
};

// MINB = CTAs resident per SM: 1 (all registers) or 2 (at most 128 registers a thread, twice the warps to hide
// the latency of the gathers and barriers when two CTAs' shared memory fits an SM)
template <int MINB>
__global__ void __launch_bounds__(256, MINB) nce_chunk_kernel(const __grid_constant__ NceJob jb, int32_t w_smem) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ NceCtl ctl;
    const int r = blockIdx.x;
    if (r >= jb.R) return;
    const NceDev &m = jb.m;
    const SmemPlan sp = SmemPlan::make(m);
    unsigned long long *dh = reinterpret_cast<unsigned long long *>(smem + sp.dh);
    float *X = reinterpret_cast<float *>(smem + sp.X);
    int32_t *src = reinterpret_cast<int32_t *>(smem + sp.src);
    float *wbuf = reinterpret_cast<float *>(smem + sp.w);
    int32_t *ent_site = reinterpret_cast<int32_t *>(smem + sp.ent);
    int32_t *ent_pos = ent_site + 2 * m.w0max;
    int8_t *ent_sig = reinterpret_cast<int8_t *>(ent_pos + 2 * m.w0max);
    LayerW lw[kMaxLayers]; const float *lin, *hw;
    stage_weights(m, w_smem != 0, wbuf, lw, lin, hw);
    __shared__ __align__(8) uint64_t tc_mbar;
    __shared__ uint32_t tc_slot;
    TcCtx tcx;
    if (m.tc) tc_begin(m.D, tcx, smem + sp.wt, &tc_mbar, &tc_slot);
    const int t = jb.slot_of_rep[r];
    double E = jb.E[r];
    int64_t nacc = 0, nnear = 0;
    NceCtx cx; cx.rank = 0; cx.CL = 1; cx.lctl = &ctl;
    for (int64_t s = 0; s < jb.n_steps; ++s) {
        nce_step<false>(jb, r, t, s, ctl, dh, X, src, lw, lin, hw, ent_site, ent_pos, ent_sig, E, nacc, nnear, cx, m.tc ? &tcx : nullptr);
        if (threadIdx.x == 0 && jb.E_samples && (s + 1) % jb.sample_interval == 0)
            jb.E_samples[((s + 1) / jb.sample_interval - 1) * jb.R + t] = E;
        __syncthreads();
    }
    if (threadIdx.x == 0) { jb.E[r] = E; jb.n_acc[r] += nacc; if (jb.n_near) jb.n_near[r] += nnear; }
    if (m.tc) tc_end(m.D, tcx);
}

// the same chunk with each replica spread over a thread-block cluster of gridDim.x / R CTAs
template <int MINB>
__global__ void __launch_bounds__(256, MINB) nce_chunk_cluster_kernel(const __grid_constant__ NceJob jb, int32_t w_smem) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ NceCtl ctl;
    cg::cluster_group cluster = cg::this_cluster();
    const int CL = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
    const int r = blockIdx.x / CL;
    if (r >= jb.R) return;                           // whole clusters only: gridDim.x == R * CL
    const NceDev &m = jb.m;
    const SmemPlan sp = SmemPlan::make(m);
    unsigned long long *dh = reinterpret_cast<unsigned long long *>(smem + sp.dh);
    float *X = reinterpret_cast<float *>(smem + sp.X);
    int32_t *src = reinterpret_cast<int32_t *>(smem + sp.src);
    float *wbuf = reinterpret_cast<float *>(smem + sp.w);
    int32_t *ent_site = reinterpret_cast<int32_t *>(smem + sp.ent);
    int32_t *ent_pos = ent_site + 2 * m.w0max;
    int8_t *ent_sig = reinterpret_cast<int8_t *>(ent_pos + 2 * m.w0max);
    LayerW lw[kMaxLayers]; const float *lin, *hw;
    stage_weights(m, w_smem != 0, wbuf, lw, lin, hw);
    __shared__ __align__(8) uint64_t tc_mbar;
    __shared__ uint32_t tc_slot;
    TcCtx tcx;
    if (m.tc) tc_begin(m.D, tcx, smem + sp.wt, &tc_mbar, &tc_slot);
    NceCtx cx; cx.rank = rank; cx.CL = CL; cx.lctl = cluster.map_shared_rank(&ctl, 0);
    cluster.sync();
    const int t = jb.slot_of_rep[r];
    double E = jb.E[r];
    int64_t nacc = 0, nnear = 0;
    for (int64_t s = 0; s < jb.n_steps; ++s) {
        nce_step<true>(jb, r, t, s, ctl, dh, X, src, lw, lin, hw, ent_site, ent_pos, ent_sig, E, nacc, nnear, cx, m.tc ? &tcx : nullptr);
        if (rank == 0 && threadIdx.x == 0 && jb.E_samples && (s + 1) % jb.sample_interval == 0)
            jb.E_samples[((s + 1) / jb.sample_interval - 1) * jb.R + t] = E;
    }
    if (rank == 0 && threadIdx.x == 0) { jb.E[r] = E; jb.n_acc[r] += nacc; if (jb.n_near) jb.n_near[r] += nnear; }
    cluster.sync();                                   // no CTA leaves while others may still read its shared memory
    if (m.tc) tc_end(m.D, tcx);
}

// Commit of the swaps kept by a force = -2 chunk (nce_nce_local_delta): one CTA per replica writes the new layer-0,
// hidden and site-energy rows from the step scratch into the caches, swaps the two sites and adds dE to the carried
// energy, where accept[r] != 0 (the reference's commit, neuralce/nce/local_update_implicit.py:185-194, plus the
// driver's occupancy and energy update, neuralce/nce/mcmc.py:180-185).  Every kept swap is consumed.
__global__ void __launch_bounds__(256) nce_commit_kernel(const __grid_constant__ NceJob jb, const int32_t *__restrict__ accept) {
    const int r = blockIdx.x;
    if (r >= jb.R) return;
    const NceDev &m = jb.m;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    const NcePending pd = jb.pend[r];
    __syncthreads();                                   // every thread has read the record before it is consumed
    if (tid == 0) jb.pend[r].valid = 0;
    if (!pd.valid || !accept[r]) return;
    if (tid == 0) jb.n_acc[r] += 1;
    if (pd.same) return;                               // same species: an accepted no-op
    const int64_t N = m.N;
    int8_t *sig = jb.sigma + (int64_t)r * N;
    float *h0 = jb.h0 + (size_t)r * N * m.C0;
    float *e = jb.e + (size_t)r * N;
    const int32_t *list = jb.list + (size_t)r * m.nmax;
    float *nb = jb.newbuf + (size_t)r * jb.scratch_stride;
    const float *en = jb.e_new + (size_t)r * m.nmax;
    if (tid == 0) { sig[pd.si] = (int8_t)pd.ssj; sig[pd.sj] = (int8_t)pd.ssi; jb.E[r] += pd.dE; }
    const float *nb0 = level_buf(jb, nb, 0);
    for (int p = warp; p < pd.nl[0]; p += nw)
        for (int c = lane; c < m.C0; c += 32) h0[(size_t)list[p] * m.C0 + c] = nb0[(size_t)p * m.C0 + c];
    for (int lvl = 1; lvl < m.depth; ++lvl) {
        float *hm = jb.hmid + ((size_t)(lvl - 1) * jb.R + r) * N * m.D;
        const float *src = level_buf(jb, nb, lvl);
        for (int p = warp; p < pd.nl[lvl]; p += nw)
            for (int c = lane; c < m.D; c += 32) hm[(size_t)list[p] * m.D + c] = src[(size_t)p * m.D + c];
    }
    for (int p = tid; p < pd.nl[m.depth]; p += nt) e[list[p]] = en[p];
}

// Metropolis decisions of R replicas from the dE of n_models models (mean over the models: the reference's ensemble)
__global__ void nce_accept_kernel(const double *__restrict__ dE, int32_t n_models, int32_t R, double scale_eV,
                                  const float *__restrict__ beta_slot, const int32_t *__restrict__ slot_of_rep,
                                  const double *__restrict__ u, int32_t *__restrict__ accept) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double s = 0.0;
    for (int k = 0; k < n_models; ++k) s += dE[(size_t)k * R + r];
    const double dEeV = s / n_models * scale_eV;
    const double beta = (double)beta_slot[slot_of_rep[r]];
    accept[r] = (dEeV == dEeV) && ((dEeV <= 0.0) || (u[r] < exp(-beta * dEeV)));
}

// ── full cache ─────────────────────────────────────────────────────────────────────────────────────
// Layer 0 of every site, bit-sliced (+-1 point functions): one plane per basis holds the sign bit of each site,
// each (k0, k1) row twice over (2 d2 bits) so that any offset in [0, d2) reads 32 consecutive bits.  A thread takes
// 32 consecutive sites along k2 and, for every reverse row of their basis (all slots: every cluster instance that
// contains the site), XORs the members' shifted plane words: bit j is the parity of site j's product.  Odd parities
// are counted per site in a vertical (bit-sliced) counter while the rows of one channel go by; the channel value is
// then (rows - 2 odd) w - mu / sd, as the float64 row sum gives.
__global__ void nce_plane_kernel(NceDev m, const int8_t *__restrict__ sigma, int32_t R, int32_t W2, uint32_t *__restrict__ planes) {
    const int64_t d0d1 = (int64_t)m.d0 * m.d1;
    const int64_t rows = (int64_t)R * m.nB * d0d1;
    const int lane = threadIdx.x & 31;
    const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < rows; w += wstride) {
        const int64_t kk = w % d0d1;
        const int64_t t = w / d0d1;
        const int b = (int)(t % m.nB);
        const int64_t r = t / m.nB;
        const int M = m.Mb[b];
        const uint8_t *ts = m.thsign + (size_t)M * m.maxP * m.maxM;          // point function 0 of M species
        const int8_t *sg = sigma + r * m.N + kk * m.d2 * m.nB + b;
        uint32_t *out = planes + w * W2;
        for (int q = 0; q < W2; ++q) {
            const int pos = q * 32 + lane;
            uint32_t bit = 0;
            if (pos < 2 * m.d2) {
                const int k2 = pos < m.d2 ? pos : pos - m.d2;
                bit = ts[sg[(int64_t)k2 * m.nB] & 3];
            }
            const uint32_t word = __ballot_sync(0xffffffffu, bit != 0u);
            if (lane == 0) out[q] = word;
        }
    }
}

// grid (blocks, nB x S, R): threads over the (k0, k1, 32-site word) items of basis blockIdx.y / S, replica
// blockIdx.z; slice blockIdx.y % S takes the rows and channels [h0s_row, h0s_ch] .. of the next slice (slices cut
// the rows of a basis at channel boundaries, so small cells still fill the GPU)
__global__ void __launch_bounds__(128) nce_h0_bits_kernel(NceDev m, const uint32_t *__restrict__ planes, int32_t W2, float *h0) {
    const int S = m.h0_slices, b = blockIdx.y / S, sl = blockIdx.y % S, r = blockIdx.z;
    const int2 lo = m.h0_slice[b * (S + 1) + sl], hi = m.h0_slice[b * (S + 1) + sl + 1];   // (first row, first channel)
    const int d0 = m.d0, d1 = m.d1, d2 = m.d2;
    const int Wn = (d2 + 31) >> 5;
    const int64_t items = (int64_t)d0 * d1 * Wn;
    const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= items) return;
    const int w = (int)(it % Wn);
    const int64_t kk = it / Wn;
    const int k1 = (int)(kk % d1), k0 = (int)(kk / d1);
    const int nv = min(32, d2 - 32 * w);
    const uint32_t mask = nv >= 32 ? 0xffffffffu : ((1u << nv) - 1u);
    const uint32_t *pr = planes + (int64_t)r * m.nB * d0 * d1 * W2;
    const int C0 = m.C0;
    // site j of the word: canonical index ((k0 d1 + k1) d2 + 32 w + j) nB + b
    float *out0 = h0 + (((int64_t)r * m.N) + ((int64_t)(k0 * d1 + k1) * d2 + 32 * w) * m.nB + b) * C0;
    const int64_t sstride = (int64_t)m.nB * C0;
    if (m.Mb[b] < 2) {                                       // inactive sites: zeros
        for (int j = 0; j < nv; ++j) for (int c = sl ? lo.y : 0; c < hi.y; ++c) out0[j * sstride + c] = 0.f;
        return;
    }
    if (sl == 0) {
        const float ch0 = (float)((1.0 - (double)m.mu[0]) / (double)m.sd[0]);
        for (int j = 0; j < nv; ++j) out0[j * sstride] = ch0;
    }
    constexpr int NQ = 13;                                    // vertical counter planes: up to 8191 rows per channel
    uint32_t cnt[NQ];
    auto flush = [&](int ch, int nrows) {
        const double wc = m.col_w[ch], base = (double)m.mu[ch] / (double)m.sd[ch];
        for (int j = 0; j < nv; ++j) {
            int odd = 0;
#pragma unroll
            for (int q = 0; q < NQ; ++q) odd |= (int)((cnt[q] >> j) & 1u) << q;
            out0[j * sstride + ch] = (float)((double)(nrows - 2 * odd) * wc - base);
        }
    };
    int ch_cur = lo.y, nrows = 0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) cnt[q] = 0u;
    const int4 *mem = m.h0mem + (size_t)b * m.J * m.mo;
    for (int jr = lo.x; jr < hi.x; ++jr) {
        const int e = b * m.J + jr;
        if (m.Rv_wfix[e] == 0) continue;
        const int ch = m.Rv_col[e] + 1;
        if (ch != ch_cur) {
            flush(ch_cur, nrows);
#pragma unroll
            for (int q = 0; q < NQ; ++q) cnt[q] = 0u;
            for (int c = ch_cur + 1; c < ch; ++c) flush(c, 0);
            ch_cur = ch; nrows = 0;
        }
        uint32_t par = 0;
        for (int mm = 0; mm < m.mo; ++mm) {
            const int4 d = mem[jr * m.mo + mm];                // (member basis or -1, uo0, uo1, uo2)
            if (d.x < 0) continue;
            int a0 = k0 + d.y; a0 -= a0 >= d0 ? d0 : 0;
            int a1 = k1 + d.z; a1 -= a1 >= d1 ? d1 : 0;
            const int pos = 32 * w + d.w;
            const uint32_t *row = pr + (((int64_t)d.x * d0 + a0) * d1 + a1) * W2 + (pos >> 5);
            par ^= __funnelshift_r(__ldg(row), __ldg(row + 1), (unsigned)(pos & 31));
        }
        // add the odd-parity bits into the vertical counter (ripple carry)
        uint32_t carry = par & mask;
#pragma unroll
        for (int q = 0; q < NQ; ++q) { const uint32_t t = cnt[q] & carry; cnt[q] ^= carry; carry = t; }
        ++nrows;
    }
    if (ch_cur < hi.y) flush(ch_cur, nrows);
#pragma unroll
    for (int q = 0; q < NQ; ++q) cnt[q] = 0u;
    for (int c = ch_cur + 1; c < hi.y; ++c) flush(c, 0);
}

// Layer 0 of every site for general point functions: every reverse row of each site pulled in float64 (fixed
// order, deterministic), standardised, float32
__global__ void nce_h0_kernel(NceDev m, const int8_t *sigma, int32_t R, float *h0) {
    const int64_t total = (int64_t)R * m.N;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / m.N, s = idx % m.N;
        const int8_t *sig = sigma + r * m.N;
        int32_t b, k[3]; coords(m, s, b, k);
        float *out = h0 + (size_t)idx * m.C0;
        const bool active = m.Mb[b] > 1;
        double acc[64];
        for (int c = 0; c < m.C0; ++c) acc[c] = 0.0;
        for (int jr = 0; jr < m.J; ++jr) {
            const int e = b * m.J + jr;
            const double w = m.Rv_w[e];
            if (w == 0.0) continue;
            double pr = 1.0;
            for (int mm = 0; mm < m.mo; ++mm) {
                const int em = e * m.mo + mm;
                if (!m.Rv_m[em]) continue;
                const int64_t q = site_at(m, k, m.Rv_uo + 3 * em, m.Rv_b[em]);
                const double *th = m.theta + ((size_t)m.Mb[m.Rv_b[em]] * m.maxP + m.Rv_p[em]) * m.maxM;
                pr *= th[sig[q]];
            }
            acc[m.Rv_col[e] + 1] += pr * w;      // Rv_w already carries 1/sd of the column
        }
        if (!active) { for (int c = 0; c < m.C0; ++c) out[c] = 0.f; continue; }
        // channel 0: the active indicator, standardised; columns: standardised sums (mu/sd folded: acc already / sd)
        out[0] = (float)((1.0 - (double)m.mu[0]) / (double)m.sd[0]);
        for (int c = 1; c < m.C0; ++c) out[c] = (float)(acc[c] - (double)m.mu[c] / (double)m.sd[c]);
    }
}

// one layer on all sites: out = layer(in); e accumulation on the last layer (weights read from global memory)
__global__ void __launch_bounds__(256, 1) nce_layer_all_kernel(NceJob jb, int lvl, int32_t r, const float *in, float *out,
                                                             float *e_out, int64_t chunk0, int64_t chunk_n) {
    extern __shared__ __align__(16) unsigned char smem[];
    const NceDev &m = jb.m;
    const int TM = tile_tm(m.D, m.tc, m.mma);
    const SmemPlan sp = SmemPlan::make(m, false);
    float *X = reinterpret_cast<float *>(smem + sp.X);
    int32_t *src = reinterpret_cast<int32_t *>(smem + sp.src);
    const int64_t per = ((chunk_n + gridDim.x - 1) / gridDim.x + TM - 1) / TM * TM;
    const int64_t a = chunk0 + (int64_t)blockIdx.x * per, cnt = max((int64_t)0, min(per, chunk0 + chunk_n - a));
    if (cnt <= 0) return;
    __shared__ __align__(8) uint64_t tc_mbar;
    __shared__ uint32_t tc_slot;
    TcCtx tcx;
    if (m.tc) tc_begin(m.D, tcx, smem + sp.wt, &tc_mbar, &tc_slot);
    TcCtx *tcp = m.tc ? &tcx : nullptr;
    const float *h0 = jb.h0 + (size_t)r * m.N * m.C0;
    const int D = m.D, ncg = D / 4;
    LayerW LW; LW.W = m.Wc[lvl]; LW.b = m.bias[lvl]; LW.G = m.gate ? m.G[lvl] : nullptr; LW.gb = m.gate ? m.gb[lvl] : nullptr;
    if (out) {
        layer_tiles(jb, lvl, LW, in, nullptr, nullptr, 0, nullptr, 0, cnt, &a, X, src, [&](int64_t pos, int c0, const float *v, int32_t, int32_t) {
            if (pos >= 0) *reinterpret_cast<float4 *>(out + (size_t)(a + pos) * D + c0) = make_float4(v[0], v[1], v[2], v[3]);
        }, 0, 1, tcp);
    } else {
        layer_tiles(jb, lvl, LW, in, nullptr, nullptr, 0, nullptr, 0, cnt, &a, X, src, [&](int64_t pos, int c0, const float *v, int32_t, int32_t) {
            const int64_t st = a + pos;
            const float tot = site_energy(v, c0, m.head_w, pos >= 0 ? h0 + (size_t)st * m.C0 : nullptr, m.lin, m.C0, ncg);
            if (pos >= 0 && c0 == 0) e_out[st] = (m.Mb[st % m.nB] > 1) ? tot : 0.f;
        }, 0, 1, tcp);
    }
    if (m.tc) tc_end(m.D, tcx);
}

__global__ void nce_e0_kernel(NceDev m, const float *h0, int64_t n, float *e) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t site = s % m.N;
        float l0 = 0.f;
        for (int c = 0; c < m.C0; ++c) l0 = fmaf(h0[(size_t)s * m.C0 + c], __ldg(m.lin + c), l0);
        e[s] = m.Mb[site % m.nB] > 1 ? l0 : 0.f;
    }
}

// E[r] = sum_s e[r, s] / norm + head_b, fixed point (order independent)
__global__ void nce_energy_kernel(NceDev m, const float *e, int32_t R, double *E, unsigned long long *acc) {
    const int r = blockIdx.y;
    unsigned long long local = 0ull;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m.N; s += (int64_t)gridDim.x * blockDim.x)
        local += (unsigned long long)llrint((double)e[(size_t)r * m.N + s] * kFix);
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&acc[r], local);
}

__global__ void nce_energy_finish(NceDev m, const unsigned long long *acc, int32_t R, double *E) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) E[r] = (double)(long long)acc[r] * kInvFix / m.norm + (double)m.head_b;
}

}  // namespace nce

// ───────────────────────────── host side ──────────────────────────────────────────────────────

struct nce_nce_model {
    nce::NceDev dev;
    std::vector<void *> allocs;
    std::mutex mu;
    int32_t *err = nullptr;
    // scratch for R replicas
    int32_t *slot = nullptr, *list = nullptr; float *newbuf = nullptr, *e_new = nullptr; int64_t stride = 0; int32_t R_alloc = 0;
    nce::NcePending *pend = nullptr;            // (R_alloc) swaps kept by nce_nce_local_delta
};


namespace nce {

template <typename T>
static int dup(nce_nce_model *h, const T *src, size_t n, const T *&dst) {
    dst = nullptr;
    if (!n || !src) return NCE_OK;
    void *p = nullptr;
    NCE_CUDA(cudaMalloc(&p, sizeof(T) * n));
    h->allocs.push_back(p);
    NCE_CUDA(cudaMemcpy(p, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    dst = (const T *)p;
    return NCE_OK;
}

// dynamic shared memory of the step kernels: 227 KB per CTA less the kernels' static shared memory
constexpr size_t kStepSmemMax = 232448 - 1024;
// two CTAs per SM: 228 KB of shared memory per SM, less 1 KB reserved per CTA and the static shared memory
constexpr size_t kStepSmemMax2 = 233472 / 2 - 2048;

static size_t tile_smem(const NceDev &m) {
    return SmemPlan::make(m, false).tile_end;
}

static size_t step_smem(const NceDev &m, bool w_smem) {
    const SmemPlan p = SmemPlan::make(m);
    return w_smem ? p.total_w : p.w;
}

static int ensure_scratch(nce_nce_model *h, int32_t R) {
    if (h->R_alloc >= R) return NCE_OK;
    for (void *p : {(void *)h->slot, (void *)h->list, (void *)h->newbuf, (void *)h->e_new, (void *)h->pend}) if (p) cudaFree(p);
    h->slot = h->list = nullptr; h->newbuf = h->e_new = nullptr; h->pend = nullptr; h->R_alloc = 0;
    const NceDev &m = h->dev;
    h->stride = (int64_t)l0_floats(m) + (int64_t)std::max(0, m.depth - 1) * m.nmax * m.D;
    NCE_CUDA(cudaMalloc((void **)&h->slot, sizeof(int32_t) * (size_t)R * m.N));
    NCE_CUDA(cudaMemset(h->slot, 0xFF, sizeof(int32_t) * (size_t)R * m.N));
    NCE_CUDA(cudaMalloc((void **)&h->list, sizeof(int32_t) * (size_t)R * m.nmax));
    NCE_CUDA(cudaMalloc((void **)&h->newbuf, sizeof(float) * (size_t)R * std::max<int64_t>(h->stride, 1)));
    NCE_CUDA(cudaMalloc((void **)&h->e_new, sizeof(float) * (size_t)R * m.nmax));
    NCE_CUDA(cudaMalloc((void **)&h->pend, sizeof(NcePending) * (size_t)R));
    NCE_CUDA(cudaMemset(h->pend, 0, sizeof(NcePending) * (size_t)R));
    h->R_alloc = R;
    return NCE_OK;
}

static NceJob make_nce_job(nce_nce_model *h, const nce_nce_state *st);

// the step kernels of one chunk: one CTA per replica, or a thread-block cluster of CL CTAs per replica
static int launch_steps(nce_nce_model *h, const NceJob &jb, int cluster, int ctas_per_sm, cudaStream_t stream) {
    const int per_sm = ctas_per_sm > 1 ? ctas_per_sm : 1;
    NCE_CHECK(per_sm <= 2, "nce_nce_run_chunk: ctas_per_sm must be 1 or 2");
    const size_t lim = per_sm == 2 ? kStepSmemMax2 : kStepSmemMax;
    const bool w_smem = step_smem(h->dev, true) <= lim;
    const size_t sm = step_smem(h->dev, w_smem);
    NCE_CHECK(sm <= lim, "nce_nce_run_chunk: %zu bytes of shared memory per CTA do not fit %d CTAs per SM", sm, per_sm);
    const int CL = cluster > 1 ? cluster : 1;
    NCE_CHECK(CL == 1 || CL == 2 || CL == 4 || CL == 8, "nce_nce_run_chunk: cluster must be 1, 2, 4 or 8");
    if (CL == 1 || h->dev.depth == 0) {
        auto kern = per_sm == 2 ? nce_chunk_kernel<2> : nce_chunk_kernel<1>;
        NCE_CUDA(::nce::raise_smem_limit((const void *)kern, sm));
        kern<<<jb.R, 256, sm, stream>>>(jb, w_smem ? 1 : 0);
    } else {
        auto kern = per_sm == 2 ? nce_chunk_cluster_kernel<2> : nce_chunk_cluster_kernel<1>;
        NCE_CUDA(::nce::raise_smem_limit((const void *)kern, sm));
        cudaLaunchConfig_t cfg; std::memset(&cfg, 0, sizeof(cfg));
        cfg.gridDim = dim3((unsigned)(jb.R * CL)); cfg.blockDim = dim3(256); cfg.dynamicSmemBytes = sm;
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)CL; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr; cfg.numAttrs = 1;
        NCE_CUDA(cudaLaunchKernelEx(&cfg, kern, jb, (int32_t)(w_smem ? 1 : 0)));
    }
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

static NceJob make_nce_job(nce_nce_model *h, const nce_nce_state *st) {
    NceJob j; std::memset(&j, 0, sizeof(j));
    j.m = h->dev;
    j.sigma = st->sigma; j.h0 = st->h0; j.hmid = st->hmid; j.e = st->e; j.E = st->E; j.beta_slot = st->beta_slot;
    j.slot_of_rep = st->slot_of_rep; j.n_acc = st->n_acc; j.R = st->R;
    j.slot = h->slot; j.list = h->list; j.newbuf = h->newbuf; j.e_new = h->e_new; j.scratch_stride = h->stride; j.pend = h->pend;
    j.err = h->err; j.sample_interval = 1;
    return j;
}

}  // namespace nce

using namespace nce;

namespace nce {
int nce_model_dims(nce_nce_handle h, int64_t *N, int32_t *C0, int32_t *D, int32_t *depth) {
    NCE_CHECK(h, "null NCE handle");
    *N = h->dev.N; *C0 = h->dev.C0; *D = h->dev.D; *depth = h->dev.depth;
    return NCE_OK;
}
// ── tensor-core tile GEMM (tcgen05) ────────────────────────────────────────────────────────────
// C[M x N] = A[M x K] B[K x N] (float32, row-major) on the tile path of the NeuralCE layers: one CTA of 4 warps
// per 128 rows stages A and B^T as bf16 (hi, and lo = bf16(x - hi) when split) in the core-matrix layout, one
// thread issues the MMAs into tensor memory, every warp reads its 32-lane quarter back.
__global__ void __launch_bounds__(128) nce_tc_gemm_kernel(const float *A, const float *B, float *C, int32_t N, int32_t K,
                                                          int32_t Kp, int32_t split, int32_t *err) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t row0 = (int64_t)blockIdx.x * 128;
    const size_t abytes = (size_t)128 * Kp * 2, bbytes = (size_t)N * Kp * 2;
    uint8_t *A0 = smem, *A1 = smem + abytes, *B0 = smem + (split ? 2 : 1) * abytes, *B1 = B0 + bbytes;
    auto put = [&](uint8_t *hi, uint8_t *lo, uint32_t off, float v) {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        *reinterpret_cast<__nv_bfloat16 *>(hi + off) = h;
        if (split) *reinterpret_cast<__nv_bfloat16 *>(lo + off) = __float2bfloat16_rn(v - __bfloat162float(h));
    };
    for (int idx = tid; idx < 128 * Kp; idx += blockDim.x) {
        const int r = idx / Kp, k = idx % Kp;
        put(A0, A1, umma::core_off(r, k, Kp), k < K ? A[(row0 + r) * K + k] : 0.f);
    }
    for (int idx = tid; idx < N * Kp; idx += blockDim.x) {
        const int n = idx / Kp, k = idx % Kp;
        put(B0, B1, umma::core_off(n, k, Kp), k < K ? B[(size_t)k * N + n] : 0.f);
    }
    umma::fence_async_smem();
    if (warp == 0) umma::tmem_alloc(&tslot, umma::tmem_cols(N));
    if (tid == 0) umma::mbar_init(&mbar, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    if (tid == 0) umma::issue_tile(tmem, A0, A1, B0, B1, N, Kp, split ? 3 : 1, &mbar);
    const bool done = umma::mbar_wait(&mbar, 0);
    if (__syncthreads_or(!done)) {                           // gave up: drain (bounded), free, report; no loads
        if (tid == 0) atomicOr(err, 1);
        umma::mbar_wait(&mbar, 0);
        umma::fence_before();
        __syncthreads();
        if (warp == 0) umma::tmem_free(tmem, umma::tmem_cols(N));
        return;
    }
    umma::fence_after();
    const int64_t row = row0 + warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) C[row * N + c0 + i] = v[i];
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, umma::tmem_cols(N));
}

}  // namespace nce

namespace nce {
// A tensor-core completion wait that runs out on purpose: tensor memory and the mbarrier are set up as in the layer
// tiles, no MMA is issued, so nothing ever arrives; the bounded wait gives up after `limit` polls and the kernel
// takes the same way out as a layer tile (flag 32 in the model's error word, bounded drain, tensor memory freed).
__global__ void __launch_bounds__(128) nce_tc_wait_selftest_kernel(int32_t *err, uint32_t limit) {
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t slot;
    TcCtx tc;
    tc_begin(32, tc, nullptr, &mbar, &slot);
    tc_wait(tc, err, limit);                                // nothing was issued: gives up, sets flag 32 and `failed`
    tc_end(32, tc, limit);
}

int nce_error_peek(nce_nce_handle h, int32_t *flags) {
    NCE_CHECK(h && flags, "nce_error_peek: null argument");
    NCE_CUDA(cudaMemcpy(flags, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return NCE_OK;
}
const char *nce_error_text(int32_t f) {
    if (f & 32) return "a tensor-core completion wait timed out";
    if (f & 8) return "a row member was outside the layer-0 ball";
    if (f & 4) return "a receptive field exceeded its tables";
    if (f & 1) return "a proposal index was out of range";
    return "no error";
}
}  // namespace nce

extern "C" {

int nce_tc_gemm(const float *A, const float *B, float *C, int32_t M, int32_t N, int32_t K, int32_t split, void *stream) {
    NCE_CHECK(A && B && C, "nce_tc_gemm: null argument");
    NCE_CHECK(M > 0 && M % 128 == 0, "nce_tc_gemm: M must be a positive multiple of 128");
    NCE_CHECK(N >= 16 && N <= 256 && N % 16 == 0, "nce_tc_gemm: N must be a multiple of 16 in [16, 256]");
    const int32_t Kp = (K + 15) / 16 * 16;
    NCE_CHECK(K >= 1 && Kp <= 256, "nce_tc_gemm: K must be in [1, 256]");
    const size_t sm = (size_t)(split ? 2 : 1) * ((size_t)128 * Kp * 2 + (size_t)N * Kp * 2);
    NCE_CHECK(sm <= 200 * 1024, "nce_tc_gemm: tiles of %zu bytes exceed shared memory", sm);
    cudaStream_t s = (cudaStream_t)stream;
    int32_t *err = nullptr;
    NCE_CUDA(cudaMallocAsync((void **)&err, sizeof(int32_t), s));
    NCE_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
    NCE_CUDA(::nce::raise_smem_limit((const void *)nce_tc_gemm_kernel, sm));
    nce_tc_gemm_kernel<<<M / 128, 128, sm, s>>>(A, B, C, N, K, Kp, split ? 1 : 0, err);
    NCE_CUDA(cudaGetLastError());
    int32_t h = 0;
    NCE_CUDA(cudaMemcpyAsync(&h, err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    NCE_CUDA(cudaStreamSynchronize(s));
    cudaFreeAsync(err, s);
    NCE_CHECK(h == 0, "nce_tc_gemm: tensor-core completion wait timed out");
    return NCE_OK;
}

int nce_nce_create(const nce_nce_desc *d, nce_nce_handle *out) {
    NCE_CHECK(d && out, "nce_nce_create: null argument");
    NCE_CHECK(d->depth >= 0 && d->depth <= kMaxLayers, "nce_nce_create: depth must be 0..%d", kMaxLayers);
    NCE_CHECK(d->C0 >= 1 && d->C0 <= 64, "nce_nce_create: layer-0 channels must be 1..64");
    NCE_CHECK(d->depth == 0 || d->D == 16 || d->D == 32 || d->D == 64 || d->D == 128, "nce_nce_create: width must be 16, 32, 64 or 128");
    NCE_CHECK(d->mo >= 1 && d->mo <= 8 && d->P >= 1 && d->P <= 8 && d->W >= 1, "nce_nce_create: mo/P/W out of range");
    NCE_CHECK(d->nB >= 1 && d->J >= 1 && d->n_cells == d->d[0] * d->d[1] * d->d[2] && d->n_cells <= 0xFFFFFFFFll,
              "nce_nce_create: bad lattice");
    NCE_CHECK(d->act == 0 || d->act == 1, "nce_nce_create: act must be 0 (tanh) or 1 (silu)");
    NCE_CHECK(d->norm > 0.0, "nce_nce_create: norm must be > 0");
    NCE_CHECK(d->mma >= 0 && d->mma <= 4, "nce_nce_create: mma must be 0, 1, 2, 3 or 4");
    NCE_CHECK(d->mma == 0 || !d->gate, "nce_nce_create: the tensor-core forms need an ungated model");
    const int64_t N = d->n_cells * d->nB;
    NCE_CHECK(N < (1ll << 31) - 1, "nce_nce_create: more than 2^31 sites");
    NCE_CHECK(d->n_groups >= 1 && d->max_gb >= 1 && d->act_b && d->act_nb && d->grp_cum, "nce_nce_create: no swap group");
    for (int g = 0; g < d->n_groups; ++g) {
        NCE_CHECK(d->act_nb[g] >= 1 && d->act_nb[g] <= d->max_gb, "nce_nce_create: act_nb out of range");
        for (int q = 0; q < d->act_nb[g]; ++q)
            NCE_CHECK(d->act_b[g * d->max_gb + q] >= 0 && d->act_b[g * d->max_gb + q] < d->nB, "nce_nce_create: act_b out of range");
    }
    NCE_CHECK(d->maxM >= 1 && d->maxP >= 1, "nce_nce_create: maxM/maxP must be >= 1");
    for (int b = 0; b < d->nB; ++b) NCE_CHECK(d->Mb[b] >= 1 && d->Mb[b] <= d->maxM, "nce_nce_create: Mb out of range");
    // host-side range checks of every table index
    const size_t nr = (size_t)d->nB * d->J * d->mo;
    for (size_t i = 0; i < nr; ++i) {
        NCE_CHECK(d->Rv_b[i] >= 0 && d->Rv_b[i] < d->nB && d->Rv_p[i] >= 0 && d->Rv_p[i] < d->maxP, "nce_nce_create: Rv_b/Rv_p out of range");
        NCE_CHECK(d->Mb[d->Rv_b[i]] >= 1 && d->Mb[d->Rv_b[i]] <= d->maxM, "nce_nce_create: Mb out of range");
        for (int c = 0; c < 3; ++c) NCE_CHECK(d->Rv_uo[3 * i + c] >= 0 && d->Rv_uo[3 * i + c] < d->d[c], "nce_nce_create: Rv_uo out of [0,d)");
    }
    for (size_t i = 0; i < (size_t)d->nB * d->J; ++i)
        NCE_CHECK(d->Rv_col[i] >= 0 && d->Rv_col[i] + 1 < d->C0, "nce_nce_create: Rv_col out of range");
    const size_t ns = (size_t)d->nB * d->P * d->W;
    for (size_t i = 0; i < ns; ++i) {
        NCE_CHECK(d->Sh_b[i] >= 0 && d->Sh_b[i] < d->nB, "nce_nce_create: Sh_b out of range");
        for (int c = 0; c < 3; ++c) NCE_CHECK(d->Sh_uo[3 * i + c] >= 0 && d->Sh_uo[3 * i + c] < d->d[c], "nce_nce_create: Sh_uo out of [0,d)");
    }
    const size_t nbl = (size_t)d->nB * d->wL;
    for (size_t i = 0; i < nbl; ++i) {
        NCE_CHECK(d->ball_b[i] >= 0 && d->ball_b[i] < d->nB, "nce_nce_create: ball_b out of range");
        for (int c = 0; c < 3; ++c) NCE_CHECK(d->ball_uo[3 * i + c] >= 0 && d->ball_uo[3 * i + c] < d->d[c], "nce_nce_create: ball_uo out of [0,d)");
    }
    int n0max = 0, nLmax = 0;
    for (int b = 0; b < d->nB; ++b) {
        for (int l = 0; l <= d->depth; ++l) {
            const int e1 = d->ball_end[b * (d->depth + 1) + l], e0 = l ? d->ball_end[b * (d->depth + 1) + l - 1] : 0;
            NCE_CHECK(e0 <= e1 && e1 <= d->wL, "nce_nce_create: ball_end not monotone within [0, wL]");
        }
        n0max = std::max(n0max, d->ball_end[b * (d->depth + 1)]);
        nLmax = std::max(nLmax, d->ball_end[b * (d->depth + 1) + d->depth]);
    }
    nce_nce_model *h = new nce_nce_model();
    NceDev &m = h->dev;
    std::memset(&m, 0, sizeof(m));
    m.nB = d->nB; m.J = d->J; m.mo = d->mo; m.P = d->P; m.W = d->W; m.depth = d->depth; m.C0 = d->C0; m.D = d->D;
    m.maxM = d->maxM; m.maxP = d->maxP; m.d0 = (int32_t)d->d[0]; m.d1 = (int32_t)d->d[1]; m.d2 = (int32_t)d->d[2];
    m.N = N; m.n_cells = d->n_cells; m.wL = d->wL; m.act = d->act; m.gate = d->gate; m.norm = d->norm; m.scale_eV = d->scale_eV;
    m.mma = d->mma;
    m.tc = (d->mma == 2 || d->mma == 4) && d->depth > 0 ? 1 : 0;
    m.tc_split = d->mma == 4 ? 1 : 0;
    m.tc_ks = kpad16(tile_kin(d->P, d->C0, d->D));     // the whole K extent of the widest layer in one A tile
    m.head_b = (float)d->head_b;
    m.n0max = 2 * n0max; m.nmax = 2 * nLmax; m.w0max = n0max;
    NCE_CHECK(d->Rv_loc, "nce_nce_create: Rv_loc required");
    for (size_t i = 0; i < nr; ++i)
        if (d->Rv_m[i]) {
            const int b = (int)(i / ((size_t)d->J * d->mo));
            NCE_CHECK(d->Rv_loc[i] < d->ball_end[b * (d->depth + 1)], "nce_nce_create: Rv_loc outside ball 0");
        }
    int rc = NCE_OK;
    auto chk = [&](int x) { if (!rc) rc = x; };
    chk(dup(h, d->Rv_b, nr, m.Rv_b)); chk(dup(h, d->Rv_uo, nr * 3, m.Rv_uo)); chk(dup(h, d->Rv_p, nr, m.Rv_p));
    chk(dup(h, d->Rv_m, nr, m.Rv_m)); chk(dup(h, d->Rv_loc, nr, m.Rv_loc)); chk(dup(h, d->Rv_col, (size_t)d->nB * d->J, m.Rv_col)); chk(dup(h, d->Rv_w, (size_t)d->nB * d->J, m.Rv_w));
    chk(dup(h, d->Mb, (size_t)d->nB, m.Mb)); chk(dup(h, d->theta, (size_t)(d->maxM + 1) * d->maxP * d->maxM, m.theta));
    {
        const std::vector<float> z((size_t)kZeroRow, 0.f);
        chk(dup(h, z.data(), z.size(), m.zrow));
    }
    {
        // +-1 point functions on every (M, p, species) a row can use -> exact integer layer-0 changes
        const size_t nth = (size_t)(d->maxM + 1) * d->maxP * d->maxM;
        std::vector<uint8_t> ts(nth, 0);
        bool bin = true;
        for (size_t i = 0; i < nr && bin; ++i) {
            if (!d->Rv_m[i]) continue;
            const int M = d->Mb[d->Rv_b[i]], pi = d->Rv_p[i];
            for (int sp = 0; sp < M; ++sp) {
                const double v = d->theta[((size_t)M * d->maxP + pi) * d->maxM + sp];
                if (v == 1.0) ts[((size_t)M * d->maxP + pi) * d->maxM + sp] = 0;
                else if (v == -1.0) ts[((size_t)M * d->maxP + pi) * d->maxM + sp] = 1;
                else { bin = false; break; }
            }
        }
        bin = bin && d->maxM <= 4;
        for (int b = 0; b < d->nB; ++b)
            for (int q = 0; q < d->ball_end[b * (d->depth + 1)]; ++q) bin = bin && q < 0x10000;
        m.l0bin = bin ? 1 : 0;
        if (bin) {
            std::vector<long long> wf((size_t)d->nB * d->J);
            for (size_t i = 0; i < wf.size(); ++i) wf[i] = llrint(2.0 * d->Rv_w[i] * kFix);
            std::vector<long long> cw((size_t)d->C0, 0);
            std::vector<char> cseen((size_t)d->C0, 0);
            for (size_t i = 0; i < wf.size() && bin; ++i) {
                if (wf[i] == 0) continue;
                const int ch = d->Rv_col[i] + 1;
                if (ch < 0 || ch >= d->C0) { bin = false; break; }
                if (!cseen[ch]) { cseen[ch] = 1; cw[ch] = wf[i]; }
                else if (cw[ch] != wf[i]) bin = false;
            }
            m.l0bin = bin ? 1 : 0;
            std::vector<int32_t> dsc(nr, 0);
            for (size_t i = 0; i < nr; ++i) {
                if (!d->Rv_m[i]) continue;
                const int M = d->Mb[d->Rv_b[i]], pi = d->Rv_p[i];
                int32_t v = (int32_t)d->Rv_loc[i] | (1 << 16);
                for (int sp = 0; sp < M; ++sp) v |= (int32_t)ts[((size_t)M * d->maxP + pi) * d->maxM + sp] << (20 + sp);
                dsc[i] = v;
            }
            chk(dup(h, wf.data(), wf.size(), m.Rv_wfix)); chk(dup(h, ts.data(), ts.size(), m.thsign));
            chk(dup(h, dsc.data(), dsc.size(), m.Rv_desc));
            chk(dup(h, cw.data(), cw.size(), m.col_wfix));
            // bit-sliced layer 0: every member on point function 0, rows of a basis sorted by channel, at most 8191
            // rows per channel (13-bit counters), channel weights w
            bool hb = m.l0bin != 0 && d->C0 >= 2;
            std::vector<int4> hm(nr, make_int4(-1, 0, 0, 0));
            std::vector<double> cwd((size_t)d->C0, 0.0);
            for (int b = 0; b < d->nB && hb; ++b) {
                int last = 0, run = 0;
                for (int j = 0; j < d->J && hb; ++j) {
                    const size_t e = (size_t)b * d->J + j;
                    if (wf[e] == 0) continue;
                    const int ch = d->Rv_col[e] + 1;
                    if (ch < last) hb = false;
                    run = ch == last ? run + 1 : 1; last = ch;
                    if (run > 8191) hb = false;
                    cwd[ch] = d->Rv_w[e];
                    for (int k = 0; k < d->mo; ++k) {
                        const size_t i = e * d->mo + k;
                        if (!d->Rv_m[i]) continue;
                        if (d->Rv_p[i] != 0) hb = false;
                        hm[i] = make_int4(d->Rv_b[i], d->Rv_uo[3 * i], d->Rv_uo[3 * i + 1], d->Rv_uo[3 * i + 2]);
                    }
                }
            }
            if (hb) {
                chk(dup(h, hm.data(), hm.size(), m.h0mem)); chk(dup(h, cwd.data(), cwd.size(), m.col_w));
                // slices of each basis's rows, cut where the channel changes, about equal in rows
                const int S = 8;
                std::vector<int2> sl((size_t)d->nB * (S + 1));
                for (int b = 0; b < d->nB; ++b) {
                    std::vector<int> start_row, start_ch;            // candidate cuts: first row of each channel run
                    int nrows = 0, last = -1;
                    for (int j = 0; j < d->J; ++j) {
                        const size_t e = (size_t)b * d->J + j;
                        if (wf[e] == 0) continue;
                        const int ch = d->Rv_col[e] + 1;
                        if (ch != last) { start_row.push_back(j); start_ch.push_back(ch); last = ch; }
                        ++nrows;
                    }
                    int2 *o = &sl[(size_t)b * (S + 1)];
                    o[0] = make_int2(0, 1);
                    int k = 1, seen = 0, ci = 0;
                    for (int j = 0; j < d->J && k < S; ++j) {
                        const size_t e = (size_t)b * d->J + j;
                        if (wf[e] == 0) continue;
                        while (ci < (int)start_row.size() && start_row[ci] < j) ++ci;
                        if (ci < (int)start_row.size() && start_row[ci] == j && j > 0 && seen >= (int64_t)k * nrows / S &&
                            start_ch[ci] > o[k - 1].y)
                            o[k++] = make_int2(j, start_ch[ci]);
                        ++seen;
                    }
                    for (; k <= S; ++k) o[k] = make_int2(d->J, d->C0);      // empty trailing slices
                    o[S] = make_int2(d->J, d->C0);
                }
                chk(dup(h, sl.data(), sl.size(), m.h0_slice));
                m.h0_slices = S;
                m.h0bits = 1;
            }
        }
    }
    chk(dup(h, d->Sh_b, ns, m.Sh_b)); chk(dup(h, d->Sh_uo, ns * 3, m.Sh_uo)); chk(dup(h, d->Sh_m, ns, m.Sh_m));
    chk(dup(h, d->Sh_inv, (size_t)d->nB * d->P, m.Sh_inv));
    chk(dup(h, d->ball_b, nbl, m.ball_b)); chk(dup(h, d->ball_uo, nbl * 3, m.ball_uo));
    chk(dup(h, d->ball_end, (size_t)d->nB * (d->depth + 1), m.ball_end));
    chk(dup(h, d->lin, (size_t)d->C0, m.lin)); chk(dup(h, d->head_w, (size_t)std::max(d->D, 1), m.head_w));
    chk(dup(h, d->mu, (size_t)d->C0, m.mu)); chk(dup(h, d->sd, (size_t)d->C0, m.sd));
    m.n_groups = d->n_groups; m.max_gb = d->max_gb;
    chk(dup(h, d->act_b, (size_t)d->n_groups * d->max_gb, m.act_b)); chk(dup(h, d->act_nb, (size_t)d->n_groups, m.act_nb));
    chk(dup(h, d->grp_cum, (size_t)d->n_groups, m.grp_cum));
    for (int l = 0; l < d->depth; ++l) {
        const int Cin = l == 0 ? d->C0 : d->D;
        chk(dup(h, d->W_cat[l], (size_t)(1 + d->P) * Cin * d->D, m.Wc[l]));
        chk(dup(h, d->bias[l], (size_t)d->D, m.bias[l]));
        if (d->gate) { chk(dup(h, d->G_cat[l], (size_t)d->P * Cin * d->D, m.G[l])); chk(dup(h, d->gate_b[l], (size_t)d->D, m.gb[l])); }
        if (m.tc) {
            // B operand of the tcgen05 tiles: B[n][k] = W[k][n] in bf16 core-matrix layout, hi then lo (split)
            const int Kin = (1 + d->P) * Cin, Kp = kpad16(Kin);
            const size_t half = (size_t)Kp * d->D * 2;
            std::vector<uint8_t> wt(half * (m.tc_split ? 2 : 1), 0);
            for (int n = 0; n < d->D; ++n)
                for (int k = 0; k < Kin; ++k) {
                    const float v = d->W_cat[l][(size_t)k * d->D + n];
                    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
                    const uint32_t off = umma::core_off(n, k, Kp);
                    std::memcpy(&wt[off], &hi, 2);
                    if (m.tc_split) {
                        const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
                        std::memcpy(&wt[half + off], &lo, 2);
                    }
                }
            chk(dup(h, wt.data(), wt.size(), m.Wt[l]));
        }
    }
    if (!rc) {
        cudaError_t e = cudaMalloc((void **)&h->err, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMemset(h->err, 0, sizeof(int32_t));
        if (e != cudaSuccess) rc = fail(NCE_ERR_CUDA, "nce_nce_create: %s", cudaGetErrorString(e));
    }
    if (!rc && m.tc && step_smem(m, false) > kStepSmemMax) {
        // the whole A operand does not fit next to the B operand: stage A in two K slices of every layer whose K
        // extent divides into them (widths 128 split: self channels, then shell means)
        const int kp_max = kpad16(tile_kin(m.P, m.C0, m.D)), ks = kp_max / 2;
        bool ok = kp_max % 32 == 0;
        for (int l = 0; l < m.depth && ok; ++l) {
            const int kp = kpad16((1 + m.P) * (l == 0 ? m.C0 : m.D));
            ok = kp <= ks || kp % ks == 0;
        }
        if (ok) m.tc_ks = ks;
    }
    if (!rc && step_smem(m, false) > kStepSmemMax)
        rc = fail(NCE_ERR_UNSUPPORTED, "nce_nce_create: receptive field%s too large for shared memory (%zu bytes)",
                  m.tc ? " and tensor-core tiles" : "", step_smem(m, false));
    if (rc) {
        for (void *p : h->allocs) cudaFree(p);
        delete h;
        return rc;
    }
    *out = h;
    return NCE_OK;
}

int nce_nce_destroy(nce_nce_handle h) {
    if (!h) return NCE_OK;
    cudaDeviceSynchronize();
    for (void *p : h->allocs) cudaFree(p);
    for (void *p : {(void *)h->slot, (void *)h->list, (void *)h->newbuf, (void *)h->e_new, (void *)h->err, (void *)h->pend})
        if (p) cudaFree(p);
    delete h;
    return NCE_OK;
}

int nce_nce_full_cache(nce_nce_handle h, const nce_nce_state *st, void *stream) {
    NCE_CHECK(h && st && st->sigma && st->h0 && st->e && st->E && st->R >= 1, "nce_nce_full_cache: bad argument");
    NCE_CHECK(st->N == h->dev.N, "nce_nce_full_cache: N mismatch");
    NCE_CHECK(h->dev.depth < 2 || st->hmid, "nce_nce_full_cache: hmid required for depth >= 2");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaStream_t s = (cudaStream_t)stream;
    const NceDev &m = h->dev;
    const int64_t tot = (int64_t)st->R * m.N;
    if (m.h0bits && st->R <= 65535) {
        const int32_t W2 = (2 * m.d2 + 31) / 32 + 1;
        StreamScratch planes;
        NCE_CUDA(planes.alloc(sizeof(uint32_t) * (size_t)st->R * m.nB * m.d0 * m.d1 * W2, s));
        const int64_t prow = (int64_t)st->R * m.nB * m.d0 * m.d1;
        nce_plane_kernel<<<(int)std::min<int64_t>((prow + 7) / 8, 1 << 20), 256, 0, s>>>(m, st->sigma, st->R, W2, (uint32_t *)planes.p);
        NCE_CUDA(cudaGetLastError());
        const int64_t items = (int64_t)m.d0 * m.d1 * ((m.d2 + 31) / 32);
        nce_h0_bits_kernel<<<dim3((unsigned)((items + 127) / 128), m.nB * m.h0_slices, st->R), 128, 0, s>>>(
            m, (const uint32_t *)planes.p, W2, st->h0);
    } else {
        nce_h0_kernel<<<(int)std::min<int64_t>((tot + 127) / 128, 65535), 128, 0, s>>>(m, st->sigma, st->R, st->h0);
    }
    NCE_CUDA(cudaGetLastError());
    NceJob jb = make_nce_job(h, st);
    const size_t xs = tile_smem(m);
    NCE_CUDA(::nce::raise_smem_limit((const void *)nce_layer_all_kernel, xs));
    const int blocks = (int)std::min<int64_t>((m.N + tile_tm(m.D, m.tc, m.mma) - 1) / tile_tm(m.D, m.tc, m.mma), 1216);
    if (m.depth == 0) {
        nce_e0_kernel<<<(int)std::min<int64_t>((tot + 255) / 256, 65535), 256, 0, s>>>(m, st->h0, tot, st->e);
        NCE_CUDA(cudaGetLastError());
    }
    // hidden layers: hmid[l-1] for l = 1..depth-1, then the last layer into e
    for (int32_t r = 0; r < st->R && m.depth > 0; ++r) {
        for (int l = 0; l < m.depth; ++l) {
            const float *in = l == 0 ? st->h0 + (size_t)r * m.N * m.C0 : st->hmid + ((size_t)(l - 1) * st->R + r) * m.N * m.D;
            if (l + 1 < m.depth) {
                float *outp = st->hmid + ((size_t)l * st->R + r) * m.N * m.D;
                nce_layer_all_kernel<<<blocks, 256, xs, s>>>(jb, l, r, in, outp, nullptr, 0, m.N);
            } else {
                nce_layer_all_kernel<<<blocks, 256, xs, s>>>(jb, l, r, in, nullptr, st->e + (size_t)r * m.N, 0, m.N);
            }
            NCE_CUDA(cudaGetLastError());
        }
    }
    StreamScratch eacc;
    NCE_CUDA(eacc.alloc(sizeof(unsigned long long) * st->R, s));
    NCE_CUDA(cudaMemsetAsync(eacc.p, 0, sizeof(unsigned long long) * st->R, s));
    dim3 g((unsigned)std::min<int64_t>((m.N + 255) / 256, 1024), st->R);
    nce_energy_kernel<<<g, 256, 0, s>>>(m, st->e, st->R, st->E, (unsigned long long *)eacc.p);
    NCE_CUDA(cudaGetLastError());
    nce_energy_finish<<<(st->R + 127) / 128, 128, 0, s>>>(m, (const unsigned long long *)eacc.p, st->R, st->E);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

int nce_nce_run_chunk(nce_nce_handle h, const nce_nce_state *st, const nce_nce_chunk *ck, void *stream) {
    NCE_CHECK(h && st && ck, "nce_nce_run_chunk: null argument");
    NCE_CHECK(st->N == h->dev.N && st->R >= 1, "nce_nce_run_chunk: state size mismatch");
    NCE_CHECK(st->sigma && st->h0 && st->e && st->E && st->beta_slot && st->slot_of_rep && st->n_acc, "nce_nce_run_chunk: null state pointer");
    NCE_CHECK(h->dev.depth < 2 || st->hmid, "nce_nce_run_chunk: hmid required for depth >= 2");
    NCE_CHECK((ck->prop_a == nullptr) == (ck->prop_b == nullptr) && (ck->prop_a == nullptr) == (ck->prop_u == nullptr),
              "nce_nce_run_chunk: prop_a/prop_b/prop_u must be all set or all NULL");
    NCE_CHECK(!ck->E_samples || ck->sample_interval > 0, "nce_nce_run_chunk: sample_interval must be > 0");
    NCE_CHECK(ck->n_steps >= 0 && ck->force >= -1 && ck->force <= 1, "nce_nce_run_chunk: bad n_steps/force");
    std::lock_guard<std::mutex> lk(h->mu);
    int rc = ensure_scratch(h, st->R); if (rc) return rc;
    NceJob jb = make_nce_job(h, st);
    jb.n_steps = ck->n_steps; jb.step0 = ck->step0; jb.prop_a = ck->prop_a; jb.prop_b = ck->prop_b; jb.prop_u = ck->prop_u;
    jb.seed = ck->seed; jb.sample_interval = ck->sample_interval > 0 ? ck->sample_interval : 1; jb.E_samples = ck->E_samples;
    jb.dE_out = ck->dE_out; jb.force = ck->force;
    NCE_CHECK(ck->near_eV >= 0.0, "nce_nce_run_chunk: near_eV must be >= 0");
    jb.n_near = st->n_near;
    jb.near_eV = ck->near_eV > 0.0 ? ck->near_eV : ((h->dev.mma == 1 || h->dev.mma == 2) ? 1e-2 : 1e-4);
    if (ck->n_steps == 0) return NCE_OK;
    rc = launch_steps(h, jb, ck->cluster, ck->ctas_per_sm, (cudaStream_t)stream);
    if (rc) return rc;
    if (ck->exchange_rounds > 0 && st->R > 1) {
        NCE_CHECK(st->rep_of_slot && st->ladder_id && st->n_ex, "nce_nce_run_chunk: exchange needs rep_of_slot/ladder_id/n_ex");
        rc = launch_exchange(st->R, st->E, h->dev.scale_eV, st->beta_slot, st->rep_of_slot, st->slot_of_rep, st->ladder_id,
                             st->n_ex, ck->seed, ck->step0 + ck->n_steps, ck->ex_parity, ck->ex_u, ck->exchange_rounds,
                             (cudaStream_t)stream);
        if (rc) return rc;
    }
    return NCE_OK;
}

int nce_nce_local_delta(nce_nce_handle h, const nce_nce_state *st, const int32_t *prop_a, const int32_t *prop_b, double *dE_out,
                        void *stream) {
    NCE_CHECK(h && st && prop_a && prop_b && dE_out, "nce_nce_local_delta: null argument");
    NCE_CHECK(st->N == h->dev.N && st->R >= 1, "nce_nce_local_delta: state size mismatch");
    NCE_CHECK(st->sigma && st->h0 && st->e && st->E && st->beta_slot && st->slot_of_rep && st->n_acc,
              "nce_nce_local_delta: null state pointer");
    NCE_CHECK(h->dev.depth < 2 || st->hmid, "nce_nce_local_delta: hmid required for depth >= 2");
    std::lock_guard<std::mutex> lk(h->mu);
    int rc = ensure_scratch(h, st->R); if (rc) return rc;
    NceJob jb = make_nce_job(h, st);
    jb.n_steps = 1; jb.step0 = 0; jb.prop_a = prop_a; jb.prop_b = prop_b; jb.prop_u = nullptr;
    jb.dE_out = dE_out; jb.force = -2; jb.rep_index = 1; jb.near_eV = 0.0;
    return launch_steps(h, jb, 1, 1, (cudaStream_t)stream);
}

int nce_nce_commit(nce_nce_handle h, const nce_nce_state *st, const int32_t *accept, void *stream) {
    NCE_CHECK(h && st && accept, "nce_nce_commit: null argument");
    NCE_CHECK(st->N == h->dev.N && st->R >= 1, "nce_nce_commit: state size mismatch");
    NCE_CHECK(st->sigma && st->h0 && st->e && st->E && st->n_acc, "nce_nce_commit: null state pointer");
    NCE_CHECK(h->dev.depth < 2 || st->hmid, "nce_nce_commit: hmid required for depth >= 2");
    std::lock_guard<std::mutex> lk(h->mu);
    NCE_CHECK(h->R_alloc >= st->R && h->pend, "nce_nce_commit: no swap was evaluated on this model (nce_nce_local_delta)");
    NceJob jb = make_nce_job(h, st);
    nce_commit_kernel<<<st->R, 256, 0, (cudaStream_t)stream>>>(jb, accept);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

int nce_nce_accept(const double *dE, int32_t n_models, int32_t R, double scale_eV, const float *beta_slot,
                   const int32_t *slot_of_rep, const double *u, int32_t *accept, void *stream) {
    NCE_CHECK(dE && beta_slot && slot_of_rep && u && accept && n_models >= 1 && R >= 1, "nce_nce_accept: bad argument");
    nce_accept_kernel<<<(R + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dE, n_models, R, scale_eV, beta_slot, slot_of_rep, u,
                                                                         accept);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

int nce_nce_tc_wait_selftest(nce_nce_handle h, int32_t limit, void *stream) {
    NCE_CHECK(h && limit >= 1, "nce_nce_tc_wait_selftest: bad argument");
    nce_tc_wait_selftest_kernel<<<1, 128, 0, (cudaStream_t)stream>>>(h->err, (uint32_t)limit);
    NCE_CUDA(cudaGetLastError());
    return NCE_OK;
}

int nce_nce_errors(nce_nce_handle h, int32_t *flags) {
    NCE_CHECK(h && flags, "nce_nce_errors: null argument");
    NCE_CUDA(cudaMemcpy(flags, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    NCE_CUDA(cudaMemset(h->err, 0, sizeof(int32_t)));
    return NCE_OK;
}

}  // extern "C"
