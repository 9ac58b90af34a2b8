// pairhmm.cu -- batched 2D pair-HMM forward / backward / E-step for GB300
// (sm_103a), behind the C ABI declared in include/pairhmm.h.
//
// Algorithm (the reference's, evoldoers/tkf-mixdom python/tkfmixdom/jax/
// dp/hmm.py:1120-1973): forward F[i,j,k] = e[i,j,k] sum_s F[pred_k(i,j),s]
// chi[s,k], backward B[i,j,s] = sum_k chi[s,k] e[succ_k] B[succ_k,k], expected
// transitions n[s,k] = sum_cells F chi e B / P, evaluated here in float32
// probability space instead of float64 log space.
//
// GB300 design:
//  * Work unit = a STRIPE of 32 lattice rows of one pair (all columns).  A
//    CTA sweeps its stripe along anti-diagonals: at step t lane r of every
//    warp owns cell (i0 + r, t - r); warp w owns the 4-state "quad" w of the
//    cell's state vector.  Two __syncthreads per step, no global traffic on
//    the critical path except the halo row.
//  * Stripes of one pair are PIPELINED across CTAs: stripe s+1 consumes the
//    bottom row of stripe s through a global edge buffer, in chunks of 32
//    columns published with release/acquire progress counters.  A persistent
//    grid pops (pair, stripe) items from an atomic queue ordered
//    longest-pair-first, so long pairs spread over many SMs and short pairs
//    fill the gaps.  A stripe only ever waits for a stripe popped before it,
//    so progress needs no co-residency guarantee; every wait is bounded.
//  * Scaling: each cell's state vector is renormalised by an exact power of
//    two (its own exponent, int32), so the DP has no underflow and the only
//    rounding is that of the float32 multiply-adds.
//  * The E-step backward kernel fuses: the backward recursion, posteriors,
//    per-group character-indexed emission counts (float64 shared-memory
//    bins) and the transition-count outer products (float32 per-thread
//    accumulators with Kahan compensation, float64 at the flush).  The
//    forward pass of an E-step stores the scaled forward lattice (stripe-
//    diagonal layout, read back with cp.async one diagonal ahead).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pairhmm.h"

namespace {

constexpr int TH = 32;             // rows per stripe == lanes per warp
constexpr int HC = 32;             // halo chunk width (columns)
constexpr int MAXS = 168;          // max padded state slots (42 quads): the wide kernels
constexpr int GMAXS = 64;          // max padded slots of the generic, warp and block kernels
constexpr int MAXQ = MAXS / 4;
constexpr int NBIN = 441 + 21 + 21;
constexpr int EXP_NONE = -(1 << 28);
constexpr double LN2 = 0.69314718055994530942;
constexpr double NEG_INF_LL = -1e30;  // reference NEG_INF (dp/hmm.py:108)
// iterations of a bounded inter-CTA wait (each one poll plus a 128 ns sleep:
// about 5 s) unless phmm_set_spin_limit chose another bound
constexpr long long kSpinLimit = 40LL * 1000 * 1000;
enum { T_S = 0, T_M = 1, T_I = 2, T_D = 3, T_E = 4, T_NONE = 5 };

struct PairMeta {
    int64_t x_off, y_off;
    int64_t lat_base;    // first cell of the pair's lattice (stripe-diagonal layout)
    int64_t edge_base;   // first cell of the pair's edge rows
    int64_t tab_base;    // first cell of the pair's optional row-major tables
    int64_t row_base;    // rows 0..Lx of the pairs before this one (band-layout outputs)
    int32_t Lx, Ly;
    int32_t n_stripes;
    int32_t stripe_base;
};

struct KParams {
    int N, NS, NQ, G, e_idx, s_slot;
    int kbeg[3], kend[3];               // slot ranges of the M, I, D groups
    int16_t slot_orig[MAXS];            // original state index or -1
    int8_t slot_type[MAXS];             // T_M/T_I/T_D dest, T_S start, T_NONE pad
    int16_t slot_group[MAXS];
    int8_t quad_type[MAXQ];
    int16_t w_orig[MAXS];               // warp kernels: source slot -> state (start last)
    int16_t w_group[MAXS];              // warp kernels: dest slot -> emission group
    const uint8_t *res;
    const PairMeta *meta;
    const int2 *items;
    int n_items;
    int *counter;
    const float *chi;
    int64_t chi_stride;
    const float *eM, *eI, *eD;
    int64_t eM_stride, eID_stride;
    float *lat;
    int *lat_exp;
    float *blat;                        // split E-step: backward lattice
    int *blat_exp;
    int *bprogress;                     // split E-step: backward edge pipeline
    float *bedge;
    int *bedge_exp;
    int count_wait;                     // count pass waits for the stripes it reads
    float *edge;
    int *edge_exp;
    int *progress;
    double *ll;
    int *status;
    double *n_trans, *cntM, *cntI, *cntD;
    double *F_log, *B_log, *post;
    int max_ly;
    long long spin_limit;
    const int *wave_ctr;                // overlapped count pass: forward, backward claim counters
    const unsigned char *cmask;         // per-cell type mask (bit 0 M, 1 I, 2 D) at tab_base, or null
    // two-warp stripes under a cell mask: columns [x, y] of the cells the mask
    // leaves live in each stripe (global stripe index), or null (all columns)
    const int2 *srange;
    float beam_scale;                   // > 0: forward states below max * beam_scale pruned (generic kernels)
    // wide kernels, stripe-edge checkpointing: lattice cell offset of each
    // stripe (global stripe index) in the current group's scratch, or null
    // for the full-lattice layout (PairMeta::lat_base)
    const int64_t *stripe_lat;
    int recompute;                      // 1: stripes recomputed from complete edge rows (no waits, no
                                        // edge / progress / log-likelihood writes)
    int ckpt;                           // count pass: row 0 of the stripe below from its backward edge row
    // factored MixDom transitions (phmm_batch.nest), or null: the two-warp
    // stripes of a shape with a nested instantiation contract through them
    const float *nest;
    int64_t nest_stride;
    int nest_K, nest_F;
};

struct SmemLayout {
    int chi, chiE, tM, tI, tD, ring, raw, mx, halo, fst, ft, ut;  // float offsets
    int ringE, haloE, fstE;                                         // int offsets
    int bins;                                                       // double offset
    int ys;                                                         // byte offset
    int bytes;
};

__host__ __device__ inline int al4(int v) { return (v + 3) & ~3; }

__host__ __device__ inline SmemLayout make_layout(int NS, int NQ, int G, int max_ly, bool bwd) {
    SmemLayout L;
    int o = 0;
    L.chi = o; o += NS * NS;
    L.chiE = o; o += al4(NS);
    L.tM = o; o += al4(G * 441);
    L.tI = o; o += al4(G * 21);
    L.tD = o; o += al4(G * 21);
    L.ring = o; o += 3 * NS * TH;
    L.raw = o; o += NS * TH;
    L.mx = o; o += al4(NQ * TH);
    L.halo = o; o += al4(2 * NS * (HC + 1));
    if (bwd) {
        L.fst = o; o += 2 * TH * NS;
        L.ft = o; o += TH * NS;
        L.ut = o; o += TH * NS;
    } else {
        L.fst = L.ft = L.ut = -1;
    }
    L.ringE = o; o += 3 * TH;
    L.haloE = o; o += al4(2 * (HC + 1));
    if (bwd) { L.fstE = o; o += 2 * TH; } else { L.fstE = -1; }
    o = (o + 3) & ~3;
    if (bwd) { L.bins = o / 2; o += 2 * G * NBIN; } else { L.bins = -1; }
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 1;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

// 2^e as a float, exact for e in [-149, 127]; 0 below.
__device__ __forceinline__ float pow2f(int e) {
    if (e >= -126) return __int_as_float((min(e, 127) + 127) << 23);
    if (e >= -149) return __int_as_float(1 << (e + 149));
    return 0.0f;
}

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Bounded wait until *p >= need.  Returns false when the bound is hit.
__device__ bool wait_geq(const int *p, int need, long long limit) {
    long long it = 0;
    while (ld_acquire(p) < need) {
        if (++it > limit) return false;
        __nanosleep(128);
    }
    return true;
}

// The split E-step's count pass runs while the wavefronts still run: an item
// of stripe si of pair m may start once that stripe is complete in both
// directions, the stripe below in the backward one (its first row is read),
// and the pair's last forward stripe (the log-likelihood).  Wavefronts publish
// completion as progress value Ly + 2.  Bounded like every other wait.
__device__ bool count_ready(const KParams &P, const PairMeta &m, int si) {
    const int done = m.Ly + 2;
    const int *f = P.progress + m.stripe_base, *b = P.bprogress + m.stripe_base;
    if (!wait_geq(f + si, done, P.spin_limit)) return false;
    if (!wait_geq(b + si, done, P.spin_limit)) return false;
    if (si + 1 < m.n_stripes && !wait_geq(b + si + 1, done, P.spin_limit)) return false;
    return wait_geq(f + m.n_stripes - 1, done, P.spin_limit);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Claim the next count item.  The overlapped count grid holds SM slots while
// it waits for the wavefront kernels, and other work on the GPU (batches on
// other streams) can keep those kernels from becoming resident at all, so an
// overlapped CTA claims only once both wavefront kernels have claimed their
// first stripe: a kernel that has claimed one is resident and drains its whole
// list, so every later wait ends.  A CTA that sees no start within the window
// leaves the remaining items to the tail grid, which runs after both
// wavefronts on its own stream and waits on nothing.
constexpr unsigned long long COUNT_START_WINDOW_NS = 200000;

__device__ int count_claim(const KParams &P) {
    if (P.count_wait) {
        const unsigned long long t0 = globaltimer_ns();
        while (ld_acquire(P.wave_ctr) == 0 || ld_acquire(P.wave_ctr + 1) == 0) {
            if (globaltimer_ns() - t0 > COUNT_START_WINDOW_NS) return P.n_items;
            __nanosleep(256);
        }
    }
    return atomicAdd(P.counter, 1);
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ float4 f4scale(float4 a, float s) {
    return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}
__device__ __forceinline__ float f4max(float4 a) { return fmaxf(fmaxf(a.x, a.y), fmaxf(a.z, a.w)); }
__device__ __forceinline__ float f4get(float4 a, int u) {
    return u == 0 ? a.x : (u == 1 ? a.y : (u == 2 ? a.z : a.w));
}

// Load the per-pair model into shared memory: transitions in slot layout
// (transposed for the backward pass), End column, emission tables, and the
// descendant residues.  Returns nothing; ends with __syncthreads().
__device__ void load_pair_model(const KParams &P, int p, const PairMeta &m, const SmemLayout &L,
                                float *sm, unsigned char *smb, bool transpose) {
    const int NS = P.NS, N = P.N, G = P.G;
    const int tid = threadIdx.x, nt = blockDim.x;
    const float *chi = P.chi + (int64_t)p * P.chi_stride;
    float *chiS = sm + L.chi;
    for (int idx = tid; idx < NS * NS; idx += nt) {
        int s = idx / NS, k = idx % NS;
        int os = P.slot_orig[s], ok = P.slot_orig[k];
        int kt = P.slot_type[k];
        float v = 0.0f;
        if (os >= 0 && ok >= 0 && (kt == T_M || kt == T_I || kt == T_D)) v = __ldg(chi + os * N + ok);
        if (transpose) chiS[k * NS + s] = v; else chiS[s * NS + k] = v;
    }
    for (int s = tid; s < NS; s += nt) {
        int os = P.slot_orig[s];
        sm[L.chiE + s] = (os >= 0) ? __ldg(chi + os * N + P.e_idx) : 0.0f;
    }
    const float *eM = P.eM + (int64_t)p * P.eM_stride;
    const float *eI = P.eI + (int64_t)p * P.eID_stride;
    const float *eD = P.eD + (int64_t)p * P.eID_stride;
    for (int idx = tid; idx < G * 441; idx += nt) sm[L.tM + idx] = __ldg(eM + idx);
    for (int idx = tid; idx < G * 21; idx += nt) {
        sm[L.tI + idx] = __ldg(eI + idx);
        sm[L.tD + idx] = __ldg(eD + idx);
    }
    unsigned char *ys = smb + L.ys;
    for (int j = tid; j <= m.Ly; j += nt) {
        int c = 0;
        if (j >= 1) {
            c = P.res[m.y_off + j - 1];
            if (c > 20) { c = 20; atomicOr(P.status + p, PHMM_ST_BAD_RESIDUE); }
        }
        ys[j] = (unsigned char)c;
    }
    __syncthreads();
}

// Per-thread emission lookup bases of the 4 slots of quad q for row char xi.
struct EmitBase {
    int off[4];
    float mask[4];
    int type;
};

__device__ __forceinline__ EmitBase emit_base(const KParams &P, const SmemLayout &L, int q, int xi) {
    EmitBase eb;
    eb.type = P.quad_type[q];
    for (int u = 0; u < 4; ++u) {
        int k = 4 * q + u;
        int kt = P.slot_type[k];
        int g = P.slot_group[k];
        bool em = (kt == T_M || kt == T_I || kt == T_D);
        eb.mask[u] = em ? 1.0f : 0.0f;
        if (!em) g = 0;
        if (eb.type == T_M) eb.off[u] = L.tM + g * 441 + xi * 21;   // + y_j
        else if (eb.type == T_I) eb.off[u] = L.tI + g * 21;          // + y_j
        else eb.off[u] = L.tD + g * 21 + xi;                         // (no y)
    }
    return eb;
}

__device__ __forceinline__ float4 emit4(const float *sm, const EmitBase &eb, int yj) {
    int add = (eb.type == T_D) ? 0 : yj;
    return make_float4(sm[eb.off[0] + add] * eb.mask[0], sm[eb.off[1] + add] * eb.mask[1],
                       sm[eb.off[2] + add] * eb.mask[2], sm[eb.off[3] + add] * eb.mask[3]);
}

// ---------------------------------------------------------------- forward
__device__ void forward_stripe(const KParams &P, int p, int si, const SmemLayout &L, float *sm,
                               unsigned char *smb, int *s_flag) {
    const PairMeta m = P.meta[p];
    const int NS = P.NS, NQ = P.NQ, N = P.N;
    const int Lx = m.Lx, Ly = m.Ly;
    const int i0 = si * TH;
    const int nrows = min(TH, Lx + 1 - i0);
    const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
    const int r = lane;
    const int i = i0 + r;
    const bool has_below = si + 1 < m.n_stripes;
    int *prog_above = (si > 0) ? P.progress + m.stripe_base + si - 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_above = P.edge + (m.edge_base + (int64_t)(si - 1) * (Ly + 1)) * NS;
    const int *edgeE_above = P.edge_exp + m.edge_base + (int64_t)(si - 1) * (Ly + 1);
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * NS;
    int *edgeE_mine = P.edge_exp + m.edge_base + (int64_t)si * (Ly + 1);
    const int64_t latc = m.lat_base + (int64_t)si * (TH + Ly) * TH;  // this stripe's first lattice cell

    load_pair_model(P, p, m, L, sm, smb, false);
    const unsigned char *ys = smb + L.ys;
    int xi = 0;
    if (r < nrows && i >= 1) {
        xi = P.res[m.x_off + i - 1];
        if (xi > 20) { xi = 20; atomicOr(P.status + p, PHMM_ST_BAD_RESIDUE); }
    }
    const EmitBase eb = emit_base(P, L, q, xi);
    const float4 *chi4 = reinterpret_cast<const float4 *>(sm + L.chi) + q;
    float *ring = sm + L.ring;
    int *ringE = reinterpret_cast<int *>(sm) + L.ringE;
    float *halo = sm + L.halo;
    int *haloE = reinterpret_cast<int *>(sm) + L.haloE;
    float *raw = sm + L.raw;
    float *mx = sm + L.mx;
    const int T_last = (nrows - 1) + Ly;
    const int qt = eb.type;
    bool aborted = false;

    for (int t = 0; t <= T_last; ++t) {
        // ---- top halo chunk (row i0-1 from the stripe above)
        if (si > 0 && (t % HC) == 0 && t <= Ly) {
            const int c = t / HC;
            const int cbeg = c * HC, cend = min(cbeg + HC, Ly + 1);
            if (threadIdx.x == 0) *s_flag = wait_geq(prog_above, cend, P.spin_limit) ? 0 : 1;
            __syncthreads();
            if (*s_flag) { aborted = true; break; }
            float *hb = halo + (c & 1) * NS * (HC + 1);
            int *hbE = haloE + (c & 1) * (HC + 1);
            const int ncol = cend - cbeg;
            for (int idx = threadIdx.x; idx < ncol * NS; idx += blockDim.x) {
                int col = idx / NS, s = idx % NS;
                hb[s * (HC + 1) + col] = __ldcg(edge_above + (int64_t)(cbeg + col) * NS + s);
            }
            for (int col = threadIdx.x; col < ncol; col += blockDim.x) hbE[col] = __ldcg(edgeE_above + cbeg + col);
            __syncthreads();
        }
        // ---- phase A: raw state values of this diagonal
        const int j = t - r;
        const bool valid = (r < nrows) && (j >= 0) && (j <= Ly);
        int Eref = EXP_NONE;
        const int mb = (P.cmask && valid) ? (int)P.cmask[m.tab_base + (int64_t)i * (Ly + 1) + j] : 7;
        if (valid) {
            const float *pp = nullptr;
            int pst = TH, Ep = EXP_NONE;
            // I pred (i, j-1): diag t-1, row r; a type the cell mask rules out
            // here takes no part (nor its exponent)
            const bool hasI = j >= 1 && (mb & 2);
            const bool hasD = i >= 1 && (mb & 4);
            const bool hasM = i >= 1 && j >= 1 && (mb & 1);
            int EI_ = EXP_NONE, ED_ = EXP_NONE, EM_ = EXP_NONE;
            const float *pI = ring + ((t + 2) % 3) * NS * TH + r;
            const float *pD = nullptr, *pM = nullptr;
            int stD = TH, stM = TH;
            if (hasI) EI_ = ringE[((t + 2) % 3) * TH + r];
            if (hasD) {
                if (r >= 1) {
                    pD = ring + ((t + 2) % 3) * NS * TH + (r - 1);
                    ED_ = ringE[((t + 2) % 3) * TH + r - 1];
                } else {
                    pD = halo + ((j / HC) & 1) * NS * (HC + 1) + (j % HC);
                    stD = HC + 1;
                    ED_ = haloE[((j / HC) & 1) * (HC + 1) + (j % HC)];
                }
            }
            if (hasM) {
                if (r >= 1) {
                    pM = ring + ((t + 1) % 3) * NS * TH + (r - 1);
                    EM_ = ringE[((t + 1) % 3) * TH + r - 1];
                } else {
                    const int jm = j - 1;
                    pM = halo + ((jm / HC) & 1) * NS * (HC + 1) + (jm % HC);
                    stM = HC + 1;
                    EM_ = haloE[((jm / HC) & 1) * (HC + 1) + (jm % HC)];
                }
            }
            Eref = max(max(hasI ? EI_ : EXP_NONE, hasD ? ED_ : EXP_NONE), hasM ? EM_ : EXP_NONE);
            bool have = false;
            if (qt == T_M && hasM) { pp = pM; pst = stM; Ep = EM_; have = true; }
            if (qt == T_I && hasI) { pp = pI; pst = TH; Ep = EI_; have = true; }
            if (qt == T_D && hasD) { pp = pD; pst = stD; Ep = ED_; have = true; }
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            if (have && Ep > EXP_NONE) {
                for (int s = 0; s < NS; s += 4) {
                    const float v0 = pp[(s + 0) * pst], v1 = pp[(s + 1) * pst];
                    const float v2 = pp[(s + 2) * pst], v3 = pp[(s + 3) * pst];
                    const float4 c0 = chi4[(s + 0) * NQ], c1 = chi4[(s + 1) * NQ];
                    const float4 c2 = chi4[(s + 2) * NQ], c3 = chi4[(s + 3) * NQ];
                    acc.x = fmaf(v0, c0.x, acc.x); acc.y = fmaf(v0, c0.y, acc.y);
                    acc.z = fmaf(v0, c0.z, acc.z); acc.w = fmaf(v0, c0.w, acc.w);
                    acc.x = fmaf(v1, c1.x, acc.x); acc.y = fmaf(v1, c1.y, acc.y);
                    acc.z = fmaf(v1, c1.z, acc.z); acc.w = fmaf(v1, c1.w, acc.w);
                    acc.x = fmaf(v2, c2.x, acc.x); acc.y = fmaf(v2, c2.y, acc.y);
                    acc.z = fmaf(v2, c2.z, acc.z); acc.w = fmaf(v2, c2.w, acc.w);
                    acc.x = fmaf(v3, c3.x, acc.x); acc.y = fmaf(v3, c3.y, acc.y);
                    acc.z = fmaf(v3, c3.z, acc.z); acc.w = fmaf(v3, c3.w, acc.w);
                }
                const float4 e = emit4(sm, eb, ys[j]);
                const float sc = pow2f(Ep - Eref);
                acc = make_float4(acc.x * e.x * sc, acc.y * e.y * sc, acc.z * e.z * sc, acc.w * e.w * sc);
            }
            float *rw = raw + (4 * q) * TH + r;
            rw[0] = acc.x; rw[TH] = acc.y; rw[2 * TH] = acc.z; rw[3 * TH] = acc.w;
            mx[q * TH + r] = f4max(acc);
        }
        __syncthreads();
        // ---- phase B: per-cell power-of-two renormalisation
        if (valid) {
            float mval = 0.0f;
            for (int qq = 0; qq < NQ; ++qq) mval = fmaxf(mval, mx[qq * TH + r]);
            const float *rw = raw + (4 * q) * TH + r;
            float4 v = make_float4(rw[0], rw[TH], rw[2 * TH], rw[3 * TH]);
            if (P.beam_scale > 0.f) {   // beam: states below max * e^-width drop out (hmm_beam.py:188-195)
                const float thr = mval * P.beam_scale;
                v = make_float4(v.x < thr ? 0.f : v.x, v.y < thr ? 0.f : v.y, v.z < thr ? 0.f : v.z,
                                v.w < thr ? 0.f : v.w);
            }
            int Ecell = EXP_NONE;
            if (mval > 0.0f) {
                int e;
                frexpf(mval, &e);
                v = make_float4(ldexpf(v.x, -e), ldexpf(v.y, -e), ldexpf(v.z, -e), ldexpf(v.w, -e));
                Ecell = Eref + e;
            } else {
                v = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (i == 0 && j == 0 && mb != 0) {  // origin: F[0,0,start] = 1 (dp/hmm.py:1212)
                v = make_float4(0.f, 0.f, 0.f, 0.f);
                const int ss = P.s_slot;
                if (ss / 4 == q) {
                    if (ss % 4 == 0) v.x = 1.f; else if (ss % 4 == 1) v.y = 1.f;
                    else if (ss % 4 == 2) v.z = 1.f; else v.w = 1.f;
                }
                Ecell = 0;
            }
            float *rg = ring + (t % 3) * NS * TH + (4 * q) * TH + r;
            rg[0] = v.x; rg[TH] = v.y; rg[2 * TH] = v.z; rg[3 * TH] = v.w;
            if (q == 0) ringE[(t % 3) * TH + r] = Ecell;
            if (has_below && r == TH - 1) {
                reinterpret_cast<float4 *>(edge_mine + (int64_t)j * NS)[q] = v;
                if (q == 0) edgeE_mine[j] = Ecell;
            }
            if (P.lat) {
                const int64_t cell = latc + (int64_t)t * TH + r;
                reinterpret_cast<float4 *>(P.lat + cell * NS)[q] = v;
                if (q == 0) P.lat_exp[cell] = Ecell;
            }
            if (P.F_log) {
                const int64_t cell = m.tab_base + (int64_t)i * (Ly + 1) + j;
                for (int u = 0; u < 4; ++u) {
                    const int os = P.slot_orig[4 * q + u];
                    if (os < 0) continue;
                    const float x = f4get(v, u);
                    P.F_log[cell * N + os] = (x > 0.f && Ecell > EXP_NONE)
                        ? log((double)x) + (double)Ecell * LN2 : NEG_INF_LL;
                }
            }
        }
        __syncthreads();
        // ---- publish bottom-row progress for the stripe below
        if (has_below && threadIdx.x == 0) {
            const int jb = t - (TH - 1);
            if (jb >= 0 && jb <= Ly && (((jb + 1) % HC) == 0 || jb == Ly)) {
                __threadfence();
                st_release(prog_mine, jb + 1);
            }
        }
    }
    if (aborted) {
        if (threadIdx.x == 0) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (has_below) { __threadfence(); st_release(prog_mine, Ly + 1); }
            if (si + 1 == m.n_stripes) P.ll[p] = NEG_INF_LL;
        }
        __syncthreads();
        return;
    }
    // ---- log-likelihood at the terminal cell (dp/hmm.py:1913)
    if (si + 1 == m.n_stripes && q == 0) {
        const int rT = Lx - i0;
        const float *cellv = ring + (T_last % 3) * NS * TH + rT;
        double acc = 0.0;
        for (int s = lane; s < NS; s += 32) acc += (double)cellv[s * TH] * (double)sm[L.chiE + s];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            const int E = ringE[(T_last % 3) * TH + rT];
            double ll = NEG_INF_LL;
            if (acc > 0.0 && isfinite(acc) && E > EXP_NONE) ll = log(acc) + (double)E * LN2;
            else atomicOr(P.status + p, PHMM_ST_ZERO_LL);
            P.ll[p] = ll;
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(512) forward_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    __shared__ int s_flag;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemLayout L = make_layout(P.NS, P.NQ, P.G, P.max_ly, false);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        forward_stripe(P, w.x, w.y, L, sm, smem_raw, &s_flag);
    }
}

// ---------------------------------------------------------------- backward + counts
__device__ void backward_stripe(const KParams &P, int p, int si, const SmemLayout &L, float *sm,
                                unsigned char *smb, int *s_flag) {
    const PairMeta m = P.meta[p];
    const int NS = P.NS, NQ = P.NQ, N = P.N, G = P.G;
    const int Lx = m.Lx, Ly = m.Ly;
    const int i0 = si * TH;
    const int nrows = min(TH, Lx + 1 - i0);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, q = tid >> 5;
    const int r = lane;
    const int i = i0 + r;
    const bool has_below = si + 1 < m.n_stripes;
    const bool has_above = si > 0;
    int *prog_below = has_below ? P.progress + m.stripe_base + si + 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_below = P.edge + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * NS;
    const int *edgeE_below = P.edge_exp + m.edge_base + (int64_t)(si + 1) * (Ly + 1);
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * NS;
    int *edgeE_mine = P.edge_exp + m.edge_base + (int64_t)si * (Ly + 1);
    const int64_t latc = m.lat_base + (int64_t)si * (TH + Ly) * TH;

    const double llv = P.ll[p];
    if (!(llv > -1e29)) {  // forward failed: no counts for this pair
        __syncthreads();
        if (tid == 0 && has_above) { __threadfence(); st_release(prog_mine, Ly + 1); }
        return;
    }
    const double lam = llv / LN2;
    const double Epd = floor(lam);
    const int Ep = (int)Epd;
    const float rfrac = (float)exp2(-(lam - Epd));

    load_pair_model(P, p, m, L, sm, smb, true);
    double *bins = reinterpret_cast<double *>(sm) + L.bins;
    for (int idx = tid; idx < G * NBIN; idx += nt) bins[idx] = 0.0;
    const unsigned char *ys = smb + L.ys;
    int xi = 0;
    if (r < nrows && i >= 1) xi = min((int)P.res[m.x_off + i - 1], 20);
    const EmitBase eb = emit_base(P, L, q, xi);
    const int qt = eb.type;
    float *ring = sm + L.ring;
    int *ringE = reinterpret_cast<int *>(sm) + L.ringE;
    float *halo = sm + L.halo;
    int *haloE = reinterpret_cast<int *>(sm) + L.haloE;
    float *raw = sm + L.raw;
    float *mx = sm + L.mx;
    float *fst = sm + L.fst;
    int *fstE = reinterpret_cast<int *>(sm) + L.fstE;
    float4 *ft4 = reinterpret_cast<float4 *>(sm + L.ft);
    float4 *ut4 = reinterpret_cast<float4 *>(sm + L.ut);
    const float4 *chiB4 = reinterpret_cast<const float4 *>(sm + L.chi) + q;  // chiB[k][4q..]

    // count-phase role: (source quad sq, dest quad kq, row group rg)
    const int npairs = NQ * NQ;
    const int RG = nt / npairs;
    const int cp = tid % npairs, rg = tid / npairs;
    const int sq = cp / NQ, kq = cp % NQ;
    const bool counter_role = rg < RG && P.quad_type[kq] != T_NONE;
    float csum[16], ccomp[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) { csum[u] = 0.f; ccomp[u] = 0.f; }

    const int T_last = (nrows - 1) + Ly;
    // lattice prefetch (cp.async): diagonal t goes to buffer t & 1
    auto prefetch = [&](int t) {
        if (t >= 0) {
            const float *src = P.lat + (latc + (int64_t)t * TH) * NS;
            float *dst = fst + (t & 1) * TH * NS;
            for (int idx = tid; idx < TH * NS / 4; idx += nt) cp_async16(dst + 4 * idx, src + 4 * idx);
            const int *srcE = P.lat_exp + latc + (int64_t)t * TH;
            int *dstE = fstE + (t & 1) * TH;
            for (int idx = tid; idx < TH / 4; idx += nt) cp_async16(dstE + 4 * idx, srcE + 4 * idx);
        }
        cp_commit();
    };
    prefetch(T_last);
    bool aborted = false;

    for (int t = T_last; t >= 0; --t) {
        prefetch(t - 1);
        // ---- bottom halo chunk (row i0+TH from the stripe below)
        const int jb = t - (nrows - 1);
        if (has_below && jb >= 0 && jb <= Ly && (jb == Ly || (jb % HC) == HC - 1)) {
            const int c = jb / HC;
            const int cbeg = c * HC, cend = min(cbeg + HC, Ly + 1);
            if (tid == 0) *s_flag = wait_geq(prog_below, Ly + 1 - cbeg, P.spin_limit) ? 0 : 1;
            __syncthreads();
            if (*s_flag) { aborted = true; break; }
            float *hb = halo + (c & 1) * NS * (HC + 1);
            int *hbE = haloE + (c & 1) * (HC + 1);
            const int ncol = cend - cbeg;
            for (int idx = tid; idx < ncol * NS; idx += nt) {
                int col = idx / NS, s = idx % NS;
                hb[s * (HC + 1) + col] = __ldcg(edge_below + (int64_t)(cbeg + col) * NS + s);
            }
            for (int col = tid; col < ncol; col += nt) hbE[col] = __ldcg(edgeE_below + cbeg + col);
            __syncthreads();
        }
        // ---- phase A: raw backward values for source slots 4q..4q+3
        const int j = t - r;
        const bool valid = (r < nrows) && (j >= 0) && (j <= Ly);
        const bool terminal = valid && i == Lx && j == Ly;
        int Eref = EXP_NONE;
        // successor pointers/exponents, kept for the count preparation
        const float *wM = nullptr, *wI = nullptr, *wD = nullptr;
        int sM = TH, sI = TH, sD = TH;
        int EM_ = EXP_NONE, EI_ = EXP_NONE, ED_ = EXP_NONE;
        if (valid) {
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            if (terminal) {
                acc = reinterpret_cast<const float4 *>(sm + L.chiE)[q];
                Eref = 0;
            } else {
                const bool hasI = j + 1 <= Ly;
                const bool hasD = i + 1 <= Lx;
                const bool hasM = hasI && hasD;
                if (hasI) {
                    wI = ring + ((t + 1) % 3) * NS * TH + r;
                    EI_ = ringE[((t + 1) % 3) * TH + r];
                }
                if (hasD) {
                    if (r + 1 < nrows) {
                        wD = ring + ((t + 1) % 3) * NS * TH + r + 1;
                        ED_ = ringE[((t + 1) % 3) * TH + r + 1];
                    } else {
                        wD = halo + ((j / HC) & 1) * NS * (HC + 1) + (j % HC);
                        sD = HC + 1;
                        ED_ = haloE[((j / HC) & 1) * (HC + 1) + (j % HC)];
                    }
                }
                if (hasM) {
                    if (r + 1 < nrows) {
                        wM = ring + ((t + 2) % 3) * NS * TH + r + 1;
                        EM_ = ringE[((t + 2) % 3) * TH + r + 1];
                    } else {
                        const int jm = j + 1;
                        wM = halo + ((jm / HC) & 1) * NS * (HC + 1) + (jm % HC);
                        sM = HC + 1;
                        EM_ = haloE[((jm / HC) & 1) * (HC + 1) + (jm % HC)];
                    }
                }
                Eref = max(max(EI_, ED_), EM_);
                const float *wp[3] = {wM, wI, wD};
                const int ws[3] = {sM, sI, sD};
                const int we[3] = {EM_, EI_, ED_};
                for (int ty = 0; ty < 3; ++ty) {
                    if (wp[ty] == nullptr || we[ty] <= EXP_NONE) continue;
                    const float *w = wp[ty];
                    const int st = ws[ty];
                    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
                    for (int k = P.kbeg[ty]; k < P.kend[ty]; ++k) {
                        const float wv = w[k * st];
                        const float4 c = chiB4[k * NQ];
                        a.x = fmaf(wv, c.x, a.x); a.y = fmaf(wv, c.y, a.y);
                        a.z = fmaf(wv, c.z, a.z); a.w = fmaf(wv, c.w, a.w);
                    }
                    const float sc = pow2f(we[ty] - Eref);
                    acc.x = fmaf(a.x, sc, acc.x); acc.y = fmaf(a.y, sc, acc.y);
                    acc.z = fmaf(a.z, sc, acc.z); acc.w = fmaf(a.w, sc, acc.w);
                }
            }
            float *rw = raw + (4 * q) * TH + r;
            rw[0] = acc.x; rw[TH] = acc.y; rw[2 * TH] = acc.z; rw[3 * TH] = acc.w;
            mx[q * TH + r] = f4max(acc);
        }
        cp_wait1();
        __syncthreads();
        // ---- phase B: normalise, store w = e*b, prepare count operands
        float4 ftv = make_float4(0.f, 0.f, 0.f, 0.f), utv = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid) {
            float mval = 0.0f;
            for (int qq = 0; qq < NQ; ++qq) mval = fmaxf(mval, mx[qq * TH + r]);
            const float *rw = raw + (4 * q) * TH + r;
            float4 b = make_float4(rw[0], rw[TH], rw[2 * TH], rw[3 * TH]);
            int Eb = EXP_NONE;
            if (mval > 0.0f) {
                int e;
                frexpf(mval, &e);
                b = make_float4(ldexpf(b.x, -e), ldexpf(b.y, -e), ldexpf(b.z, -e), ldexpf(b.w, -e));
                Eb = Eref + e;
            } else {
                b = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            float4 e4 = emit4(sm, eb, ys[j]);
            int Ew = Eb;   // exponent of w; none where no type may emit
            if (P.cmask) {   // a masked type emits nothing here: w = 0, so no predecessor sees it
                const int mb = P.cmask[m.tab_base + (int64_t)i * (Ly + 1) + j];
                const bool off = (qt == T_M && !(mb & 1)) || (qt == T_I && !(mb & 2)) || (qt == T_D && !(mb & 4));
                if (off) e4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (mb == 0) Ew = EXP_NONE;
            }
            if (P.beam_scale > 0.f && fstE[(t & 1) * TH + r] <= EXP_NONE) {
                // pruned run: a cell the forward left empty is no successor (hmm_beam.py:231, 270)
                e4 = make_float4(0.f, 0.f, 0.f, 0.f);
                Ew = EXP_NONE;
            }
            const float4 w = make_float4(b.x * e4.x, b.y * e4.y, b.z * e4.z, b.w * e4.w);
            float *rg = ring + (t % 3) * NS * TH + (4 * q) * TH + r;
            rg[0] = w.x; rg[TH] = w.y; rg[2 * TH] = w.z; rg[3 * TH] = w.w;
            if (q == 0) ringE[(t % 3) * TH + r] = Ew;
            if (has_above && r == 0) {
                reinterpret_cast<float4 *>(edge_mine + (int64_t)j * NS)[q] = w;
                if (q == 0) edgeE_mine[j] = Ew;
            }
            // forward values of this cell
            const float4 f = reinterpret_cast<const float4 *>(fst + (t & 1) * TH * NS + r * NS)[q];
            const int Ef = fstE[(t & 1) * TH + r];
            if (Ef > EXP_NONE && Eb > EXP_NONE) {
                int d = Ef + Eb - Ep;
                if (d > 126) { d = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                const float sc = ldexpf(rfrac, max(d, -200));
                ftv = f4scale(f, sc);
                // transition-count successor operand for the quad's own dest slots
                const float *ws = (qt == T_M) ? wM : (qt == T_I) ? wI : (qt == T_D) ? wD : nullptr;
                const int wst = (qt == T_M) ? sM : (qt == T_I) ? sI : sD;
                const int wex = (qt == T_M) ? EM_ : (qt == T_I) ? EI_ : ED_;
                if (ws != nullptr && wex > EXP_NONE) {
                    const float us = pow2f(min(wex - Eb, 126));
                    for (int u = 0; u < 4; ++u) {
                        const float val = ws[(4 * q + u) * wst] * us;
                        if (u == 0) utv.x = val; else if (u == 1) utv.y = val;
                        else if (u == 2) utv.z = val; else utv.w = val;
                    }
                }
            }
            // posteriors -> per-group character bins
            const float4 post4 = make_float4(ftv.x * b.x, ftv.y * b.y, ftv.z * b.z, ftv.w * b.w);
            if (qt != T_NONE) {
                for (int u = 0; u < 4; ++u) {
                    const int k = 4 * q + u;
                    const int kt = P.slot_type[k];
                    const float pv = f4get(post4, u);
                    if (pv == 0.f || !(kt == T_M || kt == T_I || kt == T_D)) continue;
                    const int g = P.slot_group[k];
                    int bi;
                    if (kt == T_M) bi = g * NBIN + xi * 21 + ys[j];
                    else if (kt == T_I) bi = g * NBIN + 441 + ys[j];
                    else bi = g * NBIN + 462 + xi;
                    atomicAdd(bins + bi, (double)pv);
                }
            }
            if (terminal) {  // expected End transitions (dp/hmm.py:1969-1971)
                for (int u = 0; u < 4; ++u) {
                    const int os = P.slot_orig[4 * q + u];
                    if (os >= 0) atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + P.e_idx,
                                           (double)f4get(post4, u));
                }
            }
            if (P.post || P.B_log) {
                const int64_t cell = m.tab_base + (int64_t)i * (Ly + 1) + j;
                for (int u = 0; u < 4; ++u) {
                    const int os = P.slot_orig[4 * q + u];
                    if (os < 0) continue;
                    if (P.post) {
                        const double pv = (double)f4get(post4, u);
                        P.post[cell * N + os] = P.beam_scale > 0.f ? fmin(pv, 1.0) : pv;
                    }
                    if (P.B_log) {
                        const float x = f4get(b, u);
                        P.B_log[cell * N + os] = (x > 0.f && Eb > EXP_NONE)
                            ? log((double)x) + (double)Eb * LN2 : NEG_INF_LL;
                    }
                }
            }
        }
        ft4[r * NQ + q] = ftv;
        ut4[r * NQ + q] = utv;
        __syncthreads();
        // ---- publish top-row progress for the stripe above
        if (has_above && tid == 0 && t <= Ly && (t % HC) == 0) {
            __threadfence();
            st_release(prog_mine, Ly + 1 - t);
        }
        // ---- phase C: transition-count outer products over the diagonal's cells
        if (counter_role) {
            float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f), p1 = p0, p2 = p0, p3 = p0;
            for (int rr = rg; rr < nrows; rr += RG) {
                const float4 fv = ft4[rr * NQ + sq];
                const float4 uv = ut4[rr * NQ + kq];
                p0.x = fmaf(fv.x, uv.x, p0.x); p0.y = fmaf(fv.x, uv.y, p0.y);
                p0.z = fmaf(fv.x, uv.z, p0.z); p0.w = fmaf(fv.x, uv.w, p0.w);
                p1.x = fmaf(fv.y, uv.x, p1.x); p1.y = fmaf(fv.y, uv.y, p1.y);
                p1.z = fmaf(fv.y, uv.z, p1.z); p1.w = fmaf(fv.y, uv.w, p1.w);
                p2.x = fmaf(fv.z, uv.x, p2.x); p2.y = fmaf(fv.z, uv.y, p2.y);
                p2.z = fmaf(fv.z, uv.z, p2.z); p2.w = fmaf(fv.z, uv.w, p2.w);
                p3.x = fmaf(fv.w, uv.x, p3.x); p3.y = fmaf(fv.w, uv.y, p3.y);
                p3.z = fmaf(fv.w, uv.z, p3.z); p3.w = fmaf(fv.w, uv.w, p3.w);
            }
            const float pv[16] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w,
                                  p2.x, p2.y, p2.z, p2.w, p3.x, p3.y, p3.z, p3.w};
#pragma unroll
            for (int u = 0; u < 16; ++u) {  // Kahan compensated accumulation
                const float y = pv[u] - ccomp[u];
                const float tt = csum[u] + y;
                ccomp[u] = (tt - csum[u]) - y;
                csum[u] = tt;
            }
        }
    }
    if (aborted) {
        if (tid == 0) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (has_above) { __threadfence(); st_release(prog_mine, Ly + 1); }
        }
        cp_wait1();
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
        return;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    // ---- flush transition counts: n[s,k] = chi[s,k] * sum f~ u~
    if (counter_role) {
        const float *chi = P.chi + (int64_t)p * P.chi_stride;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int s = 4 * sq + (u >> 2), k = 4 * kq + (u & 3);
            const int os = P.slot_orig[s], ok = P.slot_orig[k];
            const int kt = P.slot_type[k];
            const float val = csum[u] - ccomp[u];
            if (os < 0 || ok < 0 || !(kt == T_M || kt == T_I || kt == T_D) || val == 0.f) continue;
            const double c = (double)__ldg(chi + os * N + ok);
            atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + ok, (double)val * c);
        }
    }
    __syncthreads();
    // ---- flush emission bins
    for (int idx = tid; idx < G * NBIN; idx += nt) {
        const double v = bins[idx];
        if (v == 0.0) continue;
        const int g = idx / NBIN, b = idx % NBIN;
        if (b < 441) atomicAdd(P.cntM + ((int64_t)p * G + g) * 441 + b, v);
        else if (b < 462) atomicAdd(P.cntI + ((int64_t)p * G + g) * 21 + (b - 441), v);
        else atomicAdd(P.cntD + ((int64_t)p * G + g) * 21 + (b - 462), v);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(512) backward_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    __shared__ int s_flag;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemLayout L = make_layout(P.NS, P.NQ, P.G, P.max_ly, true);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        backward_stripe(P, w.x, w.y, L, sm, smem_raw, &s_flag);
    }
}

__global__ void fill_f64(double *p, int64_t n, double v) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x)
        p[idx] = v;
}

// Live column range of each stripe under a cell mask: one CTA per forward
// stripe item (pair, stripe) scans the stripe's rows of the mask and writes
// the smallest and largest column with a nonzero entry to range[stripe_base +
// stripe], or (RANGE_EMPTY_LO, RANGE_EMPTY_HI) when the mask leaves nothing.
// The terminal cell (Lx, Ly) always counts, so the stripe holding it visits
// the cell the log-likelihood is read from.  Off its range a stripe's forward
// and backward values are zero (no cell there may emit), which is what lets
// the recursions skip those anti-diagonal steps.
constexpr int RANGE_EMPTY_LO = 1 << 30, RANGE_EMPTY_HI = -(1 << 30);

__global__ void stripe_range_kernel(const KParams P, int rows, int2 *range) {
    const int2 w = P.items[blockIdx.x];
    const PairMeta m = P.meta[w.x];
    const int si = w.y, i0 = si * rows, nrows = min(rows, m.Lx + 1 - i0);
    __shared__ int s_lo, s_hi;
    if (threadIdx.x == 0) { s_lo = RANGE_EMPTY_LO; s_hi = RANGE_EMPTY_HI; }
    __syncthreads();
    int lo = RANGE_EMPTY_LO, hi = RANGE_EMPTY_HI;
    for (int r = 0; r < nrows; ++r) {
        const unsigned char *row = P.cmask + m.tab_base + (int64_t)(i0 + r) * (m.Ly + 1);
        for (int j = threadIdx.x; j <= m.Ly; j += blockDim.x)
            if (row[j]) { lo = min(lo, j); hi = max(hi, j); }
    }
    if (si + 1 == m.n_stripes && threadIdx.x == 0) { lo = min(lo, m.Ly); hi = max(hi, m.Ly); }
    if (lo <= hi) { atomicMin(&s_lo, lo); atomicMax(&s_hi, hi); }
    __syncthreads();
    if (threadIdx.x == 0) range[m.stripe_base + si] = make_int2(s_lo, s_hi);
}

// Band-layout posteriors from the split E-step's two-warp lattices: one CTA
// per forward stripe item; position (i, b) of a pair's rows takes
// f~ b~ 2^(Ef + Eb) / P at cell (i, center[i] - W + b) for the emitting
// states and the start (source slots 0..nsrc-1, start last); cells off the
// stripe's live columns or off the lattice stay 0 (set by the caller).
__global__ void band_post_kernel(const KParams P, int rows, int stride, int nsrc, const int32_t *center, int W,
                                 double *out) {
    const int2 w = P.items[blockIdx.x];
    const int p = w.x, si = w.y;
    const PairMeta m = P.meta[p];
    const double llv = P.ll[p];
    if (!(llv > -1e29)) return;
    const double lam = llv / LN2;
    const int i0 = si * rows, nrows = min(rows, m.Lx + 1 - i0), BW = 2 * W + 1;
    const int2 rg = P.srange[m.stripe_base + si];
    const int jlo = max(0, rg.x), jhi = min(m.Ly, rg.y);
    const int64_t latc = m.lat_base + (int64_t)si * (rows + m.Ly) * rows;
    for (int idx = threadIdx.x; idx < nrows * BW; idx += blockDim.x) {
        const int r = idx / BW, b = idx - r * BW, i = i0 + r;
        const int j = center[m.row_base + i] - W + b;
        if (j < jlo || j > jhi) continue;
        const int64_t cell = latc + (int64_t)(j + r) * rows + r;
        const int Ef = P.lat_exp[cell], Eb = P.blat_exp[cell];
        if (Ef <= EXP_NONE || Eb <= EXP_NONE) continue;
        const double sc = exp2((double)(Ef + Eb) - lam);
        double *o = out + ((m.row_base + i) * BW + b) * P.N;
        for (int s = 0; s < nsrc; ++s)
            o[P.w_orig[s]] = (double)P.lat[cell * stride + s] * (double)P.blat[cell * stride + s] * sc;
    }
}

}  // namespace

#include "estep_warp.cuh"
#include "estep_split.cuh"
#include "estep_twowarp.cuh"
#include "estep_block.cuh"
#include "estep_block_split.cuh"
#include "estep_wide.cuh"
#include "estep_wide_nest.cuh"

namespace {

// ---------------------------------------------------------------- host side
thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(PHMM_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

// error channel shared with the other translation units of the library
extern "C" __attribute__((visibility("hidden"))) void phmm_internal_set_error(const char *msg) { g_err = msg; }

struct phmm_plan {
    KParams base;
    int sm_count = 0;
    int launches = 0;
    // device scratch (grown on demand)
    void *meta = nullptr; size_t meta_cap = 0;
    void *items = nullptr; size_t items_cap = 0;
    int *counters = nullptr;
    float *lat = nullptr; size_t lat_cap = 0;
    int *lat_exp = nullptr; size_t latE_cap = 0;
    float *edge = nullptr; size_t edge_cap = 0;
    int *edge_exp = nullptr; size_t edgeE_cap = 0;
    int *progress = nullptr; size_t prog_cap = 0;
    float *blat = nullptr; size_t blat_cap = 0;      // split E-step
    int *blat_exp = nullptr; size_t blatE_cap = 0;
    float *bedge = nullptr; size_t bedge_cap = 0;
    int *bedge_exp = nullptr; size_t bedgeE_cap = 0;
    int64_t *slat = nullptr; size_t slat_cap = 0;    // checkpointed wide E-step: stripe offsets per group
    // split E-step: one side stream (+ fork / join events) per caller stream
    // (prio: the wavefront streams were created at the greatest priority and the
    // count streams at the least, and the forward runs on sidef)
    struct Side {
        cudaStream_t user, side, side2, side3, sidef;
        cudaEvent_t fork, join, join2, join3, fwd_done, joinf;
        bool prio;
    };
    std::vector<Side> sides;
    std::vector<PairMeta> h_meta;
    std::vector<int2> h_items;
    // optional per-kernel CUDA-event timing on the launching stream
    bool timing = false;
    bool timed_bwd = false;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool timed_count = false;
    // a call that ran in groups (batch larger than free memory): summed per-kernel times
    bool grouped = false;
    float group_ms[3] = {0.f, 0.f, 0.f};
    // register-resident warp kernels for this state space (null: generic kernels)
    int w_nm = 0, w_ni = 0, w_nd = 0;
    int grid_div = 1;       // persistent grids use 1/grid_div of the resident slots
    int launch_per_sm = 0;  // > 0: the next launch takes this many resident CTAs per SM (at most occ)
    phmm_tuning tuning = {0, 0, -1, 0, 0, 0};   // phmm_set_tuning (variant is `variant` below)
    int variant = 0;        // 0 automatic, 1 generic, 2 warp, 3 block, 4/5 split warp/block E-step, 6 wide,
                            // 7 split E-step on two-warp stripes
    bool two_warp = false;  // the last warp-family call ran the two-warp stripe kernels
    int last_variant = 0;
    long long spin_limit = 0;   // bound of the inter-CTA waits (0: kSpinLimit)
    size_t total_mem = 0;       // device memory (the automatic checkpointing rule)
    int ckpt_groups = 0;        // stripe groups of the last checkpointed call (0: full lattices)
    // checkpointed E-step of the wide kernels: the stripe groups (host)
    std::vector<int64_t> h_stripe_lat;
    int desc_mode = 0;   // 1: a _ws call writes the work description only; 2: it launches only
};

namespace {

template <typename T>
int ensure(T **ptr, size_t *cap, size_t n) {
    if (n <= *cap && *ptr) return 0;
    // grow by half again for small buffers (fewer reallocations); exactly for
    // buffers above 1 GiB, where the headroom would cost real HBM
    size_t want = n * sizeof(T) > ((size_t)1 << 30) ? n : std::max(n, (size_t)(*cap * 3 / 2));
    if (*ptr) { cudaDeviceSynchronize(); cudaFree(*ptr); *ptr = nullptr; *cap = 0; }
    cudaError_t e = cudaMalloc((void **)ptr, std::max<size_t>(want, 1) * sizeof(T));
    if (e != cudaSuccess) return fail(PHMM_E_CUDA, std::string("cudaMalloc scratch: ") + cudaGetErrorString(e));
    *cap = want;
    return 0;
}

// ---- launchers of the register-resident warp kernels, one per state-space shape
// kind: 0 forward, 1 fused backward + counts, 2 backward recursion (split), 3 counts (split);
// the block launchers take 4 for the combined forward + backward-recursion kernel
using WarpLauncher = int (*)(phmm_plan *, KParams &, int, int, int, cudaStream_t);

template <class SH>
int launch_warp(phmm_plan *plan, KParams &K, int n_items, int max_ly, int kind, cudaStream_t stream);

template <int NM, int NI, int ND>
int launch_warp_shape(phmm_plan *plan, KParams &K, int n_items, int max_ly, int kind, cudaStream_t stream) {
    return launch_warp<warp2::Shape<NM, NI, ND>>(plan, K, n_items, max_ly, kind, stream);
}

struct WarpShapeEntry { int nm, ni, nd; WarpLauncher fn; };
const WarpShapeEntry kWarpShapes[] = {
    {1, 1, 1, launch_warp_shape<1, 1, 1>},   // TKF91 / TKF92
    {1, 2, 2, launch_warp_shape<1, 2, 2>},   // MixDom K=1 F=1
    {2, 2, 2, launch_warp_shape<2, 2, 2>},   // MixFrag F=2
    {3, 3, 3, launch_warp_shape<3, 3, 3>},   // MixFrag F=3
    {2, 4, 4, launch_warp_shape<2, 4, 4>},   // MixDom K*F=2
    {3, 6, 6, launch_warp_shape<3, 6, 6>},   // MixDom K*F=3 (17 states)
    {4, 8, 8, launch_warp_shape<4, 8, 8>},   // MixDom K*F=4 (22 states)
};

// ---- launchers of the quad-per-warp block kernels, one per padded state count
// kind: as for the warp kernels
using BlockLauncher = int (*)(phmm_plan *, KParams &, int, int, int, cudaStream_t);

template <class SH>
int launch_block(phmm_plan *plan, KParams &K, int n_items, int max_ly, int kind, cudaStream_t stream);

struct BlockShapeEntry { int ns; BlockLauncher fn; };
const BlockShapeEntry kBlockShapes[] = {
    {12, launch_block<blk::BShape<12>>},   // TKF91/92, MixDom K*F=1..2 with few states
    {20, launch_block<blk::BShape<20>>},   // MixDom K*F=3 (17 states)
    {24, launch_block<blk::BShape<24>>},   // MixDom K*F=4 (22 states)
    {44, launch_block<blk::BShape<44>>},   // MixDom K*F=8 (42 states)
};

BlockLauncher find_block_launcher(int ns) {
    for (const auto &e : kBlockShapes)
        if (e.ns == ns) return e.fn;
    return nullptr;
}

WarpLauncher find_warp_launcher(int nm, int ni, int nd) {
    for (const auto &e : kWarpShapes)
        if (e.nm == nm && e.ni == ni && e.nd == nd) return e.fn;
    return nullptr;
}

// ---- factored MixDom transitions (phmm_batch.nest)
int64_t nest_record_len(int K, int F) { return 20LL * K * F + 25LL * K * F * F; }

// the wide kernels contract through the record where one quad of slots is one
// (domain, sub-state) block: F = 4, the type groups in state order (MM_d; MI_d,
// II_d per domain; MD_d, DD_d per domain), the start state after them
bool wide_nest_layout(const KParams &K, int nK, int nF) {
    if (nF != 4 || nK < 1 || K.N != 2 + 20 * nK) return false;
    if (K.kbeg[0] != 0 || K.kend[0] != 4 * nK || K.kbeg[1] != 4 * nK || K.kend[1] != 12 * nK ||
        K.kbeg[2] != 12 * nK || K.kend[2] != 20 * nK || K.s_slot < 20 * nK)
        return false;
    for (int q = 0; q < 5 * nK; ++q) {
        int d, uv;
        if (q < nK) { d = q; uv = 0; }
        else if (q < 3 * nK) { const int i = q - nK; d = i / 2; uv = (i & 1) ? 3 : 1; }
        else { const int i = q - 3 * nK; d = i / 2; uv = (i & 1) ? 4 : 2; }
        for (int u = 0; u < 4; ++u)
            if (K.slot_orig[4 * q + u] != 2 + d * 20 + uv * 4 + u) return false;
    }
    return true;
}

// (K, F) layouts with a nested instantiation of the two-warp stripes
bool has_nest_tw(int nm, int K, int F) { return nm == 3 && K == 3 && F == 1; }

// the record must describe the plan's state space, and the plan's two-warp
// slot order must be the canonical MixDom order the nested kernels assume
// (M states, then I, then D, each in state order)
int check_nest(const phmm_plan *plan, const phmm_batch *b) {
    const int K = b->nest_dom, F = b->nest_frag;
    if (K < 1 || F < 1 || plan->base.N != 2 + 5 * K * F || plan->w_nm != K * F || plan->w_ni != 2 * K * F ||
        plan->w_nd != 2 * K * F)
        return fail(PHMM_E_ARG, "phmm_batch.nest: nest_dom / nest_frag do not match the plan's MixDom state space");
    const int NM = K * F, NI = 2 * K * F, NE = 5 * K * F;
    for (int s = 0; s < NE; ++s) {
        int d, u, f;
        if (s < NM) { d = s / F; u = 0; f = s % F; }
        else if (s < NM + NI) { const int w = (s - NM) % (2 * F); d = (s - NM) / (2 * F); u = w < F ? 1 : 3; f = w % F; }
        else { const int w = (s - NM - NI) % (2 * F); d = (s - NM - NI) / (2 * F); u = w < F ? 2 : 4; f = w % F; }
        if (plan->base.w_orig[s] != 2 + d * 5 * F + u * F + f)
            return fail(PHMM_E_ARG, "phmm_batch.nest: the plan's state types are not the MixDom layout "
                                    "(state 2 + d*5F + uv*F + f)");
    }
    return 0;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// The split E-step: forward on the caller's stream and backward recursion on
// a side stream at the same time, then the count pass once both are done.
// side streams (and fork / join events) of one caller stream, created once
int get_side(phmm_plan *plan, cudaStream_t stream, bool prio, phmm_plan::Side **out) {
    for (auto &e : plan->sides)
        if (e.user == stream && e.prio == prio) { *out = &e; return 0; }
    phmm_plan::Side e{};
    e.user = stream;
    e.prio = prio;
    int least = 0, greatest = 0;
    if (prio) CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CUDA_TRY(cudaStreamCreateWithPriority(&e.side, cudaStreamNonBlocking, greatest));
    CUDA_TRY(cudaStreamCreateWithPriority(&e.side2, cudaStreamNonBlocking, least));
    CUDA_TRY(cudaStreamCreateWithPriority(&e.side3, cudaStreamNonBlocking, least));
    if (prio) CUDA_TRY(cudaStreamCreateWithPriority(&e.sidef, cudaStreamNonBlocking, greatest));
    CUDA_TRY(cudaEventCreateWithFlags(&e.fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e.join, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e.join2, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e.join3, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e.fwd_done, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e.joinf, cudaEventDisableTiming));
    plan->sides.push_back(e);
    *out = &plan->sides.back();
    return 0;
}

int launch_split(phmm_plan *plan, KParams K, WarpLauncher wl, bool combined, int n_items, int n_citems, int stripes,
                 int max_ly, void *d_items, int *d_counters, int *d_progress, float *d_bedge, int *d_bedge_exp,
                 cudaStream_t stream) {
    int rc;
    const phmm_tuning &tu = plan->tuning;
    // the count pass of the warp kernels (second side stream) overlaps the
    // wavefronts: its items wait for the stripes they read and its grid takes
    // half the resident slots (or tu.count_per_sm CTAs per SM; none at 0)
    KParams C = K;
    C.items = (const int2 *)d_items + 2 * n_items;
    C.n_items = n_citems;
    C.counter = d_counters + 2;
    C.progress = d_progress;
    C.bprogress = d_progress + stripes;
    C.count_wait = 1;
    C.wave_ctr = d_counters;
    if (combined) {
        // one persistent launch pops forward and backward stripes from one list
        KParams FB = K;
        FB.items = (const int2 *)d_items;
        FB.n_items = 2 * n_items;
        FB.counter = d_counters;
        FB.progress = d_progress;
        FB.bprogress = d_progress + stripes;
        FB.bedge = d_bedge;
        FB.bedge_exp = d_bedge_exp;
        // the count pass follows on the same stream: a 256-thread count CTA
        // holds half an SM's registers, so count CTAs waiting beside the
        // wavefront kernel could crowd it out of the SMs
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[0], stream));
        plan->launch_per_sm = tu.wave_per_sm;
        rc = wl(plan, FB, 2 * n_items, max_ly, 4, stream);
        plan->launch_per_sm = 0;
        if (rc) return rc;
        if (plan->timing) {
            CUDA_TRY(cudaEventRecord(plan->ev[1], stream));
            CUDA_TRY(cudaEventRecord(plan->ev[2], stream));
            CUDA_TRY(cudaEventRecord(plan->ev[3], stream));
        }
        C.count_wait = 0;
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[4], stream));
        if ((rc = wl(plan, C, n_citems, max_ly, 3, stream))) return rc;
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[5], stream));
        plan->launches += 2;
        plan->timed_bwd = true;
        plan->timed_count = true;
        return 0;
    }
    phmm_plan::Side *sd = nullptr;
    const bool prio = tu.priorities != 0;
    if ((rc = get_side(plan, stream, prio, &sd))) return rc;
    CUDA_TRY(cudaEventRecord(sd->fork, stream));
    CUDA_TRY(cudaStreamWaitEvent(sd->side, sd->fork, 0));
    CUDA_TRY(cudaStreamWaitEvent(sd->side2, sd->fork, 0));
    CUDA_TRY(cudaStreamWaitEvent(sd->side3, sd->fork, 0));
    // forward: on the caller's stream, or with priorities on a greatest-priority side stream
    cudaStream_t fs = stream;
    if (prio) {
        fs = sd->sidef;
        CUDA_TRY(cudaStreamWaitEvent(fs, sd->fork, 0));
    }
    KParams F = K;
    F.items = (const int2 *)d_items;
    F.n_items = n_items;
    F.counter = d_counters;
    F.progress = d_progress;
    F.blat = nullptr;
    F.blat_exp = nullptr;
    // the two wavefronts share the GPU: each persistent grid takes half the
    // resident slots (or tu.wave_per_sm CTAs per SM), so neither waits for
    // the other to drain
    plan->grid_div = 2;
    plan->launch_per_sm = tu.wave_per_sm;
    const int kf = plan->two_warp ? 5 : 0, kb = plan->two_warp ? 6 : 2;
    auto reset = [&]() { plan->grid_div = 1; plan->launch_per_sm = 0; };
    if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[0], fs));
    if ((rc = wl(plan, F, n_items, max_ly, kf, fs))) { reset(); return rc; }
    if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[1], fs));
    CUDA_TRY(cudaEventRecord(sd->fwd_done, fs));
    // backward recursion (side stream): own edge rows and progress counters
    KParams B = K;
    B.items = (const int2 *)d_items + n_items;
    B.n_items = n_items;
    B.counter = d_counters + 1;
    B.progress = d_progress + stripes;
    B.edge = d_bedge;
    B.edge_exp = d_bedge_exp;
    B.lat = nullptr;
    B.lat_exp = nullptr;
    if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[2], sd->side));
    rc = wl(plan, B, n_items, max_ly, kb, sd->side);
    reset();
    if (rc) return rc;
    if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[3], sd->side));
    CUDA_TRY(cudaEventRecord(sd->join, sd->side));
    // counts from both lattices (second side stream, overlapping the wavefronts)
    int launched = 3;
    if (tu.count_per_sm != 0) {
        plan->grid_div = 2;
        plan->launch_per_sm = tu.count_per_sm > 0 ? tu.count_per_sm : 0;
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[4], sd->side2));
        rc = wl(plan, C, n_citems, max_ly, 3, sd->side2);
        reset();
        if (rc) return rc;
        ++launched;
    }
    CUDA_TRY(cudaEventRecord(sd->join2, sd->side2));
    // the overlapped grid holds part of the slots; once both wavefronts are
    // done a second, full-size grid pops the remaining count items from the
    // same counter (all of them ready, so it waits on nothing)
    CUDA_TRY(cudaStreamWaitEvent(sd->side3, sd->fwd_done, 0));
    CUDA_TRY(cudaStreamWaitEvent(sd->side3, sd->join, 0));
    KParams C2 = C;
    C2.count_wait = 0;
    if (plan->timing && tu.count_per_sm == 0) CUDA_TRY(cudaEventRecord(plan->ev[4], sd->side3));
    if ((rc = wl(plan, C2, n_citems, max_ly, 3, sd->side3))) return rc;
    CUDA_TRY(cudaEventRecord(sd->join3, sd->side3));
    if (prio) CUDA_TRY(cudaStreamWaitEvent(stream, sd->fwd_done, 0));
    CUDA_TRY(cudaStreamWaitEvent(stream, sd->join, 0));
    CUDA_TRY(cudaStreamWaitEvent(stream, sd->join2, 0));
    CUDA_TRY(cudaStreamWaitEvent(stream, sd->join3, 0));
    if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[5], stream));
    plan->launches += launched;
    plan->timed_bwd = true;
    plan->timed_count = true;
    return 0;
}

// The wide kernels (estep_wide.cuh): forward and backward recursion in one
// persistent launch, then the count pass; lattice and edge records of NS + 4
// floats per cell (values, exponent, maximum).
int run_wide(phmm_plan *plan, const phmm_batch *b, bool estep, double *ll, double *n_trans, double *cntM,
             double *cntI, double *cntD, int32_t *status, cudaStream_t stream, void *ws, size_t ws_bytes,
             size_t *ws_need) {
    KParams K = plan->base;
    const int P_ = b->n_pairs, N = K.N, G = K.G, NS = K.NS;
    const int KS = K.kend[2], NQd = KS / 4, NQ = NS / 4;
    const int ES = wide::ls_of(NS);
    const int rows = wide::RW;
    if (NQd > 48 || ((NQ + wide::SPL - 1) / wide::SPL) * NQd > wide::CT * wide::CTPT)
        return fail(PHMM_E_ARG, "state space too large for the wide kernels");
    if (!ws_need) plan->last_variant = 6;
    // forward contraction on the tensor cores (phmm_tuning.tensor), for
    // forward-only calls: a warp's 16 destinations form its m16n8 tiles, so
    // every warp needs four whole destination quads of one type.  (In an
    // E-step the forward's 3xTF32 rounding no longer cancels against the
    // float32 backward's: counts went 1e-3 off at 162 states.)
    bool tc = !estep && plan->tuning.tensor != 0 && NQd % 4 == 0;
    for (int w = 0; tc && w < NQd / 4; ++w)
        for (int q = 1; q < 4; ++q)
            if (K.quad_type[4 * w + q] != K.quad_type[4 * w]) tc = false;
    auto fb_kernel = tc ? wide::fwdbwd_wide_kernel<true> : wide::fwdbwd_wide_kernel<false>;
    auto f_kernel = tc ? wide::forward_wide_kernel<true> : wide::forward_wide_kernel<false>;
    // factored MixDom transitions (phmm_batch.nest): the wide_nest kernels where
    // the slot layout allows (checked per plan) and neither the tensor-core
    // forward nor stripe-edge checkpointing is asked for (decided below)
    if (b->nest) {
        const int rc = check_nest(plan, b);
        if (rc) return rc;
    }
    bool wnest = b->nest && !tc && wide_nest_layout(K, b->nest_dom, b->nest_frag);
    std::vector<int> order(P_);
    for (int p = 0; p < P_; ++p) {
        if (b->Lx_host[p] < 0 || b->Ly_host[p] < 0) return fail(PHMM_E_ARG, "negative length");
        order[p] = p;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return (int64_t)(b->Lx_host[a] + 1) * (b->Ly_host[a] + 1) >
               (int64_t)(b->Lx_host[c] + 1) * (b->Ly_host[c] + 1);
    });
    plan->h_meta.resize(P_);
    int64_t lat_cells = 0, edge_cells = 0;
    int stripes = 0, max_ly = 0;
    for (int p = 0; p < P_; ++p) {
        PairMeta &m = plan->h_meta[p];
        m.Lx = b->Lx_host[p];
        m.Ly = b->Ly_host[p];
        m.x_off = b->x_off_host[p];
        m.y_off = b->y_off_host[p];
        m.n_stripes = (m.Lx + 1 + rows - 1) / rows;
        m.stripe_base = stripes;
        m.lat_base = lat_cells;
        m.edge_base = edge_cells;
        m.tab_base = 0;
        stripes += m.n_stripes;
        if (estep) lat_cells += (int64_t)m.n_stripes * (rows + m.Ly) * rows;
        edge_cells += (int64_t)m.n_stripes * (m.Ly + 1);
        max_ly = std::max(max_ly, m.Ly);
    }
    // work lists: forward / backward stripes interleaved, then the count items
    plan->h_items.clear();
    std::vector<int2> fw, bw;
    for (int p : order)
        for (int s = 0; s < plan->h_meta[p].n_stripes; ++s) fw.push_back(make_int2(p, s));
    for (int p : order)
        for (int s = plan->h_meta[p].n_stripes - 1; s >= 0; --s) bw.push_back(make_int2(p, s | blk::BWD_ITEM));
    const int n_items = (int)fw.size();
    // Stripe-edge checkpointing (E-step): the wavefronts keep no lattice, only
    // the edge rows every RW rows (their halo exchange) and the log-likelihood;
    // the count pass then runs in groups of stripes, each stripe's forward and
    // backward recursion recomputed from the edge rows above and below it into
    // a group scratch first.  Scratch: O(edge rows + group) instead of
    // O(lattice).  On with tuning.checkpoint = 1; automatic (0) when one pair's
    // two lattices alone exceed 40 % of the device's memory (a batch that is
    // only too large as a whole runs in groups of pairs, which is faster).
    bool ckpt = false;
    if (estep) {
        int64_t big = 0;
        for (int p = 0; p < P_; ++p) {
            const PairMeta &m = plan->h_meta[p];
            big = std::max(big, (int64_t)m.n_stripes * (rows + m.Ly) * rows);
        }
        const double pair_bytes = 2.0 * sizeof(float) * (double)big * ES;
        ckpt = plan->tuning.checkpoint == 1 ||
               (plan->tuning.checkpoint == 0 && pair_bytes > 0.4 * (double)plan->total_mem);
    }
    if (ckpt) wnest = false;   // the recompute passes run the dense kernels
    struct CkGroup { size_t rc_off, n_rc, c_off, n_c; };
    std::vector<CkGroup> groups;
    int64_t grp_cells = 0;   // scratch cells of the largest group (each lattice)
    plan->h_stripe_lat.clear();
    if (estep) {
        for (int i = 0; i < n_items; ++i) { plan->h_items.push_back(fw[i]); plan->h_items.push_back(bw[i]); }
        if (!ckpt) {
            for (auto it = order.rbegin(); it != order.rend(); ++it)   // shortest pairs first (ready first)
                for (int s = 0; s < plan->h_meta[*it].n_stripes; ++s)
                    for (int h = 0; h < wide::SPL; ++h) plan->h_items.push_back(make_int2(*it, (s << 4) | h));
        } else {
            // groups of one wave of the recompute kernel (two items per stripe,
            // forward and backward), longest pairs first
            const int threads = 32 * ((NQd + 3) / 4);
            const int rbytes = std::max(wide::make_smem_wd(NS, KS, max_ly, false).bytes,
                                        wide::make_smem_wd(NS, KS, max_ly, true).bytes);
            CUDA_TRY(cudaFuncSetAttribute(fb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, rbytes));
            int rocc = 0;
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rocc, fb_kernel, threads, rbytes));
            const int gmax = std::max(1, plan->sm_count * std::max(rocc, 1) / 2);
            std::vector<int2> members;
            auto close = [&]() {
                if (members.empty()) return;
                CkGroup g;
                std::vector<int64_t> tab(stripes, -1);
                int64_t off = 0;
                g.rc_off = plan->h_items.size();
                for (const int2 &st : members) {
                    const PairMeta &m = plan->h_meta[st.x];
                    tab[m.stripe_base + st.y] = off;
                    off += (int64_t)(rows + m.Ly) * rows;
                    plan->h_items.push_back(make_int2(st.x, st.y));
                    plan->h_items.push_back(make_int2(st.x, st.y | blk::BWD_ITEM));
                }
                g.n_rc = plan->h_items.size() - g.rc_off;
                g.c_off = plan->h_items.size();
                for (const int2 &st : members)
                    for (int h = 0; h < wide::SPL; ++h) plan->h_items.push_back(make_int2(st.x, (st.y << 4) | h));
                g.n_c = plan->h_items.size() - g.c_off;
                plan->h_stripe_lat.insert(plan->h_stripe_lat.end(), tab.begin(), tab.end());
                grp_cells = std::max(grp_cells, off);
                groups.push_back(g);
                members.clear();
            };
            for (int p : order)
                for (int s = 0; s < plan->h_meta[p].n_stripes; ++s) {
                    members.push_back(make_int2(p, s));
                    if ((int)members.size() == gmax) close();
                }
            close();
        }
    } else {
        plan->h_items = fw;
    }
    if (!ws_need) plan->ckpt_groups = (int)groups.size();
    const int n_fb = estep ? 2 * n_items : n_items;
    const int n_citems = estep ? n_items * wide::SPL : 0;
    if (ckpt) lat_cells = grp_cells;   // the lattices are one group's scratch
    // ---- scratch
    const size_t o_meta = 0;
    const size_t o_items = align256(o_meta + sizeof(PairMeta) * P_);
    const size_t o_cnt = align256(o_items + sizeof(int2) * plan->h_items.size());
    const size_t o_prog = align256(o_cnt + 4 * sizeof(int));
    const size_t o_edge = align256(o_prog + sizeof(int) * 2 * (size_t)stripes);
    const size_t o_bedge = align256(o_edge + sizeof(float) * (size_t)edge_cells * ES);
    const size_t o_lat = align256(o_bedge + (estep ? sizeof(float) * (size_t)edge_cells * ES : 0));
    const size_t o_blat = align256(o_lat + (estep ? sizeof(float) * (size_t)lat_cells * ES : 0));
    const size_t o_slat = align256(o_blat + (estep ? sizeof(float) * (size_t)lat_cells * ES : 0));
    const size_t need = align256(o_slat + sizeof(int64_t) * plan->h_stripe_lat.size());
    if (ws_need) { *ws_need = need; return 0; }
    void *d_meta, *d_items;
    int *d_counters, *d_progress;
    float *d_edge, *d_bedge = nullptr, *d_lat = nullptr, *d_blat = nullptr;
    int64_t *d_slat = nullptr;
    int rc;
    if (ws) {
        if (ws_bytes < need) {
            char msg[200];
            snprintf(msg, sizeof msg, "workspace of %zu bytes is too small: this batch needs %zu bytes", ws_bytes, need);
            return fail(PHMM_E_ARG, msg);
        }
        unsigned char *w = (unsigned char *)ws;
        d_meta = w + o_meta;
        d_items = w + o_items;
        d_counters = (int *)(w + o_cnt);
        d_progress = (int *)(w + o_prog);
        d_edge = (float *)(w + o_edge);
        if (estep) {
            d_bedge = (float *)(w + o_bedge);
            d_lat = (float *)(w + o_lat);
            d_blat = (float *)(w + o_blat);
        }
        if (ckpt) d_slat = (int64_t *)(w + o_slat);
    } else {
        if ((rc = ensure((char **)&plan->meta, &plan->meta_cap, sizeof(PairMeta) * P_))) return rc;
        if ((rc = ensure((char **)&plan->items, &plan->items_cap, sizeof(int2) * plan->h_items.size()))) return rc;
        if ((rc = ensure(&plan->edge, &plan->edge_cap, (size_t)edge_cells * ES))) return rc;
        if ((rc = ensure(&plan->progress, &plan->prog_cap, (size_t)2 * stripes))) return rc;
        if (estep) {
            if ((rc = ensure(&plan->bedge, &plan->bedge_cap, (size_t)edge_cells * ES))) return rc;
            if ((rc = ensure(&plan->lat, &plan->lat_cap, (size_t)lat_cells * ES))) return rc;
            if ((rc = ensure(&plan->blat, &plan->blat_cap, (size_t)lat_cells * ES))) return rc;
        }
        if (ckpt) {
            if ((rc = ensure(&plan->slat, &plan->slat_cap, plan->h_stripe_lat.size()))) return rc;
            d_slat = plan->slat;
        }
        d_meta = plan->meta;
        d_items = plan->items;
        d_counters = plan->counters;
        d_progress = plan->progress;
        d_edge = plan->edge;
        d_bedge = plan->bedge;
        d_lat = plan->lat;
        d_blat = plan->blat;
    }
    if (plan->desc_mode != 2) {   // the work description (launch-only calls find it in the workspace)
        CUDA_TRY(cudaMemcpyAsync(d_meta, plan->h_meta.data(), sizeof(PairMeta) * P_, cudaMemcpyHostToDevice,
                                 stream));
        CUDA_TRY(cudaMemcpyAsync(d_items, plan->h_items.data(), sizeof(int2) * plan->h_items.size(),
                                 cudaMemcpyHostToDevice, stream));
        if (ckpt)
            CUDA_TRY(cudaMemcpyAsync(d_slat, plan->h_stripe_lat.data(), sizeof(int64_t) * plan->h_stripe_lat.size(),
                                     cudaMemcpyHostToDevice, stream));
    }
    if (plan->desc_mode == 1) return 0;
    CUDA_TRY(cudaMemsetAsync(d_counters, 0, 3 * sizeof(int), stream));
    CUDA_TRY(cudaMemsetAsync(d_progress, 0, sizeof(int) * 2 * stripes, stream));
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int32_t) * P_, stream));
    if (estep) {
        CUDA_TRY(cudaMemsetAsync(n_trans, 0, sizeof(double) * (size_t)P_ * N * N, stream));
        CUDA_TRY(cudaMemsetAsync(cntM, 0, sizeof(double) * (size_t)P_ * G * 441, stream));
        CUDA_TRY(cudaMemsetAsync(cntI, 0, sizeof(double) * (size_t)P_ * G * 21, stream));
        CUDA_TRY(cudaMemsetAsync(cntD, 0, sizeof(double) * (size_t)P_ * G * 21, stream));
    }
    K.res = b->residues;
    K.meta = (const PairMeta *)d_meta;
    K.chi = b->chi;
    K.chi_stride = b->chi_per_pair ? (int64_t)N * N : 0;
    K.eM = b->emit_M;
    K.eI = b->emit_I;
    K.eD = b->emit_D;
    K.eM_stride = b->emit_per_pair ? (int64_t)G * 441 : 0;
    K.eID_stride = b->emit_per_pair ? (int64_t)G * 21 : 0;
    K.lat = ckpt ? nullptr : d_lat;      // checkpointed: the wavefronts write edge rows only
    K.lat_exp = nullptr;
    K.blat = ckpt ? nullptr : d_blat;
    K.blat_exp = nullptr;
    K.edge = d_edge;
    K.edge_exp = nullptr;
    K.bedge = d_bedge;
    K.bedge_exp = nullptr;
    K.progress = d_progress;
    K.bprogress = d_progress + stripes;
    K.stripe_lat = nullptr;
    K.recompute = 0;
    K.ckpt = 0;
    K.ll = ll;
    K.status = status;
    K.n_trans = n_trans;
    K.cntM = cntM;
    K.cntI = cntI;
    K.cntD = cntD;
    K.F_log = K.B_log = K.post = nullptr;
    K.max_ly = max_ly;
    K.spin_limit = plan->spin_limit > 0 ? plan->spin_limit : kSpinLimit;
    K.wave_ctr = nullptr;
    K.cmask = nullptr;
    K.srange = nullptr;
    K.beam_scale = 0.f;
    // ---- wavefronts, then the count pass (both on the caller's stream: a wide
    // wavefront CTA needs most of an SM's shared memory, so a count CTA waiting
    // beside it would only take its place)
    {
        K.items = (const int2 *)d_items;
        K.n_items = n_fb;
        K.counter = d_counters;
        const int threads = 32 * ((NQd + 3) / 4);
        int bytes = std::max(wide::make_smem_wd(NS, KS, max_ly, false).bytes,
                             estep ? wide::make_smem_wd(NS, KS, max_ly, true).bytes : 0);
        auto kern = estep ? fb_kernel : f_kernel;
        if (wnest) {   // the factored contraction: no dense chi in shared memory
            K.nest = b->nest;
            K.nest_stride = b->chi_per_pair ? nest_record_len(b->nest_dom, b->nest_frag) : 0;
            K.nest_K = b->nest_dom;
            K.nest_F = b->nest_frag;
            kern = estep ? wide::wide_nest_kernel<false> : wide::wide_nest_kernel<true>;
            bytes = std::max(wide::make_smem_wn(NS, KS, max_ly, false).bytes,
                             estep ? wide::make_smem_wn(NS, KS, max_ly, true).bytes : 0);
        }
        CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        int occ = 0;
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, bytes));
        if (occ < 1) return fail(PHMM_E_ARG, "wide kernel does not fit on an SM (shared memory)");
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[0], stream));
        const int per_sm = plan->tuning.wave_per_sm > 0 ? std::min(plan->tuning.wave_per_sm, occ) : occ;
        kern<<<std::min(n_fb, plan->sm_count * per_sm), threads, bytes, stream>>>(K);
        CUDA_TRY(cudaGetLastError());
        if (plan->timing) {
            CUDA_TRY(cudaEventRecord(plan->ev[1], stream));
            CUDA_TRY(cudaEventRecord(plan->ev[2], stream));
            CUDA_TRY(cudaEventRecord(plan->ev[3], stream));
        }
        plan->launches++;
    }
    // ---- counts (checkpointed: per group, the group's stripes recomputed first)
    if (estep) {
        K.count_wait = 0;
        const int bytes = wide::make_smem_wc(NS, KS, K.kend[0] - K.kbeg[0], K.kend[1] - K.kbeg[1],
                                             K.kend[2] - K.kbeg[2]).bytes;
        CUDA_TRY(cudaFuncSetAttribute(wide::count_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        int occ = 0;
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, wide::count_wide_kernel, wide::CT, bytes));
        if (occ < 1) return fail(PHMM_E_ARG, "wide count kernel does not fit on an SM (shared memory)");
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[4], stream));
        if (!ckpt) {
            K.items = (const int2 *)d_items + n_fb;
            K.n_items = n_citems;
            K.counter = d_counters + 2;
            wide::count_wide_kernel<<<std::min(n_citems, plan->sm_count * occ), wide::CT, bytes, stream>>>(K);
            CUDA_TRY(cudaGetLastError());
            plan->launches++;
        } else {
            const int threads = 32 * ((NQd + 3) / 4);
            const int rbytes = std::max(wide::make_smem_wd(NS, KS, max_ly, false).bytes,
                                        wide::make_smem_wd(NS, KS, max_ly, true).bytes);
            int rocc = 0;
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rocc, fb_kernel, threads, rbytes));
            if (rocc < 1) return fail(PHMM_E_ARG, "wide kernel does not fit on an SM (shared memory)");
            K.lat = d_lat;
            K.blat = d_blat;
            for (size_t gi = 0; gi < groups.size(); ++gi) {
                const CkGroup &g = groups[gi];
                K.stripe_lat = d_slat + gi * (size_t)stripes;
                CUDA_TRY(cudaMemsetAsync(d_counters, 0, 2 * sizeof(int), stream));
                // recompute the group's stripes (both directions) from the edge rows
                K.recompute = 1;
                K.ckpt = 0;
                K.items = (const int2 *)d_items + g.rc_off;
                K.n_items = (int)g.n_rc;
                K.counter = d_counters;
                fb_kernel<<<std::min((int)g.n_rc, plan->sm_count * rocc), threads, rbytes, stream>>>(K);
                CUDA_TRY(cudaGetLastError());
                // counts of the group from its scratch lattices
                K.recompute = 0;
                K.ckpt = 1;
                K.items = (const int2 *)d_items + g.c_off;
                K.n_items = (int)g.n_c;
                K.counter = d_counters + 1;
                wide::count_wide_kernel<<<std::min((int)g.n_c, plan->sm_count * occ), wide::CT, bytes, stream>>>(K);
                CUDA_TRY(cudaGetLastError());
                plan->launches += 2;
            }
        }
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[5], stream));
    }
    plan->timed_bwd = estep;
    plan->timed_count = estep;
    return 0;
}

// One call of the forward (estep false) or E-step kernels.  Scratch comes from
// the plan (grown on demand) unless the caller passes a workspace `ws` of
// `ws_bytes`; with `ws_need` set, nothing runs and the workspace size the
// call would need is stored there (only the host fields of the batch are read).
// An NVTX range for the host side of one call (visible to a profiler that
// attaches one; a pointer check otherwise).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

int run_core(phmm_plan *plan, const phmm_batch *b, bool estep, double *ll, double *n_trans,
             double *cntM, double *cntI, double *cntD, int32_t *status, double *F_log, double *B_log,
             double *post, void *stream_, void *ws, size_t ws_bytes, size_t *ws_need) {
    if (!plan || !b) return fail(PHMM_E_ARG, "null plan or batch");
    cudaStream_t stream = (cudaStream_t)stream_;
    if (!ws_need) plan->launches = 0;
    plan->grouped = false;
    const int P_ = b->n_pairs;
    if (P_ < 0) return fail(PHMM_E_ARG, "n_pairs < 0");
    if (ws_need) *ws_need = 0;
    if (P_ == 0) return 0;
    if (!b->Lx_host || !b->Ly_host || !b->x_off_host || !b->y_off_host)
        return fail(PHMM_E_ARG, "null batch length or offset array");
    if (!ws_need && plan->desc_mode != 1) {
        if (!b->residues || !b->chi || !b->emit_M || !b->emit_I || !b->emit_D || !ll || !status)
            return fail(PHMM_E_ARG, "null batch pointer");
        if (estep && (!n_trans || !cntM || !cntI || !cntD)) return fail(PHMM_E_ARG, "null E-step output");
        if (ws && ((uintptr_t)ws & 255)) return fail(PHMM_E_ARG, "workspace must be 256-byte aligned");
    }
    KParams K = plan->base;
    const int N = K.N, G = K.G;
    const bool masked = b->cell_mask != nullptr;
    const bool beam = b->beam_log_width > 0.0;
    if (b->beam_log_width < 0.0 || b->beam_log_width != b->beam_log_width)
        return fail(PHMM_E_ARG, "beam_log_width must be >= 0 (0 = no pruning)");
    if ((masked || beam) && (K.NS > GMAXS || plan->variant == 6))
        return fail(PHMM_E_ARG, "cell masks and beam pruning need a state space of at most 60 emitting states");
    if (masked && plan->variant >= 2 && plan->variant <= 5)
        return fail(PHMM_E_ARG, "cell masks run on the generic (1) or two-warp (7) kernels only");
    if (beam && plan->variant >= 2)
        return fail(PHMM_E_ARG, "beam pruning runs on the generic kernels (variant 1) only");
    // large state spaces (more than 64 padded slots) run on the wide kernels
    if (K.NS > GMAXS || plan->variant == 6) {
        if (F_log || B_log || post)
            return fail(PHMM_E_ARG, "lattice tables are not available for state spaces of more than 60 emitting states");
        return run_wide(plan, b, estep, ll, n_trans, cntM, cntI, cntD, status, stream, ws, ws_bytes, ws_need);
    }
    // kernel family: register-resident warp kernels when the shape has one and
    // no lattice tables are requested; the generic quad kernels otherwise
    WarpLauncher wl = nullptr;
    BlockLauncher bl = nullptr;
    bool split = false;   // E-step as forward || backward recursion, then counts
    const bool tables = F_log || B_log || post;
    // automatic choice (measured on GB300): the two-warp stripe kernels where
    // the state space has a compiled warp shape -- the split E-step at 17
    // states takes 2.95 ms per 200-pair batch against 3.5 ms on one-warp
    // stripes and 8.7 ms on the block kernels; the TKF91 forward takes 0.21 ms
    // per 64-pair batch against 0.30 ms on the block kernels -- else the block
    // kernels
    bool two_warp = false;
    if (!tables && plan->variant == 0 && !beam) {
        if (estep) {
            wl = find_warp_launcher(plan->w_nm, plan->w_ni, plan->w_nd);
            if (!wl && !masked) bl = find_block_launcher(K.NS);
            split = wl != nullptr || bl != nullptr;
            two_warp = wl != nullptr;
        } else {   // forward only: the two-warp stripes where the shape has them
            wl = find_warp_launcher(plan->w_nm, plan->w_ni, plan->w_nd);
            two_warp = wl != nullptr;
            if (!wl && !masked) bl = find_block_launcher(K.NS);
        }
    }
    if (!tables && (plan->variant == 3 || plan->variant == 5)) bl = find_block_launcher(K.NS);
    if (!tables && plan->variant == 5) split = estep && bl != nullptr;
    if (!tables && (plan->variant == 2 || plan->variant == 4)) wl = find_warp_launcher(plan->w_nm, plan->w_ni, plan->w_nd);
    if (!tables && plan->variant == 4) split = estep && wl != nullptr;
    if (!tables && plan->variant == 7) {
        wl = find_warp_launcher(plan->w_nm, plan->w_ni, plan->w_nd);
        split = estep && wl != nullptr;
        two_warp = wl != nullptr;
    }
    if ((plan->variant == 2 || plan->variant == 4 || plan->variant == 7) && !wl)
        return fail(PHMM_E_ARG, "no warp kernel for this state space");
    if ((plan->variant == 3 || plan->variant == 5) && !bl) return fail(PHMM_E_ARG, "no block kernel for this state space");
    const int rows = bl ? blk::ROWS : (wl ? warp2::ROWS : TH);
    const int stride = bl ? K.NS : (wl ? ((plan->w_nm + plan->w_ni + plan->w_nd + 1 + 3) & ~3) : K.NS);
    const int estride = bl ? blk::nbp_of(K.NS / 4) : 1;   // exponents per cell
    if (!ws_need) {
        plan->last_variant = two_warp ? 7 : (bl ? (split ? 5 : 3) : (split ? 4 : (wl ? 2 : 1)));
        plan->two_warp = two_warp;
    }
    // factored transitions: checked against the plan's state space; used by
    // the two-warp stripes (unmasked) where the shape has an instantiation
    if (b->nest) {
        const int rc = check_nest(plan, b);
        if (rc) return rc;
    }
    const bool use_nest = b->nest && two_warp && !masked && !beam && has_nest_tw(plan->w_nm, b->nest_dom, b->nest_frag);
    // ---- plan: stripes, offsets, longest-first order
    std::vector<int> order(P_);
    for (int p = 0; p < P_; ++p) {
        if (b->Lx_host[p] < 0 || b->Ly_host[p] < 0) return fail(PHMM_E_ARG, "negative length");
        order[p] = p;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return (int64_t)(b->Lx_host[a] + 1) * (b->Ly_host[a] + 1) >
               (int64_t)(b->Lx_host[c] + 1) * (b->Ly_host[c] + 1);
    });
    plan->h_meta.resize(P_);
    int64_t lat_cells = 0, edge_cells = 0, tab_cells = 0, row_cells = 0;
    int stripes = 0, max_ly = 0;
    for (int p = 0; p < P_; ++p) {
        PairMeta &m = plan->h_meta[p];
        m.Lx = b->Lx_host[p];
        m.Ly = b->Ly_host[p];
        m.x_off = b->x_off_host[p];
        m.y_off = b->y_off_host[p];
        m.n_stripes = (m.Lx + 1 + rows - 1) / rows;
        m.stripe_base = stripes;
        m.lat_base = lat_cells;
        m.edge_base = edge_cells;
        m.tab_base = tab_cells;
        m.row_base = row_cells;
        row_cells += m.Lx + 1;
        stripes += m.n_stripes;
        if (estep) lat_cells += (int64_t)m.n_stripes * (rows + m.Ly) * rows;
        edge_cells += (int64_t)m.n_stripes * (m.Ly + 1);
        tab_cells += (int64_t)(m.Lx + 1) * (m.Ly + 1);
        max_ly = std::max(max_ly, m.Ly);
    }
    plan->h_items.clear();
    // stripe items in pop order; a stripe only waits on stripes of its pair
    // popped before it.  Unmasked: pair by pair, longest pairs first (a pair's
    // stripes all run at once, one behind the other, and the longest pairs set
    // the critical path).  Under a cell mask (two-warp kernels, which skip the
    // steps off each stripe's live columns): a narrow band keeps only a couple
    // of a pair's stripes busy at a time, so pair-by-pair order would park most
    // CTAs on stripes that cannot start yet -- there the items go stripe by
    // stripe (the first stripe of every pair, then the second, ...; the
    // backward from the last stripe up).
    const bool by_stripe = masked && two_warp;
    int max_stripes = 0;
    for (int p = 0; p < P_; ++p) max_stripes = std::max(max_stripes, plan->h_meta[p].n_stripes);
    if (by_stripe) {
        for (int s = 0; s < max_stripes; ++s)
            for (int p : order)
                if (s < plan->h_meta[p].n_stripes) plan->h_items.push_back(make_int2(p, s));
    } else {
        for (int p : order)
            for (int s = 0; s < plan->h_meta[p].n_stripes; ++s) plan->h_items.push_back(make_int2(p, s));
    }
    const int n_items = (int)plan->h_items.size();
    if (estep && by_stripe) {
        for (int k = 0; k < max_stripes; ++k)
            for (int p : order)
                if (k < plan->h_meta[p].n_stripes)
                    plan->h_items.push_back(make_int2(p, plan->h_meta[p].n_stripes - 1 - k));
    } else if (estep) {
        for (int p : order)
            for (int s = plan->h_meta[p].n_stripes - 1; s >= 0; --s) plan->h_items.push_back(make_int2(p, s));
    }
    int n_citems = 0;
    const int cch = warp2::CCH;
    if (split) {   // count chunks: (pair, stripe << 12 | chunk), shortest pairs first (ready first)
        for (auto it = order.rbegin(); it != order.rend(); ++it) {
            const int p = *it;
            const PairMeta &m = plan->h_meta[p];
            for (int s = 0; s < m.n_stripes; ++s) {
                const int nrows = std::min(rows, m.Lx + 1 - s * rows);
                const int nch = (nrows + m.Ly + cch - 1) / cch;
                if (nch > 4096 || s >= (1 << 19)) return fail(PHMM_E_ARG, "pair too long for the count chunk index");
                for (int c = 0; c < nch; ++c) plan->h_items.push_back(make_int2(p, (s << 12) | c));
                n_citems += nch;
            }
        }
        if (bl) {   // one launch runs both wavefronts: interleave the two lists
            std::vector<int2> both(2 * (size_t)n_items);
            for (int i = 0; i < n_items; ++i) {
                both[2 * i] = plan->h_items[i];
                both[2 * i + 1] = make_int2(plan->h_items[n_items + i].x, plan->h_items[n_items + i].y | blk::BWD_ITEM);
            }
            std::copy(both.begin(), both.end(), plan->h_items.begin());
        }
    }
    int rc;
    // masked two-warp calls: the stripes' live column ranges follow the items
    const size_t n_range = (masked && two_warp) ? (size_t)stripes : 0;
    // ---- scratch: plan-owned buffers, or carved from the caller's workspace
    const size_t o_meta = 0;
    const size_t o_items = align256(o_meta + sizeof(PairMeta) * P_);
    const size_t o_cnt = align256(o_items + sizeof(int2) * (plan->h_items.size() + n_range));
    const size_t o_prog = align256(o_cnt + 4 * sizeof(int));
    const size_t o_edge = align256(o_prog + sizeof(int) * 2 * (size_t)stripes);
    const size_t o_edgeE = align256(o_edge + sizeof(float) * (size_t)edge_cells * stride);
    const size_t o_lat = align256(o_edgeE + sizeof(int) * (size_t)edge_cells * estride);
    const size_t o_latE = align256(o_lat + (estep ? sizeof(float) * (size_t)lat_cells * stride : 0));
    const size_t o_blat = align256(o_latE + (estep ? sizeof(int) * (size_t)lat_cells * estride : 0));
    const size_t o_blatE = align256(o_blat + (split ? sizeof(float) * (size_t)lat_cells * stride : 0));
    const size_t o_bedge = align256(o_blatE + (split ? sizeof(int) * (size_t)lat_cells * estride : 0));
    const size_t o_bedgeE = align256(o_bedge + (split ? sizeof(float) * (size_t)edge_cells * stride : 0));
    const size_t need = align256(o_bedgeE + (split ? sizeof(int) * (size_t)edge_cells * estride : 0));
    if (ws_need) { *ws_need = need; return 0; }
    void *d_meta, *d_items;
    int *d_counters, *d_progress, *d_edge_exp, *d_lat_exp, *d_blat_exp = nullptr, *d_bedge_exp = nullptr;
    float *d_edge, *d_lat, *d_blat = nullptr, *d_bedge = nullptr;
    if (ws) {
        if (ws_bytes < need) {
            char msg[200];
            snprintf(msg, sizeof msg, "workspace of %zu bytes is too small: this batch needs %zu bytes", ws_bytes,
                     need);
            return fail(PHMM_E_ARG, msg);
        }
        unsigned char *w = (unsigned char *)ws;
        d_meta = w + o_meta;
        d_items = w + o_items;
        d_counters = (int *)(w + o_cnt);
        d_progress = (int *)(w + o_prog);
        d_edge = (float *)(w + o_edge);
        d_edge_exp = (int *)(w + o_edgeE);
        d_lat = estep ? (float *)(w + o_lat) : nullptr;
        d_lat_exp = estep ? (int *)(w + o_latE) : nullptr;
        if (split) {
            d_blat = (float *)(w + o_blat);
            d_blat_exp = (int *)(w + o_blatE);
            d_bedge = (float *)(w + o_bedge);
            d_bedge_exp = (int *)(w + o_bedgeE);
        }
    } else {
        if ((rc = ensure((char **)&plan->meta, &plan->meta_cap, sizeof(PairMeta) * P_))) return rc;
        if ((rc = ensure((char **)&plan->items, &plan->items_cap, sizeof(int2) * (plan->h_items.size() + n_range))))
            return rc;
        if ((rc = ensure(&plan->edge, &plan->edge_cap, (size_t)edge_cells * stride))) return rc;
        if ((rc = ensure(&plan->edge_exp, &plan->edgeE_cap, (size_t)edge_cells * estride))) return rc;
        if ((rc = ensure(&plan->progress, &plan->prog_cap, (size_t)2 * stripes))) return rc;
        if (estep) {
            if ((rc = ensure(&plan->lat, &plan->lat_cap, (size_t)lat_cells * stride))) return rc;
            if ((rc = ensure(&plan->lat_exp, &plan->latE_cap, (size_t)lat_cells * estride))) return rc;
        }
        d_meta = plan->meta;
        d_items = plan->items;
        d_counters = plan->counters;
        d_progress = plan->progress;
        d_edge = plan->edge;
        d_edge_exp = plan->edge_exp;
        d_lat = plan->lat;
        d_lat_exp = plan->lat_exp;
        if (split) {
            if ((rc = ensure(&plan->blat, &plan->blat_cap, (size_t)lat_cells * stride))) return rc;
            if ((rc = ensure(&plan->blat_exp, &plan->blatE_cap, (size_t)lat_cells * estride))) return rc;
            if ((rc = ensure(&plan->bedge, &plan->bedge_cap, (size_t)edge_cells * stride))) return rc;
            if ((rc = ensure(&plan->bedge_exp, &plan->bedgeE_cap, (size_t)edge_cells * estride))) return rc;
            d_blat = plan->blat;
            d_blat_exp = plan->blat_exp;
            d_bedge = plan->bedge;
            d_bedge_exp = plan->bedge_exp;
        }
    }
    if (plan->desc_mode != 2) {   // the work description (launch-only calls find it in the workspace)
        CUDA_TRY(cudaMemcpyAsync(d_meta, plan->h_meta.data(), sizeof(PairMeta) * P_, cudaMemcpyHostToDevice,
                                 stream));
        CUDA_TRY(cudaMemcpyAsync(d_items, plan->h_items.data(), sizeof(int2) * plan->h_items.size(),
                                 cudaMemcpyHostToDevice, stream));
    }
    if (plan->desc_mode == 1) return 0;
    CUDA_TRY(cudaMemsetAsync(d_counters, 0, 3 * sizeof(int), stream));
    CUDA_TRY(cudaMemsetAsync(d_progress, 0, sizeof(int) * 2 * stripes, stream));
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int32_t) * P_, stream));
    if (estep) {
        CUDA_TRY(cudaMemsetAsync(n_trans, 0, sizeof(double) * (size_t)P_ * N * N, stream));
        CUDA_TRY(cudaMemsetAsync(cntM, 0, sizeof(double) * (size_t)P_ * G * 441, stream));
        CUDA_TRY(cudaMemsetAsync(cntI, 0, sizeof(double) * (size_t)P_ * G * 21, stream));
        CUDA_TRY(cudaMemsetAsync(cntD, 0, sizeof(double) * (size_t)P_ * G * 21, stream));
    }
    if (F_log) { fill_f64<<<256, 256, 0, stream>>>(F_log, tab_cells * N, NEG_INF_LL); plan->launches++; }
    if (B_log) { fill_f64<<<256, 256, 0, stream>>>(B_log, tab_cells * N, NEG_INF_LL); plan->launches++; }
    if (post) CUDA_TRY(cudaMemsetAsync(post, 0, sizeof(double) * (size_t)tab_cells * N, stream));

    K.res = b->residues;
    K.meta = (const PairMeta *)d_meta;
    K.n_items = n_items;
    K.chi = b->chi;
    K.chi_stride = b->chi_per_pair ? (int64_t)N * N : 0;
    if (use_nest) {
        K.nest = b->nest;
        K.nest_stride = b->chi_per_pair ? nest_record_len(b->nest_dom, b->nest_frag) : 0;
        K.nest_K = b->nest_dom;
        K.nest_F = b->nest_frag;
    }
    K.eM = b->emit_M;
    K.eI = b->emit_I;
    K.eD = b->emit_D;
    K.eM_stride = b->emit_per_pair ? (int64_t)G * 441 : 0;
    K.eID_stride = b->emit_per_pair ? (int64_t)G * 21 : 0;
    K.lat = estep ? d_lat : nullptr;
    K.lat_exp = estep ? d_lat_exp : nullptr;
    K.blat = d_blat;
    K.blat_exp = d_blat_exp;
    K.edge = d_edge;
    K.edge_exp = d_edge_exp;
    K.ll = ll;
    K.status = status;
    K.n_trans = n_trans;
    K.cntM = cntM;
    K.cntI = cntI;
    K.cntD = cntD;
    K.F_log = F_log;
    K.B_log = B_log;
    K.post = post;
    K.max_ly = max_ly;
    K.spin_limit = plan->spin_limit > 0 ? plan->spin_limit : kSpinLimit;
    K.wave_ctr = nullptr;
    K.cmask = b->cell_mask;
    K.beam_scale = b->beam_log_width > 0.0 ? (float)exp(-b->beam_log_width) : 0.f;
    K.srange = nullptr;
    if (n_range) {
        int2 *range = (int2 *)d_items + plan->h_items.size();
        K.items = (const int2 *)d_items;
        stripe_range_kernel<<<n_items, 256, 0, stream>>>(K, rows, range);
        CUDA_TRY(cudaGetLastError());
        plan->launches++;
        K.srange = range;
    }
    if (split) return launch_split(plan, K, wl ? wl : bl, bl != nullptr, n_items, n_citems, stripes, max_ly, d_items,
                                   d_counters, d_progress, d_bedge, d_bedge_exp, stream);
    for (int pass = 0; pass < (estep ? 2 : 1); ++pass) {
        const bool bwd = pass == 1;
        K.items = (const int2 *)d_items + (bwd ? n_items : 0);
        K.counter = d_counters + (bwd ? 1 : 0);
        K.progress = d_progress + (bwd ? stripes : 0);
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[bwd ? 2 : 0], stream));
        if (bl) {
            if ((rc = bl(plan, K, n_items, max_ly, bwd, stream))) return rc;
        } else if (wl) {
            if ((rc = wl(plan, K, n_items, max_ly, two_warp ? 5 : (int)bwd, stream))) return rc;
        } else {
            const int threads = 32 * K.NQ;
            const SmemLayout L = make_layout(K.NS, K.NQ, G, max_ly, bwd);
            auto kern = bwd ? backward_kernel : forward_kernel;
            CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
            int occ = 0;
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, L.bytes));
            if (occ < 1) return fail(PHMM_E_ARG, "kernel does not fit on an SM (shared memory)");
            const int grid = std::min(n_items, plan->sm_count * occ);
            kern<<<grid, threads, L.bytes, stream>>>(K);
            CUDA_TRY(cudaGetLastError());
        }
        if (plan->timing) CUDA_TRY(cudaEventRecord(plan->ev[bwd ? 3 : 1], stream));
        plan->launches++;
    }
    plan->timed_bwd = estep;
    plan->timed_count = false;
    return 0;
}

// A pair whose wavefront or count pass gave up a bounded wait (status bit
// PHMM_ST_TIMEOUT, set by whichever kernel timed out) has incomplete lattices;
// after the call's kernels its log-likelihood becomes the reference's failure
// value NEG_INF, whatever the kernels wrote, so a caller filtering on the
// log-likelihood (train_pfam.py:2859) drops it.
__global__ void timeout_epilogue_kernel(double *ll, const int32_t *status, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n && (status[p] & PHMM_ST_TIMEOUT)) ll[p] = NEG_INF_LL;
}

int launch_timeout_epilogue(double *ll, const int32_t *status, int n, cudaStream_t stream) {
    if (n <= 0) return 0;
    timeout_epilogue_kernel<<<(n + 255) / 256, 256, 0, stream>>>(ll, status, n);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

// One call of the kernels (run_core) followed by the timeout epilogue.
int run(phmm_plan *plan, const phmm_batch *b, bool estep, double *ll, double *n_trans,
        double *cntM, double *cntI, double *cntD, int32_t *status, double *F_log, double *B_log,
        double *post, void *stream_, void *ws = nullptr, size_t ws_bytes = 0, size_t *ws_need = nullptr) {
    const int rc = run_core(plan, b, estep, ll, n_trans, cntM, cntI, cntD, status, F_log, B_log, post, stream_,
                            ws, ws_bytes, ws_need);
    if (rc || ws_need || b->n_pairs <= 0 || plan->desc_mode == 1) return rc;
    const int rc2 = launch_timeout_epilogue(ll, status, b->n_pairs, (cudaStream_t)stream_);
    if (!rc2) plan->launches++;
    return rc2;
}

template <class SH>
int launch_block(phmm_plan *plan, KParams &K, int n_items, int max_ly, int kind, cudaStream_t stream) {
    void (*kern)(const KParams) = nullptr;
    int bytes = 0, threads = 0;
    if (kind == 3) {
        bytes = blk::make_smem_cb(SH::NS, K.G, max_ly, K.kend[0] - K.kbeg[0], K.kend[1] - K.kbeg[1],
                                  K.kend[2] - K.kbeg[2]).bytes;
        kern = blk::count_block_kernel<SH>;
        threads = blk::CNT_THREADS;
    } else {
        bytes = blk::make_smem_b(SH::NS, SH::NB, 1, K.G, max_ly, kind == 1).bytes;
        kern = kind == 0 ? blk::forward_block_kernel<SH>
                         : (kind == 1 ? blk::backward_block_kernel<SH> : blk::fwdbwd_block_kernel<SH>);
        threads = 32 * (SH::NB + (kind == 1 ? blk::NCW : 0));
    }
    CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    int occ = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, bytes));
    if (occ < 1) return fail(PHMM_E_ARG, "block kernel does not fit on an SM (shared memory)");
    const int grid = std::min(n_items, plan->launch_per_sm > 0
                                           ? plan->sm_count * std::min(plan->launch_per_sm, occ)
                                           : std::max(1, plan->sm_count * occ / plan->grid_div));
    kern<<<grid, threads, bytes, stream>>>(K);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

// the nested two-warp stripe kernel of shape SH for the MixDom layout (K, F),
// with its shared-memory coefficient floats, or null where none is compiled
template <class SH>
void (*nest_tw_kernel(bool bwd, int K, int F, int &floats))(const KParams) {
    if constexpr (SH::NM == 3 && SH::NI == 6 && SH::ND == 6) {
        if (K == 3 && F == 1) {
            using NT = warp2::Nest<3, 1>;
            floats = warp2::NestSlots<SH, NT>::FLOATS;
            return bwd ? warp2::stripe_tw_kernel<SH, true, false, NT> : warp2::stripe_tw_kernel<SH, false, false, NT>;
        }
    }
    floats = 0;
    return nullptr;
}

template <class SH>
int launch_warp(phmm_plan *plan, KParams &K, int n_items, int max_ly, int kind, cudaStream_t stream) {
    void (*kern)(const KParams) = nullptr;
    int bytes = 0, threads = 32;
    if (kind == 3 && plan->two_warp) {   // count pass of the two-warp split E-step
        bytes = warp2::make_smem_ct(SH::SP, SH::KP, SH::NI, K.G, max_ly).bytes;
        kern = K.srange ? warp2::count_tw_kernel<SH, true> : warp2::count_tw_kernel<SH, false>;
        threads = warp2::TWT;
    } else if (kind == 3) {
        bytes = warp2::make_smem_c(SH::SP, SH::KP, SH::NI, K.G, max_ly).bytes;
        kern = warp2::count_warp_kernel<SH>;
    } else if (kind == 5 || kind == 6) {   // two-warp stripes: forward / backward recursion
        int nest_floats = 0;
        if (K.nest) kern = nest_tw_kernel<SH>(kind == 6, K.nest_K, K.nest_F, nest_floats);
        bytes = warp2::make_smem_tw(SH::SP, SH::KP, SH::NI, K.G, max_ly, kind == 6, nest_floats).bytes;
        if (kern) {
        } else if (K.cmask) {
            kern = kind == 5 ? warp2::stripe_tw_kernel<SH, false, true> : warp2::stripe_tw_kernel<SH, true, true>;
        } else {
            kern = kind == 5 ? warp2::stripe_tw_kernel<SH, false, false> : warp2::stripe_tw_kernel<SH, true, false>;
        }
        threads = warp2::TWT;
    } else {
        bytes = warp2::make_smem_w(SH::SP, SH::KP, SH::NI, K.G, max_ly, kind != 0, kind == 1).bytes;
        kern = kind == 0 ? warp2::forward_warp_kernel<SH>
                         : (kind == 1 ? warp2::backward_warp_kernel<SH> : warp2::backward_rec_warp_kernel<SH>);
    }
    CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    int occ = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, bytes));
    if (occ < 1) return fail(PHMM_E_ARG, "warp kernel does not fit on an SM (shared memory)");
    const int grid = std::min(n_items, plan->launch_per_sm > 0
                                           ? plan->sm_count * std::min(plan->launch_per_sm, occ)
                                           : std::max(1, plan->sm_count * occ / plan->grid_div));
    kern<<<grid, threads, bytes, stream>>>(K);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

// Batches whose scratch would not fit in the device memory that is free run
// as consecutive groups of pairs (contiguous index ranges), one after the
// other on the same stream, each within the budget.
size_t plan_scratch_bytes(const phmm_plan *plan) {
    return plan->meta_cap + plan->items_cap + sizeof(int64_t) * plan->slat_cap +
           sizeof(float) * (plan->lat_cap + plan->edge_cap + plan->blat_cap +
           plan->bedge_cap) + sizeof(int) * (plan->latE_cap + plan->edgeE_cap + plan->prog_cap + plan->blatE_cap +
           plan->bedgeE_cap);
}

int run_groups(phmm_plan *plan, const phmm_batch *b, bool estep, double *ll, double *n_trans, double *cntM,
               double *cntI, double *cntD, int32_t *status, void *stream) {
    NvtxRange range(estep ? "phmm_estep" : "phmm_forward");
    if (!plan || !b) return fail(PHMM_E_ARG, "null plan or batch");
    size_t need = 0;
    int rc = run(plan, b, estep, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                 stream, nullptr, 0, &need);
    if (rc) return rc;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = (size_t)-1 / 2;
    const size_t budget = (size_t)((double)(free_b + plan_scratch_bytes(plan)) * 0.85);
    if (need <= budget || b->n_pairs <= 1)
        return run(plan, b, estep, ll, n_trans, cntM, cntI, cntD, status, nullptr, nullptr, nullptr, stream);
    const int N = plan->base.N, G = plan->base.G;
    int launches = 0, p0 = 0;
    int64_t mask_off = 0;   // cells of the pairs before p0 (the cell mask is concatenated per pair)
    float acc[3] = {0.f, 0.f, 0.f};
    bool any_bwd = false, any_count = false;
    while (p0 < b->n_pairs) {
        // the largest contiguous group from p0 that fits the budget (at least one pair)
        int lo = 1, hi = b->n_pairs - p0;
        phmm_batch g = *b;
        auto group = [&](int n) {
            g.n_pairs = n;
            g.Lx_host = b->Lx_host + p0;
            g.Ly_host = b->Ly_host + p0;
            g.x_off_host = b->x_off_host + p0;
            g.y_off_host = b->y_off_host + p0;
            g.chi = b->chi + (b->chi_per_pair ? (int64_t)p0 * N * N : 0);
            if (b->nest) g.nest = b->nest + (b->chi_per_pair ? (int64_t)p0 * nest_record_len(b->nest_dom, b->nest_frag) : 0);
            g.emit_M = b->emit_M + (b->emit_per_pair ? (int64_t)p0 * G * 441 : 0);
            g.emit_I = b->emit_I + (b->emit_per_pair ? (int64_t)p0 * G * 21 : 0);
            g.emit_D = b->emit_D + (b->emit_per_pair ? (int64_t)p0 * G * 21 : 0);
            g.cell_mask = b->cell_mask ? b->cell_mask + mask_off : nullptr;
        };
        while (lo < hi) {   // binary search on the group size
            const int mid = (lo + hi + 1) / 2;
            group(mid);
            size_t n2 = 0;
            if ((rc = run(plan, &g, estep, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                          nullptr, stream, nullptr, 0, &n2)))
                return rc;
            if (n2 <= budget) lo = mid; else hi = mid - 1;
        }
        group(lo);
        rc = run(plan, &g, estep, ll + p0, estep ? n_trans + (int64_t)p0 * N * N : nullptr,
                 estep ? cntM + (int64_t)p0 * G * 441 : nullptr, estep ? cntI + (int64_t)p0 * G * 21 : nullptr,
                 estep ? cntD + (int64_t)p0 * G * 21 : nullptr, status + p0, nullptr, nullptr, nullptr, stream);
        if (rc) return rc;
        launches += plan->launches;
        if (plan->timing) {   // each group's events are re-recorded by the next group: read them now
            for (int w = 0; w < 3; ++w) {
                if ((w == 1 && !plan->timed_bwd) || (w == 2 && !plan->timed_count)) continue;
                float ms = 0.f;
                CUDA_TRY(cudaEventSynchronize(plan->ev[2 * w + 1]));
                CUDA_TRY(cudaEventElapsedTime(&ms, plan->ev[2 * w], plan->ev[2 * w + 1]));
                acc[w] += ms;
            }
            any_bwd |= plan->timed_bwd;
            any_count |= plan->timed_count;
        }
        for (int p = p0; p < p0 + lo; ++p) mask_off += (int64_t)(b->Lx_host[p] + 1) * (b->Ly_host[p] + 1);
        p0 += lo;
    }
    plan->launches = launches;
    if (plan->timing) {
        plan->grouped = true;
        plan->timed_bwd = any_bwd;
        plan->timed_count = any_count;
        for (int w = 0; w < 3; ++w) plan->group_ms[w] = acc[w];
    }
    return 0;
}

}  // namespace

extern "C" {

int phmm_version(void) { return 1; }

int phmm_last_error(char *buf, size_t len) {
    if (buf && len) {
        size_t n = std::min(len - 1, g_err.size());
        memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return (int)g_err.size();
}

int phmm_nest_supported(int32_t n_dom, int32_t n_frag) {
    // the two-warp stripes of 17 states; the wide kernels at F = 4 (K = 4..8:
    // more than 64 slots, one quad of slots per (domain, sub-state) block)
    const bool wide_ok = n_frag == 4 && n_dom >= 4 && 20 * n_dom <= 160;
    return (has_nest_tw(n_dom * n_frag, n_dom, n_frag) || wide_ok) ? 1 : 0;
}

int phmm_plan_create(const phmm_model_desc *md, phmm_plan **out) {
    if (!md || !out || !md->state_types || md->n_states < 2) return fail(PHMM_E_ARG, "bad model description");
    const int N = md->n_states;
    if (md->state_types[0] != T_S) return fail(PHMM_E_ARG, "state 0 must be the start state (type S)");
    int e_idx = -1;
    for (int k = 0; k < N; ++k)
        if (md->state_types[k] == T_E) { e_idx = k; break; }
    if (e_idx < 0) return fail(PHMM_E_ARG, "no End (type E) state");
    if (md->n_groups < 1 || md->n_groups > 64) return fail(PHMM_E_ARG, "n_groups must be in 1..64");
    std::vector<int> byType[3];
    for (int k = 0; k < N; ++k) {
        int t = md->state_types[k];
        if (t == T_M || t == T_I || t == T_D) {
            int g = md->state_group ? md->state_group[k] : 0;
            if (g < 0 || g >= md->n_groups) return fail(PHMM_E_ARG, "state group out of range");
            byType[t - 1].push_back(k);
        } else if (t < 0 || t > T_E) {
            return fail(PHMM_E_ARG, "unknown state type");
        }
    }
    KParams K;
    memset(&K, 0, sizeof(K));
    std::vector<int> slot_orig, slot_type;
    int s_slot = -1;
    for (int ty = 0; ty < 3; ++ty) {
        K.kbeg[ty] = (int)slot_orig.size();
        for (int k : byType[ty]) { slot_orig.push_back(k); slot_type.push_back(ty + 1); }
        while (slot_orig.size() % 4) {
            if (s_slot < 0) { s_slot = (int)slot_orig.size(); slot_orig.push_back(0); slot_type.push_back(T_S); }
            else { slot_orig.push_back(-1); slot_type.push_back(T_NONE); }
        }
        K.kend[ty] = (int)slot_orig.size();
    }
    if (s_slot < 0) {
        s_slot = (int)slot_orig.size();
        slot_orig.push_back(0); slot_type.push_back(T_S);
        while (slot_orig.size() % 4) { slot_orig.push_back(-1); slot_type.push_back(T_NONE); }
    }
    const int NS = (int)slot_orig.size();
    if (NS > MAXS) return fail(PHMM_E_ARG, "too many emitting states for the generic kernels (max 164)");
    K.N = N;
    K.NS = NS;
    K.NQ = NS / 4;
    K.G = md->n_groups;
    K.e_idx = e_idx;
    K.s_slot = s_slot;
    for (int s = 0; s < NS; ++s) {
        K.slot_orig[s] = (int16_t)slot_orig[s];
        K.slot_type[s] = (int8_t)slot_type[s];
        int g = 0;
        if (slot_type[s] >= T_M && slot_type[s] <= T_D && md->state_group) g = md->state_group[slot_orig[s]];
        K.slot_group[s] = (int16_t)g;
    }
    for (int q = 0; q < K.NQ; ++q) {
        int t = T_NONE;
        for (int ty = 0; ty < 3; ++ty)
            if (4 * q >= K.kbeg[ty] && 4 * q < K.kend[ty]) t = ty + 1;
        K.quad_type[q] = (int8_t)t;
    }
    // warp-kernel slot layout: M, I, D states in order, then the start state
    {
        int ns = 0;
        for (int ty = 0; ty < 3; ++ty)
            for (int k : byType[ty]) {
                K.w_orig[ns] = (int16_t)k;
                K.w_group[ns] = (int16_t)(md->state_group ? md->state_group[k] : 0);
                ++ns;
            }
        if (ns + 1 <= MAXS) K.w_orig[ns] = 0;
    }
    phmm_plan *plan = new phmm_plan();
    plan->base = K;
    plan->w_nm = (int)byType[0].size();
    plan->w_ni = (int)byType[1].size();
    plan->w_nd = (int)byType[2].size();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&plan->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) {
        size_t fr = 0;
        e = cudaMemGetInfo(&fr, &plan->total_mem);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&plan->counters, 4 * sizeof(int));
    if (e != cudaSuccess) {
        delete plan;
        return fail(PHMM_E_CUDA, std::string("plan create: ") + cudaGetErrorString(e));
    }
    *out = plan;
    return 0;
}

int phmm_set_timing(phmm_plan *plan, int enable) {
    if (!plan) return fail(PHMM_E_ARG, "null plan");
    if (enable && !plan->ev[0]) {
        for (int k = 0; k < 6; ++k) CUDA_TRY(cudaEventCreate(&plan->ev[k]));
    }
    plan->timing = enable != 0;
    return 0;
}

int phmm_kernel_time(phmm_plan *plan, int which, float *ms) {
    if (!plan || !plan->timing) return fail(PHMM_E_ARG, "timing is not enabled on this plan");
    if (!ms || which < 0 || which > 2) return fail(PHMM_E_ARG, "bad kernel index");
    if ((which == 1 && !plan->timed_bwd) || (which == 2 && !plan->timed_count)) { *ms = 0.f; return 0; }
    if (plan->grouped) { *ms = plan->group_ms[which]; return 0; }
    CUDA_TRY(cudaEventSynchronize(plan->ev[2 * which + 1]));
    CUDA_TRY(cudaEventElapsedTime(ms, plan->ev[2 * which], plan->ev[2 * which + 1]));
    return 0;
}

int phmm_kernel_times(phmm_plan *plan, float *fwd_ms, float *bwd_ms) {
    if (!plan || !plan->timing) return fail(PHMM_E_ARG, "timing is not enabled on this plan");
    float a = 0.f, b = 0.f;
    if (plan->grouped) {
        if (fwd_ms) *fwd_ms = plan->group_ms[0];
        if (bwd_ms) *bwd_ms = plan->timed_bwd ? plan->group_ms[1] : 0.f;
        return 0;
    }
    CUDA_TRY(cudaEventSynchronize(plan->ev[1]));
    CUDA_TRY(cudaEventElapsedTime(&a, plan->ev[0], plan->ev[1]));
    if (plan->timed_bwd) {
        CUDA_TRY(cudaEventSynchronize(plan->ev[3]));
        CUDA_TRY(cudaEventElapsedTime(&b, plan->ev[2], plan->ev[3]));
    }
    if (fwd_ms) *fwd_ms = a;
    if (bwd_ms) *bwd_ms = b;
    return 0;
}

void phmm_plan_destroy(phmm_plan *plan) {
    if (!plan) return;
    cudaDeviceSynchronize();
    for (int k = 0; k < 6; ++k)
        if (plan->ev[k]) cudaEventDestroy(plan->ev[k]);
    for (auto &e : plan->sides) {
        cudaEventDestroy(e.fork);
        cudaEventDestroy(e.join);
        cudaEventDestroy(e.join2);
        cudaEventDestroy(e.join3);
        cudaEventDestroy(e.fwd_done);
        cudaEventDestroy(e.joinf);
        if (e.sidef) cudaStreamDestroy(e.sidef);
        cudaStreamDestroy(e.side);
        cudaStreamDestroy(e.side2);
        cudaStreamDestroy(e.side3);
    }
    cudaFree(plan->blat);
    cudaFree(plan->blat_exp);
    cudaFree(plan->bedge);
    cudaFree(plan->bedge_exp);
    cudaFree(plan->meta);
    cudaFree(plan->items);
    cudaFree(plan->counters);
    cudaFree(plan->lat);
    cudaFree(plan->lat_exp);
    cudaFree(plan->edge);
    cudaFree(plan->edge_exp);
    cudaFree(plan->progress);
    cudaFree(plan->slat);
    delete plan;
}

int phmm_forward(phmm_plan *plan, const phmm_batch *batch, double *ll_out, int32_t *status_out,
                 void *stream) {
    return run_groups(plan, batch, false, ll_out, nullptr, nullptr, nullptr, nullptr, status_out, stream);
}

int phmm_estep(phmm_plan *plan, const phmm_batch *batch, double *ll_out, double *n_trans, double *cnt_M,
               double *cnt_I, double *cnt_D, int32_t *status_out, void *stream) {
    return run_groups(plan, batch, true, ll_out, n_trans, cnt_M, cnt_I, cnt_D, status_out, stream);
}

int phmm_estep_tables(phmm_plan *plan, const phmm_batch *batch, double *ll_out, double *n_trans,
                      double *cnt_M, double *cnt_I, double *cnt_D, int32_t *status_out, double *log_F,
                      double *log_B, double *post, void *stream) {
    return run(plan, batch, true, ll_out, n_trans, cnt_M, cnt_I, cnt_D, status_out, log_F, log_B, post,
               stream);
}

int phmm_estep_band(phmm_plan *plan, const phmm_batch *batch, const int32_t *band_center, int32_t band_half_width,
                    double *ll_out, double *n_trans, double *cnt_M, double *cnt_I, double *cnt_D,
                    int32_t *status_out, double *post_band, void *stream) {
    NvtxRange range("phmm_estep_band");
    if (!plan || !batch) return fail(PHMM_E_ARG, "null plan or batch");
    if (!batch->cell_mask) return fail(PHMM_E_ARG, "phmm_estep_band: the batch carries no band (cell mask)");
    if (!band_center || !post_band || band_half_width < 0) return fail(PHMM_E_ARG, "phmm_estep_band: bad band output");
    if (batch->beam_log_width > 0.0) return fail(PHMM_E_ARG, "phmm_estep_band: beam pruning is not banded");
    if (plan->variant != 0 && plan->variant != 7)
        return fail(PHMM_E_ARG, "phmm_estep_band runs on the two-warp kernels (variant 0 or 7)");
    if (!find_warp_launcher(plan->w_nm, plan->w_ni, plan->w_nd))
        return fail(PHMM_E_ARG, "phmm_estep_band: no two-warp kernels for this state space");
    int rc = run(plan, batch, true, ll_out, n_trans, cnt_M, cnt_I, cnt_D, status_out, nullptr, nullptr, nullptr,
                 stream);
    if (rc) return rc;
    if (!plan->two_warp || plan->last_variant != 7)
        return fail(PHMM_E_ARG, "phmm_estep_band: the E-step did not run on the two-warp kernels");
    cudaStream_t st = (cudaStream_t)stream;
    const int N = plan->base.N, BW = 2 * band_half_width + 1;
    int64_t rows = 0;
    for (int p = 0; p < batch->n_pairs; ++p) rows += batch->Lx_host[p] + 1;
    CUDA_TRY(cudaMemsetAsync(post_band, 0, sizeof(double) * (size_t)rows * BW * N, st));
    // the E-step's work description and lattices stay in the plan's buffers;
    // the forward stripe items come first in the item list, the stripe
    // ranges right after the whole list
    KParams K = plan->base;
    K.meta = (const PairMeta *)plan->meta;
    K.items = (const int2 *)plan->items;
    K.lat = plan->lat;
    K.lat_exp = plan->lat_exp;
    K.blat = plan->blat;
    K.blat_exp = plan->blat_exp;
    K.ll = ll_out;
    K.srange = (const int2 *)plan->items + plan->h_items.size();
    int n_items = 0;
    for (int p = 0; p < batch->n_pairs; ++p) n_items += plan->h_meta[p].n_stripes;
    const int nsrc = plan->w_nm + plan->w_ni + plan->w_nd + 1;
    const int stride = (nsrc + 3) & ~3;
    band_post_kernel<<<n_items, 256, 0, st>>>(K, warp2::ROWS, stride, nsrc, band_center, band_half_width, post_band);
    CUDA_TRY(cudaGetLastError());
    plan->launches++;
    return 0;
}

int phmm_workspace_bytes(phmm_plan *plan, const phmm_batch *batch, int estep, size_t *bytes) {
    if (!bytes) return fail(PHMM_E_ARG, "null output");
    return run(plan, batch, estep != 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
               nullptr, nullptr, nullptr, 0, bytes);
}

int phmm_forward_ws(phmm_plan *plan, const phmm_batch *batch, void *workspace, size_t workspace_bytes,
                    double *ll_out, int32_t *status_out, void *stream) {
    if (!workspace) return fail(PHMM_E_ARG, "null workspace");
    return run(plan, batch, false, ll_out, nullptr, nullptr, nullptr, nullptr, status_out, nullptr, nullptr,
               nullptr, stream, workspace, workspace_bytes);
}

int phmm_estep_ws(phmm_plan *plan, const phmm_batch *batch, void *workspace, size_t workspace_bytes,
                  double *ll_out, double *n_trans, double *cnt_M, double *cnt_I, double *cnt_D,
                  int32_t *status_out, void *stream) {
    if (!workspace) return fail(PHMM_E_ARG, "null workspace");
    return run(plan, batch, true, ll_out, n_trans, cnt_M, cnt_I, cnt_D, status_out, nullptr, nullptr, nullptr,
               stream, workspace, workspace_bytes);
}

int phmm_estep_ws_prepare(phmm_plan *plan, const phmm_batch *batch, void *workspace, size_t workspace_bytes,
                          void *stream) {
    if (!plan || !workspace) return fail(PHMM_E_ARG, "null plan or workspace");
    plan->desc_mode = 1;
    const int rc = run(plan, batch, true, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                       nullptr, stream, workspace, workspace_bytes);
    plan->desc_mode = 0;
    return rc;
}

int phmm_estep_ws_launch(phmm_plan *plan, const phmm_batch *batch, void *workspace, size_t workspace_bytes,
                         double *ll_out, double *n_trans, double *cnt_M, double *cnt_I, double *cnt_D,
                         int32_t *status_out, void *stream) {
    if (!plan || !workspace) return fail(PHMM_E_ARG, "null plan or workspace");
    plan->desc_mode = 2;
    const int rc = run(plan, batch, true, ll_out, n_trans, cnt_M, cnt_I, cnt_D, status_out, nullptr, nullptr,
                       nullptr, stream, workspace, workspace_bytes);
    plan->desc_mode = 0;
    return rc;
}

int phmm_last_launch_count(const phmm_plan *plan) { return plan ? plan->launches : 0; }

int phmm_set_variant(phmm_plan *plan, int variant) {
    if (!plan || variant < 0 || variant > 7) return fail(PHMM_E_ARG, "bad variant");
    if ((variant == 2 || variant == 4 || variant == 7) && !find_warp_launcher(plan->w_nm, plan->w_ni, plan->w_nd))
        return fail(PHMM_E_ARG, "no warp kernel for this state space");
    if ((variant == 3 || variant == 5) && !find_block_launcher(plan->base.NS))
        return fail(PHMM_E_ARG, "no block kernel for this state space");
    plan->variant = variant;
    return 0;
}

int phmm_last_variant(const phmm_plan *plan) { return plan ? plan->last_variant : 0; }

int phmm_set_tuning(phmm_plan *plan, const phmm_tuning *t) {
    if (!plan || !t) return fail(PHMM_E_ARG, "null plan or tuning");
    if (t->wave_per_sm < 0 || t->wave_per_sm > 64 || t->count_per_sm < -1 || t->count_per_sm > 64 ||
        t->priorities < 0 || t->priorities > 1 || t->checkpoint < 0 || t->checkpoint > 2 ||
        t->tensor < 0 || t->tensor > 1)
        return fail(PHMM_E_ARG, "tuning out of range (wave_per_sm 0..64, count_per_sm -1..64, priorities 0/1, "
                                "checkpoint 0..2, tensor 0/1)");
    int rc = phmm_set_variant(plan, t->variant);
    if (rc) return rc;
    plan->tuning = *t;
    return 0;
}

int phmm_get_tuning(const phmm_plan *plan, phmm_tuning *t) {
    if (!plan || !t) return fail(PHMM_E_ARG, "null plan or tuning");
    *t = plan->tuning;
    t->variant = plan->variant;
    return 0;
}

int phmm_set_spin_limit(phmm_plan *plan, long long iterations) {
    if (!plan || iterations < 0) return fail(PHMM_E_ARG, "null plan or negative spin limit");
    plan->spin_limit = iterations;
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- allocation-free E-step
//
// phmm_estep_static runs the same kernels as phmm_estep with every scratch
// buffer carved out of one file-scope __device__ array, for callers that
// cannot allocate device memory.  The array is PHMM_STATIC_SCRATCH_BYTES
// large and lives on every GPU that loads this library until the process
// exits.  Host code cannot pass the array's name to a kernel (on the host it
// is only a stand-in for the symbol); its device address is looked up with
// cudaGetSymbolAddress once per device, with that device current, by the
// first call made on that device.
namespace {

__device__ __align__(256) unsigned char g_static_scratch[PHMM_STATIC_SCRATCH_BYTES];

constexpr int kStaticMaxDevices = 64;
constexpr int kStaticMaxPairs = 4096;
constexpr int kStaticMaxItems = 2 * 32768;
unsigned char *g_static_dev[kStaticMaxDevices] = {};
int g_static_sms[kStaticMaxDevices] = {};
// host staging of the per-call work description (static: no heap either)
PairMeta g_static_meta[kStaticMaxPairs];
int2 g_static_items[kStaticMaxItems];
int g_static_order[kStaticMaxPairs];

// Model slot tables for a description (same layout as phmm_plan_create).
int static_model(const phmm_model_desc *md, KParams *K, int *nm, int *ni, int *nd) {
    if (!md || !md->state_types || md->n_states < 2) return fail(PHMM_E_ARG, "bad model description");
    const int N = md->n_states;
    if (md->state_types[0] != T_S) return fail(PHMM_E_ARG, "state 0 must be the start state (type S)");
    int e_idx = -1;
    for (int k = 0; k < N; ++k)
        if (md->state_types[k] == T_E) { e_idx = k; break; }
    if (e_idx < 0) return fail(PHMM_E_ARG, "no End (type E) state");
    if (md->n_groups < 1 || md->n_groups > 64) return fail(PHMM_E_ARG, "n_groups must be in 1..64");
    int byType[3][MAXS];
    int cnt[3] = {0, 0, 0};
    for (int k = 0; k < N; ++k) {
        const int t = md->state_types[k];
        if (t == T_M || t == T_I || t == T_D) {
            const int g = md->state_group ? md->state_group[k] : 0;
            if (g < 0 || g >= md->n_groups) return fail(PHMM_E_ARG, "state group out of range");
            if (cnt[t - 1] >= MAXS) return fail(PHMM_E_ARG, "too many emitting states");
            byType[t - 1][cnt[t - 1]++] = k;
        } else if (t < 0 || t > T_E) {
            return fail(PHMM_E_ARG, "unknown state type");
        }
    }
    memset(K, 0, sizeof(*K));
    int ns = 0, s_slot = -1;
    int slot_orig[2 * MAXS], slot_type[2 * MAXS];
    for (int ty = 0; ty < 3; ++ty) {
        K->kbeg[ty] = ns;
        for (int q = 0; q < cnt[ty]; ++q) {
            if (ns >= GMAXS) return fail(PHMM_E_ARG, "phmm_estep_static: at most 60 emitting states");
            slot_orig[ns] = byType[ty][q]; slot_type[ns] = ty + 1; ++ns;
        }
        while (ns % 4) {
            if (ns >= GMAXS) return fail(PHMM_E_ARG, "phmm_estep_static: at most 60 emitting states");
            if (s_slot < 0) { s_slot = ns; slot_orig[ns] = 0; slot_type[ns] = T_S; }
            else { slot_orig[ns] = -1; slot_type[ns] = T_NONE; }
            ++ns;
        }
        K->kend[ty] = ns;
    }
    if (s_slot < 0) {
        if (ns + 4 > GMAXS) return fail(PHMM_E_ARG, "phmm_estep_static: at most 60 emitting states");
        s_slot = ns; slot_orig[ns] = 0; slot_type[ns] = T_S; ++ns;
        while (ns % 4) { slot_orig[ns] = -1; slot_type[ns] = T_NONE; ++ns; }
    }
    K->N = N;
    K->NS = ns;
    K->NQ = ns / 4;
    K->G = md->n_groups;
    K->e_idx = e_idx;
    K->s_slot = s_slot;
    for (int s = 0; s < ns; ++s) {
        K->slot_orig[s] = (int16_t)slot_orig[s];
        K->slot_type[s] = (int8_t)slot_type[s];
        int g = 0;
        if (slot_type[s] >= T_M && slot_type[s] <= T_D && md->state_group) g = md->state_group[slot_orig[s]];
        K->slot_group[s] = (int16_t)g;
    }
    for (int q = 0; q < K->NQ; ++q) {
        int t = T_NONE;
        for (int ty = 0; ty < 3; ++ty)
            if (4 * q >= K->kbeg[ty] && 4 * q < K->kend[ty]) t = ty + 1;
        K->quad_type[q] = (int8_t)t;
    }
    int w = 0;
    for (int ty = 0; ty < 3; ++ty)
        for (int q = 0; q < cnt[ty]; ++q) {
            const int k = byType[ty][q];
            K->w_orig[w] = (int16_t)k;
            K->w_group[w] = (int16_t)(md->state_group ? md->state_group[k] : 0);
            ++w;
        }
    if (w < MAXS) K->w_orig[w] = 0;
    *nm = cnt[0];
    *ni = cnt[1];
    *nd = cnt[2];
    return 0;
}

}  // namespace

extern "C" int phmm_estep_static(const phmm_model_desc *md, const phmm_batch *b, double *ll,
                                 double *n_trans, double *cntM, double *cntI, double *cntD,
                                 int32_t *status, void *stream_) {
    NvtxRange range("phmm_estep_static");
    if (!b) return fail(PHMM_E_ARG, "null batch");
    KParams K;
    int nm = 0, ni = 0, nd = 0, rc;
    if ((rc = static_model(md, &K, &nm, &ni, &nd))) return rc;
    cudaStream_t stream = (cudaStream_t)stream_;
    const int P_ = b->n_pairs;
    if (P_ < 0) return fail(PHMM_E_ARG, "n_pairs < 0");
    if (P_ == 0) return 0;
    if (!b->Lx_host || !b->Ly_host || !b->x_off_host || !b->y_off_host || !b->residues || !b->chi ||
        !b->emit_M || !b->emit_I || !b->emit_D || !ll || !status || !n_trans || !cntM || !cntI || !cntD)
        return fail(PHMM_E_ARG, "null batch pointer or output");
    if (P_ > kStaticMaxPairs) return fail(PHMM_E_ARG, "phmm_estep_static: more than 4096 pairs in one call");
    if (b->cell_mask) return fail(PHMM_E_ARG, "phmm_estep_static: cell masks are not supported (use phmm_estep)");
    if (b->beam_log_width != 0.0)
        return fail(PHMM_E_ARG, "phmm_estep_static: beam pruning is not supported (use phmm_estep)");
    // ---- device set-up, once per device (the first call on a device does it)
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticMaxDevices) return fail(PHMM_E_ARG, "device ordinal out of range");
    if (!g_static_dev[dev]) {
        void *ptr = nullptr;
        CUDA_TRY(cudaGetSymbolAddress(&ptr, g_static_scratch));
        int sms = 0;
        CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        g_static_sms[dev] = sms;
        g_static_dev[dev] = (unsigned char *)ptr;
    }
    unsigned char *base = g_static_dev[dev];
    const int N = K.N, G = K.G;
    const WarpLauncher wl = find_warp_launcher(nm, ni, nd);
    const int rows = wl ? warp2::ROWS : TH;
    const int stride = wl ? ((nm + ni + nd + 1 + 3) & ~3) : K.NS;
    // ---- work description and scratch layout
    int64_t lat_cells = 0, edge_cells = 0;
    int stripes = 0, max_ly = 0;
    for (int p = 0; p < P_; ++p) {
        if (b->Lx_host[p] < 0 || b->Ly_host[p] < 0) return fail(PHMM_E_ARG, "negative length");
        PairMeta &m = g_static_meta[p];
        m.Lx = b->Lx_host[p];
        m.Ly = b->Ly_host[p];
        m.x_off = b->x_off_host[p];
        m.y_off = b->y_off_host[p];
        m.n_stripes = (m.Lx + 1 + rows - 1) / rows;
        m.stripe_base = stripes;
        m.lat_base = lat_cells;
        m.edge_base = edge_cells;
        m.tab_base = 0;
        stripes += m.n_stripes;
        lat_cells += (int64_t)m.n_stripes * (rows + m.Ly) * rows;
        edge_cells += (int64_t)m.n_stripes * (m.Ly + 1);
        max_ly = std::max(max_ly, m.Ly);
        g_static_order[p] = p;
    }
    if (2 * (int64_t)stripes > kStaticMaxItems)
        return fail(PHMM_E_ARG, "phmm_estep_static: batch has more than 32768 row stripes");
    const size_t off_meta = 0;
    const size_t off_items = align256(off_meta + sizeof(PairMeta) * P_);
    const size_t off_cnt = align256(off_items + sizeof(int2) * 2 * stripes);
    const size_t off_prog = align256(off_cnt + 4 * sizeof(int));
    const size_t off_edge = align256(off_prog + sizeof(int) * 2 * stripes);
    const size_t off_edgeE = align256(off_edge + sizeof(float) * (size_t)edge_cells * stride);
    const size_t off_lat = align256(off_edgeE + sizeof(int) * (size_t)edge_cells);
    const size_t off_latE = align256(off_lat + sizeof(float) * (size_t)lat_cells * stride);
    const size_t need = align256(off_latE + sizeof(int) * (size_t)lat_cells);
    if (need > (size_t)PHMM_STATIC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "phmm_estep_static: batch needs %zu bytes of scratch, more than the %zu bytes the "
                 "allocation-free entry point holds; split the batch or use phmm_estep",
                 need, (size_t)PHMM_STATIC_SCRATCH_BYTES);
        return fail(PHMM_E_ARG, msg);
    }
    std::sort(g_static_order, g_static_order + P_, [&](int a, int c) {
        const int64_t ca = (int64_t)(b->Lx_host[a] + 1) * (b->Ly_host[a] + 1);
        const int64_t cc = (int64_t)(b->Lx_host[c] + 1) * (b->Ly_host[c] + 1);
        return ca != cc ? ca > cc : a < c;
    });
    int n_items = 0;
    for (int q = 0; q < P_; ++q) {
        const int p = g_static_order[q];
        for (int s = 0; s < g_static_meta[p].n_stripes; ++s) g_static_items[n_items++] = make_int2(p, s);
    }
    for (int q = 0; q < P_; ++q) {
        const int p = g_static_order[q];
        for (int s = g_static_meta[p].n_stripes - 1; s >= 0; --s) g_static_items[n_items++] = make_int2(p, s);
    }
    // ---- copy the work description, clear what must start at zero
    CUDA_TRY(cudaMemcpyAsync(base + off_meta, g_static_meta, sizeof(PairMeta) * P_, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(base + off_items, g_static_items, sizeof(int2) * 2 * stripes,
                             cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemsetAsync(base + off_cnt, 0, 4 * sizeof(int), stream));
    CUDA_TRY(cudaMemsetAsync(base + off_prog, 0, sizeof(int) * 2 * stripes, stream));
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int32_t) * P_, stream));
    CUDA_TRY(cudaMemsetAsync(n_trans, 0, sizeof(double) * (size_t)P_ * N * N, stream));
    CUDA_TRY(cudaMemsetAsync(cntM, 0, sizeof(double) * (size_t)P_ * G * 441, stream));
    CUDA_TRY(cudaMemsetAsync(cntI, 0, sizeof(double) * (size_t)P_ * G * 21, stream));
    CUDA_TRY(cudaMemsetAsync(cntD, 0, sizeof(double) * (size_t)P_ * G * 21, stream));
    K.res = b->residues;
    K.meta = (const PairMeta *)(base + off_meta);
    K.n_items = stripes;
    K.chi = b->chi;
    K.chi_stride = b->chi_per_pair ? (int64_t)N * N : 0;
    K.eM = b->emit_M;
    K.eI = b->emit_I;
    K.eD = b->emit_D;
    K.eM_stride = b->emit_per_pair ? (int64_t)G * 441 : 0;
    K.eID_stride = b->emit_per_pair ? (int64_t)G * 21 : 0;
    K.lat = (float *)(base + off_lat);
    K.lat_exp = (int *)(base + off_latE);
    K.edge = (float *)(base + off_edge);
    K.edge_exp = (int *)(base + off_edgeE);
    K.ll = ll;
    K.status = status;
    K.n_trans = n_trans;
    K.cntM = cntM;
    K.cntI = cntI;
    K.cntD = cntD;
    K.F_log = K.B_log = K.post = nullptr;
    K.max_ly = max_ly;
    K.spin_limit = kSpinLimit;
    K.wave_ctr = nullptr;
    K.cmask = nullptr;
    K.srange = nullptr;
    K.beam_scale = 0.f;
    phmm_plan launch_ctx;   // carries the SM count for the shared launchers; owns no memory
    launch_ctx.sm_count = g_static_sms[dev];
    for (int pass = 0; pass < 2; ++pass) {
        const bool bwd = pass == 1;
        K.items = (const int2 *)(base + off_items) + (bwd ? stripes : 0);
        K.counter = (int *)(base + off_cnt) + (bwd ? 1 : 0);
        K.progress = (int *)(base + off_prog) + (bwd ? stripes : 0);
        if (wl) {
            if ((rc = wl(&launch_ctx, K, stripes, max_ly, bwd, stream))) return rc;
        } else {
            const int threads = 32 * K.NQ;
            const SmemLayout L = make_layout(K.NS, K.NQ, G, max_ly, bwd);
            auto kern = bwd ? backward_kernel : forward_kernel;
            CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
            int occ = 0;
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, L.bytes));
            if (occ < 1) return fail(PHMM_E_ARG, "kernel does not fit on an SM (shared memory)");
            kern<<<std::min(stripes, g_static_sms[dev] * occ), threads, L.bytes, stream>>>(K);
            CUDA_TRY(cudaGetLastError());
        }
    }
    return launch_timeout_epilogue(ll, status, P_, stream);
}
