// estep_warp.cuh -- register-resident warp-per-stripe E-step kernels for
// small pair-HMM state spaces (included by pairhmm.cu).
//
// One warp (= one CTA) sweeps a STRIPE of 64 lattice rows of one pair along
// anti-diagonals.  Lane L owns rows 2L and 2L+1; at step t it computes cells
// A = (i0+2L, t-2L) and B = (i0+2L+1, t-2L-1), both on anti-diagonal i0+t.
// The state vectors of the last two steps stay in registers:
//   forward  A: I-pred = A(t-1), D-pred = lane L-1's B(t-1) (one __shfl_up),
//              M-pred = the D-pred received at step t-1;
//            B: I-pred = B(t-1), D-pred = A(t-1), M-pred = A(t-2);
//   backward B: I-succ = B(t+1), D-succ = lane L+1's A(t+1) (one __shfl_down),
//              M-succ = the D-succ received at step t+1;
//            A: I-succ = A(t+1), D-succ = B(t+1), M-succ = B(t+2).
// Lane 0 / lane 31 take the stripe-boundary neighbour from the halo row of
// the adjacent stripe (global edge buffer, 32-column chunks published with
// st.release by the single lane that writes them, polled with ld.acquire).
// The numbers of M, I and D states are template parameters, so each
// multiply-add reads the predecessor of its destination's type without a
// select; transition rows are warp-broadcast float4 loads, 8 FMAs per load.
// No __syncthreads anywhere: a warp is the whole CTA.

namespace warp2 {

constexpr int R = 2;          // rows per lane
constexpr int ROWS = 32 * R;  // rows per stripe
constexpr int HCW = 32;       // (layout) halo staging width
constexpr int PUB = 4;        // edge-row progress is published every PUB columns

template <int NM_, int NI_, int ND_>
struct Shape {
    static constexpr int NM = NM_, NI = NI_, ND = ND_;
    static constexpr int NE = NM + NI + ND;       // emitting states (dest slots 0..NE-1)
    static constexpr int NSRC = NE + 1;           // + start state (slot NE)
    static constexpr int SP = (NSRC + 3) & ~3;    // padded source stride
    static constexpr int KP = (NE + 3) & ~3;      // padded dest stride
    static constexpr int SPP = SP + 4, KPP = KP + 4;   // padded staging row strides
    static constexpr int BS = SP / 4, BK = KP / 4, NBLK = BS * BK;
    static constexpr int GROUPS = 32 / NBLK;      // count-phase lane groups
    static_assert(NBLK <= 32, "count blocks must fit in a warp");
    __host__ __device__ static constexpr int type_of(int k) { return k < NM ? T_M : (k < NM + NI ? T_I : T_D); }
};

struct SmemW {
    int chi, chiE, tM, tI, tD, halo, fst, ust;   // float offsets
    int haloE, fstE;                              // int offsets
    int bins;                                     // float offset (I-type bins [G][21])
    int colI;                                     // float offset (I-type column ring [ROWS][NI])
    int ys;                                       // byte offset
    int bytes;
};

// bwd: transposed chi; counts: the count-phase staging of the fused backward
__host__ __device__ inline SmemW make_smem_w(int SP, int KP, int NI, int G, int max_ly, bool bwd, bool counts) {
    SmemW L;
    int o = 0;
    const int SPP = SP + 4, KPP = KP + 4;
    L.chi = o; o += bwd ? KP * SP : SP * KP;
    L.chiE = o; o += SP;
    L.tM = o; o += al4(G * 441);
    L.tI = o; o += al4(G * 21);
    L.tD = o; o += al4(G * 21);
    L.halo = o; o += HCW * al4(KP > SP ? KP : SP);
    if (counts) {
        L.fst = o; o += 2 * ROWS * SPP;
        L.ust = o; o += ROWS * KPP;
        L.bins = o; o += al4(G * 21);
        L.colI = o; o += al4(ROWS * (NI > 0 ? NI : 1));
    } else {
        L.fst = L.ust = L.bins = L.colI = -1;
    }
    L.haloE = o; o += HCW;
    if (counts) { L.fstE = o; o += 2 * ROWS; } else { L.fstE = -1; }
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 1;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

__host__ __device__ inline SmemW make_smem_w(int SP, int KP, int NI, int G, int max_ly, bool bwd) {
    return make_smem_w(SP, KP, NI, G, max_ly, bwd, bwd);
}

// Per-stripe model load into shared memory (one warp).  chi layouts:
// 0 forward chi[s*KP + k]; 1 backward (transposed) chi[k*SP + s]; 2 forward
// with source pairs interleaved, chi[(s/2)*2KP + 2k + s%2] (one float4 holds
// sources s, s+1 for destinations k, k+1); 3 backward with destination pairs
// interleaved, chi[(k/2)*2SP + 2s + k%2].
constexpr int CHI_FWD = 0, CHI_BWD = 1, CHI_FWD_PAIRS = 2, CHI_BWD_PAIRS = 3;

template <class SH>
__device__ void load_model_w(const KParams &P, int p, const PairMeta &m, const SmemW &L, float *sm,
                             unsigned char *smb, int layout) {
    const int lane = threadIdx.x & 31;
    const int N = P.N, G = P.G;
    const float *chi = P.chi + (int64_t)p * P.chi_stride;
    for (int idx = lane; idx < SH::SP * SH::KP; idx += 32) {
        const int s = idx / SH::KP, k = idx % SH::KP;
        float v = 0.f;
        if (s < SH::NSRC && k < SH::NE) v = __ldg(chi + P.w_orig[s] * N + P.w_orig[k]);
        int at;
        if (layout == CHI_FWD) at = s * SH::KP + k;
        else if (layout == CHI_BWD) at = k * SH::SP + s;
        else if (layout == CHI_FWD_PAIRS) at = (s >> 1) * (2 * SH::KP) + 2 * k + (s & 1);
        else at = (k >> 1) * (2 * SH::SP) + 2 * s + (k & 1);
        sm[L.chi + at] = v;
    }
    for (int s = lane; s < SH::SP; s += 32)
        sm[L.chiE + s] = (s < SH::NSRC) ? __ldg(chi + P.w_orig[s] * N + P.e_idx) : 0.f;
    const float *eM = P.eM + (int64_t)p * P.eM_stride;
    const float *eI = P.eI + (int64_t)p * P.eID_stride;
    const float *eD = P.eD + (int64_t)p * P.eID_stride;
    for (int idx = lane; idx < G * 441; idx += 32) sm[L.tM + idx] = __ldg(eM + idx);
    for (int idx = lane; idx < G * 21; idx += 32) {
        sm[L.tI + idx] = __ldg(eI + idx);
        sm[L.tD + idx] = __ldg(eD + idx);
    }
    unsigned char *ys = smb + L.ys;
    for (int j = lane; j <= m.Ly; j += 32) {
        int c = 0;
        if (j >= 1) {
            c = P.res[m.y_off + j - 1];
            if (c > 20) { c = 20; atomicOr(P.status + p, PHMM_ST_BAD_RESIDUE); }
        }
        ys[j] = (unsigned char)c;
    }
    if (L.bins >= 0) {
        for (int idx = lane; idx < G * 21; idx += 32) sm[L.bins + idx] = 0.f;
        for (int idx = lane; idx < ROWS * (SH::NI > 0 ? SH::NI : 1); idx += 32) sm[L.colI + idx] = 0.f;
    }
    __syncwarp();
}

__device__ __forceinline__ int row_char(const KParams &P, int p, const PairMeta &m, int i) {
    if (i < 1 || i > m.Lx) return 0;
    int c = P.res[m.x_off + i - 1];
    return c > 20 ? 20 : c;
}

// exponent e with m * 2^-e in [0.5, 1) for m > 0 (normal or subnormal)
__device__ __forceinline__ int exp_of(float m) {
    const int b = (__float_as_int(m) >> 23) & 0xff;
    if (b != 0) return b - 126;
    int e;
    frexpf(m, &e);
    return e;
}

__device__ __forceinline__ float scale_pow2(float v, int e) {
    // v * 2^e for e possibly outside the normal range of a single factor
    if (e >= -126 && e <= 127) return v * pow2f(e);
    return ldexpf(v, e);
}

// ---------------------------------------------------------------- forward
template <class SH>
__device__ void fwd_stripe_w(const KParams &P, int p, int si, const SmemW &L, float *sm,
                             unsigned char *smb) {
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, KP = SH::KP, NM = SH::NM, NI = SH::NI;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int lane = threadIdx.x & 31;
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const int *prog_above = (si > 0) ? P.progress + m.stripe_base + si - 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_above = P.edge + (m.edge_base + (int64_t)(si - 1) * (Ly + 1)) * SP;
    const int *edgeE_above = P.edge_exp + m.edge_base + (int64_t)(si - 1) * (Ly + 1);
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * SP;
    int *edgeE_mine = P.edge_exp + m.edge_base + (int64_t)si * (Ly + 1);
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;

    load_model_w<SH>(P, p, m, L, sm, smb, false);
    const unsigned char *ys = smb + L.ys;
    const float4 *chi4 = reinterpret_cast<const float4 *>(sm + L.chi);

    // per-row constants: emission bases
    int rowi[R], xch[R];
    float eD[R][SH::ND > 0 ? SH::ND : 1];
    int offM[R][NM > 0 ? NM : 1];
#pragma unroll
    for (int c = 0; c < R; ++c) {
        rowi[c] = i0 + R * lane + c;
        xch[c] = row_char(P, p, m, rowi[c]);
#pragma unroll
        for (int k = 0; k < NM; ++k) offM[c][k] = L.tM + P.w_group[k] * 441 + xch[c] * 21;
#pragma unroll
        for (int k = 0; k < SH::ND; ++k) eD[c][k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xch[c]];
    }
    int offI[NI > 0 ? NI : 1];
#pragma unroll
    for (int k = 0; k < NI; ++k) offI[k] = L.tI + P.w_group[NM + k] * 21;

    float prev[R][NSRC], pp[NSRC], d0[NSRC], m0[NSRC];
    int Eprev[R], Epp = EXP_NONE, Em0 = EXP_NONE;
#pragma unroll
    for (int s = 0; s < NSRC; ++s) {
        prev[0][s] = 0.f; prev[1][s] = 0.f; pp[s] = 0.f; d0[s] = 0.f; m0[s] = 0.f;
    }
    Eprev[0] = Eprev[1] = EXP_NONE;
    const int T_last = (nrows - 1) + Ly;
    bool aborted = false;
    // halo prefetch state (lane 0 of a stripe that has one above)
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (si > 0 && lane == 0) pv = ld_acquire(prog_above);

    for (int t = 0; t <= T_last; ++t) {
        // ---- halo (row i0-1, column t) for lane 0's cell A: normally prefetched
        // into registers during step t-1; fetched synchronously otherwise
        if (si > 0 && t <= Ly) {
            int ok = 1;
            if (lane == 0 && hx_col != t) {
                if (!wait_geq(prog_above, t + 1, P.spin_limit)) {
                    ok = 0;
                } else {
                    const float4 *src = reinterpret_cast<const float4 *>(edge_above + (int64_t)t * SP);
#pragma unroll
                    for (int q = 0; q < SP / 4; ++q) {
                        const float4 v = __ldcg(src + q);
                        hx[4 * q] = v.x; hx[4 * q + 1] = v.y; hx[4 * q + 2] = v.z; hx[4 * q + 3] = v.w;
                    }
                    hxE = __ldcg(edgeE_above + t);
                    hx_col = t;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) { aborted = true; break; }
        }
        int jc[R];
        bool valid[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            jc[c] = t - (R * lane + c);
            valid[c] = (R * lane + c < nrows) && jc[c] >= 0 && jc[c] <= Ly;
        }
        // ---- predecessor exponents
        int EdA = __shfl_up_sync(0xffffffffu, Eprev[R - 1], 1);
        const bool lane0_halo = (lane == 0) && (si > 0) && (t <= Ly);
        if (lane == 0) EdA = lane0_halo ? hxE : EXP_NONE;
        // existence of predecessors
        const bool hasI0 = jc[0] >= 1, hasD0 = rowi[0] >= 1, hasM0 = hasI0 && hasD0;
        const bool hasI1 = jc[1] >= 1, hasD1 = rowi[1] >= 1, hasM1 = hasI1 && hasD1;
        const int EI0 = hasI0 ? Eprev[0] : EXP_NONE, ED0 = hasD0 ? EdA : EXP_NONE, EM0 = hasM0 ? Em0 : EXP_NONE;
        const int EI1 = hasI1 ? Eprev[1] : EXP_NONE, ED1 = hasD1 ? Eprev[0] : EXP_NONE, EM1 = hasM1 ? Epp : EXP_NONE;
        const int Eref0 = max(max(EI0, ED0), EM0), Eref1 = max(max(EI1, ED1), EM1);
        // ---- the contraction: acc[c][k] = sum_s pred_type(k)[s] chi[s][k]
        float acc[R][NE];
#pragma unroll
        for (int c = 0; c < R; ++c)
#pragma unroll
            for (int k = 0; k < NE; ++k) acc[c][k] = 0.f;
#pragma unroll
        for (int s = 0; s < NSRC; ++s) {
            float dA = __shfl_up_sync(0xffffffffu, prev[R - 1][s], 1);
            if (lane == 0) dA = lane0_halo ? hx[s] : 0.f;
            d0[s] = dA;
            const float pI0 = prev[0][s], pD0 = dA, pM0 = m0[s];
            const float pI1 = prev[1][s], pD1 = prev[0][s], pM1 = pp[s];
            const float4 *row = chi4 + s * (KP / 4);
#pragma unroll
            for (int kq = 0; kq < KP / 4; ++kq) {
                const float4 cv = row[kq];
                const float cvs[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = 4 * kq + u;
                    if (k < NE) {
                        const int ty = SH::type_of(k);
                        const float p0 = ty == T_M ? pM0 : (ty == T_I ? pI0 : pD0);
                        const float p1 = ty == T_M ? pM1 : (ty == T_I ? pI1 : pD1);
                        acc[0][k] = fmaf(p0, cvs[u], acc[0][k]);
                        acc[1][k] = fmaf(p1, cvs[u], acc[1][k]);
                    }
                }
            }
        }
        // ---- emissions, type scales, per-cell renormalisation
        const float sM0 = hasM0 ? pow2f(EM0 - Eref0) : 0.f, sI0 = hasI0 ? pow2f(EI0 - Eref0) : 0.f;
        const float sD0 = hasD0 ? pow2f(ED0 - Eref0) : 0.f;
        const float sM1 = hasM1 ? pow2f(EM1 - Eref1) : 0.f, sI1 = hasI1 ? pow2f(EI1 - Eref1) : 0.f;
        const float sD1 = hasD1 ? pow2f(ED1 - Eref1) : 0.f;
        int Enew[R];
        float mx[R] = {0.f, 0.f};
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int yj = valid[c] ? ys[jc[c]] : 0;
            const float sM = c == 0 ? sM0 : sM1, sI = c == 0 ? sI0 : sI1, sD = c == 0 ? sD0 : sD1;
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                float e;
                const int ty = SH::type_of(k);
                if (ty == T_M) e = sm[offM[c][k] + yj] * sM;
                else if (ty == T_I) e = sm[offI[k - NM] + yj] * sI;
                else e = eD[c][k - NM - NI] * sD;
                acc[c][k] = valid[c] ? acc[c][k] * e : 0.f;
                mx[c] = fmaxf(mx[c], acc[c][k]);
            }
            const int Eref = c == 0 ? Eref0 : Eref1;
            if (mx[c] > 0.f) {
                const int e = exp_of(mx[c]);
                const float sc = pow2f(-e);
                if (-e >= -126 && -e <= 127) {
#pragma unroll
                    for (int k = 0; k < NE; ++k) acc[c][k] *= sc;
                } else {
#pragma unroll
                    for (int k = 0; k < NE; ++k) acc[c][k] = ldexpf(acc[c][k], -e);
                }
                Enew[c] = Eref + e;
            } else {
                Enew[c] = EXP_NONE;
            }
        }
        // origin: F[0,0,start] = 1
        float sNew[R] = {0.f, 0.f};
        if (valid[0] && rowi[0] == 0 && jc[0] == 0) { sNew[0] = 1.f; Enew[0] = 0; }
        // ---- outputs: lattice, edge row, log-likelihood
#pragma unroll
        for (int c = 0; c < R; ++c) {
            if (!valid[c]) continue;
            const int rho = R * lane + c;
            if (P.lat) {
                float4 *dst = reinterpret_cast<float4 *>(P.lat + (latc + (int64_t)t * ROWS + rho) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        v[u] = s < NE ? acc[c][s] : (s == NE ? sNew[c] : 0.f);
                    }
                    dst[q] = make_float4(v[0], v[1], v[2], v[3]);
                }
                P.lat_exp[latc + (int64_t)t * ROWS + rho] = Enew[c];
            }
            if (has_below && rho == ROWS - 1) {
                float4 *dst = reinterpret_cast<float4 *>(edge_mine + (int64_t)jc[c] * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        v[u] = s < NE ? acc[c][s] : (s == NE ? sNew[c] : 0.f);
                    }
                    dst[q] = make_float4(v[0], v[1], v[2], v[3]);
                }
                edgeE_mine[jc[c]] = Enew[c];
                const int jb = jc[c];
                if (((jb + 1) % PUB) == 0 || jb == Ly) st_release(prog_mine, jb + 1);
            }
            if (rowi[c] == Lx && jc[c] == Ly && si + 1 == m.n_stripes) {
                double a = 0.0;
#pragma unroll
                for (int s = 0; s < NE; ++s) a += (double)acc[c][s] * (double)sm[L.chiE + s];
                a += (double)sNew[c] * (double)sm[L.chiE + NE];
                double ll = NEG_INF_LL;
                if (a > 0.0 && isfinite(a) && Enew[c] > EXP_NONE) ll = log(a) + (double)Enew[c] * LN2;
                else atomicOr(P.status + p, PHMM_ST_ZERO_LL);
                P.ll[p] = ll;
            }
        }
        // ---- shift the register history
#pragma unroll
        for (int s = 0; s < NSRC; ++s) {
            m0[s] = d0[s];
            pp[s] = prev[0][s];
            prev[0][s] = s < NE ? acc[0][s] : (s == NE ? sNew[0] : 0.f);
            prev[1][s] = s < NE ? acc[1][s] : (s == NE ? sNew[1] : 0.f);
        }
        Em0 = EdA;
        Epp = Eprev[0];
        Eprev[0] = Enew[0];
        Eprev[1] = Enew[1];
        // ---- prefetch halo column t+1 when the progress read last step covers it
        if (si > 0 && lane == 0 && t + 1 <= Ly) {
            if (pv > t + 1) {
                const float4 *src = reinterpret_cast<const float4 *>(edge_above + (int64_t)(t + 1) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    const float4 v = __ldcg(src + q);
                    hx[4 * q] = v.x; hx[4 * q + 1] = v.y; hx[4 * q + 2] = v.z; hx[4 * q + 3] = v.w;
                }
                hxE = __ldcg(edgeE_above + t + 1);
                hx_col = t + 1;
            }
            // poll the stripe above only when its last known progress does not
            // cover the next prefetch (an acquire load per step is costly)
            if (pv <= t + 2) pv = ld_acquire(prog_above);
        }
    }
    if (aborted) {
        if (lane == 31 && has_below) st_release(prog_mine, Ly + 1);
        if (lane == 0) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (si + 1 == m.n_stripes) P.ll[p] = NEG_INF_LL;
        }
    }
    // stripe complete (lattice and, for the last stripe, the log-likelihood):
    // the count pass of the split E-step may start on it
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(prog_mine, Ly + 2);
}

template <class SH>
__global__ void __launch_bounds__(32) forward_warp_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemW L = make_smem_w(SH::SP, SH::KP, SH::NI, P.G, P.max_ly, false);
    for (;;) {
        int it = 0;
        if ((threadIdx.x & 31) == 0) it = atomicAdd(P.counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        fwd_stripe_w<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

// ---------------------------------------------------------------- backward + counts
template <class SH>
__device__ void bwd_stripe_w(const KParams &P, int p, int si, const SmemW &L, float *sm,
                             unsigned char *smb) {
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, KP = SH::KP, NM = SH::NM, NI = SH::NI;
    constexpr int ND = SH::ND, SPP = SH::SPP, KPP = SH::KPP;
    const PairMeta m = P.meta[p];
    const int N = P.N, G = P.G;
    const int Lx = m.Lx, Ly = m.Ly;
    const int lane = threadIdx.x & 31;
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const bool has_above = si > 0;
    const int *prog_below = has_below ? P.progress + m.stripe_base + si + 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_below = P.edge + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * SP;
    const int *edgeE_below = P.edge_exp + m.edge_base + (int64_t)(si + 1) * (Ly + 1);
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * SP;
    int *edgeE_mine = P.edge_exp + m.edge_base + (int64_t)si * (Ly + 1);
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;

    const double llv = P.ll[p];
    if (!(llv > -1e29)) {
        if (lane == 0 && has_above) st_release(prog_mine, Ly + 1);
        __syncwarp();
        return;
    }
    const double lam = llv / LN2;
    const double Epd = floor(lam);
    const int Ep = (int)Epd;
    const float rfrac = (float)exp2(-(lam - Epd));

    load_model_w<SH>(P, p, m, L, sm, smb, true);
    const unsigned char *ys = smb + L.ys;
    const float4 *chiB4 = reinterpret_cast<const float4 *>(sm + L.chi);   // chiB[k][s]
    float *fst = sm + L.fst;
    int *fstE = reinterpret_cast<int *>(sm) + L.fstE;
    float *ust = sm + L.ust;
    float *bins = sm + L.bins;
    float *colI = sm + L.colI;
    // D-type emission counts: the row character is fixed per lane -> registers (Kahan)
    float dcnt[R][ND > 0 ? ND : 1], dcmp[R][ND > 0 ? ND : 1];
#pragma unroll
    for (int c = 0; c < R; ++c)
#pragma unroll
        for (int k = 0; k < ND; ++k) { dcnt[c][k] = 0.f; dcmp[c][k] = 0.f; }
    double *cntM_pair = P.cntM + (int64_t)p * G * 441;

    int rowi[R], xch[R];
    float eD[R][SH::ND > 0 ? SH::ND : 1];
    int offM[R][NM > 0 ? NM : 1];
#pragma unroll
    for (int c = 0; c < R; ++c) {
        rowi[c] = i0 + R * lane + c;
        xch[c] = row_char(P, p, m, rowi[c]);
#pragma unroll
        for (int k = 0; k < NM; ++k) offM[c][k] = L.tM + P.w_group[k] * 441 + xch[c] * 21;
#pragma unroll
        for (int k = 0; k < SH::ND; ++k) eD[c][k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xch[c]];
    }
    int offI[NI > 0 ? NI : 1];
#pragma unroll
    for (int k = 0; k < NI; ++k) offI[k] = L.tI + P.w_group[NM + k] * 21;

    // count-phase role
    const int blk = lane % SH::NBLK, grp = lane / SH::NBLK;
    const bool counter = grp < SH::GROUPS;
    const int bs = blk / SH::BK, bk = blk % SH::BK;
    float csum[16], ccomp[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) { csum[u] = 0.f; ccomp[u] = 0.f; }

    // successor histories (w = e * b of dest slots)
    float wn[R][NE], wnn1[NE], dR[NE], mR[NE];
    int Ewn[R] = {EXP_NONE, EXP_NONE}, Ewnn1 = EXP_NONE, EmR = EXP_NONE;
#pragma unroll
    for (int k = 0; k < NE; ++k) { wn[0][k] = 0.f; wn[1][k] = 0.f; wnn1[k] = 0.f; dR[k] = 0.f; mR[k] = 0.f; }

    const int T_last = (nrows - 1) + Ly;
    auto prefetch = [&](int t) {
        if (t >= 0) {
            const float *src = P.lat + (latc + (int64_t)t * ROWS) * SP;
            float *dst = fst + (t & 1) * ROWS * SPP;
            for (int idx = lane; idx < ROWS * SP / 4; idx += 32) {
                const int r = idx / (SP / 4), q = idx % (SP / 4);
                cp_async16(dst + r * SPP + 4 * q, src + 4 * idx);
            }
            const int *srcE = P.lat_exp + latc + (int64_t)t * ROWS;
            int *dstE = fstE + (t & 1) * ROWS;
            for (int idx = lane; idx < ROWS / 4; idx += 32) cp_async16(dstE + 4 * idx, srcE + 4 * idx);
        }
        cp_commit();
    };
    prefetch(T_last);
    bool aborted = false;
    // halo prefetch state (lane 31 of a stripe that has one below)
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (has_below && lane == 31) pv = ld_acquire(prog_below);

    for (int t = T_last; t >= 0; --t) {
        prefetch(t - 1);
        // ---- halo (row i0+64, column t-63) for lane 31's cell B: normally
        // prefetched into registers during step t+1; fetched synchronously otherwise
        const int jb = t - (ROWS - 1);
        if (has_below && jb >= 0 && jb <= Ly) {
            int ok = 1;
            if (lane == 31 && hx_col != jb) {
                if (!wait_geq(prog_below, Ly + 1 - jb, P.spin_limit)) {
                    ok = 0;
                } else {
                    const float4 *src = reinterpret_cast<const float4 *>(edge_below + (int64_t)jb * SP);
#pragma unroll
                    for (int q = 0; q < SP / 4; ++q) {
                        const float4 v = __ldcg(src + q);
                        hx[4 * q] = v.x; hx[4 * q + 1] = v.y; hx[4 * q + 2] = v.z; hx[4 * q + 3] = v.w;
                    }
                    hxE = __ldcg(edgeE_below + jb);
                    hx_col = jb;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 31);
            if (!ok) { aborted = true; break; }
        }
        int jc[R];
        bool valid[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            jc[c] = t - (R * lane + c);
            valid[c] = (R * lane + c < nrows) && jc[c] >= 0 && jc[c] <= Ly;
        }
        const bool lane31_halo = (lane == 31) && has_below && jc[1] >= 0 && jc[1] <= Ly;
        int EdRn = __shfl_down_sync(0xffffffffu, Ewn[0], 1);
        if (lane == 31) EdRn = lane31_halo ? hxE : EXP_NONE;
        // successor existence and exponents
        const bool term0 = valid[0] && rowi[0] == Lx && jc[0] == Ly;
        const bool term1 = valid[1] && rowi[1] == Lx && jc[1] == Ly;
        const bool hI0 = jc[0] + 1 <= Ly, hD0 = rowi[0] + 1 <= Lx, hM0 = hI0 && hD0;
        const bool hI1 = jc[1] + 1 <= Ly, hD1 = rowi[1] + 1 <= Lx, hM1 = hI1 && hD1;
        // cell A: I = A(t+1), D = B(t+1), M = B(t+2); cell B: I = B(t+1), D = lane+1 A(t+1), M = saved
        const int EI0 = hI0 ? Ewn[0] : EXP_NONE, ED0 = hD0 ? Ewn[1] : EXP_NONE, EM0 = hM0 ? Ewnn1 : EXP_NONE;
        const int EI1 = hI1 ? Ewn[1] : EXP_NONE, ED1 = hD1 ? EdRn : EXP_NONE, EM1 = hM1 ? EmR : EXP_NONE;
        const int Eref0 = term0 ? 0 : max(max(EI0, ED0), EM0);
        const int Eref1 = term1 ? 0 : max(max(EI1, ED1), EM1);
        const float sM0 = (hM0 && !term0) ? pow2f(EM0 - Eref0) : 0.f, sI0 = (hI0 && !term0) ? pow2f(EI0 - Eref0) : 0.f;
        const float sD0 = (hD0 && !term0) ? pow2f(ED0 - Eref0) : 0.f;
        const float sM1 = (hM1 && !term1) ? pow2f(EM1 - Eref1) : 0.f, sI1 = (hI1 && !term1) ? pow2f(EI1 - Eref1) : 0.f;
        const float sD1 = (hD1 && !term1) ? pow2f(ED1 - Eref1) : 0.f;
        float acc[R][NSRC];
#pragma unroll
        for (int s = 0; s < NSRC; ++s) { acc[0][s] = 0.f; acc[1][s] = 0.f; }
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            float dk = __shfl_down_sync(0xffffffffu, wn[0][k], 1);
            if (lane == 31) dk = lane31_halo ? hx[k] : 0.f;
            dR[k] = dk;
            const int ty = SH::type_of(k);
            const float w0 = ty == T_M ? wnn1[k] * sM0 : (ty == T_I ? wn[0][k] * sI0 : wn[1][k] * sD0);
            const float w1 = ty == T_M ? mR[k] * sM1 : (ty == T_I ? wn[1][k] * sI1 : dk * sD1);
            const float4 *col = chiB4 + k * (SP / 4);
#pragma unroll
            for (int sq = 0; sq < SP / 4; ++sq) {
                const float4 cv = col[sq];
                const float cvs[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = 4 * sq + u;
                    if (s < NSRC) {
                        acc[0][s] = fmaf(w0, cvs[u], acc[0][s]);
                        acc[1][s] = fmaf(w1, cvs[u], acc[1][s]);
                    }
                }
            }
        }
        // terminal cell: b[s] = chi[s, End]
        if (term0) {
#pragma unroll
            for (int s = 0; s < NSRC; ++s) acc[0][s] = sm[L.chiE + s];
        }
        if (term1) {
#pragma unroll
            for (int s = 0; s < NSRC; ++s) acc[1][s] = sm[L.chiE + s];
        }
        // ---- renormalise, w = e*b, count operands
        cp_wait1();
        __syncwarp();
        float wnew[R][NE];
        int Eb[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            float mxv = 0.f;
#pragma unroll
            for (int s = 0; s < NSRC; ++s) {
                if (!valid[c]) acc[c][s] = 0.f;
                mxv = fmaxf(mxv, acc[c][s]);
            }
            const int Eref = c == 0 ? Eref0 : Eref1;
            int e = 0;
            if (mxv > 0.f) {
                e = exp_of(mxv);
#pragma unroll
                for (int s = 0; s < NSRC; ++s) acc[c][s] = scale_pow2(acc[c][s], -e);
                Eb[c] = Eref + e;
            } else {
                Eb[c] = EXP_NONE;
            }
            const int yj = valid[c] ? ys[jc[c]] : 0;
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                float ev;
                const int ty = SH::type_of(k);
                if (ty == T_M) ev = sm[offM[c][k] + yj];
                else if (ty == T_I) ev = sm[offI[k - NM] + yj];
                else ev = eD[c][k - NM - NI];
                wnew[c][k] = acc[c][k] * ev;
            }
            const int rho = R * lane + c;
            // forward values of this cell -> f~ (in place in the staging buffer)
            float *fcell = fst + (t & 1) * ROWS * SPP + rho * SPP;
            const int Ef = fstE[(t & 1) * ROWS + rho];
            float fsc = 0.f;
            if (valid[c] && Ef > EXP_NONE && Eb[c] > EXP_NONE) {
                int d = Ef + Eb[c] - Ep;
                if (d > 126) { d = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                fsc = scale_pow2(rfrac, max(d, -200));
            }
            float post[NSRC];
#pragma unroll
            for (int q = 0; q < SP / 4; ++q) {
                const float4 fv = reinterpret_cast<const float4 *>(fcell)[q];
                const float fa[4] = {fv.x, fv.y, fv.z, fv.w};
                float ftq[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = 4 * q + u;
                    ftq[u] = (s < NSRC && fsc > 0.f) ? fa[u] * fsc : 0.f;
                    if (s < NSRC) post[s] = ftq[u] * acc[c][s];
                }
                reinterpret_cast<float4 *>(fcell)[q] = make_float4(ftq[0], ftq[1], ftq[2], ftq[3]);
            }
            // u~[k] = w_succ(k)[k] * 2^(E_succ - Eb)
            const float uM = mxv > 0.f ? fminf(scale_pow2(c == 0 ? sM0 : sM1, -e), 3e38f) : 0.f;
            const float uI = mxv > 0.f ? fminf(scale_pow2(c == 0 ? sI0 : sI1, -e), 3e38f) : 0.f;
            const float uD = mxv > 0.f ? fminf(scale_pow2(c == 0 ? sD0 : sD1, -e), 3e38f) : 0.f;
            float *ucell = ust + rho * KPP;
#pragma unroll
            for (int q = 0; q < KP / 4; ++q) {
                float uq[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int k = 4 * q + v;
                    float u = 0.f;
                    if (k < NE) {
                        const int ty = SH::type_of(k);
                        if (c == 0) u = ty == T_M ? wnn1[k] * uM : (ty == T_I ? wn[0][k] * uI : wn[1][k] * uD);
                        else u = ty == T_M ? mR[k] * uM : (ty == T_I ? wn[1][k] * uI : dR[k] * uD);
                    }
                    uq[v] = (valid[c] && fsc > 0.f) ? u : 0.f;
                }
                reinterpret_cast<float4 *>(ucell)[q] = make_float4(uq[0], uq[1], uq[2], uq[3]);
            }
            if (valid[c]) {
                // posteriors -> emission counts: M straight to float64 global
                // reductions, I into this column's ring slot, D into registers
#pragma unroll
                for (int k = 0; k < NE; ++k) {
                    const int ty = SH::type_of(k);
                    if (ty == T_M) {
                        if (post[k] != 0.f)
                            atomicAdd(cntM_pair + P.w_group[k] * 441 + xch[c] * 21 + yj, (double)post[k]);
                    } else if (ty == T_I) {
                        colI[(jc[c] % ROWS) * NI + (k - NM)] += post[k];
                    } else {
                        const int kd = k - NM - NI;
                        const float y = post[k] - dcmp[c][kd];
                        const float tt = dcnt[c][kd] + y;
                        dcmp[c][kd] = (tt - dcnt[c][kd]) - y;
                        dcnt[c][kd] = tt;
                    }
                }
                if ((c == 0 && term0) || (c == 1 && term1)) {
#pragma unroll
                    for (int s = 0; s < NSRC; ++s)
                        atomicAdd(P.n_trans + ((int64_t)p * N + P.w_orig[s]) * N + P.e_idx, (double)post[s]);
                }
                if (has_above && rowi[c] == i0) {   // top row -> edge for the stripe above
                    float4 *dst = reinterpret_cast<float4 *>(edge_mine + (int64_t)jc[c] * SP);
#pragma unroll
                    for (int q = 0; q < SP / 4; ++q) {
                        float v[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int k = 4 * q + u;
                            v[u] = k < NE ? wnew[c][k] : 0.f;
                        }
                        dst[q] = make_float4(v[0], v[1], v[2], v[3]);
                    }
                    edgeE_mine[jc[c]] = Eb[c];
                    if ((jc[c] % PUB) == 0) st_release(prog_mine, Ly + 1 - jc[c]);
                }
            }
        }
        __syncwarp();
        // ---- column t is complete once row i0 (lane 0, cell A) has visited it
        if (lane == 0 && t <= Ly) {
            const int slot = t % ROWS;
            const int yj = ys[t];
#pragma unroll
            for (int k = 0; k < NI; ++k) {
                bins[P.w_group[NM + k] * 21 + yj] += colI[slot * NI + k];
                colI[slot * NI + k] = 0.f;
            }
        }
        // ---- transition-count outer products over the 64 cells of this step
        if (counter) {
            float pz[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) pz[u] = 0.f;
            const int r0 = grp * ROWS / SH::GROUPS, r1 = (grp + 1) * ROWS / SH::GROUPS;
            for (int rr = r0; rr < r1; ++rr) {
                const float4 fv = reinterpret_cast<const float4 *>(fst + (t & 1) * ROWS * SPP + rr * SPP)[bs];
                const float4 uv = reinterpret_cast<const float4 *>(ust + rr * KPP)[bk];
                const float fa[4] = {fv.x, fv.y, fv.z, fv.w};
                const float ua[4] = {uv.x, uv.y, uv.z, uv.w};
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) pz[4 * a + b] = fmaf(fa[a], ua[b], pz[4 * a + b]);
            }
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const float y = pz[u] - ccomp[u];
                const float tt = csum[u] + y;
                ccomp[u] = (tt - csum[u]) - y;
                csum[u] = tt;
            }
        }
        __syncwarp();
        // ---- shift histories
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            mR[k] = dR[k];
            wnn1[k] = wn[1][k];
            wn[0][k] = valid[0] ? wnew[0][k] : 0.f;
            wn[1][k] = valid[1] ? wnew[1][k] : 0.f;
        }
        EmR = EdRn;
        Ewnn1 = Ewn[1];
        Ewn[0] = valid[0] ? Eb[0] : EXP_NONE;
        Ewn[1] = valid[1] ? Eb[1] : EXP_NONE;
        // ---- prefetch halo column jb-1 when the progress read last step covers it
        if (has_below && lane == 31 && jb - 1 >= 0 && jb - 1 <= Ly) {
            if (pv >= Ly + 1 - (jb - 1)) {
                const float4 *src = reinterpret_cast<const float4 *>(edge_below + (int64_t)(jb - 1) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    const float4 v = __ldcg(src + q);
                    hx[4 * q] = v.x; hx[4 * q + 1] = v.y; hx[4 * q + 2] = v.z; hx[4 * q + 3] = v.w;
                }
                hxE = __ldcg(edgeE_below + jb - 1);
                hx_col = jb - 1;
            }
            if (pv < Ly + 3 - jb) pv = ld_acquire(prog_below);   // only when the next prefetch needs more
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (aborted) {
        if (lane == 0) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (has_above) st_release(prog_mine, Ly + 1);
        }
        __syncwarp();
        return;
    }
    // ---- flush transition counts n[s,k] = chi[s,k] * sum f~ u~
    if (counter) {
        const float *chi = P.chi + (int64_t)p * P.chi_stride;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int s = 4 * bs + (u >> 2), k = 4 * bk + (u & 3);
            const float val = csum[u] - ccomp[u];
            if (s >= NSRC || k >= NE || val == 0.f) continue;
            const int os = P.w_orig[s], ok = P.w_orig[k];
            atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + ok, (double)val * (double)__ldg(chi + os * N + ok));
        }
    }
#pragma unroll
    for (int c = 0; c < R; ++c) {
        const int rho = R * lane + c;
        if (rho >= nrows || rowi[c] < 1) continue;
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            const float v = dcnt[c][k] - dcmp[c][k];
            if (v != 0.f)
                atomicAdd(P.cntD + ((int64_t)p * G + P.w_group[NM + NI + k]) * 21 + xch[c], (double)v);
        }
    }
    __syncwarp();
    for (int idx = lane; idx < G * 21; idx += 32) {
        const float v = bins[idx];
        if (v != 0.f) atomicAdd(P.cntI + (int64_t)p * G * 21 + idx, (double)v);
    }
    __syncwarp();
}

template <class SH>
__global__ void __launch_bounds__(32) backward_warp_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemW L = make_smem_w(SH::SP, SH::KP, SH::NI, P.G, P.max_ly, true);
    for (;;) {
        int it = 0;
        if ((threadIdx.x & 31) == 0) it = atomicAdd(P.counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        bwd_stripe_w<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

}  // namespace warp2
