// estep_twowarp.cuh -- two-warp stripe kernels of the split E-step (included
// by pairhmm.cu after estep_split.cuh).
//
// The one-warp kernels give each lane two rows of a 64-row stripe, so one
// anti-diagonal step costs a lane two cells' contractions (about 1,100 warp
// instructions at 17 states).  The wavefront's critical path is a chain of
// such steps, so its length is steps x per-step latency, and a lone warp
// issues at well under one instruction per cycle.  Here a stripe is a CTA of
// 64 threads, one lattice row each: thread r computes cell (i0 + r, t - r)
// at step t, half the work per step of the one-warp kernels.  Inside a warp
// the neighbour row comes by __shfl; across the two warps (row 31 -> row 32)
// it goes through a double-buffered shared-memory slot, written by the
// producing thread at the end of step t and read at step t+1, with one
// __syncthreads per step.
//
// The lattice layout (cell (t, rho) of stripe si at lat_base + si*(64+Ly)*64
// + t*64 + rho), the edge rows and the progress counters are those of the
// one-warp kernels, so count_warp_kernel reads these lattices unchanged.

namespace warp2 {

constexpr int TWT = 64;   // threads per stripe CTA (= ROWS)

struct SmemTW {
    SmemW w;        // model tables, halo staging and the y characters
    int bnd;        // float offset: boundary slots [2][SP]
    int bndE;       // int offset: boundary exponents [2]
    int flag;       // int offset: [0], [1] abort flags by step parity, [2] popped item
    int bytes;
};

__host__ __device__ inline SmemTW make_smem_tw(int SP, int KP, int NI, int G, int max_ly, bool bwd) {
    SmemTW L;
    L.w = make_smem_w(SP, KP, NI, G, max_ly, bwd, false);
    int o = L.w.bytes / 4;   // L.w.bytes is a multiple of 16
    L.bnd = o; o += 2 * SP;
    L.bndE = o; o += 4;
    L.flag = o; o += 4;
    L.bytes = o * 4;
    return L;
}

template <class SH>
__device__ void fwd_stripe_tw(const KParams &P, int p, int si, const SmemTW &LT, float *sm,
                              unsigned char *smb) {
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, KP = SH::KP, NM = SH::NM, NI = SH::NI;
    const SmemW &L = LT.w;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int r = threadIdx.x, lane = r & 31;
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
    float *bnd = sm + LT.bnd;
    int *bndE = reinterpret_cast<int *>(sm) + LT.bndE;
    volatile int *s_abort = reinterpret_cast<int *>(sm) + LT.flag;

    if (r < 32) load_model_w<SH>(P, p, m, L, sm, smb, false);
    if (r < 2 * SP) bnd[r] = 0.f;
    if (r < 2) bndE[r] = EXP_NONE;
    if (r < 2) s_abort[r] = 0;
    __syncthreads();
    const unsigned char *ys = smb + L.ys;
    const float4 *chi4 = reinterpret_cast<const float4 *>(sm + L.chi);

    const int rowi = i0 + r;
    const int xch = row_char(P, p, m, rowi);
    float eD[SH::ND > 0 ? SH::ND : 1];
    int offM[NM > 0 ? NM : 1];
#pragma unroll
    for (int k = 0; k < NM; ++k) offM[k] = L.tM + P.w_group[k] * 441 + xch * 21;
#pragma unroll
    for (int k = 0; k < SH::ND; ++k) eD[k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xch];
    int offI[NI > 0 ? NI : 1];
#pragma unroll
    for (int k = 0; k < NI; ++k) offI[k] = L.tI + P.w_group[NM + k] * 21;

    float prev[NSRC], d0[NSRC], m0[NSRC];
    int Eprev = EXP_NONE, Em0 = EXP_NONE;
#pragma unroll
    for (int s = 0; s < NSRC; ++s) { prev[s] = 0.f; d0[s] = 0.f; m0[s] = 0.f; }
    const int T_last = (nrows - 1) + Ly;
    // M- and I-type emission factors of the cell of the next step, loaded one
    // step ahead (the y character and the table lookup are two dependent loads)
    float eMI[NM + NI > 0 ? NM + NI : 1];
    auto load_emit = [&](int tt) {
        const int j = tt - r;
        const int yj = (r < nrows && j >= 0 && j <= Ly) ? ys[j] : 0;
#pragma unroll
        for (int k = 0; k < NM; ++k) eMI[k] = sm[offM[k] + yj];
#pragma unroll
        for (int k = 0; k < NI; ++k) eMI[NM + k] = sm[offI[k] + yj];
    };
    load_emit(0);
    bool aborted = false;
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (si > 0 && r == 0) pv = ld_acquire(prog_above);

    for (int t = 0; t <= T_last; ++t) {
        // halo (row i0-1, column t) for thread 0: normally prefetched during step t-1
        if (si > 0 && t <= Ly && r == 0 && hx_col != t) {
            if (!wait_geq(prog_above, t + 1, P.spin_limit)) {
                s_abort[t & 1] = 1;   // read by all threads after this step's barrier
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
        const int jc = t - r;
        const bool valid = r < nrows && jc >= 0 && jc <= Ly;
        const bool halo = (r == 0) && (si > 0) && (t <= Ly);
        const int slot = (t + 1) & 1;   // written by thread 31 at step t-1
        // the row above at step t-1: shuffles for lanes 1..31; lane 0 takes the
        // halo (thread 0) or the boundary slot (thread 32).  The slot is read by
        // the whole CTA as broadcast loads and merged by selects, so nothing in
        // the contraction waits on a divergent branch.
        float bv[SP];
        {
            const float4 *b4 = reinterpret_cast<const float4 *>(bnd + slot * SP);
#pragma unroll
            for (int q = 0; q < SP / 4; ++q) {
                const float4 v = b4[q];
                bv[4 * q] = v.x; bv[4 * q + 1] = v.y; bv[4 * q + 2] = v.z; bv[4 * q + 3] = v.w;
            }
        }
        const bool l0 = lane == 0, top = r == 0;
        int EdA = __shfl_up_sync(0xffffffffu, Eprev, 1);
        EdA = l0 ? (top ? (halo ? hxE : EXP_NONE) : bndE[slot]) : EdA;
#pragma unroll
        for (int s = 0; s < NSRC; ++s) {
            const float v = __shfl_up_sync(0xffffffffu, prev[s], 1);
            d0[s] = l0 ? (top ? (halo ? hx[s] : 0.f) : bv[s]) : v;
        }
        const bool hasI = jc >= 1, hasD = rowi >= 1, hasM = hasI && hasD;
        const int EI = hasI ? Eprev : EXP_NONE, ED = hasD ? EdA : EXP_NONE, EM = hasM ? Em0 : EXP_NONE;
        const int Eref = max(max(EI, ED), EM);
        float acc[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) acc[k] = 0.f;
#pragma unroll
        for (int s = 0; s < NSRC; ++s) {
            const float pI = prev[s], pD = d0[s], pM = m0[s];
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
                        const float pk = ty == T_M ? pM : (ty == T_I ? pI : pD);
                        acc[k] = fmaf(pk, cvs[u], acc[k]);
                    }
                }
            }
        }
        // emissions, type scales, per-cell renormalisation
        const float sM = hasM ? pow2f(EM - Eref) : 0.f, sI = hasI ? pow2f(EI - Eref) : 0.f;
        const float sD = hasD ? pow2f(ED - Eref) : 0.f;
        int Enew;
        float mx = 0.f;
        {
            float mxs[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                float e;
                const int ty = SH::type_of(k);
                if (ty == T_M) e = eMI[k] * sM;
                else if (ty == T_I) e = eMI[k] * sI;
                else e = eD[k - NM - NI] * sD;
                acc[k] = valid ? acc[k] * e : 0.f;
                mxs[k & 3] = fmaxf(mxs[k & 3], acc[k]);
            }
            mx = fmaxf(fmaxf(mxs[0], mxs[1]), fmaxf(mxs[2], mxs[3]));
            if (mx > 0.f) {
                const int e = exp_of(mx);
                if (-e >= -126 && -e <= 127) {
                    const float sc = pow2f(-e);
#pragma unroll
                    for (int k = 0; k < NE; ++k) acc[k] *= sc;
                } else {
#pragma unroll
                    for (int k = 0; k < NE; ++k) acc[k] = ldexpf(acc[k], -e);
                }
                Enew = Eref + e;
            } else {
                Enew = EXP_NONE;
            }
        }
        // origin: F[0,0,start] = 1
        float sNew = 0.f;
        if (valid && rowi == 0 && jc == 0) { sNew = 1.f; Enew = 0; }
        if (valid) {
            if (P.lat) {
                float4 *dst = reinterpret_cast<float4 *>(P.lat + (latc + (int64_t)t * ROWS + r) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        v[u] = s < NE ? acc[s] : (s == NE ? sNew : 0.f);
                    }
                    dst[q] = make_float4(v[0], v[1], v[2], v[3]);
                }
                P.lat_exp[latc + (int64_t)t * ROWS + r] = Enew;
            }
            if (has_below && r == ROWS - 1) {
                float4 *dst = reinterpret_cast<float4 *>(edge_mine + (int64_t)jc * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        v[u] = s < NE ? acc[s] : (s == NE ? sNew : 0.f);
                    }
                    dst[q] = make_float4(v[0], v[1], v[2], v[3]);
                }
                edgeE_mine[jc] = Enew;
                if (((jc + 1) % PUB) == 0 || jc == Ly) st_release(prog_mine, jc + 1);
            }
            if (rowi == Lx && jc == Ly && si + 1 == m.n_stripes) {
                double a = 0.0;
#pragma unroll
                for (int s = 0; s < NE; ++s) a += (double)acc[s] * (double)sm[L.chiE + s];
                a += (double)sNew * (double)sm[L.chiE + NE];
                double ll = NEG_INF_LL;
                if (a > 0.0 && isfinite(a) && Enew > EXP_NONE) ll = log(a) + (double)Enew * LN2;
                else atomicOr(P.status + p, PHMM_ST_ZERO_LL);
                P.ll[p] = ll;
            }
        }
        // shift the register history
#pragma unroll
        for (int s = 0; s < NSRC; ++s) {
            m0[s] = d0[s];
            prev[s] = s < NE ? acc[s] : (s == NE ? sNew : 0.f);
        }
        Em0 = EdA;
        Eprev = Enew;
        // row 31 hands its new state to row 32 for step t+1
        if (r == 31) {
#pragma unroll
            for (int s = 0; s < SP; ++s) bnd[(t & 1) * SP + s] = s < NSRC ? prev[s] : 0.f;
            bndE[t & 1] = Eprev;
        }
        load_emit(t + 1);
        // prefetch halo column t+1 when the progress read last step covers it
        if (si > 0 && r == 0 && t + 1 <= Ly) {
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
            if (pv <= t + 2) pv = ld_acquire(prog_above);
        }
        __syncthreads();
        // the flag of step t is written only before this barrier, and the
        // next write goes to the other parity: every thread sees the same value
        if (s_abort[t & 1]) { aborted = true; break; }
    }
    if (aborted) {
        if (r == ROWS - 1 && has_below) st_release(prog_mine, Ly + 1);
        if (r == 0) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (si + 1 == m.n_stripes) P.ll[p] = NEG_INF_LL;
        }
    }
    // stripe complete: the count pass may start on it
    __threadfence();
    __syncthreads();
    if (r == 0) st_release(prog_mine, Ly + 2);
}

template <class SH>
__device__ void bwd_rec_stripe_tw(const KParams &P, int p, int si, const SmemTW &LT, float *sm,
                                  unsigned char *smb) {
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, NM = SH::NM, NI = SH::NI;
    const SmemW &L = LT.w;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int r = threadIdx.x, lane = r & 31;
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
    float *bnd = sm + LT.bnd;
    int *bndE = reinterpret_cast<int *>(sm) + LT.bndE;
    volatile int *s_abort = reinterpret_cast<int *>(sm) + LT.flag;

    if (r < 32) load_model_w<SH>(P, p, m, L, sm, smb, true);
    if (r < 2 * SP) bnd[r] = 0.f;
    if (r < 2) bndE[r] = EXP_NONE;
    if (r < 2) s_abort[r] = 0;
    __syncthreads();
    const unsigned char *ys = smb + L.ys;
    const float4 *chiB4 = reinterpret_cast<const float4 *>(sm + L.chi);   // chiB[k][s]

    const int rowi = i0 + r;
    const int xch = row_char(P, p, m, rowi);
    float eD[SH::ND > 0 ? SH::ND : 1];
    int offM[NM > 0 ? NM : 1];
#pragma unroll
    for (int k = 0; k < NM; ++k) offM[k] = L.tM + P.w_group[k] * 441 + xch * 21;
#pragma unroll
    for (int k = 0; k < SH::ND; ++k) eD[k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xch];
    int offI[NI > 0 ? NI : 1];
#pragma unroll
    for (int k = 0; k < NI; ++k) offI[k] = L.tI + P.w_group[NM + k] * 21;

    // successors: I = own cell at step t+1 (wn), D = row r+1 at step t+1
    // (dR, received by shuffle or boundary slot), M = the D received at t+1 (mR)
    float wn[NE], dR[NE], mR[NE];
    int Ewn = EXP_NONE, EmR = EXP_NONE;
#pragma unroll
    for (int k = 0; k < NE; ++k) { wn[k] = 0.f; dR[k] = 0.f; mR[k] = 0.f; }

    const int T_last = (nrows - 1) + Ly;
    // M- and I-type emission factors of the cell of the next step, loaded one step ahead
    float eMI[NM + NI > 0 ? NM + NI : 1];
    auto load_emit = [&](int tt) {
        const int j = tt - r;
        const int yj = (r < nrows && j >= 0 && j <= Ly) ? ys[j] : 0;
#pragma unroll
        for (int k = 0; k < NM; ++k) eMI[k] = sm[offM[k] + yj];
#pragma unroll
        for (int k = 0; k < NI; ++k) eMI[NM + k] = sm[offI[k] + yj];
    };
    load_emit(T_last);
    bool aborted = false;
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (has_below && r == ROWS - 1) pv = ld_acquire(prog_below);

    for (int t = T_last; t >= 0; --t) {
        const int jb = t - (ROWS - 1);
        if (has_below && jb >= 0 && jb <= Ly && r == ROWS - 1 && hx_col != jb) {
            if (!wait_geq(prog_below, Ly + 1 - jb, P.spin_limit)) {
                s_abort[t & 1] = 1;   // read by all threads after this step's barrier
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
        const int jc = t - r;
        const bool valid = r < nrows && jc >= 0 && jc <= Ly;
        const bool halo = (r == ROWS - 1) && has_below && jc >= 0 && jc <= Ly;
        const int slot = (t + 1) & 1;   // written by thread 32 at step t+1
        // the row below at step t+1: shuffles for lanes 0..30; lane 31 takes the
        // halo (thread 63) or the boundary slot (thread 31), merged by selects
        float bv[SP];
        {
            const float4 *b4 = reinterpret_cast<const float4 *>(bnd + slot * SP);
#pragma unroll
            for (int q = 0; q < SP / 4; ++q) {
                const float4 v = b4[q];
                bv[4 * q] = v.x; bv[4 * q + 1] = v.y; bv[4 * q + 2] = v.z; bv[4 * q + 3] = v.w;
            }
        }
        const bool l31 = lane == 31, bottom = r == ROWS - 1;
        int EdRn = __shfl_down_sync(0xffffffffu, Ewn, 1);
        EdRn = l31 ? (bottom ? (halo ? hxE : EXP_NONE) : bndE[slot]) : EdRn;
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const float v = __shfl_down_sync(0xffffffffu, wn[k], 1);
            dR[k] = l31 ? (bottom ? (halo ? hx[k] : 0.f) : bv[k]) : v;
        }
        const bool term = valid && rowi == Lx && jc == Ly;
        const bool hI = jc + 1 <= Ly, hD = rowi + 1 <= Lx, hM = hI && hD;
        const int EI = hI ? Ewn : EXP_NONE, ED = hD ? EdRn : EXP_NONE, EM = hM ? EmR : EXP_NONE;
        const int Eref = term ? 0 : max(max(EI, ED), EM);
        const float sM = (hM && !term) ? pow2f(EM - Eref) : 0.f, sI = (hI && !term) ? pow2f(EI - Eref) : 0.f;
        const float sD = (hD && !term) ? pow2f(ED - Eref) : 0.f;
        float acc[NSRC];
#pragma unroll
        for (int s = 0; s < NSRC; ++s) acc[s] = 0.f;
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const float dk = dR[k];
            const int ty = SH::type_of(k);
            const float w = ty == T_M ? mR[k] * sM : (ty == T_I ? wn[k] * sI : dk * sD);
            const float4 *col = chiB4 + k * (SP / 4);
#pragma unroll
            for (int sq = 0; sq < SP / 4; ++sq) {
                const float4 cv = col[sq];
                const float cvs[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = 4 * sq + u;
                    if (s < NSRC) acc[s] = fmaf(w, cvs[u], acc[s]);
                }
            }
        }
        if (term) {
#pragma unroll
            for (int s = 0; s < NSRC; ++s) acc[s] = sm[L.chiE + s];
        }
        float wnew[NE];
        int Eb;
        {
            float mxs[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int s = 0; s < NSRC; ++s) {
                if (!valid) acc[s] = 0.f;
                mxs[s & 3] = fmaxf(mxs[s & 3], acc[s]);
            }
            const float mxv = fmaxf(fmaxf(mxs[0], mxs[1]), fmaxf(mxs[2], mxs[3]));
            if (mxv > 0.f) {
                const int e = exp_of(mxv);
#pragma unroll
                for (int s = 0; s < NSRC; ++s) acc[s] = scale_pow2(acc[s], -e);
                Eb = Eref + e;
            } else {
                Eb = EXP_NONE;
            }
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                float ev;
                const int ty = SH::type_of(k);
                if (ty == T_M || ty == T_I) ev = eMI[k];
                else ev = eD[k - NM - NI];
                wnew[k] = acc[k] * ev;
            }
        }
        if (valid) {
            float4 *dst = reinterpret_cast<float4 *>(P.blat + (latc + (int64_t)t * ROWS + r) * SP);
#pragma unroll
            for (int q = 0; q < SP / 4; ++q) {
                float v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = 4 * q + u;
                    v[u] = s < NSRC ? acc[s] : 0.f;
                }
                dst[q] = make_float4(v[0], v[1], v[2], v[3]);
            }
            P.blat_exp[latc + (int64_t)t * ROWS + r] = Eb;
            if (has_above && rowi == i0) {   // top row -> edge for the stripe above
                float4 *e = reinterpret_cast<float4 *>(edge_mine + (int64_t)jc * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int k = 4 * q + u;
                        v[u] = k < NE ? wnew[k] : 0.f;
                    }
                    e[q] = make_float4(v[0], v[1], v[2], v[3]);
                }
                edgeE_mine[jc] = Eb;
                if ((jc % PUB) == 0) st_release(prog_mine, Ly + 1 - jc);
            }
        }
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            mR[k] = dR[k];
            wn[k] = valid ? wnew[k] : 0.f;
        }
        EmR = EdRn;
        Ewn = valid ? Eb : EXP_NONE;
        // row 32 hands its new state to row 31 for step t-1
        if (r == 32) {
#pragma unroll
            for (int k = 0; k < SP; ++k) bnd[(t & 1) * SP + k] = k < NE ? wn[k] : 0.f;
            bndE[t & 1] = Ewn;
        }
        load_emit(t - 1);
        if (has_below && r == ROWS - 1 && jb - 1 >= 0 && jb - 1 <= Ly) {
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
            if (pv < Ly + 3 - jb) pv = ld_acquire(prog_below);
        }
        __syncthreads();
        // the flag of step t is written only before this barrier, and the
        // next write goes to the other parity: every thread sees the same value
        if (s_abort[t & 1]) { aborted = true; break; }
    }
    if (aborted && r == 0) {
        atomicOr(P.status + p, PHMM_ST_TIMEOUT);
        if (has_above) st_release(prog_mine, Ly + 1);
    }
    __threadfence();   // stripe complete: the count pass may start on it
    __syncthreads();
    if (r == 0) st_release(prog_mine, Ly + 2);
}

// Persistent two-warp CTAs popping stripe items (forward: kind 5; backward
// recursion: kind 6).
template <class SH, bool BWD>
__global__ void __launch_bounds__(TWT) stripe_tw_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemTW L = make_smem_tw(SH::SP, SH::KP, SH::NI, P.G, P.max_ly, BWD);
    int *s_item = reinterpret_cast<int *>(sm) + L.flag + 2;
    for (;;) {
        if (threadIdx.x == 0) *s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = *s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        if (BWD) bwd_rec_stripe_tw<SH>(P, w.x, w.y, L, sm, smem_raw);
        else fwd_stripe_tw<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

}  // namespace warp2
