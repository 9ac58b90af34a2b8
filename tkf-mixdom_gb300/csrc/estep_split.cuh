// estep_split.cuh -- the split E-step for the register-resident warp kernels
// (included by pairhmm.cu after estep_warp.cuh).
//
// The fused backward kernel does the backward recursion and the expected
// counts in one pass, so every anti-diagonal step of the critical path pays
// for the count work.  The split E-step removes the counts from both
// wavefronts:
//   1. forward_warp_kernel writes the forward lattice F (unchanged);
//   2. backward_rec_warp_kernel runs the backward recursion alone and writes
//      the backward lattice B (values b~ before the emission, one exponent
//      per cell, the same stripe-diagonal layout as F).  It does not read F,
//      so it runs at the same time as the forward kernel, on a second stream;
//   3. count_warp_kernel then reads both lattices in independent chunks of
//      64 anti-diagonal steps of one stripe and accumulates posteriors,
//      emission counts and the transition-count outer products.  Nothing in
//      it waits on anything: it is a throughput kernel.
// The critical path of a batch becomes max(forward, backward recursion)
// plus the count pass, instead of forward + fused backward.

namespace warp2 {

constexpr int CCH = 64;   // anti-diagonal steps per count chunk

// ---------------------------------------------------------------- backward recursion only
template <class SH>
__device__ void bwd_rec_stripe_w(const KParams &P, int p, int si, const SmemW &L, float *sm,
                                 unsigned char *smb) {
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, NM = SH::NM, NI = SH::NI;
    const PairMeta m = P.meta[p];
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

    load_model_w<SH>(P, p, m, L, sm, smb, true);
    const unsigned char *ys = smb + L.ys;
    const float4 *chiB4 = reinterpret_cast<const float4 *>(sm + L.chi);   // chiB[k][s]

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

    float wn[R][NE], wnn1[NE], dR[NE], mR[NE];
    int Ewn[R] = {EXP_NONE, EXP_NONE}, Ewnn1 = EXP_NONE, EmR = EXP_NONE;
#pragma unroll
    for (int k = 0; k < NE; ++k) { wn[0][k] = 0.f; wn[1][k] = 0.f; wnn1[k] = 0.f; dR[k] = 0.f; mR[k] = 0.f; }

    const int T_last = (nrows - 1) + Ly;
    bool aborted = false;
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (has_below && lane == 31) pv = ld_acquire(prog_below);

    for (int t = T_last; t >= 0; --t) {
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
        const bool term0 = valid[0] && rowi[0] == Lx && jc[0] == Ly;
        const bool term1 = valid[1] && rowi[1] == Lx && jc[1] == Ly;
        const bool hI0 = jc[0] + 1 <= Ly, hD0 = rowi[0] + 1 <= Lx, hM0 = hI0 && hD0;
        const bool hI1 = jc[1] + 1 <= Ly, hD1 = rowi[1] + 1 <= Lx, hM1 = hI1 && hD1;
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
        if (term0) {
#pragma unroll
            for (int s = 0; s < NSRC; ++s) acc[0][s] = sm[L.chiE + s];
        }
        if (term1) {
#pragma unroll
            for (int s = 0; s < NSRC; ++s) acc[1][s] = sm[L.chiE + s];
        }
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
            if (mxv > 0.f) {
                const int e = exp_of(mxv);
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
            if (valid[c]) {
                const int rho = R * lane + c;
                float4 *dst = reinterpret_cast<float4 *>(P.blat + (latc + (int64_t)t * ROWS + rho) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        v[u] = s < NSRC ? acc[c][s] : 0.f;
                    }
                    dst[q] = make_float4(v[0], v[1], v[2], v[3]);
                }
                P.blat_exp[latc + (int64_t)t * ROWS + rho] = Eb[c];
                if (has_above && rowi[c] == i0) {   // top row -> edge for the stripe above
                    float4 *e = reinterpret_cast<float4 *>(edge_mine + (int64_t)jc[c] * SP);
#pragma unroll
                    for (int q = 0; q < SP / 4; ++q) {
                        float v[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int k = 4 * q + u;
                            v[u] = k < NE ? wnew[c][k] : 0.f;
                        }
                        e[q] = make_float4(v[0], v[1], v[2], v[3]);
                    }
                    edgeE_mine[jc[c]] = Eb[c];
                    if ((jc[c] % PUB) == 0) st_release(prog_mine, Ly + 1 - jc[c]);
                }
            }
        }
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
    if (aborted && lane == 0) {
        atomicOr(P.status + p, PHMM_ST_TIMEOUT);
        if (has_above) st_release(prog_mine, Ly + 1);
    }
    __threadfence();   // stripe complete: the count pass may start on it
    __syncwarp();
    if (lane == 0) st_release(prog_mine, Ly + 2);
}

template <class SH>
__global__ void __launch_bounds__(32) backward_rec_warp_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemW L = make_smem_w(SH::SP, SH::KP, SH::NI, P.G, P.max_ly, true, false);
    for (;;) {
        int it = 0;
        if ((threadIdx.x & 31) == 0) it = atomicAdd(P.counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        bwd_rec_stripe_w<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

// ---------------------------------------------------------------- counts from both lattices
// One warp per chunk of CCH anti-diagonal steps of one stripe.  The forward
// and backward lattice rows of step t-1 are copied into shared memory with
// cp.async while step t is processed (double buffer); lane 31's successor in
// the first row of the stripe below is loaded one step ahead into registers.
struct SmemC {
    int tM, tI, tD, fbuf, bbuf, ust, bins, colI;   // float offsets
    int fE, bE;                                    // int offsets
    int ys;                                        // byte offset
    int bytes;
};

__host__ __device__ inline SmemC make_smem_c(int SP, int KP, int NI, int G, int max_ly) {
    SmemC L;
    int o = 0;
    L.tM = o; o += al4(G * 441);
    L.tI = o; o += al4(G * 21);
    L.tD = o; o += al4(G * 21);
    L.fbuf = o; o += 2 * ROWS * (SP + 4);
    L.bbuf = o; o += 2 * ROWS * (SP + 4);
    L.ust = o; o += ROWS * (KP + 4);
    L.bins = o; o += al4(G * 21);
    L.colI = o; o += al4(ROWS * (NI > 0 ? NI : 1));
    L.fE = o; o += 2 * ROWS;
    L.bE = o; o += 2 * ROWS;
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 4;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

template <class SH>
__device__ void count_chunk_w(const KParams &P, int p, int si, int ch, const SmemC &L, float *sm,
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
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;
    const int64_t latb = m.lat_base + (int64_t)(si + 1) * (ROWS + Ly) * ROWS;   // stripe below (row 0)
    const int T_last = (nrows - 1) + Ly;
    const int t0 = ch * CCH;
    const int t_hi = min(T_last, t0 + CCH - 1);
    const int t_top = min(T_last, t_hi + 2);   // two steps of successor history first
    if (t0 > T_last) return;
    if (P.count_wait) {   // the wavefronts may still run: wait for the stripes read here
        int ok = 1;
        if (lane == 0) ok = count_ready(P, m, si) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
            if (lane == 0) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            return;
        }
    }
    const double llv = __ldcg(P.ll + p);
    if (!(llv > -1e29)) return;   // uniform over the warp
    const double lam = llv / LN2;
    const double Epd = floor(lam);
    const int Ep = (int)Epd;
    const float rfrac = (float)exp2(-(lam - Epd));
    float *fbuf = sm + L.fbuf, *bbuf = sm + L.bbuf, *ust = sm + L.ust, *bins = sm + L.bins, *colI = sm + L.colI;
    int *fEb = reinterpret_cast<int *>(sm) + L.fE;
    int *bEb = reinterpret_cast<int *>(sm) + L.bE;
    // the lattice rows of step t (all 64 rows; rows outside the pair hold stale
    // data that is never used unguarded)
    auto prefetch = [&](int t) {
        if (t >= t0) {
            const int buf = t & 1;
            const float *srcF = P.lat + (latc + (int64_t)t * ROWS) * SP;
            const float *srcB = P.blat + (latc + (int64_t)t * ROWS) * SP;
            for (int idx = lane; idx < ROWS * SP / 4; idx += 32) {
                const int r = idx / (SP / 4), q = idx % (SP / 4);
                if (t <= t_hi) cp_async16(fbuf + buf * ROWS * SPP + r * SPP + 4 * q, srcF + 4 * idx);
                cp_async16(bbuf + buf * ROWS * SPP + r * SPP + 4 * q, srcB + 4 * idx);
            }
            for (int idx = lane; idx < ROWS / 4; idx += 32) {
                if (t <= t_hi) cp_async16(fEb + buf * ROWS + 4 * idx, P.lat_exp + latc + (int64_t)t * ROWS + 4 * idx);
                cp_async16(bEb + buf * ROWS + 4 * idx, P.blat_exp + latc + (int64_t)t * ROWS + 4 * idx);
            }
        }
        cp_commit();
    };
    prefetch(t_top);
    // ---- tables, y characters of the chunk's columns, zeroed bins
    {
        const float *eM = P.eM + (int64_t)p * P.eM_stride;
        const float *eI = P.eI + (int64_t)p * P.eID_stride;
        const float *eDg = P.eD + (int64_t)p * P.eID_stride;
        for (int idx = lane; idx < G * 441; idx += 32) sm[L.tM + idx] = __ldg(eM + idx);
        for (int idx = lane; idx < G * 21; idx += 32) {
            sm[L.tI + idx] = __ldg(eI + idx);
            sm[L.tD + idx] = __ldg(eDg + idx);
            sm[L.bins + idx] = 0.f;
        }
        unsigned char *ysw = smb + L.ys;
        const int jlo = max(0, t0 - (ROWS - 1)), jhi = min(Ly, t_hi + 3);
        for (int j = jlo + lane; j <= jhi; j += 32) {
            int c = 0;
            if (j >= 1) c = min((int)P.res[m.y_off + j - 1], 20);
            ysw[j] = (unsigned char)c;
        }
        for (int idx = lane; idx < ROWS * (NI > 0 ? NI : 1); idx += 32) colI[idx] = 0.f;
        __syncwarp();
    }
    const unsigned char *ys = smb + L.ys;

    int rowi[R], xch[R];
    float eD[R][ND > 0 ? ND : 1];
    int offM[R][NM > 0 ? NM : 1];
#pragma unroll
    for (int c = 0; c < R; ++c) {
        rowi[c] = i0 + R * lane + c;
        xch[c] = row_char(P, p, m, rowi[c]);
#pragma unroll
        for (int k = 0; k < NM; ++k) offM[c][k] = L.tM + P.w_group[k] * 441 + xch[c] * 21;
#pragma unroll
        for (int k = 0; k < ND; ++k) eD[c][k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xch[c]];
    }
    int offI[NI > 0 ? NI : 1];
#pragma unroll
    for (int k = 0; k < NI; ++k) offI[k] = L.tI + P.w_group[NM + k] * 21;
    // the first row of the stripe below (lane 31's D / M successors)
    int offMb[NM > 0 ? NM : 1];
    float eDb[ND > 0 ? ND : 1];
    {
        const int xb = row_char(P, p, m, i0 + ROWS);
#pragma unroll
        for (int k = 0; k < NM; ++k) offMb[k] = L.tM + P.w_group[k] * 441 + xb * 21;
#pragma unroll
        for (int k = 0; k < ND; ++k) eDb[k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xb];
    }
    double *cntM_pair = P.cntM + (int64_t)p * G * 441;

    float dcnt[R][ND > 0 ? ND : 1], dcmp[R][ND > 0 ? ND : 1];
#pragma unroll
    for (int c = 0; c < R; ++c)
#pragma unroll
        for (int k = 0; k < ND; ++k) { dcnt[c][k] = 0.f; dcmp[c][k] = 0.f; }
    const int blk = lane % SH::NBLK, grp = lane / SH::NBLK;
    const bool counter = grp < SH::GROUPS;
    const int bs = blk / SH::BK, bk = blk % SH::BK;
    float csum[16], ccomp[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) { csum[u] = 0.f; ccomp[u] = 0.f; }

    // successor histories: w~ of my cells at t+1 (wn), of cell B at t+2 (wnn1),
    // and the D-successor of cell B seen at step t+1 (dR), which is cell B's
    // M-successor at step t
    float wn[R][NE], wnn1[NE], dR[NE];
    int Ewn[R] = {EXP_NONE, EXP_NONE}, Ewnn1 = EXP_NONE, EdR = EXP_NONE;
#pragma unroll
    for (int k = 0; k < NE; ++k) { wn[0][k] = 0.f; wn[1][k] = 0.f; wnn1[k] = 0.f; dR[k] = 0.f; }
    // lane 31: b~ of row i0+64 at column (t - 63), loaded one step ahead
    float bbv[SP];
    int bbE = EXP_NONE;
    auto load_below = [&](int t) {
        const int jb = t - (ROWS - 1);
        bbE = EXP_NONE;
        if (lane == 31 && has_below && t >= t0 && jb >= 0 && jb <= Ly) {
            const int64_t cell = latb + (int64_t)jb * ROWS;
            bbE = __ldcg(P.blat_exp + cell);
            const float4 *src = reinterpret_cast<const float4 *>(P.blat + cell * SP);
#pragma unroll
            for (int q = 0; q < SP / 4; ++q) {
                const float4 v = __ldcg(src + q);
                bbv[4 * q] = v.x; bbv[4 * q + 1] = v.y; bbv[4 * q + 2] = v.z; bbv[4 * q + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int s = 0; s < SP; ++s) bbv[s] = 0.f;
        }
    };
    load_below(t_top);

    for (int t = t_top; t >= t0; --t) {
        const bool count = t <= t_hi;
        const int buf = t & 1;
        prefetch(t - 1);
        cp_wait1();
        __syncwarp();
        int jc[R];
        bool valid[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            jc[c] = t - (R * lane + c);
            valid[c] = (R * lane + c < nrows) && jc[c] >= 0 && jc[c] <= Ly;
        }
        // ---- b~ and w~ = e b~ of my two cells at step t
        float wcur[R][NE];
        int Eb[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int rho = R * lane + c;
            const int E = valid[c] ? bEb[buf * ROWS + rho] : EXP_NONE;
            Eb[c] = E > EXP_NONE ? E : EXP_NONE;
            const int yj = valid[c] ? ys[jc[c]] : 0;
            const float *br = bbuf + buf * ROWS * SPP + rho * SPP;
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                const int ty = SH::type_of(k);
                float ev;
                if (ty == T_M) ev = sm[offM[c][k] + yj];
                else if (ty == T_I) ev = sm[offI[k - NM] + yj];
                else ev = eD[c][k - NM - NI];
                wcur[c][k] = Eb[c] > EXP_NONE ? br[k] * ev : 0.f;
            }
        }
        // D-successor of cell B (row 2L+2, column jc[1]): lane L+1's cell A at t+1,
        // or for lane 31 the first row of the stripe below at column jc[1]
        float dnew[NE];
        int Ednew = __shfl_down_sync(0xffffffffu, Ewn[0], 1);
#pragma unroll
        for (int k = 0; k < NE; ++k) dnew[k] = __shfl_down_sync(0xffffffffu, wn[0][k], 1);
        if (lane == 31) {
            const bool okb = has_below && jc[1] >= 0 && jc[1] <= Ly && bbE > EXP_NONE;
            const int yb = okb ? ys[jc[1]] : 0;
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                const int ty = SH::type_of(k);
                float ev;
                if (ty == T_M) ev = sm[offMb[k] + yb];
                else if (ty == T_I) ev = sm[offI[k - NM] + yb];
                else ev = eDb[k - NM - NI];
                dnew[k] = okb ? bbv[k] * ev : 0.f;
            }
            Ednew = okb ? bbE : EXP_NONE;
        }
        load_below(t - 1);
        if (count) {
            const bool term0 = valid[0] && rowi[0] == Lx && jc[0] == Ly;
            const bool term1 = valid[1] && rowi[1] == Lx && jc[1] == Ly;
            const bool hI0 = jc[0] + 1 <= Ly, hD0 = rowi[0] + 1 <= Lx, hM0 = hI0 && hD0;
            const bool hI1 = jc[1] + 1 <= Ly, hD1 = rowi[1] + 1 <= Lx, hM1 = hI1 && hD1;
            // successor exponents by type (cell A: I = A(t+1), D = B(t+1), M = B(t+2);
            // cell B: I = B(t+1), D = dnew, M = dR = the D-successor seen at t+1)
            const int EI0 = (hI0 && !term0) ? Ewn[0] : EXP_NONE, ED0 = (hD0 && !term0) ? Ewn[1] : EXP_NONE;
            const int EM0 = (hM0 && !term0) ? Ewnn1 : EXP_NONE;
            const int EI1 = (hI1 && !term1) ? Ewn[1] : EXP_NONE, ED1 = (hD1 && !term1) ? Ednew : EXP_NONE;
            const int EM1 = (hM1 && !term1) ? EdR : EXP_NONE;
#pragma unroll
            for (int c = 0; c < R; ++c) {
                const int rho = R * lane + c;
                const int Ef = valid[c] ? fEb[buf * ROWS + rho] : EXP_NONE;
                float fsc = 0.f;
                if (valid[c] && Ef > EXP_NONE && Eb[c] > EXP_NONE) {
                    int d = Ef + Eb[c] - Ep;
                    if (d > 126) { d = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                    fsc = scale_pow2(rfrac, max(d, -200));
                }
                // f~ scaled in place (the outer products read it from the buffer)
                float *fr = fbuf + buf * ROWS * SPP + rho * SPP;
                const float *br = bbuf + buf * ROWS * SPP + rho * SPP;
                float ft[NSRC];
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    const float4 v = reinterpret_cast<const float4 *>(fr)[q];
                    const float va[4] = {v.x, v.y, v.z, v.w};
                    float o[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        o[u] = (s < NSRC && fsc > 0.f) ? va[u] * fsc : 0.f;
                        if (s < NSRC) ft[s] = o[u];
                    }
                    reinterpret_cast<float4 *>(fr)[q] = make_float4(o[0], o[1], o[2], o[3]);
                }
                // u~[k] = w~_succ(k)[k] * 2^(E_succ - Eb)
                const int EM = c == 0 ? EM0 : EM1, EI = c == 0 ? EI0 : EI1, ED = c == 0 ? ED0 : ED1;
                const bool live = fsc > 0.f;
                const float uM = (live && EM > EXP_NONE) ? fminf(scale_pow2(1.f, EM - Eb[c]), 3e38f) : 0.f;
                const float uI = (live && EI > EXP_NONE) ? fminf(scale_pow2(1.f, EI - Eb[c]), 3e38f) : 0.f;
                const float uD = (live && ED > EXP_NONE) ? fminf(scale_pow2(1.f, ED - Eb[c]), 3e38f) : 0.f;
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
                            else u = ty == T_M ? dR[k] * uM : (ty == T_I ? wn[1][k] * uI : dnew[k] * uD);
                        }
                        uq[v] = u;
                    }
                    reinterpret_cast<float4 *>(ust + rho * KPP)[q] = make_float4(uq[0], uq[1], uq[2], uq[3]);
                }
                if (live) {
                    const int yj = ys[jc[c]];
#pragma unroll
                    for (int k = 0; k < NE; ++k) {
                        const float pk = ft[k] * br[k];
                        const int ty = SH::type_of(k);
                        if (ty == T_M) {
                            if (pk != 0.f) atomicAdd(cntM_pair + P.w_group[k] * 441 + xch[c] * 21 + yj, (double)pk);
                        } else if (ty == T_I) {
                            colI[(jc[c] % ROWS) * NI + (k - NM)] += pk;
                        } else {
                            const int kd = k - NM - NI;
                            const float y = pk - dcmp[c][kd];
                            const float tt = dcnt[c][kd] + y;
                            dcmp[c][kd] = (tt - dcnt[c][kd]) - y;
                            dcnt[c][kd] = tt;
                        }
                    }
                    if ((c == 0 && term0) || (c == 1 && term1)) {   // expected End transitions
#pragma unroll
                        for (int s = 0; s < NSRC; ++s)
                            atomicAdd(P.n_trans + ((int64_t)p * N + P.w_orig[s]) * N + P.e_idx,
                                      (double)(ft[s] * br[s]));
                    }
                }
            }
            __syncwarp();
            // column t is complete once row i0 (lane 0, cell A) has visited it
            if (lane == 0 && t <= Ly) {
                const int slot = t % ROWS;
                const int yj = ys[t];
#pragma unroll
                for (int k = 0; k < NI; ++k) {
                    bins[P.w_group[NM + k] * 21 + yj] += colI[slot * NI + k];
                    colI[slot * NI + k] = 0.f;
                }
            }
            if (counter) {
                float pz[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) pz[u] = 0.f;
                const float *fb = fbuf + buf * ROWS * SPP;
                auto row_outer = [&](int rr) {
                    const float4 fv = reinterpret_cast<const float4 *>(fb + rr * SPP)[bs];
                    const float4 uv = reinterpret_cast<const float4 *>(ust + rr * KPP)[bk];
                    const float fa[4] = {fv.x, fv.y, fv.z, fv.w};
                    const float ua[4] = {uv.x, uv.y, uv.z, uv.w};
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) pz[4 * a + b] = fmaf(fa[a], ua[b], pz[4 * a + b]);
                };
                if constexpr (ROWS % SH::GROUPS == 0) {   // fixed trip count: unrolled
                    constexpr int RPG = ROWS / SH::GROUPS;
                    const int r0 = grp * RPG;
#pragma unroll 4
                    for (int rr = r0; rr < r0 + RPG; ++rr) row_outer(rr);
                } else {
                    const int r0 = grp * ROWS / SH::GROUPS, r1 = (grp + 1) * ROWS / SH::GROUPS;
                    for (int rr = r0; rr < r1; ++rr) row_outer(rr);
                }
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    const float y = pz[u] - ccomp[u];
                    const float tt = csum[u] + y;
                    ccomp[u] = (tt - csum[u]) - y;
                    csum[u] = tt;
                }
            }
        }
        __syncwarp();   // the buffers of step t are free for the prefetch of step t-2
        // ---- shift histories
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            dR[k] = dnew[k];
            wnn1[k] = wn[1][k];
            wn[0][k] = wcur[0][k];
            wn[1][k] = wcur[1][k];
        }
        EdR = Ednew;
        Ewnn1 = Ewn[1];
        Ewn[0] = Eb[0];
        Ewn[1] = Eb[1];
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    // ---- flush the chunk's partial counts (float64 reductions)
    __syncwarp();
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
            if (v != 0.f) atomicAdd(P.cntD + ((int64_t)p * G + P.w_group[NM + NI + k]) * 21 + xch[c], (double)v);
        }
    }
    // I-type columns not completed inside the chunk (touched by rows below row 0)
    for (int j = max(0, t0 - (ROWS - 1)) + lane; j <= min(Ly, t0 - 1); j += 32) {
        const int slot = j % ROWS;
        const int yj = ys[j];
#pragma unroll
        for (int k = 0; k < NI; ++k) {
            const float v = colI[slot * NI + k];
            if (v != 0.f) atomicAdd(P.cntI + ((int64_t)p * G + P.w_group[NM + k]) * 21 + yj, (double)v);
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
__global__ void __launch_bounds__(32) count_warp_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemC L = make_smem_c(SH::SP, SH::KP, SH::NI, P.G, P.max_ly);
    for (;;) {
        int it = 0;
        if ((threadIdx.x & 31) == 0) it = count_claim(P);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        count_chunk_w<SH>(P, w.x, w.y >> 12, w.y & 4095, L, sm, smem_raw);
    }
}

}  // namespace warp2
