// estep_block_split.cuh -- the split E-step for the quad-per-warp block
// kernels (included by pairhmm.cu after estep_block.cuh).
//
// As for the warp kernels (estep_split.cuh): the forward block kernel writes
// the forward lattice; backward_rec_block_kernel runs only the backward
// recursion (NB warps, no count warps) at the same time on a second stream
// and writes the backward lattice b~ with per-quad exponents; then
// count_block_kernel reads both lattices in independent chunks of 64
// anti-diagonal steps of one stripe.  A count CTA has 256 threads: in phase
// A four threads per cell (rows 0..63 of the step) form the posterior of
// their quads, the emission counts and the successor operands u~; in phase
// B the threads accumulate the f~ x u~ outer products of the step's 64 cells
// in 4 x 4 tiles (Kahan), flushed with chi as float64 reductions at the end
// of the chunk.

namespace blk {

constexpr int CCHB = 64;          // anti-diagonal steps per count chunk
constexpr int CNT_THREADS = 256;  // count CTA

// ---------------------------------------------------------------- backward recursion only
template <class SH>
__device__ void bwd_rec_stripe_b(const KParams &P, int p, int si, const SmemB &L, float *sm, unsigned char *smb) {
    constexpr int NS = SH::NS, NB = SH::NB, NBP = SH::NBP, SPR = SH::SPR;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x;
    const int lane = tid & 31, q = tid >> 5;
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const bool has_above = si > 0;
    // the backward direction's own progress counters and edge rows
    const int *prog_below = has_below ? P.bprogress + m.stripe_base + si + 1 : nullptr;
    int *prog_mine = P.bprogress + m.stripe_base + si;
    const float *edge_below = P.bedge + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * NS;
    const int *edgeE_below = P.bedge_exp + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * NBP;
    float *edge_mine = P.bedge + (m.edge_base + (int64_t)si * (Ly + 1)) * NS;
    int *edgeE_mine = P.bedge_exp + (m.edge_base + (int64_t)si * (Ly + 1)) * NBP;
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;

    load_model_b(P, p, m, L, sm, smb, true);
    const unsigned char *ys = smb + L.ys;
    float *ring = sm + L.ring;
    int *ringE = reinterpret_cast<int *>(sm) + L.ringE;
    float *halo = sm + L.halo;
    int *haloE = reinterpret_cast<int *>(sm) + L.haloE;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    if (tid == 0) { misc[0] = 0; misc[1] = 0; }
    __syncthreads();
    const float4 *chi4q = reinterpret_cast<const float4 *>(sm + L.chi) + q;   // chiB[k][4q..]
    float cq[SH::CHI_REG ? NS : 1][4];
    if constexpr (SH::CHI_REG) {
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const float4 cv = chi4q[k * (NS / 4)];
            cq[k][0] = cv.x; cq[k][1] = cv.y; cq[k][2] = cv.z; cq[k][3] = cv.w;
        }
    }
    int rowi[R];
    QuadEmit qe[R];
#pragma unroll
    for (int c = 0; c < R; ++c) {
        rowi[c] = i0 + lane + 32 * c;
        int xc = 0;
        if (rowi[c] >= 1 && rowi[c] <= Lx) xc = min((int)P.res[m.x_off + rowi[c] - 1], 20);
        qe[c] = quad_emit(P, L, q, xc);
    }
    const int T_last = (nrows - 1) + Ly;
    int pv = 0, fetched = Ly + 1;   // halo columns >= fetched are in flight or landed
    if (tid == 0 && has_below) pv = ld_acquire(prog_below);
    bool aborted = false;
    int k = 0;
    for (int t = T_last; t >= 0; --t, ++k) {
        // ---- halo column t-63 (row i0+64) in shared memory before the step barrier;
        // a failed wait is flagged in misc[k & 1], read by every warp after the barrier
        const int jh = t - (ROWS - 1);
        if (tid == 0 && has_below && jh >= 0 && jh <= Ly) {
            if (fetched > jh) {
                if (!wait_geq(prog_below, Ly + 1 - jh, P.spin_limit)) {
                    misc[k & 1] = 1;
                } else {
                    const int sl = jh % 3;
                    for (int i = 0; i < NS / 4; ++i)
                        cp_async16(halo + sl * NS + 4 * i, edge_below + (int64_t)jh * NS + 4 * i);
                    for (int i = 0; i < NBP / 4; ++i)
                        cp_async16(haloE + sl * NBP + 4 * i, edgeE_below + (int64_t)jh * NBP + 4 * i);
                    cp_commit();
                    fetched = jh;
                }
            }
            cp_wait0();
        }
        bar_sync(BAR_STEP, NB * 32);
        if (misc[k & 1]) { aborted = true; break; }
        // ---- top row of step t+1 -> edge row for the stripe above
        if (tid == 0 && has_above && t + 1 <= T_last) {
            const int jt = t + 1;
            if (jt <= Ly) {
                copy_edge_cell(ring + ((t + 1) % 3) * ROWS * SPR, ringE + ((t + 1) % 3) * ROWS * NBP,
                               edge_mine + (int64_t)jt * NS, edgeE_mine + (int64_t)jt * NBP, NS, NBP);
                if ((jt % PUBB) == 0) st_release(prog_mine, Ly + 1 - jt);
            }
        }
        // ---- prefetch halo column jh-1 for the next step
        if (tid == 0 && has_below && jh - 1 >= 0 && jh - 1 <= Ly) {
            if (fetched == jh && pv >= Ly + 1 - (jh - 1)) {
                const int sl = (jh - 1) % 3;
                for (int i = 0; i < NS / 4; ++i)
                    cp_async16(halo + sl * NS + 4 * i, edge_below + (int64_t)(jh - 1) * NS + 4 * i);
                for (int i = 0; i < NBP / 4; ++i)
                    cp_async16(haloE + sl * NBP + 4 * i, edgeE_below + (int64_t)(jh - 1) * NBP + 4 * i);
                cp_commit();
                fetched = jh - 1;
            }
            if (pv < Ly + 3 - jh) pv = ld_acquire(prog_below);   // only when the next prefetch needs more
        }
        if (tid == 0) misc[(k + 1) & 1] = 0;   // every warp read it two barriers ago
        // ---- successor vectors of both cells (the zero vector when one does not exist)
        const float *zv = sm + L.zvec;
        const int *ze = reinterpret_cast<const int *>(sm) + L.zvecE;
        const float *vI[R], *vD[R], *vM[R];
        const int *eI[R], *eD[R], *eM[R];
        bool valid[R], term[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int rho = lane + 32 * c;
            const int j = t - rho;
            const int i = rowi[c];
            valid[c] = rho < nrows && j >= 0 && j <= Ly;
            term[c] = valid[c] && i == Lx && j == Ly;
            vI[c] = vD[c] = vM[c] = zv;
            eI[c] = eD[c] = eM[c] = ze;
            if (!valid[c] || term[c]) continue;
            const bool hI = j + 1 <= Ly, hD = i + 1 <= Lx, hM = hI && hD;
            if (hI) { vI[c] = ring + ((t + 1) % 3) * ROWS * SPR + rho * SPR; eI[c] = ringE + ((t + 1) % 3) * ROWS * NBP + rho * NBP; }
            if (hD) {
                if (rho + 1 < nrows) { vD[c] = ring + ((t + 1) % 3) * ROWS * SPR + (rho + 1) * SPR; eD[c] = ringE + ((t + 1) % 3) * ROWS * NBP + (rho + 1) * NBP; }
                else { vD[c] = halo + (j % 3) * NS; eD[c] = haloE + (j % 3) * NBP; }
            }
            if (hM) {
                if (rho + 1 < nrows) { vM[c] = ring + ((t + 2) % 3) * ROWS * SPR + (rho + 1) * SPR; eM[c] = ringE + ((t + 2) % 3) * ROWS * NBP + (rho + 1) * NBP; }
                else { vM[c] = halo + ((j + 1) % 3) * NS; eM[c] = haloE + ((j + 1) % 3) * NBP; }
            }
        }
        // ---- b[4q+u] = sum over destination quads d of chi[4q+u][d..] w_succ(type d)[d..],
        // both cells in one pass over the transition operands
        int Ed[R][NB];
        int Eref[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            int EvM[NBP], EvI[NBP], EvD[NBP];
#pragma unroll
            for (int ii = 0; ii < NBP / 4; ++ii) {
                const int4 a = reinterpret_cast<const int4 *>(eM[c])[ii];
                const int4 b = reinterpret_cast<const int4 *>(eI[c])[ii];
                const int4 d4 = reinterpret_cast<const int4 *>(eD[c])[ii];
                EvM[4 * ii] = a.x; EvM[4 * ii + 1] = a.y; EvM[4 * ii + 2] = a.z; EvM[4 * ii + 3] = a.w;
                EvI[4 * ii] = b.x; EvI[4 * ii + 1] = b.y; EvI[4 * ii + 2] = b.z; EvI[4 * ii + 3] = b.w;
                EvD[4 * ii] = d4.x; EvD[4 * ii + 1] = d4.y; EvD[4 * ii + 2] = d4.z; EvD[4 * ii + 3] = d4.w;
            }
            Eref[c] = EXP_NONE;
#pragma unroll
            for (int d = 0; d < NB; ++d) {
                const int dt = P.quad_type[d];
                Ed[c][d] = dt == T_M ? EvM[d] : (dt == T_I ? EvI[d] : (dt == T_D ? EvD[d] : EXP_NONE));
                Eref[c] = max(Eref[c], Ed[c][d]);
            }
        }
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
#pragma unroll
        for (int d = 0; d < NB; ++d) {
            const int dt = P.quad_type[d];
            const float *v0 = dt == T_M ? vM[0] : (dt == T_I ? vI[0] : (dt == T_D ? vD[0] : zv));
            const float *v1 = dt == T_M ? vM[1] : (dt == T_I ? vI[1] : (dt == T_D ? vD[1] : zv));
            const float s0 = pow2n(Ed[0][d] - Eref[0]), s1 = pow2n(Ed[1][d] - Eref[1]);
            const float4 x = *reinterpret_cast<const float4 *>(v0 + 4 * d);
            const float4 y = *reinterpret_cast<const float4 *>(v1 + 4 * d);
            const float xs[4] = {x.x * s0, x.y * s0, x.z * s0, x.w * s0};
            const float yv[4] = {y.x * s1, y.y * s1, y.z * s1, y.w * s1};
#pragma unroll
            for (int ii = 0; ii < 4; ++ii) {
                const int kk = 4 * d + ii;
                float c0, c1, c2, c3;
                if constexpr (SH::CHI_REG) {
                    c0 = cq[kk][0]; c1 = cq[kk][1]; c2 = cq[kk][2]; c3 = cq[kk][3];
                } else {
                    const float4 cv = chi4q[kk * (NS / 4)];
                    c0 = cv.x; c1 = cv.y; c2 = cv.z; c3 = cv.w;
                }
                a0 = fmaf(xs[ii], c0, a0); a1 = fmaf(xs[ii], c1, a1); a2 = fmaf(xs[ii], c2, a2); a3 = fmaf(xs[ii], c3, a3);
                g0 = fmaf(yv[ii], c0, g0); g1 = fmaf(yv[ii], c1, g1); g2 = fmaf(yv[ii], c2, g2); g3 = fmaf(yv[ii], c3, g3);
            }
        }
        const float4 accv[R] = {make_float4(a0, a1, a2, a3), make_float4(g0, g1, g2, g3)};
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int rho = lane + 32 * c;
            const int j = t - rho;
            float4 bq = make_float4(0.f, 0.f, 0.f, 0.f), wq = bq;
            int Eb = EXP_NONE;
            if (valid[c]) {
                int Er = Eref[c];
                if (term[c]) {
                    bq = *reinterpret_cast<const float4 *>(sm + L.chiE + 4 * q);
                    Er = 0;
                } else {
                    bq = accv[c];
                }
                const float mx = f4max(bq);
                if (mx > 0.f && Er > EXP_NONE) {
                    const int eb = warp2::exp_of(mx);
                    if (-eb >= -126 && -eb <= 127) bq = f4scale(bq, pow2f(-eb));
                    else bq = make_float4(ldexpf(bq.x, -eb), ldexpf(bq.y, -eb), ldexpf(bq.z, -eb), ldexpf(bq.w, -eb));
                    Eb = Er + eb;
                } else {
                    bq = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                const float4 e = quad_emit_vals(sm, qe[c], ys[j]);
                wq = make_float4(bq.x * e.x, bq.y * e.y, bq.z * e.z, bq.w * e.w);
                const int64_t cell = latc + (int64_t)t * ROWS + rho;
                reinterpret_cast<float4 *>(P.blat + cell * NS)[q] = bq;
                P.blat_exp[cell * NBP + q] = Eb;
            }
            const int sl = t % 3;
            *reinterpret_cast<float4 *>(ring + sl * ROWS * SPR + rho * SPR + 4 * q) = wq;
            ringE[sl * ROWS * NBP + rho * NBP + q] = Eb;
        }
    }
    bar_sync(BAR_STEP, NB * 32);   // step 0's ring is complete
    if (tid == 0) {
        cp_wait0();
        if (has_above) {
            if (!aborted)
                copy_edge_cell(ring, ringE, edge_mine, edgeE_mine, NS, NBP);   // column 0 (step 0)
            st_release(prog_mine, Ly + 1);
        }
        if (aborted) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
    }
    __threadfence();   // stripe complete: the count pass may start on it
    bar_sync(BAR_STEP, NB * 32);
    if (tid == 0) st_release(prog_mine, Ly + 2);
}

// Both wavefronts of the split E-step in one persistent launch: the work list
// interleaves forward stripes and backward stripes (bit 30 of the stripe
// field marks a backward item), each direction in its own longest-pair-first
// order, so the two share the GPU's CTA slots as they free up.  A stripe waits
// only for a stripe of its own direction popped before it.
constexpr int BWD_ITEM = 1 << 30;

template <class SH>
__global__ void __launch_bounds__(32 * SH::NB) fwdbwd_block_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemB L = make_smem_b(SH::NS, SH::NB, 1, P.G, P.max_ly, false);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        if (w.y & BWD_ITEM) bwd_rec_stripe_b<SH>(P, w.x, w.y & ~BWD_ITEM, L, sm, smem_raw);
        else fwd_stripe_b<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

// ---------------------------------------------------------------- counts from both lattices
struct SmemCB {
    int tM, tI, tD, fst, ust, rowM, rowD, colI, binsI;   // float offsets
    int ys;                                             // byte offset
    int bytes;
};

// Emission-count bins are indexed by slot (M: [row][M slot][y], I: [column
// mod 64][I slot], D: [row][D slot]): a cell's slots are owned by one thread
// each and the cells of one step have distinct rows and columns, so the bins
// need no atomics.  wM / wI / wD are the slot widths of the three types.
__host__ __device__ inline SmemCB make_smem_cb(int NS, int G, int max_ly, int wM, int wI, int wD) {
    const int SPR = spr_of(NS);
    SmemCB L;
    int o = 0;
    L.tM = o; o += al4(G * 441);
    L.tI = o; o += al4(G * 21);
    L.tD = o; o += al4(G * 21);
    L.fst = o; o += ROWS * SPR;
    L.ust = o; o += ROWS * SPR;
    L.rowM = o; o += al4(ROWS * wM * 21);
    L.rowD = o; o += al4(ROWS * wD);
    L.colI = o; o += al4(ROWS * wI);
    L.binsI = o; o += al4(G * 21);
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 2;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

// emission factors of the 4 slots of quad q at characters (xi, yj)
__device__ __forceinline__ float4 quad_emit_at(const KParams &P, const float *sm, const SmemCB &L, int q, int xi, int yj) {
    float v[4];
    const int qt = P.quad_type[q];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int k = 4 * q + u;
        const int kt = P.slot_type[k];
        const bool em = (kt == T_M || kt == T_I || kt == T_D);
        const int g = em ? P.slot_group[k] : 0;
        float e = 0.f;
        if (em) {
            if (qt == T_M) e = sm[L.tM + g * 441 + xi * 21 + yj];
            else if (qt == T_I) e = sm[L.tI + g * 21 + yj];
            else e = sm[L.tD + g * 21 + xi];
        }
        v[u] = e;
    }
    return make_float4(v[0], v[1], v[2], v[3]);
}

template <class SH>
__device__ void count_chunk_b(const KParams &P, int p, int si, int ch, const SmemCB &L, float *sm, unsigned char *smb) {
    constexpr int NS = SH::NS, NB = SH::NB, NBP = SH::NBP, SPR = SH::SPR;
    constexpr int QPT = (NB + 3) / 4;   // quads per phase-A thread
    const PairMeta m = P.meta[p];
    const int N = P.N, G = P.G;
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x;
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;
    const int64_t latb = m.lat_base + (int64_t)(si + 1) * (ROWS + Ly) * ROWS;
    const int T_last = (nrows - 1) + Ly;
    const int t0 = ch * CCHB;
    const int t_hi = min(T_last, t0 + CCHB - 1);
    if (t0 > T_last) return;
    if (P.count_wait) {   // the wavefronts may still run: wait for the stripes read here
        __shared__ int s_ok;
        if (tid == 0) {
            s_ok = count_ready(P, m, si) ? 1 : 0;
            if (!s_ok) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
        }
        __syncthreads();
        const int ok = s_ok;
        __syncthreads();
        if (!ok) return;
    }
    const double llv = __ldcg(P.ll + p);
    if (!(llv > -1e29)) return;   // uniform over the CTA
    const double lam = llv / LN2;
    const int Ep = (int)floor(lam);
    const float rfrac = (float)exp2(-(lam - floor(lam)));
    const int mb = P.kbeg[0], ib = P.kbeg[1], db = P.kbeg[2];
    const int wM = P.kend[0] - mb, wI = P.kend[1] - ib, wD = P.kend[2] - db;
    {
        const float *eM = P.eM + (int64_t)p * P.eM_stride;
        const float *eI = P.eI + (int64_t)p * P.eID_stride;
        const float *eDg = P.eD + (int64_t)p * P.eID_stride;
        for (int idx = tid; idx < G * 441; idx += CNT_THREADS) sm[L.tM + idx] = __ldg(eM + idx);
        for (int idx = tid; idx < G * 21; idx += CNT_THREADS) {
            sm[L.tI + idx] = __ldg(eI + idx);
            sm[L.tD + idx] = __ldg(eDg + idx);
            sm[L.binsI + idx] = 0.f;
        }
        for (int idx = tid; idx < ROWS * wM * 21; idx += CNT_THREADS) sm[L.rowM + idx] = 0.f;
        for (int idx = tid; idx < ROWS * wD; idx += CNT_THREADS) sm[L.rowD + idx] = 0.f;
        for (int idx = tid; idx < ROWS * wI; idx += CNT_THREADS) sm[L.colI + idx] = 0.f;
        unsigned char *ysw = smb + L.ys;
        const int jlo = max(0, t0 - (ROWS - 1)), jhi = min(Ly, t_hi + 1);
        for (int j = jlo + tid; j <= jhi; j += CNT_THREADS) {
            int c = 0;
            if (j >= 1) c = min((int)P.res[m.y_off + j - 1], 20);
            ysw[j] = (unsigned char)c;
        }
    }
    __syncthreads();
    const unsigned char *ys = smb + L.ys;
    float *fst = sm + L.fst, *ust = sm + L.ust;
    float *rowM = sm + L.rowM, *rowD = sm + L.rowD, *colI = sm + L.colI, *binsI = sm + L.binsI;
    // phase A role: cell row rho, quads sub, sub+4, ...
    const int rho = tid >> 2, sub = tid & 3;
    const int irow = i0 + rho;
    const int xc = (irow >= 1 && irow <= Lx) ? min((int)P.res[m.x_off + irow - 1], 20) : 0;
    const int xn = (irow + 1 >= 1 && irow + 1 <= Lx) ? min((int)P.res[m.x_off + irow], 20) : 0;   // row i+1
    // phase B role: 4 x 4 tile (bs, bk) over rows of group grp
    constexpr int NBLK = NB * NB;
    const int GRP = max(1, CNT_THREADS / NBLK);
    const int blk_i = tid % NBLK, grp = tid / NBLK;
    const bool blk_role = grp < GRP && NBLK <= CNT_THREADS;
    const int bs = blk_i / NB, bk = blk_i % NB;
    // tiles beyond one per thread (NB*NB > 256) are looped over
    constexpr int TPT = (NBLK + CNT_THREADS - 1) / CNT_THREADS;
    float csum[TPT][16], ccomp[TPT][16];
#pragma unroll
    for (int a = 0; a < TPT; ++a)
#pragma unroll
        for (int u = 0; u < 16; ++u) { csum[a][u] = 0.f; ccomp[a][u] = 0.f; }

    // lattice loads of one step for this thread's cell and quads; issued a step
    // ahead (before the outer products of the current step) so their latency
    // hides behind phase B
    int Ef[QPT], Eb[QPT], Es[QPT];
    float4 fv[QPT], bv[QPT], sv[QPT];
    auto issue = [&](int t) {
        const int j = t - rho;
        const bool valid = t >= t0 && rho < nrows && j >= 0 && j <= Ly;
        const int64_t cell = latc + (int64_t)t * ROWS + rho;
        const bool hI = j + 1 <= Ly, hD = irow + 1 <= Lx, hM = hI && hD;
#pragma unroll
        for (int a = 0; a < QPT; ++a) {
            const int q = sub + 4 * a;
            Ef[a] = EXP_NONE; Eb[a] = EXP_NONE; Es[a] = EXP_NONE;
            fv[a] = make_float4(0.f, 0.f, 0.f, 0.f); bv[a] = fv[a]; sv[a] = fv[a];
            if (!valid || q >= NB) continue;
            // every quad of a valid cell is written (zero values with EXP_NONE)
            Ef[a] = __ldcg(P.lat_exp + cell * NBP + q);
            Eb[a] = __ldcg(P.blat_exp + cell * NBP + q);
            fv[a] = __ldcg(reinterpret_cast<const float4 *>(P.lat + cell * NS) + q);
            bv[a] = __ldcg(reinterpret_cast<const float4 *>(P.blat + cell * NS) + q);
            const int qt = P.quad_type[q];
            int64_t sc = -1;
            if (qt == T_I && hI) sc = latc + (int64_t)(t + 1) * ROWS + rho;
            else if (qt == T_D && hD && (rho + 1 < nrows || has_below))
                sc = rho + 1 < nrows ? latc + (int64_t)(t + 1) * ROWS + rho + 1 : latb + (int64_t)j * ROWS;
            else if (qt == T_M && hM && (rho + 1 < nrows || has_below))
                sc = rho + 1 < nrows ? latc + (int64_t)(t + 2) * ROWS + rho + 1 : latb + (int64_t)(j + 1) * ROWS;
            if (sc >= 0) {
                Es[a] = __ldcg(P.blat_exp + sc * NBP + q);
                sv[a] = __ldcg(reinterpret_cast<const float4 *>(P.blat + sc * NS) + q);
            }
        }
    };
    issue(t_hi);
    for (int t = t_hi; t >= t0; --t) {
        // ================= phase A: one cell per 4 threads
        {
            const int j = t - rho;
            const bool valid = rho < nrows && j >= 0 && j <= Ly;
            int Efl = EXP_NONE;
#pragma unroll
            for (int a = 0; a < QPT; ++a) Efl = max(Efl, Ef[a]);
            Efl = max(Efl, __shfl_xor_sync(0xffffffffu, Efl, 1));
            const int Efm = max(Efl, __shfl_xor_sync(0xffffffffu, Efl, 2));
            const bool live = valid && Efm > EXP_NONE;
            const bool term = valid && irow == Lx && j == Ly;
            const int yj = valid ? ys[j] : 0;
            const int yn = (valid && j + 1 <= Ly) ? ys[j + 1] : 0;
#pragma unroll
            for (int a = 0; a < QPT; ++a) {
                const int q = sub + 4 * a;
                if (q >= NB) continue;
                float4 ft = make_float4(0.f, 0.f, 0.f, 0.f), uu = ft;
                if (live) {
                    if (Ef[a] > EXP_NONE) ft = f4scale(fv[a], pow2n(Ef[a] - Efm));
                    // posteriors of my quad -> emission counts, End transitions
                    if (Eb[a] > EXP_NONE) {
                        int dp = Eb[a] + Efm - Ep;
                        if (dp > 126) { dp = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                        const float ps = warp2::scale_pow2(rfrac, max(dp, -200));
                        const float pk[4] = {ft.x * bv[a].x * ps, ft.y * bv[a].y * ps, ft.z * bv[a].z * ps,
                                             ft.w * bv[a].w * ps};
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int s = 4 * q + u;
                            const int st = P.slot_type[s];
                            const float pv = pk[u];
                            if (pv == 0.f) continue;
                            if (st == T_M) rowM[(rho * wM + s - mb) * 21 + yj] += pv;
                            else if (st == T_I) colI[(j % ROWS) * wI + s - ib] += pv;
                            else if (st == T_D) rowD[rho * wD + s - db] += pv;
                            if (term && P.slot_orig[s] >= 0)
                                atomicAdd(P.n_trans + ((int64_t)p * N + P.slot_orig[s]) * N + P.e_idx, (double)pv);
                        }
                    }
                    // successor operand of my destination quad
                    if (Es[a] > EXP_NONE && !term) {
                        const int qt = P.quad_type[q];
                        const int xi = qt == T_I ? xc : xn;
                        const int yy = qt == T_D ? yj : yn;
                        int du = Es[a] + Efm - Ep;
                        if (du > 126) { du = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                        const float us = fminf(warp2::scale_pow2(rfrac, max(du, -200)), 3e38f);
                        const float4 e4 = quad_emit_at(P, sm, L, q, xi, yy);
                        uu = make_float4(sv[a].x * e4.x * us, sv[a].y * e4.y * us, sv[a].z * e4.z * us,
                                         sv[a].w * e4.w * us);
                    }
                }
                *reinterpret_cast<float4 *>(fst + rho * SPR + 4 * q) = ft;
                *reinterpret_cast<float4 *>(ust + rho * SPR + 4 * q) = uu;
            }
        }
        issue(t - 1);
        __syncthreads();
        // column t is complete once row 0 visited it: I-type bins
        if (tid == 0 && t <= Ly) {
            const int slot = t % ROWS;
            const int yj = ys[t];
            for (int k = 0; k < wI; ++k) {
                const int s = ib + k;
                if (P.slot_type[s] == T_I) binsI[P.slot_group[s] * 21 + yj] += colI[slot * wI + k];
                colI[slot * wI + k] = 0.f;
            }
        }
        // ================= phase B: outer products of the step's cells
#pragma unroll
        for (int a = 0; a < TPT; ++a) {
            const int bidx = tid + a * CNT_THREADS;
            const bool role = TPT > 1 ? bidx < NBLK : blk_role;
            if (!role) continue;
            const int b_s = TPT > 1 ? bidx / NB : bs, b_k = TPT > 1 ? bidx % NB : bk;
            const int r0 = TPT > 1 ? 0 : grp * ROWS / GRP, r1 = TPT > 1 ? ROWS : (grp + 1) * ROWS / GRP;
            float pz[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) pz[u] = 0.f;
            for (int rr = r0; rr < r1; ++rr) {
                const float4 fv = *reinterpret_cast<const float4 *>(fst + rr * SPR + 4 * b_s);
                const float4 uv = *reinterpret_cast<const float4 *>(ust + rr * SPR + 4 * b_k);
                const float fa[4] = {fv.x, fv.y, fv.z, fv.w};
                const float ua[4] = {uv.x, uv.y, uv.z, uv.w};
#pragma unroll
                for (int x = 0; x < 4; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) pz[4 * x + y] = fmaf(fa[x], ua[y], pz[4 * x + y]);
            }
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const float y = pz[u] - ccomp[a][u];
                const float tt = csum[a][u] + y;
                ccomp[a][u] = (tt - csum[a][u]) - y;
                csum[a][u] = tt;
            }
        }
        __syncthreads();
    }
    // ================= flush (float64 reductions)
    const float *chi = P.chi + (int64_t)p * P.chi_stride;
#pragma unroll
    for (int a = 0; a < TPT; ++a) {
        const int bidx = tid + a * CNT_THREADS;
        const bool role = TPT > 1 ? bidx < NBLK : blk_role;
        if (!role) continue;
        const int b_s = TPT > 1 ? bidx / NB : bs, b_k = TPT > 1 ? bidx % NB : bk;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int s = 4 * b_s + (u >> 2), kk = 4 * b_k + (u & 3);
            const int os = P.slot_orig[s], ok = P.slot_orig[kk];
            const int kt = P.slot_type[kk];
            const float val = csum[a][u] - ccomp[a][u];
            if (os < 0 || ok < 0 || !(kt == T_M || kt == T_I || kt == T_D) || val == 0.f) continue;
            atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + ok, (double)val * (double)__ldg(chi + os * N + ok));
        }
    }
    for (int idx = tid; idx < ROWS * wM * 21; idx += CNT_THREADS) {
        const int r = idx / (wM * 21), k = (idx / 21) % wM, y = idx % 21;
        const float v = rowM[idx];
        const int ir = i0 + r;
        if (v != 0.f && ir >= 1 && ir <= Lx && P.slot_type[mb + k] == T_M) {
            const int xr = min((int)P.res[m.x_off + ir - 1], 20);
            atomicAdd(P.cntM + ((int64_t)p * G + P.slot_group[mb + k]) * 441 + xr * 21 + y, (double)v);
        }
    }
    for (int idx = tid; idx < ROWS * wD; idx += CNT_THREADS) {
        const int r = idx / wD, k = idx % wD;
        const float v = rowD[idx];
        const int ir = i0 + r;
        if (v != 0.f && ir >= 1 && ir <= Lx && P.slot_type[db + k] == T_D) {
            const int xr = min((int)P.res[m.x_off + ir - 1], 20);
            atomicAdd(P.cntD + ((int64_t)p * G + P.slot_group[db + k]) * 21 + xr, (double)v);
        }
    }
    // I-type columns not completed inside the chunk
    for (int idx = tid; idx < ROWS * wI; idx += CNT_THREADS) {
        const int jj = max(0, t0 - (ROWS - 1)) + idx / wI, k = idx % wI;
        if (jj > min(Ly, t0 - 1) || P.slot_type[ib + k] != T_I) continue;
        const float v = colI[(jj % ROWS) * wI + k];
        if (v != 0.f) atomicAdd(P.cntI + ((int64_t)p * G + P.slot_group[ib + k]) * 21 + ys[jj], (double)v);
    }
    for (int idx = tid; idx < G * 21; idx += CNT_THREADS) {
        const float v = binsI[idx];
        if (v != 0.f) atomicAdd(P.cntI + (int64_t)p * G * 21 + idx, (double)v);
    }
    __syncthreads();
}

template <class SH>
__global__ void __launch_bounds__(CNT_THREADS, 2) count_block_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemCB L = make_smem_cb(SH::NS, P.G, P.max_ly, P.kend[0] - P.kbeg[0], P.kend[1] - P.kbeg[1],
                                  P.kend[2] - P.kbeg[2]);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        count_chunk_b<SH>(P, w.x, w.y >> 12, w.y & 4095, L, sm, smem_raw);
    }
}

}  // namespace blk
