// estep_wide_nest.cuh -- the wide E-step kernels with the factored MixDom
// transitions (phmm_batch.nest), included by pairhmm.cu after estep_wide.cuh.
//
// The dense wide kernels contract every cell over all NS source slots (about
// 26 k multiply-adds at 162 states).  Under the factored transitions a
// destination k of domain d and sub-state uv needs only
//   sum_a cin[a][k] G_a(pred)  +  sum over its same-domain block of pred[s] intra[s][k]
// (G_a = sum over sources of top-level type a of exit[s] f[s]), 3 + 12 (M-block
// sub-states MM, MI, MD) or 3 + 4 (II, DD) terms at F = 4.  With F = 4 one
// quad of slots is exactly one (domain, sub-state) block, so a thread's 4 x 4
// tile (4 rows x its quad) reads 1 or 3 partner quads of its predecessor
// ring plus three type sums per row.  The type sums of each new cell are
// gathered when the cell is produced -- every thread adds its quad's share
// into a ring of G values per row by shared-memory atomics -- so a step keeps
// the dense kernels' single __syncthreads.  The backward recursion is the
// transpose: b[s] = exit[s] Gb_{U(s)} + its block, with
// Gb_a = sM PM_a(M-succ) + sI PI_a(I-succ) + sD PD_a(D-succ), where
// P_{tau,a}(cell) = sum over the cell's destinations k of type tau of
// cin[a][k] w_k is gathered the same way (nine values per row).
//
// Rings, exponents (E, MX), edge rows, progress counters and lattice records
// are those of the dense wide kernels, so count_wide_kernel reads these
// lattices unchanged.  Stripe-edge checkpointing (recomputation) keeps the
// dense kernels.

namespace wide {

constexpr int NIA = 52;   // floats per quad of intra coefficients (12 partners x 4, padded: no bank conflicts)

struct SmemWn {
    int A, B, E, MX, G, llp, misc;   // rings as the dense kernels; G: type-sum ring
    int ex, cin, c0, chiE, ia, pq;   // coefficients (pq: ints, partner quads [NQd][3])
    int us;                          // int offset: top-level type U of each slot (3 = none) [NS]
    int ys;                          // byte offset
    int bytes;
};

// bwd: rings over the destination slots (KS) and the nine-value P ring
__host__ __device__ inline SmemWn make_smem_wn(int NS, int KS, int max_ly, bool bwd) {
    SmemWn L;
    const int NSRC = bwd ? KS : NS, NQd = KS / 4, BWd = RW + 4;
    int o = 0;
    L.A = o; o += 2 * NSRC * RW;
    L.B = o; o += 3 * NSRC * BWd;
    L.G = o; o += 4 * (bwd ? 9 : 3) * BWd;
    L.E = o; o += 4 * BWd;
    L.MX = o; o += 4 * BWd;
    L.ex = o; o += (NS + 3) & ~3;
    L.cin = o; o += 3 * KS;
    L.c0 = o; o += KS;
    L.chiE = o; o += (NS + 3) & ~3;
    L.ia = o; o += NQd * NIA;
    L.pq = o; o += (3 * NQd + 3) & ~3;
    L.us = o; o += (NS + 3) & ~3;
    o = (o + 1) & ~1;
    L.llp = o / 2; o += 2 * (KS / 4 + 4);
    L.misc = o; o += 8;
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 2;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

// (domain, sub-state) of quad q and the quad of (d, uv), F = 4 (checked by the host)
__device__ __forceinline__ void nest_quad_du(const KParams &P, int q, int &d, int &uv) {
    const int qi = P.kbeg[1] / 4, qd0 = P.kbeg[2] / 4;
    if (q < qi) { d = q; uv = 0; }
    else if (q < qd0) { const int i = q - qi; d = i >> 1; uv = (i & 1) ? 3 : 1; }
    else { const int i = q - qd0; d = i >> 1; uv = (i & 1) ? 4 : 2; }
}
__device__ __forceinline__ int nest_quad_of(const KParams &P, int d, int uv) {
    const int qi = P.kbeg[1] / 4, qd0 = P.kbeg[2] / 4;
    return uv == 0 ? d : (uv == 1 ? qi + 2 * d : (uv == 3 ? qi + 2 * d + 1 : (uv == 2 ? qd0 + 2 * d : qd0 + 2 * d + 1)));
}
__device__ __forceinline__ int nest_U(int uv) { return uv < 3 ? 0 : uv - 2; }

// exponent of a stored maximum (positive float bits): e with m 2^-e in [0.5, 1)
// for normal m; a subnormal maximum counts as 2^-126 (the predicted output
// exponent then keeps the cell's values a little below 0.5, which every
// consumer takes with its exponent)
__device__ __forceinline__ int exp_of_max_n(int mbits) { return max((mbits >> 23) & 0xff, 1) - 126; }

// Coefficients of pair p into shared memory (all threads).  bwd: intra rows by
// source quad (partners = destination slots), else by destination quad.
__device__ void load_nest_wide(const KParams &P, int p, const SmemWn &L, float *sm, bool bwd) {
    const int NS = P.NS, KS = P.kend[2], NQd = KS / 4, N = P.N;
    constexpr int F = 4, bs = 20;
    const int K = P.nest_K, nb = 5 * K * F;
    const int tid = threadIdx.x, nt = blockDim.x;
    const float *rec = P.nest + (int64_t)p * P.nest_stride;
    const float *chi = P.chi + (int64_t)p * P.chi_stride;
    int *us = reinterpret_cast<int *>(sm) + L.us;
    for (int s = tid; s < NS; s += nt) {
        float v = 0.f;
        int u = 3;
        if (s < KS) {
            int d, uv;
            nest_quad_du(P, s >> 2, d, uv);
            v = __ldg(rec + d * bs + uv * F + (s & 3));
            u = nest_U(uv);
        }
        sm[L.ex + s] = v;
        us[s] = u;
        const int os = P.slot_orig[s];
        sm[L.chiE + s] = os >= 0 ? __ldg(chi + os * N + P.e_idx) : 0.f;
    }
    for (int idx = tid; idx < 3 * KS; idx += nt) {
        const int a = idx / KS, k = idx % KS;
        int d, uv;
        nest_quad_du(P, k >> 2, d, uv);
        sm[L.cin + idx] = __ldg(rec + nb + a * nb + d * bs + uv * F + (k & 3));
    }
    for (int k = tid; k < KS; k += nt) sm[L.c0 + k] = __ldg(chi + P.slot_orig[k]);   // start -> k
    int *pq = reinterpret_cast<int *>(sm) + L.pq;
    for (int q = tid; q < NQd; q += nt) {
        int d, uv;
        nest_quad_du(P, q, d, uv);
        for (int j = 0; j < 3; ++j) pq[3 * q + j] = uv < 3 ? nest_quad_of(P, d, j) : (j == 0 ? q : -1);
    }
    for (int idx = tid; idx < NQd * 48; idx += nt) {
        const int q = idx / 48, j = (idx % 48) / 4, u = idx % 4;
        int d, uv;
        nest_quad_du(P, q, d, uv);
        const int pj = j >> 2, uu = j & 3;
        float v = 0.f;
        if (uv < 3 || pj == 0) {
            const int puv = uv < 3 ? pj : uv;           // the partner's sub-state
            const int mine = uv * F + u, other = puv * F + uu;
            const int row = bwd ? mine : other, col = bwd ? other : mine;   // intra[src][dst]
            v = __ldg(rec + 4 * nb + d * bs * bs + row * bs + col);
        }
        sm[L.ia + q * NIA + j * 4 + u] = v;
    }
}

// Emission factors of a thread's 4 destination slots (one quad, one type) at
// its 4 rows, looked up per step by the y character only: offsets into the
// M / I tables built once per stripe, D factors (fixed by the row's x) read
// once.  (The dense kernels decode slot type and group per lookup.)
struct QuadEmit {
    const float *tab;   // eM (by x and y), eI (by y) or eD (by x)
    int gb[4];          // [u] group offset
    int xo[4];          // [row] x offset (M: 21 x, D: x, I: 0)
    int ym;             // 1: add y (M, I), 0 (D)
    __device__ void init(const KParams &P, const float *eMg, const float *eIg, const float *eDg, int q, const int (&xr)[4]) {
        const int qt = P.quad_type[q];
#pragma unroll
        for (int u = 0; u < 4; ++u) gb[u] = P.slot_group[4 * q + u] * (qt == T_M ? 441 : 21);
#pragma unroll
        for (int i = 0; i < 4; ++i) xo[i] = qt == T_M ? xr[i] * 21 : (qt == T_D ? xr[i] : 0);
        tab = qt == T_M ? eMg : (qt == T_I ? eIg : eDg);
        ym = qt == T_D ? 0 : 1;
    }
    __device__ __forceinline__ float at(int i, int u, int y) const { return __ldg(tab + gb[u] + xo[i] + ym * y); }
};

// ---------------------------------------------------------------- forward
__device__ void fwd_stripe_wn(const KParams &P, int p, int si, const SmemWn &L, float *sm, unsigned char *smb) {
    const int NS = P.NS, KS = P.kend[2], NQd = KS / 4;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int rg = lane & 7, qd = 4 * warp + (lane >> 3);
    const bool active = qd < NQd;
    const int r0 = 4 * rg;
    const int i0 = si * RW;
    const int nrows = min(RW, Lx + 1 - i0);
    const bool has_above = si > 0, has_below = si + 1 < m.n_stripes;
    const int ES = ls_of(NS);
    const int *prog_above = has_above ? P.progress + m.stripe_base + si - 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_above = P.edge + (m.edge_base + (int64_t)(si - 1) * (Ly + 1)) * ES;
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * ES;
    const int64_t latc = m.lat_base + (int64_t)si * (RW + Ly) * RW;
    float *A = sm + L.A, *B = sm + L.B, *GB = sm + L.G;
    int *E = reinterpret_cast<int *>(sm) + L.E;
    int *MX = reinterpret_cast<int *>(sm) + L.MX;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    double *llp = reinterpret_cast<double *>(sm) + L.llp;
    unsigned char *ys = smb + L.ys;
    const int BW = RW + 4;
    const int GS = 3 * BW;   // one G slot: [3][BW], row r at index r + 1, the halo row at 0
    load_nest_wide(P, p, L, sm, false);
    for (int idx = tid; idx < 2 * NS * RW; idx += nt) A[idx] = 0.f;
    for (int idx = tid; idx < 3 * NS * BW; idx += nt) B[idx] = 0.f;
    for (int idx = tid; idx < 4 * GS; idx += nt) GB[idx] = 0.f;
    for (int idx = tid; idx < 4 * BW; idx += nt) { E[idx] = EXP_NONE; MX[idx] = 0; }
    for (int j = tid; j <= Ly; j += nt) {
        int c = 0;
        if (j >= 1) {
            c = P.res[m.y_off + j - 1];
            if (c > 20) { c = 20; atomicOr(P.status + p, PHMM_ST_BAD_RESIDUE); }
        }
        ys[j] = (unsigned char)c;
    }
    if (tid == 0) { misc[0] = 0; misc[1] = 0; }
    const float *eMg = P.eM + (int64_t)p * P.eM_stride;
    const float *eIg = P.eI + (int64_t)p * P.eID_stride;
    const float *eDg = P.eD + (int64_t)p * P.eID_stride;
    int xr[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int row = i0 + r0 + i;
        xr[i] = (row >= 1 && row <= Lx) ? min((int)P.res[m.x_off + row - 1], 20) : 0;
    }
    const int qt = active ? P.quad_type[qd] : T_NONE;
    int myd = 0, myuv = 0;
    if (active) nest_quad_du(P, qd, myd, myuv);
    const int myU = nest_U(myuv);
    const int T_last = (nrows - 1) + Ly;
    QuadEmit qe;
    qe.init(P, eMg, eIg, eDg, active ? qd : 0, xr);
    const int *usl = reinterpret_cast<const int *>(sm) + L.us;
    __syncthreads();   // coefficients in place
    float cinr[3][4], exr[4];
    int pqr[3] = {-1, -1, -1};
    if (active) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            exr[u] = sm[L.ex + 4 * qd + u];
#pragma unroll
            for (int a = 0; a < 3; ++a) cinr[a][u] = sm[L.cin + a * KS + 4 * qd + u];
        }
        const int *pq = reinterpret_cast<const int *>(sm) + L.pq;
#pragma unroll
        for (int j = 0; j < 3; ++j) pqr[j] = pq[3 * qd + j];
    } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            exr[u] = 0.f;
#pragma unroll
            for (int a = 0; a < 3; ++a) cinr[a][u] = 0.f;
        }
    }
    const float *iaq = sm + L.ia + (active ? qd : 0) * NIA;
    // halo column col of row i0-1: B slot (col - 1) % 3 index 0, E / MX slot
    // (col - 1) & 3, and its type sums in G slot (col - 1) & 3 index 0 (warp 0)
    // The halo column is loaded into registers one step before it is staged
    // (its L2 latency then overlaps a whole step instead of holding warp 0
    // -- and with it the step's barrier -- at the end of each step).
    constexpr int HQ = (WMAXS + 31) / 32;
    float hv[HQ];
    int hE = EXP_NONE, hMX = 0;
    auto load_halo = [&](int col) -> bool {   // warp 0
        if (!has_above || col > Ly) return true;
        int ok = 1;
        if (lane == 0) ok = wait_geq(prog_above, col + 1, P.spin_limit) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) return false;
        const float *src = edge_above + (int64_t)col * ES;
#pragma unroll
        for (int j = 0; j < HQ; ++j) {
            const int s2 = lane + 32 * j;
            hv[j] = s2 < NS ? __ldcg(src + s2) : 0.f;
        }
        if (lane == 0) {
            hE = __ldcg(reinterpret_cast<const int *>(src) + NS);
            hMX = __ldcg(reinterpret_cast<const int *>(src) + NS + 1);
        }
        return true;
    };
    auto stage_halo = [&](int col) {   // warp 0: the loaded column into B, E / MX and its type sums
        if (!has_above || col > Ly) return;
        const int bs = (col + 2) % 3, es = (col + 3) & 3;
        float g[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int j = 0; j < HQ; ++j) {
            const int s2 = lane + 32 * j;
            if (s2 < NS) {
                B[(bs * NS + s2) * BW] = hv[j];
                const int u = usl[s2];
                const float c = sm[L.ex + s2] * hv[j];
                g[0] += u == 0 ? c : 0.f;
                g[1] += u == 1 ? c : 0.f;
                g[2] += u == 2 ? c : 0.f;
            }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) g[a] += __shfl_xor_sync(0xffffffffu, g[a], o);
        if (lane == 0) {
            E[es * BW] = hE;
            MX[es * BW] = hMX;
#pragma unroll
            for (int a = 0; a < 3; ++a) GB[es * GS + a * BW] = g[a];
        }
    };
    __syncthreads();
    if (warp == 0) {
        bool ok = load_halo(0);
        if (ok) stage_halo(0);
        if (ok) ok = load_halo(1);
        if (!ok && lane == 0) misc[0] = 1;
    }
    int llE = EXP_NONE;
    bool aborted = false;
    int k = 0;
    for (int t = 0; t <= T_last; ++t, ++k) {
        __syncthreads();
        if (misc[k & 1]) { aborted = true; break; }
        if (tid == 0) misc[(k + 1) & 1] = 0;
        for (int r = tid; r < RW; r += nt) MX[((t + 1) & 3) * BW + r + 1] = 0;
        // the G slot of step t+1 starts at zero (last read at step t-1, as an M-predecessor)
        for (int idx = tid; idx < GS; idx += nt) {
            if (idx % BW != 0) GB[((t + 1) & 3) * GS + idx] = 0.f;   // index 0: the halo row, written by warp 0
        }
        if (si == 0 && tid == 0 && P.s_slot >= KS) {
            if (t == 2) A[(0 * NS + P.s_slot) * RW + 0] = 0.f;
            if (t == 3) B[(0 * NS + P.s_slot) * BW + 1] = 0.f;
        }
        // ---- bottom row of step t-1 -> edge row for the stripe below (warp 1)
        if (warp == (nt > 32 ? 1 : 0) && has_below && t >= 1) {
            const int jb = t - 1 - (RW - 1);
            if (jb >= 0 && jb <= Ly) {
                const int sl = (t - 1) % 3;
                float *dst = edge_mine + (int64_t)jb * ES;
                for (int s = lane; s < NS; s += 32) dst[s] = B[(sl * NS + s) * BW + RW];
                if (lane == 0) {
                    reinterpret_cast<int *>(dst)[NS] = E[((t - 1) & 3) * BW + RW];
                    reinterpret_cast<int *>(dst)[NS + 1] = MX[((t - 1) & 3) * BW + RW];
                }
                if (((jb + 1) % WPUB) == 0 || jb == Ly) {   // publish: this and the earlier columns' rows
                    __threadfence();
                    __syncwarp();
                    if (lane == 0) st_release(prog_mine, jb + 1);
                }
            }
        }
        if (active) {
            int Eo[4];
            float sc[4];
            bool valid[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, row = i0 + r, j = t - r;
                valid[i] = r < nrows && j >= 0 && j <= Ly;
                int EI = EXP_NONE, ED = EXP_NONE, EM = EXP_NONE;
                if (valid[i]) {
                    if (j >= 1) {
                        const int mb = MX[((t - 1) & 3) * BW + r + 1];
                        const int e = E[((t - 1) & 3) * BW + r + 1];
                        if (mb > 0 && e > EXP_NONE) EI = e + exp_of_max_n(mb);
                    }
                    if (row >= 1) {
                        const int mb = MX[((t - 1) & 3) * BW + r];
                        const int e = E[((t - 1) & 3) * BW + r];
                        if (mb > 0 && e > EXP_NONE) ED = e + exp_of_max_n(mb);
                    }
                    if (row >= 1 && j >= 1) {
                        const int mb = MX[((t - 2) & 3) * BW + r];
                        const int e = E[((t - 2) & 3) * BW + r];
                        if (mb > 0 && e > EXP_NONE) EM = e + exp_of_max_n(mb);
                    }
                }
                const int Eout = max(max(EI, ED), EM);
                Eo[i] = Eout;
                const int Emine = qt == T_I ? EI : (qt == T_D ? ED : EM);
                const int Eraw = qt == T_I ? E[((t - 1) & 3) * BW + r + 1]
                                           : (qt == T_D ? E[((t - 1) & 3) * BW + r] : E[((t - 2) & 3) * BW + r]);
                sc[i] = (Emine > EXP_NONE && Eout > EXP_NONE) ? pow2d(Eraw - Eout) : 0.f;
            }
            const float *base = qt == T_I ? A + ((t - 1) & 1) * NS * RW + r0
                                          : (qt == T_D ? B + ((t + 2) % 3) * NS * BW + r0 : B + ((t + 1) % 3) * NS * BW + r0);
            const int stride = qt == T_I ? RW : BW;
            // type sums of the predecessor rows (I: own row at t-1; D, M: row above at t-1, t-2)
            const float *gp = qt == T_I ? GB + ((t - 1) & 3) * GS + r0 + 1
                                        : (qt == T_D ? GB + ((t - 1) & 3) * GS + r0 : GB + ((t - 2) & 3) * GS + r0);
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float g0 = gp[i], g1 = gp[BW + i], g2 = gp[2 * BW + i];
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[i][u] = fmaf(cinr[2][u], g2, fmaf(cinr[1][u], g1, cinr[0][u] * g0));
            }
            // the same-domain block: 1 or 3 partner quads of the predecessor row
#pragma unroll
            for (int pj = 0; pj < 3; ++pj) {
                if (pqr[pj] < 0) continue;
#pragma unroll
                for (int uu = 0; uu < 4; ++uu) {
                    const int s = 4 * pqr[pj] + uu;
                    const float4 pv = *reinterpret_cast<const float4 *>(base + s * stride);
                    const float4 cv = *reinterpret_cast<const float4 *>(iaq + (4 * pj + uu) * 4);
                    const float pa[4] = {pv.x, pv.y, pv.z, pv.w};
                    const float ca[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int u = 0; u < 4; ++u) acc[i][u] = fmaf(pa[i], ca[u], acc[i][u]);
                }
            }
            // the start state (non-zero only at the origin) for the cells next to it
            if (si == 0 && t <= 2 && P.s_slot >= KS) {
                const float4 pv = *reinterpret_cast<const float4 *>(base + P.s_slot * stride);
                const float pa[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[i][u] = fmaf(pa[i], sm[L.c0 + 4 * qd + u], acc[i][u]);
            }
            float mxr[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, j = t - r;
                const int yj = valid[i] ? ys[j] : 0;
                const bool origin = valid[i] && i0 + r == 0 && j == 0;
                mxr[i] = 0.f;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    float v = 0.f;
                    if (valid[i] && sc[i] > 0.f) v = acc[i][u] * sc[i] * qe.at(i, u, yj);
                    if (4 * qd + u == P.s_slot) v = origin ? 1.f : 0.f;
                    acc[i][u] = v;
                    mxr[i] = fmaxf(mxr[i], v);
                }
            }
            const int sa = t & 1, sb = t % 3;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int s = 4 * qd + u;
                *reinterpret_cast<float4 *>(A + (sa * NS + s) * RW + r0) =
                    make_float4(acc[0][u], acc[1][u], acc[2][u], acc[3][u]);
#pragma unroll
                for (int i = 0; i < 4; ++i) B[(sb * NS + s) * BW + r0 + i + 1] = acc[i][u];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, row = i0 + r, j = t - r;
                const bool origin = valid[i] && row == 0 && j == 0;
                if (qd == 0) E[(t & 3) * BW + r + 1] = origin ? 0 : Eo[i];
                if (mxr[i] > 0.f) atomicMax(MX + (t & 3) * BW + r + 1, __float_as_int(mxr[i]));
                // my quad's share of the new cell's type sum
                const float g = fmaf(exr[3], acc[i][3], fmaf(exr[2], acc[i][2], fmaf(exr[1], acc[i][1], exr[0] * acc[i][0])));
                if (g != 0.f) atomicAdd(GB + (t & 3) * GS + myU * BW + r + 1, g);
                if (valid[i] && P.lat) {
                    const int64_t cell = latc + (int64_t)t * RW + r;
                    float *rec = P.lat + cell * ES;
                    *reinterpret_cast<float4 *>(rec + 4 * qd) = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
                    if (qd == 0) {
                        for (int s2 = KS; s2 < NS; ++s2) rec[s2] = (origin && s2 == P.s_slot) ? 1.f : 0.f;
                        reinterpret_cast<int *>(rec)[NS] = origin ? 0 : Eo[i];
                    }
                }
                if (valid[i] && row == Lx && j == Ly && si + 1 == m.n_stripes) {
                    double a = 0.0;
#pragma unroll
                    for (int u = 0; u < 4; ++u) a += (double)acc[i][u] * (double)sm[L.chiE + 4 * qd + u];
                    llp[qd] = a;
                    if (qd == 0) llE = origin ? 0 : Eo[i];
                }
            }
            if (si == 0 && t == 0 && qd == 0 && rg == 0 && P.s_slot >= KS) {
                A[(0 * NS + P.s_slot) * RW + 0] = 1.f;
                B[(0 * NS + P.s_slot) * BW + 1] = 1.f;
                atomicMax(MX + 0 * BW + 1, __float_as_int(1.f));
            }
        }
        if (warp == 0 && t + 1 <= T_last) {   // column t+1 (loaded last step) staged; t+2 loaded
            stage_halo(t + 1);
            if (t + 2 <= T_last && !load_halo(t + 2) && lane == 0) misc[(k + 1) & 1] = 1;
        }
    }
    __syncthreads();
    if (!aborted && has_below) {
        const int t = T_last + 1;
        const int jb = t - 1 - (RW - 1);
        if (warp == (nt > 32 ? 1 : 0) && jb >= 0 && jb <= Ly) {
            const int sl = (t - 1) % 3;
            float *dst = edge_mine + (int64_t)jb * ES;
            for (int s = lane; s < NS; s += 32) dst[s] = B[(sl * NS + s) * BW + RW];
            if (lane == 0) {
                reinterpret_cast<int *>(dst)[NS] = E[((t - 1) & 3) * BW + RW];
                reinterpret_cast<int *>(dst)[NS + 1] = MX[((t - 1) & 3) * BW + RW];
            }
            __threadfence();
        }
    }
    __syncthreads();
    if (tid == 0) {
        if (has_below) { __threadfence(); st_release(prog_mine, Ly + 1); }
        if (aborted) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (si + 1 == m.n_stripes) P.ll[p] = NEG_INF_LL;
        }
    }
    if (!aborted && si + 1 == m.n_stripes) {
        int *Eterm = misc + 4;
        const int rT = Lx - i0;
        if (active && qd == 0 && rg == (rT >> 2)) *Eterm = llE;
        __syncthreads();
        if (tid == 0) {
            double acc = 0.0;
            for (int q = 0; q < NQd; ++q) acc += llp[q];
            if (Lx == 0 && Ly == 0 && P.s_slot >= KS) acc += (double)sm[L.chiE + P.s_slot];
            const int Et = *Eterm;
            double ll = NEG_INF_LL;
            if (acc > 0.0 && isfinite(acc) && Et > EXP_NONE) ll = log(acc) + (double)Et * LN2;
            else atomicOr(P.status + p, PHMM_ST_ZERO_LL);
            P.ll[p] = ll;
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(prog_mine, Ly + 2);
}

// ---------------------------------------------------------------- backward recursion
__device__ void bwd_rec_stripe_wn(const KParams &P, int p, int si, const SmemWn &L, float *sm, unsigned char *smb) {
    const int NS = P.NS, KS = P.kend[2], NQd = KS / 4;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int rg = lane & 7, qs = 4 * warp + (lane >> 3);   // output (source) quad
    const bool active = qs < NQd;
    const int r0 = 4 * rg;
    const int i0 = si * RW;
    const int nrows = min(RW, Lx + 1 - i0);
    const bool has_above = si > 0, has_below = si + 1 < m.n_stripes;
    const int ES = ls_of(NS);
    const int *prog_below = has_below ? P.bprogress + m.stripe_base + si + 1 : nullptr;
    int *prog_mine = P.bprogress + m.stripe_base + si;
    const float *edge_below = P.bedge + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * ES;
    float *edge_mine = P.bedge + (m.edge_base + (int64_t)si * (Ly + 1)) * ES;
    const int64_t latc = m.lat_base + (int64_t)si * (RW + Ly) * RW;
    float *A = sm + L.A, *B = sm + L.B, *PR = sm + L.G;
    int *E = reinterpret_cast<int *>(sm) + L.E;
    int *MX = reinterpret_cast<int *>(sm) + L.MX;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    unsigned char *ys = smb + L.ys;
    const int BW = RW + 4;
    const int PS = 9 * BW;   // one P slot: [tau * 3 + a][BW], row r at index r + 3, the halo row at RW + 3
    load_nest_wide(P, p, L, sm, true);
    for (int idx = tid; idx < 2 * KS * RW; idx += nt) A[idx] = 0.f;
    for (int idx = tid; idx < 3 * KS * BW; idx += nt) B[idx] = 0.f;
    for (int idx = tid; idx < 4 * PS; idx += nt) PR[idx] = 0.f;
    for (int idx = tid; idx < 4 * BW; idx += nt) { E[idx] = EXP_NONE; MX[idx] = 0; }
    for (int j = tid; j <= Ly; j += nt) {
        int c = 0;
        if (j >= 1) c = min((int)P.res[m.y_off + j - 1], 20);
        ys[j] = (unsigned char)c;
    }
    if (tid == 0) { misc[0] = 0; misc[1] = 0; }
    const float *eMg = P.eM + (int64_t)p * P.eM_stride;
    const float *eIg = P.eI + (int64_t)p * P.eID_stride;
    const float *eDg = P.eD + (int64_t)p * P.eID_stride;
    int xr[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int row = i0 + r0 + i;
        xr[i] = (row >= 1 && row <= Lx) ? min((int)P.res[m.x_off + row - 1], 20) : 0;
    }
    const int T_last = (nrows - 1) + Ly;
    int myd = 0, myuv = 0;
    if (active) nest_quad_du(P, qs, myd, myuv);
    const int myU = nest_U(myuv);
    const int myT = active ? P.quad_type[qs] - T_M : 0;   // my quad as destinations: 0 M, 1 I, 2 D
    QuadEmit qe;
    qe.init(P, eMg, eIg, eDg, active ? qs : 0, xr);
    __syncthreads();
    float cinr[3][4], exr[4];
    int pqr[3] = {-1, -1, -1};
    if (active) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            exr[u] = sm[L.ex + 4 * qs + u];
#pragma unroll
            for (int a = 0; a < 3; ++a) cinr[a][u] = sm[L.cin + a * KS + 4 * qs + u];
        }
        const int *pq = reinterpret_cast<const int *>(sm) + L.pq;
#pragma unroll
        for (int j = 0; j < 3; ++j) pqr[j] = pq[3 * qs + j];
    } else {
        // (inactive: no partners)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            exr[u] = 0.f;
#pragma unroll
            for (int a = 0; a < 3; ++a) cinr[a][u] = 0.f;
        }
    }
    const float *iaq = sm + L.ia + (active ? qs : 0) * NIA;
    int tqr[3];   // the partner quads' destination types
#pragma unroll
    for (int j = 0; j < 3; ++j) tqr[j] = pqr[j] >= 0 ? P.quad_type[pqr[j]] : T_NONE;
    // halo: row i0+RW at column c: B slot (c + RW) % 3 index RW + 3, E / MX slot
    // (c + RW) & 3 index RW, its nine P sums in P slot (c + RW) & 3 index RW + 3
    constexpr int HQ = (WMAXS + 31) / 32;
    float hv[HQ];
    int hE = EXP_NONE, hMX = 0;
    auto load_halo = [&](int col) -> bool {   // warp 0 (loaded a step before staged, as in the forward)
        if (!has_below || col < 0 || col > Ly) return true;
        int ok = 1;
        if (lane == 0) ok = wait_geq(prog_below, Ly + 1 - col, P.spin_limit) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) return false;
        const float *src = edge_below + (int64_t)col * ES;
#pragma unroll
        for (int jj = 0; jj < HQ; ++jj) {
            const int kk = lane + 32 * jj;
            hv[jj] = kk < KS ? __ldcg(src + kk) : 0.f;
        }
        if (lane == 0) {
            hE = __ldcg(reinterpret_cast<const int *>(src) + NS);
            hMX = __ldcg(reinterpret_cast<const int *>(src) + NS + 1);
        }
        return true;
    };
    auto stage_halo = [&](int col) {
        if (!has_below || col < 0 || col > Ly) return;
        const int bs = (col + RW) % 3, es = (col + RW) & 3;
        float pv[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) pv[v] = 0.f;
        const int qi = P.kbeg[1] / 4, qd0 = P.kbeg[2] / 4;
#pragma unroll
        for (int jj = 0; jj < HQ; ++jj) {
            const int kk = lane + 32 * jj;
            if (kk < KS) {
                const float w = hv[jj];
                B[(bs * KS + kk) * BW + RW + 3] = w;
                const int qk = kk >> 2;
                const int tk = qk < qi ? 0 : (qk < qd0 ? 1 : 2);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float c = sm[L.cin + a * KS + kk] * w;
                    pv[0 + a] += tk == 0 ? c : 0.f;
                    pv[3 + a] += tk == 1 ? c : 0.f;
                    pv[6 + a] += tk == 2 ? c : 0.f;
                }
            }
        }
#pragma unroll
        for (int v = 0; v < 9; ++v)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) pv[v] += __shfl_xor_sync(0xffffffffu, pv[v], o);
        if (lane == 0) {
            E[es * BW + RW] = hE;
            MX[es * BW + RW] = hMX;
#pragma unroll
            for (int v = 0; v < 9; ++v) PR[es * PS + v * BW + RW + 3] = pv[v];
        }
    };
    auto publish_top = [&](int t) {
        if (!has_above || t < 0 || t > Ly) return;
        float *dst = edge_mine + (int64_t)t * ES;
        for (int kk = lane; kk < KS; kk += 32) dst[kk] = A[((t & 1) * KS + kk) * RW + 0];
        if (lane == 0) {
            reinterpret_cast<int *>(dst)[NS] = E[(t & 3) * BW + 0];
            reinterpret_cast<int *>(dst)[NS + 1] = MX[(t & 3) * BW + 0];
        }
        if ((t % WPUB) == 0) {   // publish: this and the earlier (higher) columns' rows
            __threadfence();
            __syncwarp();
            if (lane == 0) st_release(prog_mine, Ly + 1 - t);
        }
    };
    __syncthreads();
    if (warp == 0) {
        bool ok = load_halo(T_last - (RW - 1));
        if (ok) stage_halo(T_last - (RW - 1));
        if (ok) ok = load_halo(T_last - RW);
        if (!ok && lane == 0) misc[0] = 1;
    }
    bool aborted = false;
    int k = 0;
    for (int t = T_last; t >= 0; --t, ++k) {
        __syncthreads();
        if (misc[k & 1]) { aborted = true; break; }
        if (tid == 0) misc[(k + 1) & 1] = 0;
        for (int r = tid; r < RW; r += nt) MX[((t - 1) & 3) * BW + r] = 0;
        // the P slot of step t-1 starts at zero (last read at step t+1, as an
        // M-successor); its halo index RW + 3 is written by warp 0
        for (int idx = tid; idx < PS; idx += nt) {
            if (idx % BW != RW + 3) PR[((t - 1) & 3) * PS + idx] = 0.f;
        }
        if (warp == (nt > 32 ? 1 : 0)) publish_top(t + 1);
        if (active) {
            int Eo[4], EsM[4], EsI[4], EsD[4];
            bool valid[4], term[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, row = i0 + r, j = t - r;
                valid[i] = r < nrows && j >= 0 && j <= Ly;
                term[i] = valid[i] && row == Lx && j == Ly;
                int vI = EXP_NONE, vD = EXP_NONE, vM = EXP_NONE;
                EsI[i] = EsD[i] = EsM[i] = EXP_NONE;
                if (valid[i] && !term[i]) {
                    if (j + 1 <= Ly) {
                        const int mb = MX[((t + 1) & 3) * BW + r], e = E[((t + 1) & 3) * BW + r];
                        if (mb > 0 && e > EXP_NONE) { EsI[i] = e; vI = e + exp_of_max_n(mb); }
                    }
                    if (row + 1 <= Lx) {
                        const int mb = MX[((t + 1) & 3) * BW + r + 1], e = E[((t + 1) & 3) * BW + r + 1];
                        if (mb > 0 && e > EXP_NONE) { EsD[i] = e; vD = e + exp_of_max_n(mb); }
                    }
                    if (row + 1 <= Lx && j + 1 <= Ly) {
                        const int mb = MX[((t + 2) & 3) * BW + r + 1], e = E[((t + 2) & 3) * BW + r + 1];
                        if (mb > 0 && e > EXP_NONE) { EsM[i] = e; vM = e + exp_of_max_n(mb); }
                    }
                }
                Eo[i] = term[i] ? 0 : max(max(vI, vD), vM);
            }
            float sM[4], sI[4], sD[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                sM[i] = (EsM[i] > EXP_NONE) ? pow2d(EsM[i] - Eo[i]) : 0.f;
                sI[i] = (EsI[i] > EXP_NONE) ? pow2d(EsI[i] - Eo[i]) : 0.f;
                sD[i] = (EsD[i] > EXP_NONE) ? pow2d(EsD[i] - Eo[i]) : 0.f;
            }
            // Gb for my sources' type: I-successor (own row, t+1), D (row + 1, t+1), M (row + 1, t+2)
            const float *pI = PR + ((t + 1) & 3) * PS + (3 + myU) * BW + r0 + 3;
            const float *pD = PR + ((t + 1) & 3) * PS + (6 + myU) * BW + r0 + 4;
            const float *pM = PR + ((t + 2) & 3) * PS + (0 + myU) * BW + r0 + 4;
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float gb = fmaf(sD[i], pD[i], fmaf(sI[i], pI[i], sM[i] * pM[i]));
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[i][u] = exr[u] * gb;
            }
            // the same-domain block: 1 or 3 partner destination quads, each from its type's successor ring
#pragma unroll
            for (int pj = 0; pj < 3; ++pj) {
                if (pqr[pj] < 0) continue;
                const int tq = tqr[pj];
                const float *wb = tq == T_M ? B + ((t + 2) % 3) * KS * BW + r0 + 4
                                            : (tq == T_I ? A + ((t + 1) & 1) * KS * RW + r0 : B + ((t + 1) % 3) * KS * BW + r0 + 4);
                const int wst = tq == T_I ? RW : BW;
                float sw[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) sw[i] = tq == T_M ? sM[i] : (tq == T_I ? sI[i] : sD[i]);
#pragma unroll
                for (int uu = 0; uu < 4; ++uu) {
                    const int kk = 4 * pqr[pj] + uu;
                    const float4 w = *reinterpret_cast<const float4 *>(wb + kk * wst);
                    const float4 cv = *reinterpret_cast<const float4 *>(iaq + (4 * pj + uu) * 4);
                    const float wa[4] = {w.x * sw[0], w.y * sw[1], w.z * sw[2], w.w * sw[3]};
                    const float ca[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int u = 0; u < 4; ++u) acc[i][u] = fmaf(wa[i], ca[u], acc[i][u]);
                }
            }
            float bv[4][4], mxr[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, j = t - r;
                const int yj = valid[i] ? ys[j] : 0;
                mxr[i] = 0.f;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    float b = 0.f;
                    if (valid[i]) {
                        b = term[i] ? sm[L.chiE + 4 * qs + u] : acc[i][u];
                        mxr[i] = fmaxf(mxr[i], b * qe.at(i, u, yj));
                    }
                    bv[i][u] = b;
                }
            }
            const int sa = t & 1, sb = t % 3;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, j = t - r;
                const int yj = valid[i] ? ys[j] : 0;
                float wv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    wv[u] = valid[i] ? bv[i][u] * qe.at(i, u, yj) : 0.f;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    A[(sa * KS + 4 * qs + u) * RW + r] = wv[u];
                    B[(sb * KS + 4 * qs + u) * BW + r + 3] = wv[u];
                }
                // my quad's share of the new cell's P sums (my quad as destinations of type myT)
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float pa = fmaf(cinr[a][3], wv[3], fmaf(cinr[a][2], wv[2], fmaf(cinr[a][1], wv[1], cinr[a][0] * wv[0])));
                    if (pa != 0.f) atomicAdd(PR + (t & 3) * PS + (3 * myT + a) * BW + r + 3, pa);
                }
                if (qs == 0) E[(t & 3) * BW + r] = valid[i] ? Eo[i] : EXP_NONE;
                if (mxr[i] > 0.f) atomicMax(MX + (t & 3) * BW + r, __float_as_int(mxr[i]));
                if (valid[i] && P.blat) {
                    const int64_t cell = latc + (int64_t)t * RW + r;
                    float *rec = P.blat + cell * ES;
                    *reinterpret_cast<float4 *>(rec + 4 * qs) = make_float4(bv[i][0], bv[i][1], bv[i][2], bv[i][3]);
                    if (qs == 0) reinterpret_cast<int *>(rec)[NS] = Eo[i];
                }
            }
        }
        if (warp == 0) {   // column t - RW (loaded last step) staged; the next one loaded
            stage_halo(t - RW);
            if (!load_halo(t - RW - 1) && lane == 0) misc[(k + 1) & 1] = 1;
        }
    }
    __syncthreads();
    if (!aborted && warp == (nt > 32 ? 1 : 0)) publish_top(0);
    __syncthreads();
    if (tid == 0) {
        if (has_above) { __threadfence(); st_release(prog_mine, Ly + 1); }
        if (aborted) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(prog_mine, Ly + 2);
}

// Persistent CTAs over interleaved forward and backward stripe items (E-step),
// or forward items only.
template <bool FWD_ONLY>
__global__ void __launch_bounds__(384) wide_nest_kernel(const KParams P) {   // 32 x 12 warps at most (48 quads)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemWn Lf = make_smem_wn(P.NS, P.kend[2], P.max_ly, false);
    const SmemWn Lb = make_smem_wn(P.NS, P.kend[2], P.max_ly, true);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        if (!FWD_ONLY && (w.y & blk::BWD_ITEM)) bwd_rec_stripe_wn(P, w.x, w.y & ~blk::BWD_ITEM, Lb, sm, smem_raw);
        else fwd_stripe_wn(P, w.x, w.y, Lf, sm, smem_raw);
    }
}

}  // namespace wide
