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
    int nest;       // float offset: factored MixDom transition coefficients (NestSlots), or -1
    int bytes;
};

__host__ __device__ inline SmemTW make_smem_tw(int SP, int KP, int NI, int G, int max_ly, bool bwd,
                                               int nest_floats = 0) {
    SmemTW L;
    L.w = make_smem_w(SP, KP, NI, G, max_ly, bwd, false);
    int o = L.w.bytes / 4;   // L.w.bytes is a multiple of 16
    L.bnd = o; o += 2 * SP;
    L.bndE = o; o += 4;
    L.flag = o; o += 4;
    L.nest = -1;
    if (nest_floats > 0) { L.nest = o; o += al4(nest_floats); }   // o stays a multiple of 4
    L.bytes = o * 4;
    return L;
}

// ---------------------------------------------------------------- factored (nested) transitions
// The collapsed MixDom chi (models/mixdom.py:252-423) is, between body
// states, chi[s][k] = exit[s] T_exit_k[d_k][U(s)][U(k)] dest[k] plus a
// same-domain block: the inter-domain part factors through the three
// top-level types U in {M, I, D} (MM, MI, MD -> M; II -> I; DD -> D), and
// within a domain the M-block couples MM, MI, MD (3F x 3F) while II and DD
// couple only among their own fragments (F x F).  With cin[a][k] = dest[k]
// T_exit_k[d_k][a][U(k)] a destination's sum over all sources becomes
//   sum_s f[s] chi[s][k] = sum_a cin[a][k] G_a + sum_{s in block(k)} f[s] intra[s][k],
//   G_a = sum_{s: U(s) = a} exit[s] f[s],
// 3 + 3F (or 3 + F) multiply-adds instead of N, plus the three G sums per
// cell; the backward recursion is the transpose.  NoNest keeps the dense
// contraction (any chi); Nest<K, F> is the MixDom layout with K domains and
// F fragments, in the two-warp slot order (M states, then I, then D, each in
// state order: MM_df; MI_df, II_df per domain; MD_df, DD_df per domain).
struct NoNest { static constexpr int K = 0, F = 0; };
template <int K_, int F_> struct Nest { static constexpr int K = K_, F = F_; };

template <class SH, class NT>
struct NestSlots {
    static constexpr int K = NT::K, F = NT::F, NM = SH::NM, NI = SH::NI, NE = SH::NE;
    static_assert(NM == K * F && NI == 2 * K * F && SH::ND == 2 * K * F, "nested slots need the MixDom shape");
    static constexpr int IS = (3 * F + 3) & ~3;   // intra row stride (floats)
    __host__ __device__ static constexpr int dom(int s) {
        return s < NM ? s / F : (s < NM + NI ? (s - NM) / (2 * F) : (s - NM - NI) / (2 * F));
    }
    __host__ __device__ static constexpr int uv(int s) {   // 0 MM, 1 MI, 2 MD, 3 II, 4 DD
        return s < NM ? 0 : (s < NM + NI ? (((s - NM) % (2 * F)) < F ? 1 : 3) : (((s - NM - NI) % (2 * F)) < F ? 2 : 4));
    }
    __host__ __device__ static constexpr int frag(int s) {
        return s < NM ? s % F : (s < NM + NI ? ((s - NM) % (2 * F)) % F : ((s - NM - NI) % (2 * F)) % F);
    }
    __host__ __device__ static constexpr int U(int s) { return uv(s) < 3 ? 0 : uv(s) - 2; }   // 0 M, 1 I, 2 D
    __host__ __device__ static constexpr int slot(int d, int u, int f) {
        return u == 0 ? d * F + f
                      : (u == 1 ? NM + d * 2 * F + f
                                : (u == 3 ? NM + d * 2 * F + F + f
                                          : (u == 2 ? NM + NI + d * 2 * F + f : NM + NI + d * 2 * F + F + f)));
    }
    __host__ __device__ static constexpr int n_intra(int s) { return uv(s) < 3 ? 3 * F : F; }
    // the j-th same-block partner of slot s (a source of destination s in the
    // forward, a destination of source s in the backward)
    __host__ __device__ static constexpr int partner(int s, int j) {
        return uv(s) < 3 ? slot(dom(s), j / F, j % F) : slot(dom(s), uv(s), j);
    }
    __host__ __device__ static constexpr int local(int s) { return uv(s) * F + frag(s); }   // index in the domain block
    __host__ __device__ static constexpr int body(int s) { return dom(s) * 5 * F + local(s); }   // state - 2
    // shared-memory region (floats): exit[SP], cin[3][KP], chi0[KP] (start -> k), intra rows [NE][IS]
    static constexpr int OX = 0, OC = SH::SP, O0 = OC + 3 * SH::KP, OI = O0 + SH::KP;
    static constexpr int FLOATS = OI + NE * IS;
};

// Load the factored coefficients of pair p (record in state order, see
// include/pairhmm.h phmm_batch.nest) into the slot-ordered shared region; one
// warp.  BWD: intra rows by source (partners = destinations), else by destination.
template <class SH, class NT, bool BWD>
__device__ void load_nest_tw(const KParams &P, int p, float *nz) {
    using NS = NestSlots<SH, NT>;
    constexpr int K = NT::K, F = NT::F, nb = 5 * K * F, bs = 5 * F;
    const int lane = threadIdx.x & 31;
    const float *rec = P.nest + (int64_t)p * P.nest_stride;
    const float *chi = P.chi + (int64_t)p * P.chi_stride;
    for (int s = lane; s < SH::SP; s += 32) nz[NS::OX + s] = s < NS::NE ? __ldg(rec + NS::body(s)) : 0.f;
    for (int idx = lane; idx < 3 * SH::KP; idx += 32) {
        const int a = idx / SH::KP, k = idx % SH::KP;
        nz[NS::OC + idx] = k < NS::NE ? __ldg(rec + nb + a * nb + NS::body(k)) : 0.f;
    }
    for (int k = lane; k < SH::KP; k += 32) nz[NS::O0 + k] = k < NS::NE ? __ldg(chi + P.w_orig[k]) : 0.f;
    for (int idx = lane; idx < NS::NE * NS::IS; idx += 32) {
        const int s = idx / NS::IS, j = idx % NS::IS;
        float v = 0.f;
        if (j < NS::n_intra(s)) {
            const int q = NS::partner(s, j);
            const int row = BWD ? NS::local(s) : NS::local(q), col = BWD ? NS::local(q) : NS::local(s);
            v = __ldg(rec + 4 * nb + NS::dom(s) * bs * bs + row * bs + col);
        }
        nz[NS::OI + idx] = v;
    }
}

// MK: the batch carries a cell mask (a separate instantiation, so the
// unmasked recursion carries none of the mask's instructions)
// NT: NoNest (dense chi) or Nest<K, F> (factored MixDom transitions, unmasked batches)
template <class SH, bool MK, class NT = NoNest>
__device__ void fwd_stripe_tw(const KParams &P, int p, int si, const SmemTW &LT, float *sm,
                              unsigned char *smb) {
    static_assert(NT::K == 0 || !MK, "the factored contraction runs on unmasked batches");
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

    if (r < 32) load_model_w<SH>(P, p, m, L, sm, smb, CHI_FWD_PAIRS);
    if constexpr (NT::K > 0) {
        if (r >= 32) load_nest_tw<SH, NT, false>(P, p, sm + LT.nest);
    }
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

    // state vectors as pairs of sources (s, s+1): the contraction runs on
    // paired FMAs (__ffma2_rn), even and odd sources in the two halves
    constexpr int SQ = SP / 2;
    float2 prev[SQ], d0[SQ], m0[SQ];
    int Eprev = EXP_NONE, Em0 = EXP_NONE;
    // factored contraction: the type sums G_a of the M- and I-predecessors
    // (carried from earlier steps: G(m0) is the previous step's G(d0))
    float Gm[3] = {0.f, 0.f, 0.f}, Gp[3] = {0.f, 0.f, 0.f}, Gd[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < SQ; ++q) {
        prev[q] = make_float2(0.f, 0.f); d0[q] = make_float2(0.f, 0.f); m0[q] = make_float2(0.f, 0.f);
    }
    const int T_last = (nrows - 1) + Ly;
    // under a cell mask: the steps that touch the stripe's live columns, and
    // the live columns of the row above (off them every value is zero, so the
    // other steps are skipped and the halo there reads as zero)
    int t_beg = 0, t_end = T_last, hlo = 0, hhi = Ly;
    if (MK) {
        const int2 rg = P.srange[m.stripe_base + si];
        t_beg = max(0, rg.x);
        t_end = min(T_last, rg.y + nrows - 1);
        if (si > 0) {
            const int2 ra = P.srange[m.stripe_base + si - 1];
            hlo = ra.x;
            hhi = min(Ly, ra.y);
        }
    }
    // M- and I-type emission factors of the cell of the next step, loaded one
    // step ahead (the y character and the table lookup are two dependent loads)
    // (and the cell's type mask: bit 0 M, 1 I, 2 D may emit; 7 without a mask)
    float eMI[NM + NI > 0 ? NM + NI : 1];
    int mbx = 7;
    const unsigned char *mrow = MK ? P.cmask + m.tab_base + (int64_t)rowi * (Ly + 1) : nullptr;
    auto load_emit = [&](int tt) {
        const int j = tt - r;
        const bool in = r < nrows && j >= 0 && j <= Ly;
        const int yj = in ? ys[j] : 0;
#pragma unroll
        for (int k = 0; k < NM; ++k) eMI[k] = sm[offM[k] + yj];
#pragma unroll
        for (int k = 0; k < NI; ++k) eMI[NM + k] = sm[offI[k] + yj];
        if (MK) mbx = in ? (int)__ldg(mrow + j) : 7;
    };
    load_emit(t_beg);
    bool aborted = false;
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (si > 0 && r == 0) pv = ld_acquire(prog_above);
    // a stripe that starts past step 0: row 0's first M predecessor is column
    // t_beg - 1 of the row above, which the skipped step t_beg - 1 would have
    // read -- load it into the history here
    if (MK && si > 0 && r == 0 && t_beg <= t_end && t_beg - 1 >= max(hlo, 0) && t_beg - 1 <= hhi) {
        const int col = t_beg - 1;
        if (!wait_geq(prog_above, col + 1, P.spin_limit)) {
            s_abort[t_beg & 1] = 1;   // seen by all threads after the first step's barrier
        } else {
            const float *src = edge_above + (int64_t)col * SP;
#pragma unroll
            for (int q = 0; q < SQ; ++q) m0[q] = make_float2(__ldcg(src + 2 * q), __ldcg(src + 2 * q + 1));
            Em0 = __ldcg(edgeE_above + col);
        }
    }

    for (int t = t_beg; t <= t_end; ++t) {
        // halo (row i0-1, column t) for thread 0: normally prefetched during
        // step t-1; zero off the live columns above (a cell mask)
        if (si > 0 && t <= Ly && r == 0 && hx_col != t) {
            if (MK && (t < hlo || t > hhi)) {
#pragma unroll
                for (int s = 0; s < SP; ++s) hx[s] = 0.f;
                hxE = EXP_NONE;
                hx_col = t;
            } else if (!wait_geq(prog_above, t + 1, P.spin_limit)) {
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
        for (int q = 0; q < SQ; ++q) {
            if (2 * q >= NSRC) continue;   // padding pairs stay zero
            const float vx = __shfl_up_sync(0xffffffffu, prev[q].x, 1);
            const float vy = __shfl_up_sync(0xffffffffu, prev[q].y, 1);
            d0[q].x = l0 ? (top ? (halo ? hx[2 * q] : 0.f) : bv[2 * q]) : vx;
            d0[q].y = l0 ? (top ? (halo ? hx[2 * q + 1] : 0.f) : bv[2 * q + 1]) : vy;
        }
        // a type that may not emit here contributes nothing (nor its exponent);
        // outside the lattice nothing emits, so the type scales below are zero
        // there and no separate select clears the cell
        const bool hasI = valid && jc >= 1 && (mbx & 2), hasD = valid && rowi >= 1 && (mbx & 4);
        const bool hasM = valid && jc >= 1 && rowi >= 1 && (mbx & 1);
        const int EI = hasI ? Eprev : EXP_NONE, ED = hasD ? EdA : EXP_NONE, EM = hasM ? Em0 : EXP_NONE;
        const int Eref = max(max(EI, ED), EM);
        float acc[NE];
        if constexpr (NT::K > 0) {
            using NS = NestSlots<SH, NT>;
            const float *nz = sm + LT.nest;
            const float4 *nx4 = reinterpret_cast<const float4 *>(nz + NS::OX);
            const float4 *nc4 = reinterpret_cast<const float4 *>(nz + NS::OC);
            const float4 *ni4 = reinterpret_cast<const float4 *>(nz + NS::OI);
            auto comp = [](const float4 &v, int u) { return u == 0 ? v.x : (u == 1 ? v.y : (u == 2 ? v.z : v.w)); };
            auto elem = [](const float2 (&v)[SQ], int s) { return (s & 1) ? v[s >> 1].y : v[s >> 1].x; };
            // G of the D-predecessor just received
            Gd[0] = Gd[1] = Gd[2] = 0.f;
#pragma unroll
            for (int s4 = 0; s4 < SP / 4; ++s4) {
                const float4 ex = nx4[s4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int s = 4 * s4 + u;
                    if (s < NE) Gd[NS::U(s)] = fmaf(comp(ex, u), elem(d0, s), Gd[NS::U(s)]);
                }
            }
#pragma unroll
            for (int k4 = 0; k4 < KP / 4; ++k4) {
                const float4 c0 = nc4[k4], c1 = nc4[KP / 4 + k4], c2 = nc4[2 * (KP / 4) + k4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = 4 * k4 + u;
                    if (k >= NE) continue;
                    const int ty = SH::type_of(k);
                    const float g0 = ty == T_M ? Gm[0] : (ty == T_I ? Gp[0] : Gd[0]);
                    const float g1 = ty == T_M ? Gm[1] : (ty == T_I ? Gp[1] : Gd[1]);
                    const float g2 = ty == T_M ? Gm[2] : (ty == T_I ? Gp[2] : Gd[2]);
                    float a = comp(c0, u) * g0;
                    a = fmaf(comp(c1, u), g1, a);
                    a = fmaf(comp(c2, u), g2, a);
#pragma unroll
                    for (int j4 = 0; j4 < NS::IS / 4; ++j4) {
                        const float4 cv = ni4[k * (NS::IS / 4) + j4];
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            const int j = 4 * j4 + v;
                            if (j < NS::n_intra(k)) {
                                const int sj = NS::partner(k, j);
                                const float pv = ty == T_M ? elem(m0, sj) : (ty == T_I ? elem(prev, sj) : elem(d0, sj));
                                a = fmaf(comp(cv, v), pv, a);
                            }
                        }
                    }
                    acc[k] = a;
                }
            }
            // the start state is non-zero only at the origin: the cells next to it
            const float stm = elem(m0, NE), stp = elem(prev, NE), std_ = elem(d0, NE);
            if (__any_sync(0xffffffffu, stm != 0.f || stp != 0.f || std_ != 0.f)) {
#pragma unroll
                for (int k = 0; k < NE; ++k) {
                    const int ty = SH::type_of(k);
                    acc[k] = fmaf(nz[NS::O0 + k], ty == T_M ? stm : (ty == T_I ? stp : std_), acc[k]);
                }
            }
        } else {
            float2 acc2[NE];
#pragma unroll
            for (int k = 0; k < NE; ++k) acc2[k] = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < SQ; ++q) {
                if (2 * q >= NSRC) continue;
                const float4 *row = chi4 + q * (KP / 2);   // sources 2q, 2q+1 for all destinations
#pragma unroll
                for (int kp = 0; kp < KP / 2; ++kp) {
                    const float4 cv = row[kp];             // (k, k+1) x (2q, 2q+1)
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int k = 2 * kp + u;
                        if (k < NE) {
                            const int ty = SH::type_of(k);
                            const float2 pk = ty == T_M ? m0[q] : (ty == T_I ? prev[q] : d0[q]);
                            acc2[k] = __ffma2_rn(pk, u == 0 ? make_float2(cv.x, cv.y) : make_float2(cv.z, cv.w),
                                                 acc2[k]);
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < NE; ++k) acc[k] = acc2[k].x + acc2[k].y;
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
                acc[k] = acc[k] * e;
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
        if (valid && rowi == 0 && jc == 0 && mbx != 0) { sNew = 1.f; Enew = 0; }
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
                if (((jc + 1) % PUB) == 0 || jc == t_end - (ROWS - 1)) st_release(prog_mine, jc + 1);
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
        for (int q = 0; q < SQ; ++q) {
            m0[q] = d0[q];
            const int s0 = 2 * q, s1 = 2 * q + 1;
            prev[q].x = s0 < NE ? acc[s0] : (s0 == NE ? sNew : 0.f);
            prev[q].y = s1 < NE ? acc[s1] : (s1 == NE ? sNew : 0.f);
        }
        if constexpr (NT::K > 0) {   // G of the new cell (the next step's I-predecessor)
            using NS = NestSlots<SH, NT>;
            const float *nz = sm + LT.nest;
            float g[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int s = 0; s < NE; ++s) g[NS::U(s)] = fmaf(nz[NS::OX + s], acc[s], g[NS::U(s)]);
#pragma unroll
            for (int a = 0; a < 3; ++a) { Gm[a] = Gd[a]; Gp[a] = g[a]; }
        }
        Em0 = EdA;
        Eprev = Enew;
        // row 31 hands its new state to row 32 for step t+1
        if (r == 31) {
            float2 *b2 = reinterpret_cast<float2 *>(bnd + (t & 1) * SP);
#pragma unroll
            for (int q = 0; q < SQ; ++q) b2[q] = prev[q];
            bndE[t & 1] = Eprev;
        }
        load_emit(t + 1);
        // prefetch halo column t+1 when the progress read last step covers it
        // (its loads then overlap the barrier), and poll for the column after
        if (si > 0 && r == 0 && t + 1 <= Ly) {
            if (MK && (t + 1 < hlo || t + 1 > hhi)) {
#pragma unroll
                for (int s = 0; s < SP; ++s) hx[s] = 0.f;
                hxE = EXP_NONE;
                hx_col = t + 1;
            } else if (pv > t + 1) {
                const float4 *src = reinterpret_cast<const float4 *>(edge_above + (int64_t)(t + 1) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    const float4 v = __ldcg(src + q);
                    hx[4 * q] = v.x; hx[4 * q + 1] = v.y; hx[4 * q + 2] = v.z; hx[4 * q + 3] = v.w;
                }
                hxE = __ldcg(edgeE_above + t + 1);
                hx_col = t + 1;
            }
            if (t + 2 <= hhi && pv <= t + 2) pv = ld_acquire(prog_above);
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

template <class SH, bool MK, class NT = NoNest>
__device__ void bwd_rec_stripe_tw(const KParams &P, int p, int si, const SmemTW &LT, float *sm,
                                  unsigned char *smb) {
    static_assert(NT::K == 0 || !MK, "the factored contraction runs on unmasked batches");
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, KP = SH::KP, NM = SH::NM, NI = SH::NI;
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

    if (r < 32) load_model_w<SH>(P, p, m, L, sm, smb, CHI_BWD_PAIRS);
    if constexpr (NT::K > 0) {
        if (r >= 32) load_nest_tw<SH, NT, true>(P, p, sm + LT.nest);
    }
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
    // (as pairs of destinations (k, k+1): the contraction runs on paired FMAs)
    constexpr int KQ = KP / 2;
    float2 wn[KQ], dR[KQ], mR[KQ];
    int Ewn = EXP_NONE, EmR = EXP_NONE;
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
        wn[q] = make_float2(0.f, 0.f); dR[q] = make_float2(0.f, 0.f); mR[q] = make_float2(0.f, 0.f);
    }

    const int T_last = (nrows - 1) + Ly;
    // under a cell mask: the steps that touch the stripe's live columns, and
    // the live columns of the row below (as in the forward)
    int t_beg = 0, t_end = T_last, hlo = 0, hhi = Ly;
    if (MK) {
        const int2 rg = P.srange[m.stripe_base + si];
        t_beg = max(0, rg.x);
        t_end = min(T_last, rg.y + nrows - 1);
        if (has_below) {
            const int2 rb = P.srange[m.stripe_base + si + 1];
            hlo = rb.x;
            hhi = min(Ly, rb.y);
        }
    }
    // M- and I-type emission factors of the cell of the next step, loaded one step ahead
    // (and the cell's type mask, as in the forward, folded into the factors
    // here, off the step's dependency chain: eDc is eD with the D bit applied)
    float eMI[NM + NI > 0 ? NM + NI : 1];
    float eDc[SH::ND > 0 ? SH::ND : 1];
    int mbx = 7;
    const unsigned char *mrow = MK ? P.cmask + m.tab_base + (int64_t)rowi * (Ly + 1) : nullptr;
    auto load_emit = [&](int tt) {
        const int j = tt - r;
        const bool in = r < nrows && j >= 0 && j <= Ly;
        const int yj = in ? ys[j] : 0;
        if (MK) mbx = in ? (int)__ldg(mrow + j) : 7;
        const float bM = (mbx & 1) ? 1.f : 0.f, bI = (mbx & 2) ? 1.f : 0.f, bD = (mbx & 4) ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < NM; ++k) eMI[k] = sm[offM[k] + yj] * bM;
#pragma unroll
        for (int k = 0; k < NI; ++k) eMI[NM + k] = sm[offI[k] + yj] * bI;
#pragma unroll
        for (int k = 0; k < SH::ND; ++k) eDc[k] = eD[k] * bD;
    };
    load_emit(t_end);
    bool aborted = false;
    float hx[SP];
#pragma unroll
    for (int s = 0; s < SP; ++s) hx[s] = 0.f;
    int hxE = EXP_NONE, hx_col = -1, pv = 0;
    if (has_below && r == ROWS - 1) pv = ld_acquire(prog_below);
    // a stripe that ends before its last step: row 63's first M successor is
    // column jb + 1 of the row below (jb = t_end - 63), which the skipped step
    // t_end + 1 would have received -- load it into the history here
    if (MK && has_below && r == ROWS - 1 && t_beg <= t_end) {
        const int col = t_end - (ROWS - 1) + 1;
        if (col >= max(hlo, 0) && col <= hhi) {
            if (!wait_geq(prog_below, Ly + 1 - col, P.spin_limit)) {
                s_abort[t_end & 1] = 1;   // seen by all threads after the first step's barrier
            } else {
                const float *src = edge_below + (int64_t)col * SP;
#pragma unroll
                for (int q = 0; q < KQ; ++q) {
                    if (2 * q >= NE) continue;
                    mR[q] = make_float2(__ldcg(src + 2 * q), __ldcg(src + 2 * q + 1));
                }
                EmR = __ldcg(edgeE_below + col);
            }
        }
    }

    for (int t = t_end; t >= t_beg; --t) {
        const int jb = t - (ROWS - 1);
        // halo (row i0+64, column jb) for thread 63: normally prefetched during
        // step t+1; zero off the live columns below (a cell mask)
        if (has_below && jb >= 0 && jb <= Ly && r == ROWS - 1 && hx_col != jb) {
            if (MK && (jb < hlo || jb > hhi)) {
#pragma unroll
                for (int s = 0; s < SP; ++s) hx[s] = 0.f;
                hxE = EXP_NONE;
                hx_col = jb;
            } else if (!wait_geq(prog_below, Ly + 1 - jb, P.spin_limit)) {
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
        for (int q = 0; q < KQ; ++q) {
            if (2 * q >= NE) continue;   // padding pairs stay zero
            const float vx = __shfl_down_sync(0xffffffffu, wn[q].x, 1);
            const float vy = __shfl_down_sync(0xffffffffu, wn[q].y, 1);
            dR[q].x = l31 ? (bottom ? (halo ? hx[2 * q] : 0.f) : bv[2 * q]) : vx;
            dR[q].y = l31 ? (bottom ? (halo ? hx[2 * q + 1] : 0.f) : bv[2 * q + 1]) : vy;
        }
        const bool term = valid && rowi == Lx && jc == Ly;
        const bool hI = jc + 1 <= Ly, hD = rowi + 1 <= Lx, hM = hI && hD;
        const int EI = hI ? Ewn : EXP_NONE, ED = hD ? EdRn : EXP_NONE, EM = hM ? EmR : EXP_NONE;
        const int Eref = term ? 0 : max(max(EI, ED), EM);
        const float sM = (hM && !term) ? pow2f(EM - Eref) : 0.f, sI = (hI && !term) ? pow2f(EI - Eref) : 0.f;
        const float sD = (hD && !term) ? pow2f(ED - Eref) : 0.f;
        // successor weights w_k, paired (k, k+1)
        float2 w2[KQ];
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
            float wv[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int k = 2 * q + u;
                float w = 0.f;
                if (k < NE) {
                    const int ty = SH::type_of(k);
                    const float vm = u ? mR[q].y : mR[q].x, vi = u ? wn[q].y : wn[q].x, vd = u ? dR[q].y : dR[q].x;
                    w = ty == T_M ? vm * sM : (ty == T_I ? vi * sI : vd * sD);
                }
                wv[u] = w;
            }
            w2[q] = make_float2(wv[0], wv[1]);
        }
        float acc[NSRC];
        if constexpr (NT::K > 0) {
            using NS = NestSlots<SH, NT>;
            const float *nz = sm + LT.nest;
            const float4 *nx4 = reinterpret_cast<const float4 *>(nz + NS::OX);
            const float4 *nc4 = reinterpret_cast<const float4 *>(nz + NS::OC);
            const float4 *ni4 = reinterpret_cast<const float4 *>(nz + NS::OI);
            auto comp = [](const float4 &v, int u) { return u == 0 ? v.x : (u == 1 ? v.y : (u == 2 ? v.z : v.w)); };
            auto wv = [&](int k) { return (k & 1) ? w2[k >> 1].y : w2[k >> 1].x; };
            // the type sums over destinations, Gb_a = sum_k cin[a][k] w_k
            float Gb[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int k4 = 0; k4 < KP / 4; ++k4) {
                const float4 c0 = nc4[k4], c1 = nc4[KP / 4 + k4], c2 = nc4[2 * (KP / 4) + k4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = 4 * k4 + u;
                    if (k >= NE) continue;
                    Gb[0] = fmaf(comp(c0, u), wv(k), Gb[0]);
                    Gb[1] = fmaf(comp(c1, u), wv(k), Gb[1]);
                    Gb[2] = fmaf(comp(c2, u), wv(k), Gb[2]);
                }
            }
#pragma unroll
            for (int s4 = 0; s4 < SP / 4; ++s4) {
                const float4 ex = nx4[s4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int sidx = 4 * s4 + u;
                    if (sidx >= NE) continue;
                    float a = comp(ex, u) * Gb[NS::U(sidx)];
#pragma unroll
                    for (int j4 = 0; j4 < NS::IS / 4; ++j4) {
                        const float4 cv = ni4[sidx * (NS::IS / 4) + j4];
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            const int j = 4 * j4 + v;
                            if (j < NS::n_intra(sidx)) a = fmaf(comp(cv, v), wv(NS::partner(sidx, j)), a);
                        }
                    }
                    acc[sidx] = a;
                }
            }
            // the start state's backward value matters only at the origin
            acc[NE] = 0.f;
            const bool origin = valid && rowi == 0 && jc == 0;
            if (__any_sync(0xffffffffu, origin)) {
                float a = 0.f;
#pragma unroll
                for (int k = 0; k < NE; ++k) a = fmaf(nz[NS::O0 + k], wv(k), a);
                if (origin) acc[NE] = a;
            }
        } else {
            float2 acc2[NSRC];
#pragma unroll
            for (int s2 = 0; s2 < NSRC; ++s2) acc2[s2] = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < KQ; ++q) {
                if (2 * q >= NE) continue;
                const float4 *row = chiB4 + q * (SP / 2);   // destinations 2q, 2q+1 for all sources
#pragma unroll
                for (int sp = 0; sp < SP / 2; ++sp) {
                    const float4 cv = row[sp];             // (2q, 2q+1) x (s, s+1)
                    if (2 * sp < NSRC) acc2[2 * sp] = __ffma2_rn(w2[q], make_float2(cv.x, cv.y), acc2[2 * sp]);
                    if (2 * sp + 1 < NSRC)
                        acc2[2 * sp + 1] = __ffma2_rn(w2[q], make_float2(cv.z, cv.w), acc2[2 * sp + 1]);
                }
            }
#pragma unroll
            for (int s2 = 0; s2 < NSRC; ++s2) acc[s2] = acc2[s2].x + acc2[s2].y;
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
            // a type that may not emit here gets w = e b = 0 (its factor is 0)
            // and a stored b of 0, so neither its predecessors nor the count
            // pass see it
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                const int ty = SH::type_of(k);
                const float ev = (ty == T_M || ty == T_I) ? eMI[k] : eDc[k - NM - NI];
                wnew[k] = acc[k] * ev;
            }
            if (MK && mbx != 7) {
#pragma unroll
                for (int k = 0; k < NE; ++k) {
                    const int ty = SH::type_of(k);
                    const int bit = ty == T_M ? 1 : (ty == T_I ? 2 : 4);
                    if (!(mbx & bit)) acc[k] = 0.f;
                }
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
                if ((jc % PUB) == 0 || jc == t_beg) st_release(prog_mine, Ly + 1 - jc);
            }
        }
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
            mR[q] = dR[q];
            const int k0 = 2 * q, k1 = 2 * q + 1;
            wn[q].x = (valid && k0 < NE) ? wnew[k0] : 0.f;
            wn[q].y = (valid && k1 < NE) ? wnew[k1] : 0.f;
        }
        EmR = EdRn;
        Ewn = (valid && mbx != 0) ? Eb : EXP_NONE;
        // row 32 hands its new state to row 31 for step t-1
        if (r == 32) {
            float2 *b2 = reinterpret_cast<float2 *>(bnd + (t & 1) * SP);
#pragma unroll
            for (int q = 0; q < KQ; ++q) b2[q] = wn[q];
#pragma unroll
            for (int q = KQ; q < SP / 2; ++q) b2[q] = make_float2(0.f, 0.f);
            bndE[t & 1] = Ewn;
        }
        load_emit(t - 1);
        // prefetch halo column jb-1 when the progress read last step covers it,
        // and poll for the column after
        if (has_below && r == ROWS - 1 && jb - 1 >= 0 && jb - 1 <= Ly) {
            if (MK && (jb - 1 < hlo || jb - 1 > hhi)) {
#pragma unroll
                for (int s = 0; s < SP; ++s) hx[s] = 0.f;
                hxE = EXP_NONE;
                hx_col = jb - 1;
            } else if (pv >= Ly + 1 - (jb - 1)) {
                const float4 *src = reinterpret_cast<const float4 *>(edge_below + (int64_t)(jb - 1) * SP);
#pragma unroll
                for (int q = 0; q < SP / 4; ++q) {
                    const float4 v = __ldcg(src + q);
                    hx[4 * q] = v.x; hx[4 * q + 1] = v.y; hx[4 * q + 2] = v.z; hx[4 * q + 3] = v.w;
                }
                hxE = __ldcg(edgeE_below + jb - 1);
                hx_col = jb - 1;
            }
            if (jb - 2 >= hlo && pv < Ly + 3 - jb) pv = ld_acquire(prog_below);
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
template <class SH, bool BWD, bool MK, class NT = NoNest>
__global__ void __launch_bounds__(TWT) stripe_tw_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    int nest_floats = 0;
    if constexpr (NT::K > 0) nest_floats = NestSlots<SH, NT>::FLOATS;
    const SmemTW L = make_smem_tw(SH::SP, SH::KP, SH::NI, P.G, P.max_ly, BWD, nest_floats);
    int *s_item = reinterpret_cast<int *>(sm) + L.flag + 2;
    for (;;) {
        if (threadIdx.x == 0) *s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = *s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        if (BWD) bwd_rec_stripe_tw<SH, MK, NT>(P, w.x, w.y, L, sm, smem_raw);
        else fwd_stripe_tw<SH, MK, NT>(P, w.x, w.y, L, sm, smem_raw);
    }
}

}  // namespace warp2

// ---------------------------------------------------------------- two-warp count pass
// count_chunk_w with one row per thread: a 64-thread CTA takes a chunk of CCH
// anti-diagonal steps of one stripe, both warps sharing the model tables and
// the double-buffered lattice rows.  Row r's D- and M-successors come from row
// r+1 by __shfl_down inside a warp, through a shared slot across the two warps
// (row 32 -> row 31) and from the stripe below for row 63.  The outer products
// run over 64 threads: thread (group, block) owns a 4 x 4 tile of (source,
// destination) for ROWS / groups rows.
namespace warp2 {

struct SmemCT {
    SmemC c;
    int slot;    // float offset: [2][SP] w~ of row 32 at the previous step
    int slotE;   // int offset: [2]
    int item;    // int offset: popped item
    int bytes;
};

__host__ __device__ inline SmemCT make_smem_ct(int SP, int KP, int NI, int G, int max_ly) {
    SmemCT L;
    L.c = make_smem_c(SP, KP, NI, G, max_ly);
    int o = L.c.bytes / 4;
    L.slot = o; o += 2 * SP;
    L.slotE = o; o += 4;
    L.item = o; o += 4;
    L.bytes = o * 4;
    return L;
}

// MK: a cell-masked batch (the stripes' live step ranges in P.srange)
template <class SH, bool MK>
__device__ void count_chunk_tw(const KParams &P, int p, int si, int ch, const SmemCT &LT, float *sm,
                               unsigned char *smb) {
    constexpr int NE = SH::NE, NSRC = SH::NSRC, SP = SH::SP, KP = SH::KP, NM = SH::NM, NI = SH::NI;
    constexpr int ND = SH::ND, SPP = SH::SPP, KPP = SH::KPP;
    constexpr int GROUPS64 = TWT / SH::NBLK;   // outer-product row groups over 64 threads
    const SmemC &L = LT.c;
    const PairMeta m = P.meta[p];
    const int N = P.N, G = P.G;
    const int Lx = m.Lx, Ly = m.Ly;
    const int r = threadIdx.x, lane = r & 31;
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;
    const int64_t latb = m.lat_base + (int64_t)(si + 1) * (ROWS + Ly) * ROWS;   // stripe below (row 0)
    const int T_last = (nrows - 1) + Ly;
    // under a cell mask the recursions visited only the steps [t_beg, t_last]
    // of this stripe and columns [blo, bhi] of the first row below: the count
    // covers those steps of the chunk and reads the rest as zero
    int t_beg = 0, t_last = T_last, blo = 0, bhi = Ly;
    if (MK) {
        const int2 rg = P.srange[m.stripe_base + si];
        t_beg = max(0, rg.x);
        t_last = min(T_last, rg.y + nrows - 1);
        if (has_below) {
            const int2 rb = P.srange[m.stripe_base + si + 1];
            blo = rb.x;
            bhi = min(Ly, rb.y);
        }
    }
    const int t0 = ch * CCH;
    const int t_hi = min(t_last, t0 + CCH - 1);
    const int t_lo = max(t0, t_beg);
    const int t_top = min(T_last, t_hi + 2);   // two steps of successor history first
    if (t_lo > t_hi) return;                    // uniform over the CTA
    int *s_flag = reinterpret_cast<int *>(sm) + LT.slotE + 2;
    if (P.count_wait) {   // the wavefronts may still run: wait for the stripes read here
        if (r == 0) *s_flag = count_ready(P, m, si) ? 1 : 0;
        __syncthreads();
        const int ok = *s_flag;
        __syncthreads();
        if (!ok) {
            if (r == 0) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            return;
        }
    }
    const double llv = __ldcg(P.ll + p);
    if (!(llv > -1e29)) return;   // uniform over the CTA
    const double lam = llv / LN2;
    const double Epd = floor(lam);
    const int Ep = (int)Epd;
    const float rfrac = (float)exp2(-(lam - Epd));
    float *fbuf = sm + L.fbuf, *bbuf = sm + L.bbuf, *ust = sm + L.ust, *bins = sm + L.bins, *colI = sm + L.colI;
    int *fEb = reinterpret_cast<int *>(sm) + L.fE;
    int *bEb = reinterpret_cast<int *>(sm) + L.bE;
    float *slot = sm + LT.slot;
    int *slotE = reinterpret_cast<int *>(sm) + LT.slotE;
    auto prefetch = [&](int t) {
        if (t >= t_lo) {
            const int buf = t & 1;
            if (MK && t > t_last) {   // successor history past the live steps: b~ = 0
                for (int idx = r; idx < ROWS * SPP; idx += TWT) bbuf[buf * ROWS * SPP + idx] = 0.f;
                bEb[buf * ROWS + r] = EXP_NONE;
            } else {
                const float *srcF = P.lat + (latc + (int64_t)t * ROWS) * SP;
                const float *srcB = P.blat + (latc + (int64_t)t * ROWS) * SP;
                for (int idx = r; idx < ROWS * SP / 4; idx += TWT) {
                    const int rr = idx / (SP / 4), q = idx % (SP / 4);
                    if (t <= t_hi) cp_async16(fbuf + buf * ROWS * SPP + rr * SPP + 4 * q, srcF + 4 * idx);
                    cp_async16(bbuf + buf * ROWS * SPP + rr * SPP + 4 * q, srcB + 4 * idx);
                }
                if (r < ROWS / 4) {
                    if (t <= t_hi)
                        cp_async16(fEb + buf * ROWS + 4 * r, P.lat_exp + latc + (int64_t)t * ROWS + 4 * r);
                    cp_async16(bEb + buf * ROWS + 4 * r, P.blat_exp + latc + (int64_t)t * ROWS + 4 * r);
                }
            }
        }
        cp_commit();
    };
    prefetch(t_top);
    // ---- tables, y characters of the chunk's columns, zeroed bins and slots
    {
        const float *eM = P.eM + (int64_t)p * P.eM_stride;
        const float *eI = P.eI + (int64_t)p * P.eID_stride;
        const float *eDg = P.eD + (int64_t)p * P.eID_stride;
        for (int idx = r; idx < G * 441; idx += TWT) sm[L.tM + idx] = __ldg(eM + idx);
        for (int idx = r; idx < G * 21; idx += TWT) {
            sm[L.tI + idx] = __ldg(eI + idx);
            sm[L.tD + idx] = __ldg(eDg + idx);
            sm[L.bins + idx] = 0.f;
        }
        unsigned char *ysw = smb + L.ys;
        const int jlo = max(0, t0 - (ROWS - 1)), jhi = min(Ly, t_hi + 3);
        for (int j = jlo + r; j <= jhi; j += TWT) {
            int c = 0;
            if (j >= 1) c = min((int)P.res[m.y_off + j - 1], 20);
            ysw[j] = (unsigned char)c;
        }
        for (int idx = r; idx < ROWS * (NI > 0 ? NI : 1); idx += TWT) colI[idx] = 0.f;
        if (r < 2 * SP) slot[r] = 0.f;
        if (r < 2) slotE[r] = EXP_NONE;
        __syncthreads();
    }
    const unsigned char *ys = smb + L.ys;

    const int rowi = i0 + r;
    const int xch = row_char(P, p, m, rowi);
    float eD[ND > 0 ? ND : 1];
    int offM[NM > 0 ? NM : 1];
#pragma unroll
    for (int k = 0; k < NM; ++k) offM[k] = L.tM + P.w_group[k] * 441 + xch * 21;
#pragma unroll
    for (int k = 0; k < ND; ++k) eD[k] = sm[L.tD + P.w_group[NM + NI + k] * 21 + xch];
    int offI[NI > 0 ? NI : 1];
#pragma unroll
    for (int k = 0; k < NI; ++k) offI[k] = L.tI + P.w_group[NM + k] * 21;
    // the first row of the stripe below (row 63's D / M successors)
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

    float dcnt[ND > 0 ? ND : 1], dcmp[ND > 0 ? ND : 1];
#pragma unroll
    for (int k = 0; k < ND; ++k) { dcnt[k] = 0.f; dcmp[k] = 0.f; }
    const int blk = r % SH::NBLK, grp = r / SH::NBLK;
    const bool counter = grp < GROUPS64;
    const int bs = blk / SH::BK, bk = blk % SH::BK;
    float csum[16], ccomp[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) { csum[u] = 0.f; ccomp[u] = 0.f; }

    // successor histories: w~ of my cell at t+1 (wn) and the D-successor seen
    // at step t+1 (dR), which is my M-successor at step t
    float wn[NE], dR[NE];
    int Ewn = EXP_NONE, EdR = EXP_NONE;
#pragma unroll
    for (int k = 0; k < NE; ++k) { wn[k] = 0.f; dR[k] = 0.f; }
    // row 63: b~ of row i0+64 at column (t - 63), loaded one step ahead
    float bbv[SP];
    int bbE = EXP_NONE;
    auto load_below = [&](int t) {
        const int jb = t - (ROWS - 1);
        bbE = EXP_NONE;
        if (r == ROWS - 1 && has_below && t >= t_lo && jb >= blo && jb <= bhi) {
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

    for (int t = t_top; t >= t_lo; --t) {
        const bool count = t <= t_hi;
        const int buf = t & 1;
        // step t's rows have landed (this thread's copies, then everyone's),
        // and every thread is done with step t+1, whose buffer takes step t-1
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
        prefetch(t - 1);
        const int jc = t - r;
        const bool valid = r < nrows && jc >= 0 && jc <= Ly;
        // ---- b~ and w~ = e b~ of my cell at step t
        float wcur[NE];
        const int Eb0 = valid ? bEb[buf * ROWS + r] : EXP_NONE;
        const int Eb = Eb0 > EXP_NONE ? Eb0 : EXP_NONE;
        const int yj = valid ? ys[jc] : 0;
        const float *br = bbuf + buf * ROWS * SPP + r * SPP;
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const int ty = SH::type_of(k);
            float ev;
            if (ty == T_M) ev = sm[offM[k] + yj];
            else if (ty == T_I) ev = sm[offI[k - NM] + yj];
            else ev = eD[k - NM - NI];
            wcur[k] = Eb > EXP_NONE ? br[k] * ev : 0.f;
        }
        // D-successor (row r+1, column jc) = row r+1's w~ at step t+1: a shuffle
        // inside a warp, the slot written by row 32 for row 31, the stripe
        // below for row 63
        float dnew[NE];
        int Ednew = __shfl_down_sync(0xffffffffu, Ewn, 1);
#pragma unroll
        for (int k = 0; k < NE; ++k) dnew[k] = __shfl_down_sync(0xffffffffu, wn[k], 1);
        if (r == 31) {
            const int sb = (t + 1) & 1;
#pragma unroll
            for (int k = 0; k < NE; ++k) dnew[k] = slot[sb * SP + k];
            Ednew = slotE[sb];
        } else if (r == ROWS - 1) {
            const bool okb = has_below && jc >= 0 && jc <= Ly && bbE > EXP_NONE;
            const int yb = okb ? ys[jc] : 0;
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
            const bool term = valid && rowi == Lx && jc == Ly;
            const bool hI = jc + 1 <= Ly, hD = rowi + 1 <= Lx, hM = hI && hD;
            // successor exponents by type: I = mine at t+1, D = dnew, M = dR
            const int EI = (hI && !term) ? Ewn : EXP_NONE, ED = (hD && !term) ? Ednew : EXP_NONE;
            const int EM = (hM && !term) ? EdR : EXP_NONE;
            const int Ef = valid ? fEb[buf * ROWS + r] : EXP_NONE;
            float fsc = 0.f;
            if (valid && Ef > EXP_NONE && Eb > EXP_NONE) {
                int d = Ef + Eb - Ep;
                if (d > 126) { d = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                fsc = scale_pow2(rfrac, max(d, -200));
            }
            // f~ scaled in place (the outer products read it from the buffer)
            float *fr = fbuf + buf * ROWS * SPP + r * SPP;
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
            const bool live = fsc > 0.f;
            const float uM = (live && EM > EXP_NONE) ? fminf(scale_pow2(1.f, EM - Eb), 3e38f) : 0.f;
            const float uI = (live && EI > EXP_NONE) ? fminf(scale_pow2(1.f, EI - Eb), 3e38f) : 0.f;
            const float uD = (live && ED > EXP_NONE) ? fminf(scale_pow2(1.f, ED - Eb), 3e38f) : 0.f;
#pragma unroll
            for (int q = 0; q < KP / 4; ++q) {
                float uq[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int k = 4 * q + v;
                    float u = 0.f;
                    if (k < NE) {
                        const int ty = SH::type_of(k);
                        u = ty == T_M ? dR[k] * uM : (ty == T_I ? wn[k] * uI : dnew[k] * uD);
                    }
                    uq[v] = u;
                }
                reinterpret_cast<float4 *>(ust + r * KPP)[q] = make_float4(uq[0], uq[1], uq[2], uq[3]);
            }
            if (live) {
#pragma unroll
                for (int k = 0; k < NE; ++k) {
                    const float pk = ft[k] * br[k];
                    const int ty = SH::type_of(k);
                    if (ty == T_M) {
                        if (pk != 0.f) atomicAdd(cntM_pair + P.w_group[k] * 441 + xch * 21 + yj, (double)pk);
                    } else if (ty == T_I) {
                        colI[(jc % ROWS) * NI + (k - NM)] += pk;
                    } else {
                        const int kd = k - NM - NI;
                        const float y = pk - dcmp[kd];
                        const float tt = dcnt[kd] + y;
                        dcmp[kd] = (tt - dcnt[kd]) - y;
                        dcnt[kd] = tt;
                    }
                }
                if (term) {   // expected End transitions
#pragma unroll
                    for (int s = 0; s < NSRC; ++s)
                        atomicAdd(P.n_trans + ((int64_t)p * N + P.w_orig[s]) * N + P.e_idx, (double)(ft[s] * br[s]));
                }
            }
        }
        // row 32 hands its w~ at step t to row 31 for step t-1 (read after the
        // next step's first barrier; the other parity is being read now)
        if (r == 32) {
#pragma unroll
            for (int k = 0; k < NE; ++k) slot[(t & 1) * SP + k] = wcur[k];
            slotE[t & 1] = Eb;
        }
        __syncthreads();   // ust, the scaled f~ rows and colI complete for step t
        if (count) {
            // column t is complete once row i0 (thread 0) has visited it
            if (r == 0 && t <= Ly) {
                const int sl = t % ROWS;
                const int yt = ys[t];
#pragma unroll
                for (int k = 0; k < NI; ++k) {
                    bins[P.w_group[NM + k] * 21 + yt] += colI[sl * NI + k];
                    colI[sl * NI + k] = 0.f;
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
                if constexpr (ROWS % GROUPS64 == 0) {
                    constexpr int RPG = ROWS / GROUPS64;
                    const int r0 = grp * RPG;
#pragma unroll 4
                    for (int rr = r0; rr < r0 + RPG; ++rr) row_outer(rr);
                } else {
                    const int r0 = grp * ROWS / GROUPS64, r1 = (grp + 1) * ROWS / GROUPS64;
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
        // ---- shift histories
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            dR[k] = dnew[k];
            wn[k] = wcur[k];
        }
        EdR = Ednew;
        Ewn = Eb;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    // ---- flush the chunk's partial counts (float64 reductions)
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
    if (r < nrows && rowi >= 1) {
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            const float v = dcnt[k] - dcmp[k];
            if (v != 0.f) atomicAdd(P.cntD + ((int64_t)p * G + P.w_group[NM + NI + k]) * 21 + xch, (double)v);
        }
    }
    // I-type columns not completed inside the chunk (touched by rows below row 0)
    for (int j = max(0, t_lo - (ROWS - 1)) + r; j <= min(Ly, t_lo - 1); j += TWT) {
        const int sl = j % ROWS;
        const int yt = ys[j];
#pragma unroll
        for (int k = 0; k < NI; ++k) {
            const float v = colI[sl * NI + k];
            if (v != 0.f) atomicAdd(P.cntI + ((int64_t)p * G + P.w_group[NM + k]) * 21 + yt, (double)v);
        }
    }
    for (int idx = r; idx < G * 21; idx += TWT) {
        const float v = bins[idx];
        if (v != 0.f) atomicAdd(P.cntI + (int64_t)p * G * 21 + idx, (double)v);
    }
    __syncthreads();
}

template <class SH, bool MK>
__global__ void __launch_bounds__(TWT) count_tw_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemCT L = make_smem_ct(SH::SP, SH::KP, SH::NI, P.G, P.max_ly);
    int *s_item = reinterpret_cast<int *>(sm) + L.item;
    for (;;) {
        if (threadIdx.x == 0) *s_item = count_claim(P);
        __syncthreads();
        const int it = *s_item;
        __syncthreads();
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        count_chunk_tw<SH, MK>(P, w.x, w.y >> 12, w.y & 4095, L, sm, smem_raw);
    }
}

}  // namespace warp2
