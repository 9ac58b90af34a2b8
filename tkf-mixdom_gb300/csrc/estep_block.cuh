// estep_block.cuh -- quad-per-warp, latency-oriented E-step kernels (included
// by pairhmm.cu after the generic kernels).
//
// The critical path of a batch is the longest pair: Lx+Ly anti-diagonal
// steps that cannot overlap.  These kernels spread one step of a 64-row
// stripe over NB = NS/4 warps (one warp per 4-state "quad" of the padded
// state vector; states are grouped by type so a quad has one type), so a
// step costs about one quad's work:
//   * lane L owns rows 2L, 2L+1 of the stripe; warp q owns states 4q..4q+3;
//   * the transition block chi[:, 4q..4q+3] (forward) / chi[4q..4q+3, :]
//     (backward) stays in registers for the whole stripe;
//   * a warp reads only the predecessor (successor) vector of its own
//     quad's type from a 3-step shared-memory ring;
//   * every quad of every cell carries its own power-of-two exponent, so a
//     warp renormalises its own quad and no cross-warp max is needed: one
//     named barrier per step;
//   * the halo row of the neighbouring stripe is copied into shared memory
//     with cp.async one step ahead by one lane, from the release/acquire
//     edge-row pipeline shared with the other kernels.
// The backward kernel adds NC count warps that take the staged (b, u) of
// every step from a shared-memory ring (producer/consumer named barriers)
// and do the posteriors, emission counts and transition-count outer
// products off the critical path.

namespace blk {

constexpr int R = 2;
constexpr int ROWS = 64;
constexpr int PUBB = 4;            // edge progress published every PUBB columns
constexpr int KSTAGE = 3;          // count-ring depth (backward)
constexpr int BAR_STEP = 1;        // named barrier ids
constexpr int BAR_FULL0 = 2;       // 2..2+KSTAGE-1
constexpr int BAR_EMPTY0 = 2 + KSTAGE;

__device__ __forceinline__ void bar_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

template <int NS_>
struct BShape {
    static constexpr int NS = NS_;              // padded slots (multiple of 4)
    static constexpr int NB = NS / 4;           // quads == recursion warps
    // exponent row stride: a multiple of 4 that is 4 mod 8, so int4 rows of
    // consecutive lanes fall in distinct bank groups
    static constexpr int NBP = (((NB + 3) & ~3) % 8 == 0) ? ((NB + 3) & ~3) + 4 : ((NB + 3) & ~3);
    // value row stride: an odd number of float4 quads (conflict-free float4 rows)
    static constexpr int SPR = ((NS / 4) % 2 == 1) ? NS : NS + 4;
    static constexpr bool CHI_REG = NS <= 24;   // chi block in registers
};

struct SmemB {
    int chi, chiE, tM, tI, tD, ring, halo;        // float offsets
    int ringE, haloE, misc;                       // int offsets
    int zvec, zvecE;                              // an all-zero vector (float) and its exponents (int)
    int cst_b, cst_u, cst_bE, cst_uE, fst, fstE;  // backward count ring (float / int offsets)
    int colI, binsI;                              // backward emission-count scratch
    int ys;                                       // byte offset
    int bytes;
};

__host__ __device__ inline int nbp_of(int NB) {
    const int a = (NB + 3) & ~3;
    return (a % 8 == 0) ? a + 4 : a;
}
__host__ __device__ inline int spr_of(int NS) { return ((NS / 4) % 2 == 1) ? NS : NS + 4; }

__host__ __device__ inline SmemB make_smem_b(int NS, int NB, int NI, int G, int max_ly, bool bwd) {
    const int NBP = nbp_of(NB), SPR = spr_of(NS);
    SmemB L;
    int o = 0;
    L.chi = o; o += NS * NS;
    L.chiE = o; o += NS;
    L.tM = o; o += al4(G * 441);
    L.tI = o; o += al4(G * 21);
    L.tD = o; o += al4(G * 21);
    L.ring = o; o += 3 * ROWS * SPR;
    L.halo = o; o += 3 * NS;
    L.ringE = o; o += 3 * ROWS * NBP;
    L.haloE = o; o += 3 * NBP;
    L.misc = o; o += 4 * 32;
    L.zvec = o; o += al4(NS);
    L.zvecE = o; o += NBP;
    if (bwd) {
        L.cst_b = o; o += KSTAGE * ROWS * SPR;
        L.cst_u = o; o += KSTAGE * ROWS * SPR;
        L.cst_bE = o; o += KSTAGE * ROWS * NBP;
        L.cst_uE = o; o += KSTAGE * ROWS * NBP;
        L.fst = o; o += 2 * ROWS * SPR;
        L.fstE = o; o += 2 * ROWS * NBP;
        L.colI = o; o += al4(ROWS * G);
        L.binsI = o; o += al4(G * 21);
    } else {
        L.cst_b = L.cst_u = L.cst_bE = L.cst_uE = L.fst = L.fstE = L.colI = L.binsI = -1;
    }
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 1;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

// Model into shared memory (all threads of the CTA; ends with __syncthreads).
// chi slot layout [s][k] (forward) or [k][s] (backward) over the padded slots.
__device__ void load_model_b(const KParams &P, int p, const PairMeta &m, const SmemB &L, float *sm,
                             unsigned char *smb, bool bwd) {
    const int NS = P.NS, N = P.N, G = P.G;
    const int tid = threadIdx.x, nt = blockDim.x;
    const float *chi = P.chi + (int64_t)p * P.chi_stride;
    for (int idx = tid; idx < NS * NS; idx += nt) {
        const int s = idx / NS, k = idx % NS;
        const int os = P.slot_orig[s], ok = P.slot_orig[k];
        const int kt = P.slot_type[k];
        float v = 0.f;
        if (os >= 0 && ok >= 0 && (kt == T_M || kt == T_I || kt == T_D)) v = __ldg(chi + os * N + ok);
        if (bwd) sm[L.chi + k * NS + s] = v; else sm[L.chi + s * NS + k] = v;
    }
    for (int s = tid; s < NS; s += nt) {
        const int os = P.slot_orig[s];
        sm[L.chiE + s] = (os >= 0) ? __ldg(chi + os * N + P.e_idx) : 0.f;
    }
    const float *eM = P.eM + (int64_t)p * P.eM_stride;
    const float *eI = P.eI + (int64_t)p * P.eID_stride;
    const float *eD = P.eD + (int64_t)p * P.eID_stride;
    for (int idx = tid; idx < G * 441; idx += nt) sm[L.tM + idx] = __ldg(eM + idx);
    for (int idx = tid; idx < G * 21; idx += nt) {
        sm[L.tI + idx] = __ldg(eI + idx);
        sm[L.tD + idx] = __ldg(eD + idx);
    }
    for (int s = tid; s < NS; s += nt) sm[L.zvec + s] = 0.f;
    for (int b = tid; b < nbp_of(NS / 4); b += nt) reinterpret_cast<int *>(sm)[L.zvecE + b] = EXP_NONE;
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

struct QuadEmit {
    int off[4];      // table offsets (M: + y, I: + y, D: fixed)
    float mask[4];
    int type;
};

__device__ __forceinline__ QuadEmit quad_emit(const KParams &P, const SmemB &L, int q, int xi) {
    QuadEmit e;
    e.type = P.quad_type[q];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int k = 4 * q + u;
        const int kt = P.slot_type[k];
        const bool em = (kt == T_M || kt == T_I || kt == T_D);
        const int g = em ? P.slot_group[k] : 0;
        e.mask[u] = em ? 1.f : 0.f;
        if (e.type == T_M) e.off[u] = L.tM + g * 441 + xi * 21;
        else if (e.type == T_I) e.off[u] = L.tI + g * 21;
        else e.off[u] = L.tD + g * 21 + xi;
    }
    return e;
}

__device__ __forceinline__ float4 quad_emit_vals(const float *sm, const QuadEmit &e, int yj) {
    const int add = e.type == T_D ? 0 : yj;
    return make_float4(sm[e.off[0] + add] * e.mask[0], sm[e.off[1] + add] * e.mask[1],
                       sm[e.off[2] + add] * e.mask[2], sm[e.off[3] + add] * e.mask[3]);
}

// 2^d for d <= 0 (exact in the normal range, 0 below it: such terms are
// below 2^-126 of the cell's largest quad and cannot move a float32 sum)
__device__ __forceinline__ float pow2n(int d) { return d > -127 ? __int_as_float((d + 127) << 23) : 0.f; }

__device__ __forceinline__ void load_exps(const int *e, int (&E)[32], int NBP) {
    for (int i = 0; i < NBP / 4; ++i) {
        const int4 v = reinterpret_cast<const int4 *>(e)[i];
        E[4 * i] = v.x; E[4 * i + 1] = v.y; E[4 * i + 2] = v.z; E[4 * i + 3] = v.w;
    }
}

// Dot products of one quad of destinations with a predecessor vector whose
// quads carry their own exponents: out[u] = sum_b 2^(E_b - Eref) sum_{s in b}
// v[s] chi[s][4q+u].  Returns Eref (EXP_NONE when the vector is all zero).
template <class SH>
__device__ __forceinline__ int quad_contract(const float *vec, const int *vecE, const float (&cq)[SH::CHI_REG ? SH::NS : 1][4],
                                             const float4 *chi4q, float4 &out) {
    constexpr int NB = SH::NB, NS = SH::NS, NBP = SH::NBP;
    int E[NBP];
#pragma unroll
    for (int i = 0; i < NBP / 4; ++i) {
        const int4 v = reinterpret_cast<const int4 *>(vecE)[i];
        E[4 * i] = v.x; E[4 * i + 1] = v.y; E[4 * i + 2] = v.z; E[4 * i + 3] = v.w;
    }
    int Eref = EXP_NONE;
#pragma unroll
    for (int b = 0; b < NB; ++b) Eref = max(Eref, E[b]);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    if (Eref > EXP_NONE) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const float sc = pow2n(E[b] - Eref);
            const float4 v = *reinterpret_cast<const float4 *>(vec + 4 * b);
            const float vs[4] = {v.x * sc, v.y * sc, v.z * sc, v.w * sc};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int s = 4 * b + i;
                float c0, c1, c2, c3;
                if constexpr (SH::CHI_REG) {
                    c0 = cq[s][0]; c1 = cq[s][1]; c2 = cq[s][2]; c3 = cq[s][3];
                } else {
                    const float4 cv = chi4q[s * (NS / 4)];
                    c0 = cv.x; c1 = cv.y; c2 = cv.z; c3 = cv.w;
                }
                a0 = fmaf(vs[i], c0, a0); a1 = fmaf(vs[i], c1, a1);
                a2 = fmaf(vs[i], c2, a2); a3 = fmaf(vs[i], c3, a3);
            }
        }
    }
    out = make_float4(a0, a1, a2, a3);
    return Eref;
}

// quad_contract for the two cells of a lane at once: every transition
// operand loaded (or held in registers) serves both cells.  A missing
// predecessor is the zero vector with EXP_NONE exponents (no branches).
template <class SH>
__device__ __forceinline__ void quad_contract2(const float *v0, const int *e0, const float *v1, const int *e1,
                                               const float (&cq)[SH::CHI_REG ? SH::NS : 1][4], const float4 *chi4q,
                                               float4 &o0, float4 &o1, int &Eref0, int &Eref1) {
    constexpr int NB = SH::NB, NS = SH::NS, NBP = SH::NBP;
    int E0[NBP], E1[NBP];
#pragma unroll
    for (int i = 0; i < NBP / 4; ++i) {
        const int4 a = reinterpret_cast<const int4 *>(e0)[i];
        const int4 b = reinterpret_cast<const int4 *>(e1)[i];
        E0[4 * i] = a.x; E0[4 * i + 1] = a.y; E0[4 * i + 2] = a.z; E0[4 * i + 3] = a.w;
        E1[4 * i] = b.x; E1[4 * i + 1] = b.y; E1[4 * i + 2] = b.z; E1[4 * i + 3] = b.w;
    }
    Eref0 = EXP_NONE;
    Eref1 = EXP_NONE;
#pragma unroll
    for (int b = 0; b < NB; ++b) { Eref0 = max(Eref0, E0[b]); Eref1 = max(Eref1, E1[b]); }
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const float s0 = pow2n(E0[b] - Eref0), s1 = pow2n(E1[b] - Eref1);
        const float4 x = *reinterpret_cast<const float4 *>(v0 + 4 * b);
        const float4 y = *reinterpret_cast<const float4 *>(v1 + 4 * b);
        const float xs[4] = {x.x * s0, x.y * s0, x.z * s0, x.w * s0};
        const float ysv[4] = {y.x * s1, y.y * s1, y.z * s1, y.w * s1};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int s = 4 * b + i;
            float k0, k1, k2, k3;
            if constexpr (SH::CHI_REG) {
                k0 = cq[s][0]; k1 = cq[s][1]; k2 = cq[s][2]; k3 = cq[s][3];
            } else {
                const float4 cv = chi4q[s * (NS / 4)];
                k0 = cv.x; k1 = cv.y; k2 = cv.z; k3 = cv.w;
            }
            a0 = fmaf(xs[i], k0, a0); a1 = fmaf(xs[i], k1, a1); a2 = fmaf(xs[i], k2, a2); a3 = fmaf(xs[i], k3, a3);
            c0 = fmaf(ysv[i], k0, c0); c1 = fmaf(ysv[i], k1, c1); c2 = fmaf(ysv[i], k2, c2); c3 = fmaf(ysv[i], k3, c3);
        }
    }
    o0 = make_float4(a0, a1, a2, a3);
    o1 = make_float4(c0, c1, c2, c3);
}

__device__ __forceinline__ void copy_edge_cell(const float *v, const int *e, float *gv, int *ge, int NS, int NBP) {
    for (int i = 0; i < NS / 4; ++i)
        reinterpret_cast<float4 *>(gv)[i] = reinterpret_cast<const float4 *>(v)[i];
    for (int i = 0; i < NBP / 4; ++i)
        reinterpret_cast<int4 *>(ge)[i] = reinterpret_cast<const int4 *>(e)[i];
}

// ---------------------------------------------------------------- forward
template <class SH>
__device__ void fwd_stripe_b(const KParams &P, int p, int si, const SmemB &L, float *sm, unsigned char *smb) {
    constexpr int NS = SH::NS, NB = SH::NB, NBP = SH::NBP, SPR = SH::SPR;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x;
    const int lane = tid & 31, q = tid >> 5;
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const bool has_above = si > 0;
    const int *prog_above = has_above ? P.progress + m.stripe_base + si - 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_above = P.edge + (m.edge_base + (int64_t)(si - 1) * (Ly + 1)) * NS;
    const int *edgeE_above = P.edge_exp + (m.edge_base + (int64_t)(si - 1) * (Ly + 1)) * NBP;
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * NS;
    int *edgeE_mine = P.edge_exp + (m.edge_base + (int64_t)si * (Ly + 1)) * NBP;
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;

    load_model_b(P, p, m, L, sm, smb, false);
    const unsigned char *ys = smb + L.ys;
    float *ring = sm + L.ring;
    int *ringE = reinterpret_cast<int *>(sm) + L.ringE;
    float *halo = sm + L.halo;
    int *haloE = reinterpret_cast<int *>(sm) + L.haloE;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    const float4 *chi4q = reinterpret_cast<const float4 *>(sm + L.chi) + q;
    float cq[SH::CHI_REG ? NS : 1][4];
    if constexpr (SH::CHI_REG) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const float4 cv = chi4q[s * (NS / 4)];
            cq[s][0] = cv.x; cq[s][1] = cv.y; cq[s][2] = cv.z; cq[s][3] = cv.w;
        }
    }
    int rowi[R], xch[R];
    QuadEmit qe[R];
#pragma unroll
    for (int c = 0; c < R; ++c) {
        rowi[c] = i0 + lane + 32 * c;
        xch[c] = 0;
        if (rowi[c] >= 1 && rowi[c] <= Lx) xch[c] = min((int)P.res[m.x_off + rowi[c] - 1], 20);
        qe[c] = quad_emit(P, L, q, xch[c]);
    }
    const int qt = P.quad_type[q];
    const int T_last = (nrows - 1) + Ly;
    // halo pipeline state (thread 0 only)
    int pv = 0, fetched = 0;   // columns [0, fetched) of the halo row are in flight or landed
    if (tid == 0) { misc[0] = 0; if (has_above) pv = ld_acquire(prog_above); }
    double llpart = 0.0;
    int llE = EXP_NONE;

    for (int t = 0; t <= T_last; ++t) {
        // ---- halo column t (row i0-1) must be in shared memory before the step barrier
        if (tid == 0 && has_above && t <= Ly) {
            if (fetched <= t) {   // not prefetched: wait for the producer, fetch now
                if (!wait_geq(prog_above, t + 1, P.spin_limit)) {
                    misc[0] = 1;
                } else {
                    const int sl = t % 3;
                    for (int i = 0; i < NS / 4; ++i)
                        cp_async16(halo + sl * NS + 4 * i, edge_above + (int64_t)t * NS + 4 * i);
                    for (int i = 0; i < NBP / 4; ++i)
                        cp_async16(haloE + sl * NBP + 4 * i, edgeE_above + (int64_t)t * NBP + 4 * i);
                    cp_commit();
                    fetched = t + 1;
                }
            }
            cp_wait0();
        }
        bar_sync(BAR_STEP, NB * 32);
        if (misc[0]) break;                       // uniform: written before the barrier
        // ---- bottom row of step t-1 (every warp wrote its quad before the barrier):
        // thread 0 copies it to the edge row and publishes; its own release covers it
        if (tid == 0 && has_below && t >= 1) {
            const int jb = t - 1 - (ROWS - 1);
            if (jb >= 0 && jb <= Ly) {
                copy_edge_cell(ring + ((t + 2) % 3) * ROWS * SPR + (ROWS - 1) * SPR,
                               ringE + ((t + 2) % 3) * ROWS * NBP + (ROWS - 1) * NBP,
                               edge_mine + (int64_t)jb * NS, edgeE_mine + (int64_t)jb * NBP, NS, NBP);
                if (((jb + 1) % PUBB) == 0 || jb == Ly) st_release(prog_mine, jb + 1);
            }
        }
        // ---- prefetch halo column t+1 when the progress read at the last step covers it
        if (tid == 0 && has_above && t + 1 <= Ly) {
            if (fetched == t + 1 && pv > t + 1) {
                const int sl = (t + 1) % 3;
                for (int i = 0; i < NS / 4; ++i)
                    cp_async16(halo + sl * NS + 4 * i, edge_above + (int64_t)(t + 1) * NS + 4 * i);
                for (int i = 0; i < NBP / 4; ++i)
                    cp_async16(haloE + sl * NBP + 4 * i, edgeE_above + (int64_t)(t + 1) * NBP + 4 * i);
                cp_commit();
                fetched = t + 2;
            }
            if (pv <= t + 2) pv = ld_acquire(prog_above);   // only when the next prefetch needs more
        }
        // ---- my quad for both cells: predecessors, then one merged contraction
        const float *pvp[R];
        const int *pep[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int rho = lane + 32 * c;
            const int j = t - rho;
            const int i = rowi[c];
            const bool valid = rho < nrows && j >= 0 && j <= Ly;
            pvp[c] = sm + L.zvec;
            pep[c] = reinterpret_cast<const int *>(sm) + L.zvecE;
            if (!valid) continue;
            if (qt == T_I) {
                if (j >= 1) { pvp[c] = ring + ((t + 2) % 3) * ROWS * SPR + rho * SPR; pep[c] = ringE + ((t + 2) % 3) * ROWS * NBP + rho * NBP; }
            } else if (qt == T_D) {
                if (i >= 1) {
                    if (rho >= 1) { pvp[c] = ring + ((t + 2) % 3) * ROWS * SPR + (rho - 1) * SPR; pep[c] = ringE + ((t + 2) % 3) * ROWS * NBP + (rho - 1) * NBP; }
                    else { pvp[c] = halo + (j % 3) * NS; pep[c] = haloE + (j % 3) * NBP; }
                }
            } else if (qt == T_M) {
                if (i >= 1 && j >= 1) {
                    if (rho >= 1) { pvp[c] = ring + ((t + 1) % 3) * ROWS * SPR + (rho - 1) * SPR; pep[c] = ringE + ((t + 1) % 3) * ROWS * NBP + (rho - 1) * NBP; }
                    else { pvp[c] = halo + ((j - 1) % 3) * NS; pep[c] = haloE + ((j - 1) % 3) * NBP; }
                }
            }
        }
        float4 oc[R];
        int Erc[R];
        quad_contract2<SH>(pvp[0], pep[0], pvp[1], pep[1], cq, chi4q, oc[0], oc[1], Erc[0], Erc[1]);
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int rho = lane + 32 * c;
            const int j = t - rho;
            const bool valid = rho < nrows && j >= 0 && j <= Ly;
            if (!valid) continue;
            const int i = rowi[c];
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
            int Eo = EXP_NONE;
            {
                const int Eref = Erc[c];
                o = oc[c];
                const float4 e = quad_emit_vals(sm, qe[c], ys[j]);
                o = make_float4(o.x * e.x, o.y * e.y, o.z * e.z, o.w * e.w);
                const float mx = f4max(o);
                if (mx > 0.f && Eref > EXP_NONE) {
                    const int eb = warp2::exp_of(mx);
                    const float sc = pow2f(-eb);
                    if (-eb >= -126 && -eb <= 127) o = f4scale(o, sc);
                    else o = make_float4(ldexpf(o.x, -eb), ldexpf(o.y, -eb), ldexpf(o.z, -eb), ldexpf(o.w, -eb));
                    Eo = Eref + eb;
                } else {
                    o = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            if (i == 0 && j == 0 && (P.s_slot >> 2) == q) {   // origin: F[0,0,start] = 1
                const int u = P.s_slot & 3;
                o = make_float4(u == 0 ? 1.f : 0.f, u == 1 ? 1.f : 0.f, u == 2 ? 1.f : 0.f, u == 3 ? 1.f : 0.f);
                Eo = 0;
            }
            const int sl = t % 3;
            *reinterpret_cast<float4 *>(ring + sl * ROWS * SPR + rho * SPR + 4 * q) = o;
            ringE[sl * ROWS * NBP + rho * NBP + q] = Eo;
            if (P.lat) {
                const int64_t cell = latc + (int64_t)t * ROWS + rho;
                reinterpret_cast<float4 *>(P.lat + cell * NS)[q] = o;
                P.lat_exp[cell * NBP + q] = Eo;
            }
            if (i == Lx && j == Ly && si + 1 == m.n_stripes) {   // my quad's share of P(x,y)
                double a = (double)o.x * sm[L.chiE + 4 * q] + (double)o.y * sm[L.chiE + 4 * q + 1] +
                           (double)o.z * sm[L.chiE + 4 * q + 2] + (double)o.w * sm[L.chiE + 4 * q + 3];
                llpart = a;
                llE = Eo;
            }
        }
    }
    bar_sync(BAR_STEP, NB * 32);
    const bool aborted = misc[0] != 0;
    if (tid == 0 && has_below) {   // last column (or everything, after an abort)
        if (!aborted)
            copy_edge_cell(ring + (T_last % 3) * ROWS * SPR + (ROWS - 1) * SPR,
                           ringE + (T_last % 3) * ROWS * NBP + (ROWS - 1) * NBP,
                           edge_mine + (int64_t)Ly * NS, edgeE_mine + (int64_t)Ly * NBP, NS, NBP);
        st_release(prog_mine, Ly + 1);
    }
    if (aborted) {
        if (tid == 0) {
            atomicOr(P.status + p, PHMM_ST_TIMEOUT);
            if (si + 1 == m.n_stripes) P.ll[p] = NEG_INF_LL;
        }
        if (tid == 0) cp_wait0();
        __threadfence();
        bar_sync(BAR_STEP, NB * 32);
        if (tid == 0) st_release(P.progress + m.stripe_base + si, Ly + 2);
        return;
    }
    // ---- log-likelihood: combine the per-quad partial sums of the terminal cell
    double *llbuf = reinterpret_cast<double *>(misc + 32);
    int *llEbuf = misc + 64;
    if (si + 1 == m.n_stripes) {
        const int rT = Lx - i0;
        if (lane == (rT & 31)) {
            llbuf[q] = llpart;
            llEbuf[q] = llE;
        }
    }
    bar_sync(BAR_STEP, NB * 32);
    if (tid == 0 && si + 1 == m.n_stripes) {
        int Emax = EXP_NONE;
        for (int b = 0; b < NB; ++b)
            if (llbuf[b] > 0.0) Emax = max(Emax, llEbuf[b]);
        double acc = 0.0;
        for (int b = 0; b < NB; ++b)
            if (llbuf[b] > 0.0) acc += llbuf[b] * exp2((double)(llEbuf[b] - Emax));
        double ll = NEG_INF_LL;
        if (acc > 0.0 && isfinite(acc) && Emax > EXP_NONE) ll = log(acc) + (double)Emax * LN2;
        else atomicOr(P.status + p, PHMM_ST_ZERO_LL);
        P.ll[p] = ll;
    }
    // stripe complete (lattice and, for the last stripe, the log-likelihood):
    // the count pass of the split E-step may start on it
    __threadfence();
    bar_sync(BAR_STEP, NB * 32);
    if (tid == 0) st_release(P.progress + m.stripe_base + si, Ly + 2);
}

template <class SH>
__global__ void __launch_bounds__(32 * SH::NB) forward_block_kernel(const KParams P) {
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
        fwd_stripe_b<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

// ---------------------------------------------------------------- backward + counts
constexpr int NCW = 4;            // count warps per CTA
constexpr int BAR_CNT = 2 + 2 * KSTAGE;

template <class SH>
__device__ void bwd_stripe_b(const KParams &P, int p, int si, const SmemB &L, float *sm, unsigned char *smb) {
    constexpr int NS = SH::NS, NB = SH::NB, NBP = SH::NBP, SPR = SH::SPR;
    constexpr int NALL = 32 * (NB + NCW);
    const PairMeta m = P.meta[p];
    const int N = P.N, G = P.G;
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const bool rec = wid < NB;                  // recursion warp (quad wid) or count warp
    const int i0 = si * ROWS;
    const int nrows = min(ROWS, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const bool has_above = si > 0;
    const int *prog_below = has_below ? P.progress + m.stripe_base + si + 1 : nullptr;
    int *prog_mine = P.progress + m.stripe_base + si;
    const float *edge_below = P.edge + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * NS;
    const int *edgeE_below = P.edge_exp + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * NBP;
    float *edge_mine = P.edge + (m.edge_base + (int64_t)si * (Ly + 1)) * NS;
    int *edgeE_mine = P.edge_exp + (m.edge_base + (int64_t)si * (Ly + 1)) * NBP;
    const int64_t latc = m.lat_base + (int64_t)si * (ROWS + Ly) * ROWS;

    const double llv = P.ll[p];
    if (!(llv > -1e29)) {   // forward failed: nothing to count (uniform decision)
        if (tid == 0 && has_above) st_release(prog_mine, Ly + 1);
        __syncthreads();
        return;
    }
    const double lam = llv / LN2;
    load_model_b(P, p, m, L, sm, smb, true);
    const unsigned char *ys = smb + L.ys;
    float *ring = sm + L.ring;
    int *ringE = reinterpret_cast<int *>(sm) + L.ringE;
    float *halo = sm + L.halo;
    int *haloE = reinterpret_cast<int *>(sm) + L.haloE;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    float *cstb = sm + L.cst_b, *cstu = sm + L.cst_u;
    int *cstbE = reinterpret_cast<int *>(sm) + L.cst_bE, *cstuE = reinterpret_cast<int *>(sm) + L.cst_uE;
    float *fst = sm + L.fst;
    int *fstE = reinterpret_cast<int *>(sm) + L.fstE;
    float *colI = sm + L.colI, *binsI = sm + L.binsI;
    for (int idx = tid; idx < ROWS * G; idx += blockDim.x) colI[idx] = 0.f;
    for (int idx = tid; idx < G * 21; idx += blockDim.x) binsI[idx] = 0.f;
    if (tid == 0) { misc[0] = 0; misc[1] = 0; }
    __syncthreads();
    const int T_last = (nrows - 1) + Ly;
    const int nsteps = T_last + 1;

    if (rec) {
        // ======================= recursion warps: quad q of the backward vector
        const int q = wid;
        const float4 *chi4q = reinterpret_cast<const float4 *>(sm + L.chi) + q;  // chiB[k][4q..]
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
        const int qt = P.quad_type[q];
        int pv = 0, fetched = Ly + 1;   // halo columns >= fetched are in flight or landed
        if (tid == 0 && has_below) pv = ld_acquire(prog_below);
        int k = 0;
        bool aborted = false;
        for (int t = T_last; t >= 0; --t, ++k) {
            // ---- halo column t-63 (row i0+64) in shared memory before the step barrier
            const int jh = t - (ROWS - 1);
            if (tid == 0 && has_below && jh >= 0 && jh <= Ly) {
                if (fetched > jh) {
                    if (!wait_geq(prog_below, Ly + 1 - jh, P.spin_limit)) {
                        misc[0] = 1;
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
            const bool abort_now = misc[0] != 0;
            // ---- top row of step t+1 -> edge row for the stripe above
            if (!abort_now && tid == 0 && has_above && t + 1 <= T_last) {
                const int jt = t + 1;
                if (jt <= Ly) {
                    copy_edge_cell(ring + ((t + 1) % 3) * ROWS * SPR, ringE + ((t + 1) % 3) * ROWS * NBP,
                                   edge_mine + (int64_t)jt * NS, edgeE_mine + (int64_t)jt * NBP, NS, NBP);
                    if ((jt % PUBB) == 0) st_release(prog_mine, Ly + 1 - jt);
                }
            }
            // ---- count-ring slot for this step must be free
            const int cs = k % KSTAGE;
            if (k >= KSTAGE) bar_sync(BAR_EMPTY0 + cs, NALL);
            if (abort_now) {
                if (tid == 0) misc[1] = 1;
                bar_arrive(BAR_FULL0 + cs, NALL);
                aborted = true;
                break;
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
#pragma unroll
            for (int c = 0; c < R; ++c) {
                const int rho = lane + 32 * c;
                const int j = t - rho;
                const bool valid = rho < nrows && j >= 0 && j <= Ly;
                float4 bq = make_float4(0.f, 0.f, 0.f, 0.f), uq = bq, wq = bq;
                int Eb = EXP_NONE, Eu = EXP_NONE;
                if (valid) {
                    const int i = rowi[c];
                    const bool term = (i == Lx && j == Ly);
                    // successor vectors by type
                    const bool hI = j + 1 <= Ly, hD = i + 1 <= Lx, hM = hI && hD;
                    const float *vI = hI ? ring + ((t + 1) % 3) * ROWS * SPR + rho * SPR : nullptr;
                    const int *eI = hI ? ringE + ((t + 1) % 3) * ROWS * NBP + rho * NBP : nullptr;
                    const float *vD = nullptr, *vM = nullptr;
                    const int *eD = nullptr, *eM = nullptr;
                    if (hD) {
                        if (rho + 1 < nrows) { vD = ring + ((t + 1) % 3) * ROWS * SPR + (rho + 1) * SPR; eD = ringE + ((t + 1) % 3) * ROWS * NBP + (rho + 1) * NBP; }
                        else { vD = halo + (j % 3) * NS; eD = haloE + (j % 3) * NBP; }
                    }
                    if (hM) {
                        if (rho + 1 < nrows) { vM = ring + ((t + 2) % 3) * ROWS * SPR + (rho + 1) * SPR; eM = ringE + ((t + 2) % 3) * ROWS * NBP + (rho + 1) * NBP; }
                        else { vM = halo + ((j + 1) % 3) * NS; eM = haloE + ((j + 1) % 3) * NBP; }
                    }
                    // b[4q+u] = sum over dest quads d (successor of d's type)
                    int EvM[NBP], EvI[NBP], EvD[NBP];
#pragma unroll
                    for (int ii = 0; ii < NBP; ++ii) { EvM[ii] = EXP_NONE; EvI[ii] = EXP_NONE; EvD[ii] = EXP_NONE; }
#pragma unroll
                    for (int ii = 0; ii < NBP / 4; ++ii) {
                        if (eM) { const int4 v = reinterpret_cast<const int4 *>(eM)[ii]; EvM[4*ii] = v.x; EvM[4*ii+1] = v.y; EvM[4*ii+2] = v.z; EvM[4*ii+3] = v.w; }
                        if (eI) { const int4 v = reinterpret_cast<const int4 *>(eI)[ii]; EvI[4*ii] = v.x; EvI[4*ii+1] = v.y; EvI[4*ii+2] = v.z; EvI[4*ii+3] = v.w; }
                        if (eD) { const int4 v = reinterpret_cast<const int4 *>(eD)[ii]; EvD[4*ii] = v.x; EvD[4*ii+1] = v.y; EvD[4*ii+2] = v.z; EvD[4*ii+3] = v.w; }
                    }
                    int Ed[NB];
                    int Eref = EXP_NONE;
#pragma unroll
                    for (int d = 0; d < NB; ++d) {
                        const int dt = P.quad_type[d];
                        Ed[d] = dt == T_M ? EvM[d] : (dt == T_I ? EvI[d] : (dt == T_D ? EvD[d] : EXP_NONE));
                        Eref = max(Eref, Ed[d]);
                    }
                    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
                    if (term) {
                        const float4 ce = *reinterpret_cast<const float4 *>(sm + L.chiE + 4 * q);
                        a0 = ce.x; a1 = ce.y; a2 = ce.z; a3 = ce.w;
                        Eref = 0;
                    } else if (Eref > EXP_NONE) {
#pragma unroll
                        for (int d = 0; d < NB; ++d) {
                            if (Ed[d] <= EXP_NONE) continue;
                            const int dt = P.quad_type[d];
                            const float *vv = dt == T_M ? vM : (dt == T_I ? vI : vD);
                            const float sc = pow2n(Ed[d] - Eref);
                            const float4 w4 = *reinterpret_cast<const float4 *>(vv + 4 * d);
                            const float ws[4] = {w4.x * sc, w4.y * sc, w4.z * sc, w4.w * sc};
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
                                a0 = fmaf(ws[ii], c0, a0); a1 = fmaf(ws[ii], c1, a1);
                                a2 = fmaf(ws[ii], c2, a2); a3 = fmaf(ws[ii], c3, a3);
                            }
                        }
                    }
                    bq = make_float4(a0, a1, a2, a3);
                    const float mx = f4max(bq);
                    if (mx > 0.f && Eref > EXP_NONE) {
                        const int eb = warp2::exp_of(mx);
                        if (-eb >= -126 && -eb <= 127) bq = f4scale(bq, pow2f(-eb));
                        else bq = make_float4(ldexpf(bq.x, -eb), ldexpf(bq.y, -eb), ldexpf(bq.z, -eb), ldexpf(bq.w, -eb));
                        Eb = Eref + eb;
                    } else {
                        bq = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    const float4 e = quad_emit_vals(sm, qe[c], ys[j]);
                    wq = make_float4(bq.x * e.x, bq.y * e.y, bq.z * e.z, bq.w * e.w);
                    // successor values of my own dest quad (transition-count operand)
                    const float *vs = qt == T_M ? vM : (qt == T_I ? vI : (qt == T_D ? vD : nullptr));
                    const int *es = qt == T_M ? eM : (qt == T_I ? eI : (qt == T_D ? eD : nullptr));
                    if (vs != nullptr && !term) {
                        uq = *reinterpret_cast<const float4 *>(vs + 4 * q);
                        Eu = es[q];
                    }
                }
                const int sl = t % 3;
                *reinterpret_cast<float4 *>(ring + sl * ROWS * SPR + rho * SPR + 4 * q) = wq;
                ringE[sl * ROWS * NBP + rho * NBP + q] = Eb;
                *reinterpret_cast<float4 *>(cstb + (cs * ROWS + rho) * SPR + 4 * q) = bq;
                *reinterpret_cast<float4 *>(cstu + (cs * ROWS + rho) * SPR + 4 * q) = uq;
                cstbE[(cs * ROWS + rho) * NBP + q] = Eb;
                cstuE[(cs * ROWS + rho) * NBP + q] = Eu;
            }
            bar_arrive(BAR_FULL0 + cs, NALL);
        }
        // drain: wait until the count warps released the last slots
        const int kend = aborted ? k + 1 : nsteps;
        for (int kk = max(0, kend - KSTAGE); kk < kend; ++kk) bar_sync(BAR_EMPTY0 + kk % KSTAGE, NALL);
        if (tid == 0) {
            cp_wait0();
            if (has_above) {
                if (!aborted)
                    copy_edge_cell(ring, ringE, edge_mine, edgeE_mine, NS, NBP);   // column 0 (step 0)
                st_release(prog_mine, Ly + 1);
            }
        }
    } else {
        // ======================= count warps: posteriors, emission counts, outer products
        const int ct = tid - 32 * NB;             // 0 .. 32*NCW-1
        const int Ep = (int)floor(lam);
        const float rfrac = (float)exp2(-(lam - floor(lam)));
        // cell role: count thread ct < 64 owns row ct
        const int rho = ct;
        const bool cell_role = ct < ROWS;
        int xc = 0;
        const int irow = i0 + rho;
        if (cell_role && irow >= 1 && irow <= Lx) xc = min((int)P.res[m.x_off + irow - 1], 20);
        float dsum[NS], dcmp[NS];   // D-type emission counts of my row (Kahan)
#pragma unroll
        for (int s = 0; s < NS; ++s) { dsum[s] = 0.f; dcmp[s] = 0.f; }
        // block role for the outer products
        constexpr int NBLK = NB * NB;
        constexpr int NCT = 32 * NCW;
        const int GRP = max(1, NCT / NBLK);
        const int blk = ct % NBLK, grp = ct / NBLK;
        const bool blk_role = grp < GRP && NBLK <= NCT;
        const int bs = blk / NB, bk = blk % NB;
        float csum[16], ccomp[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) { csum[u] = 0.f; ccomp[u] = 0.f; }
        auto prefetch = [&](int t) {
            if (t >= 0) {
                const float *src = P.lat + (latc + (int64_t)t * ROWS) * NS;
                float *dst = fst + (t & 1) * ROWS * SPR;
                for (int idx = ct; idx < ROWS * NS / 4; idx += NCT) {
                    const int r = idx / (NS / 4), qq = idx % (NS / 4);
                    cp_async16(dst + r * SPR + 4 * qq, src + 4 * idx);
                }
                const int *srcE = P.lat_exp + (latc + (int64_t)t * ROWS) * NBP;
                int *dstE = fstE + (t & 1) * ROWS * NBP;
                for (int idx = ct; idx < ROWS * NBP / 4; idx += NCT) cp_async16(dstE + 4 * idx, srcE + 4 * idx);
            }
            cp_commit();
        };
        prefetch(T_last);
        int k = 0;
        for (int t = T_last; t >= 0; --t, ++k) {
            const int cs = k % KSTAGE;
            bar_sync(BAR_FULL0 + cs, NALL);
            if (misc[1]) { bar_arrive(BAR_EMPTY0 + cs, NALL); break; }
            cp_wait0();
            bar_sync(BAR_CNT, NCT);              // lattice rows of step t landed for all count threads
            prefetch(t - 1);
            float *fcell = fst + (t & 1) * ROWS * SPR;
            if (cell_role) {
                const int j = t - rho;
                const bool valid = rho < nrows && j >= 0 && j <= Ly;
                float *fr = fcell + rho * SPR;
                float *ur = cstu + (cs * ROWS + rho) * SPR;
                const float *br = cstb + (cs * ROWS + rho) * SPR;
                const int *fE = fstE + (t & 1) * ROWS * NBP + rho * NBP;
                const int *bE = cstbE + (cs * ROWS + rho) * NBP;
                const int *uE = cstuE + (cs * ROWS + rho) * NBP;
                int Efm = EXP_NONE;
                if (valid) {
#pragma unroll
                    for (int b = 0; b < NB; ++b) Efm = max(Efm, fE[b]);
                }
                const bool live = valid && Efm > EXP_NONE;
                const int yj = valid ? ys[j] : 0;
                float post[NS];
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                    const float4 fv = *reinterpret_cast<const float4 *>(fr + 4 * b);
                    const float4 bv = *reinterpret_cast<const float4 *>(br + 4 * b);
                    const float4 uv = *reinterpret_cast<const float4 *>(ur + 4 * b);
                    const int Ef = fE[b], Eb = bE[b], Eu = uE[b];
                    const float fs = (live && Ef > EXP_NONE) ? pow2f(Ef - Efm) : 0.f;
                    int dp = Eb + Efm - Ep;
                    if (dp > 126) { dp = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                    const float ps = (live && Eb > EXP_NONE) ? warp2::scale_pow2(rfrac, max(dp, -200)) : 0.f;
                    int du = Eu + Efm - Ep;
                    if (du > 126) { du = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                    const float us = (live && Eu > EXP_NONE) ? fminf(warp2::scale_pow2(rfrac, max(du, -200)), 3e38f) : 0.f;
                    // lattice rows of cells outside the pair are never written: never
                    // multiply them (garbage * 0 can be NaN), select instead
                    const float4 ft = fs > 0.f ? make_float4(fv.x * fs, fv.y * fs, fv.z * fs, fv.w * fs)
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
                    *reinterpret_cast<float4 *>(fr + 4 * b) = ft;
                    *reinterpret_cast<float4 *>(ur + 4 * b) = us > 0.f ? make_float4(uv.x * us, uv.y * us, uv.z * us, uv.w * us)
                                                                     : make_float4(0.f, 0.f, 0.f, 0.f);
                    post[4 * b] = ft.x * bv.x * ps; post[4 * b + 1] = ft.y * bv.y * ps;
                    post[4 * b + 2] = ft.z * bv.z * ps; post[4 * b + 3] = ft.w * bv.w * ps;
                }
                if (live) {
                    double *cntM = P.cntM + (int64_t)p * G * 441;
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        const int st = P.slot_type[s];
                        const float pv = post[s];
                        if (st == T_M) {
                            if (pv != 0.f) atomicAdd(cntM + P.slot_group[s] * 441 + xc * 21 + yj, (double)pv);
                        } else if (st == T_I) {
                            colI[(j % ROWS) * G + P.slot_group[s]] += pv;
                        } else if (st == T_D) {
                            const float y = pv - dcmp[s];
                            const float tt = dsum[s] + y;
                            dcmp[s] = (tt - dsum[s]) - y;
                            dsum[s] = tt;
                        }
                    }
                    if (irow == Lx && j == Ly) {   // expected End transitions
#pragma unroll
                        for (int s = 0; s < NS; ++s) {
                            const int os = P.slot_orig[s];
                            if (os >= 0) atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + P.e_idx, (double)post[s]);
                        }
                    }
                }
            }
            bar_sync(BAR_CNT, NCT);
            // column t is complete once row 0 visited it: I-type bins
            if (ct == 0 && t <= Ly) {
                const int slot = t % ROWS;
                const int yj = ys[t];
                for (int g = 0; g < G; ++g) {
                    binsI[g * 21 + yj] += colI[slot * G + g];
                    colI[slot * G + g] = 0.f;
                }
            }
            // transition-count outer products over the step's cells
            if (blk_role) {
                float pz[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) pz[u] = 0.f;
                const int r0 = grp * ROWS / GRP, r1 = (grp + 1) * ROWS / GRP;
                for (int rr = r0; rr < r1; ++rr) {
                    const float4 fv = *reinterpret_cast<const float4 *>(fcell + rr * SPR + 4 * bs);
                    const float4 uv = *reinterpret_cast<const float4 *>(cstu + (cs * ROWS + rr) * SPR + 4 * bk);
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
            bar_arrive(BAR_EMPTY0 + cs, NALL);
        }
        cp_wait0();
        bar_sync(BAR_CNT, NCT);
        if (misc[1] == 0) {
            // flush: transition counts n[s,k] = chi[s,k] * sum f~ u~
            if (blk_role) {
                const float *chi = P.chi + (int64_t)p * P.chi_stride;
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    const int s = 4 * bs + (u >> 2), kk = 4 * bk + (u & 3);
                    const int os = P.slot_orig[s], ok = P.slot_orig[kk];
                    const int kt = P.slot_type[kk];
                    const float val = csum[u] - ccomp[u];
                    if (os < 0 || ok < 0 || !(kt == T_M || kt == T_I || kt == T_D) || val == 0.f) continue;
                    atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + ok, (double)val * (double)__ldg(chi + os * N + ok));
                }
            }
            if (cell_role && rho < nrows && irow >= 1) {
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    if (P.slot_type[s] != T_D) continue;
                    const float v = dsum[s] - dcmp[s];
                    if (v != 0.f) atomicAdd(P.cntD + ((int64_t)p * G + P.slot_group[s]) * 21 + xc, (double)v);
                }
            }
            for (int idx = ct; idx < G * 21; idx += NCT) {
                const float v = binsI[idx];
                if (v != 0.f) atomicAdd(P.cntI + (int64_t)p * G * 21 + idx, (double)v);
            }
        }
    }
    __syncthreads();
    if (tid == 0 && misc[1]) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
    __syncthreads();
}

template <class SH>
__global__ void __launch_bounds__(32 * (SH::NB + NCW)) backward_block_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemB L = make_smem_b(SH::NS, SH::NB, 1, P.G, P.max_ly, true);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        bwd_stripe_b<SH>(P, w.x, w.y, L, sm, smem_raw);
    }
}

}  // namespace blk
