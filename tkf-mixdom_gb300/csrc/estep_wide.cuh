// estep_wide.cuh -- E-step kernels for large state spaces (more than 64
// padded slots, up to WMAXS: MixDom2 with K*F up to 33, e.g. n_dom=8,
// n_frag=4 -> 162 states).  Included by pairhmm.cu.
//
// At this size one cell is a 4NQ x NS contraction (about 26 k multiply-adds
// at 162 states), so a stripe step is a small GEMM: out[row][k] =
// sum_s pred_type(k)[row][s] chi[s][k].  A CTA sweeps a stripe of RW = 32
// rows along anti-diagonals; thread (row group rg, destination quad q) owns
// the 4 x 4 output tile rows 4rg..4rg+3 x states 4q..4q+3 and loops over the
// NS sources with two float4 loads (four rows of the predecessor, four
// transition entries) per 16 FMAs.  Lane layout: lane = 8 * (quad within the
// warp) + rg, so a warp's predecessor loads hit 8 consecutive float4s and its
// transition loads 4 consecutive float4s (one wavefront each).
//
// Predecessor rings in shared memory, source-major so rows are contiguous:
//   A[2][NS][RW]      row r at index r       (I-type predecessor: same row);
//   B[3][NS][RW + 4]  row r at index r + 1   (D / M predecessors: row r-1),
//                     index 0 = the halo row of the stripe above.
// Scaling: one power-of-two exponent per cell plus the cell's maximum value
// (E[4][RW+4], MX[4][RW+4], atomicMax on the float bits).  A cell's output
// takes exponent E_out = max over its predecessors of (E_pred +
// exponent(max_pred)), so stored values stay below ~NS and no cross-thread
// renormalisation is needed: one __syncthreads per step.
//
// The backward recursion (bwd_rec) is the transpose: out[row][s] = sum_k
// chi[s][k] w_succ(type k)[row][k], with successor rings of w = e b over the
// 4NQ destination slots (A: row r at index r, B: row r at index r + 3, halo
// row RW at index RW + 3).  Both write full lattices (values + exponent +
// maximum per cell) for the count pass.

namespace wide {

constexpr int RW = 32;           // rows per stripe
constexpr int WMAXS = 168;       // largest padded slot count
constexpr int WPUB = 4;          // edge progress published every WPUB columns

__host__ __device__ inline int ls_of(int NS) { return NS + 4; }   // lattice / edge record (floats)

struct SmemWd {
    int chi, chiE, A, B, E, MX, llp, misc;   // float / int offsets (llp: double index)
    int ys;                                   // byte offset
    int bytes;
};

// KS: destination slots (4 x destination quads); NSRC: sources of the ring
__host__ __device__ inline SmemWd make_smem_wd(int NS, int KS, int max_ly, bool bwd) {
    SmemWd L;
    const int NSRC = bwd ? KS : NS;          // ring vectors: forward sources / backward w of dests
    int o = 0;
    L.chi = o; o += bwd ? KS * KS : NS * KS;  // forward chi[s][k]; backward chiB[k][s] (s < KS)
    L.chiE = o; o += (NS + 3) & ~3;
    L.A = o; o += 2 * NSRC * RW;
    L.B = o; o += 3 * NSRC * (RW + 4);
    L.E = o; o += 4 * (RW + 4);
    L.MX = o; o += 4 * (RW + 4);
    o = (o + 1) & ~1;
    L.llp = o / 2; o += 2 * (KS / 4 + 4);
    L.misc = o; o += 8;
    int bytes = o * 4;
    L.ys = bytes;
    bytes += max_ly + 2;
    L.bytes = (bytes + 15) & ~15;
    return L;
}

__device__ __forceinline__ int exp_of_max(int mbits) {   // exponent of a positive float given as bits
    return warp2::exp_of(__int_as_float(mbits));
}

__device__ __forceinline__ float pow2d(int d) {   // 2^d for any d (0 far below the float range)
    if (d >= -126 && d <= 127) return pow2f(d);
    return d < -149 ? 0.f : ldexpf(1.f, d);
}

// emission factor of destination slot k at characters (x, y) from the global tables
__device__ __forceinline__ float emit_g(const KParams &P, const float *eM, const float *eI, const float *eD, int k,
                                        int x, int y) {
    const int kt = P.slot_type[k];
    const int g = P.slot_group[k];
    if (kt == T_M) return __ldg(eM + g * 441 + x * 21 + y);
    if (kt == T_I) return __ldg(eI + g * 21 + y);
    if (kt == T_D) return __ldg(eD + g * 21 + x);
    return 0.f;
}

// ---------------------------------------------------------------- 3xTF32 helpers
// x = hi + lo with hi = x rounded to TF32 and lo the TF32-rounded remainder;
// hi*hi + hi*lo + lo*hi then carries about 21 bits of each product.
__device__ __forceinline__ void tf32_split(float x, uint32_t &hi, uint32_t &lo) {
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    const float rem = x - __uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(rem));
    hi = h;
    lo = l;
}

// c += a b on the tensor cores (one warp; m16 n8 k8, TF32 inputs, float32
// accumulator).  Fragments: a0 (g, q), a1 (g+8, q), a2 (g, q+4), a3 (g+8, q+4);
// b0 (k q, n g), b1 (k q+4, n g); c0/c1 (g, 2q / 2q+1), c2/c3 (g+8, ...), with
// g = lane / 4, q = lane % 4.
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ---------------------------------------------------------------- forward
// TC: the step's contraction on the tensor cores (phmm_tuning.tensor; the host
// sets it only where every warp's 16 destinations share one type)
template <bool TC>
__device__ void fwd_stripe_wd(const KParams &P, int p, int si, const SmemWd &L, float *sm, unsigned char *smb) {
    const int NS = P.NS, KS = P.kend[2], NQd = KS / 4, N = P.N;
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
    const int64_t latc = P.stripe_lat ? P.stripe_lat[m.stripe_base + si] : m.lat_base + (int64_t)si * (RW + Ly) * RW;
    const bool pub = !P.recompute;   // a recomputed stripe publishes nothing (its edge rows exist)
    float *chiS = sm + L.chi, *A = sm + L.A, *B = sm + L.B;
    int *E = reinterpret_cast<int *>(sm) + L.E;
    int *MX = reinterpret_cast<int *>(sm) + L.MX;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    double *llp = reinterpret_cast<double *>(sm) + L.llp;
    unsigned char *ys = smb + L.ys;
    const int BW = RW + 4;
    // ---- model, rings, residues
    {
        const float *chi = P.chi + (int64_t)p * P.chi_stride;
        for (int idx = tid; idx < NS * KS; idx += nt) {
            const int s = idx / KS, k = idx % KS;
            const int os = P.slot_orig[s], ok = P.slot_orig[k];
            const int kt = P.slot_type[k];
            float v = 0.f;
            if (os >= 0 && ok >= 0 && (kt == T_M || kt == T_I || kt == T_D)) v = __ldg(chi + os * N + ok);
            chiS[idx] = v;
        }
        for (int s = tid; s < NS; s += nt) {
            const int os = P.slot_orig[s];
            sm[L.chiE + s] = os >= 0 ? __ldg(chi + os * N + P.e_idx) : 0.f;
        }
        for (int idx = tid; idx < 2 * NS * RW; idx += nt) A[idx] = 0.f;
        for (int idx = tid; idx < 3 * NS * BW; idx += nt) B[idx] = 0.f;
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
    }
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
    const int T_last = (nrows - 1) + Ly;
    // halo column t of row i0-1 goes to B[(t-1) % 3][s][0] (row -1 at step t-1);
    // warp 0 fetches column t+1 during step t, column 0 before the loop
    // (B slot (col - 1) % 3, exponent / maximum slot (col - 1) & 3)
    auto fetch_halo = [&](int col) -> bool {
        if (!has_above || col > Ly) return true;
        int ok = 1;
        if (lane == 0 && pub) ok = wait_geq(prog_above, col + 1, P.spin_limit) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) return false;
        const int bs = (col + 2) % 3, es = (col + 3) & 3;
        const float *src = edge_above + (int64_t)col * ES;
        for (int s = lane; s < NS; s += 32) B[(bs * NS + s) * BW] = __ldcg(src + s);
        if (lane == 0) {
            E[es * BW] = __ldcg(reinterpret_cast<const int *>(src) + NS);
            MX[es * BW] = __ldcg(reinterpret_cast<const int *>(src) + NS + 1);
        }
        return true;
    };
    __syncthreads();
    if (warp == 0 && !fetch_halo(0)) misc[0] = 1;
    int llE = EXP_NONE;
    bool aborted = false;
    int k = 0;
    for (int t = 0; t <= T_last; ++t, ++k) {
        __syncthreads();
        if (misc[k & 1]) { aborted = true; break; }
        if (tid == 0) misc[(k + 1) & 1] = 0;
        // maxima of step t+1 start at zero (slot last read at step t-1)
        for (int r = tid; r < RW; r += nt) MX[((t + 1) & 3) * BW + r + 1] = 0;
        // the origin's start-state entries (start slot outside the destination
        // quads) live two (A) / three (B) steps
        if (si == 0 && tid == 0 && P.s_slot >= KS) {
            if (t == 2) A[(0 * NS + P.s_slot) * RW + 0] = 0.f;
            if (t == 3) B[(0 * NS + P.s_slot) * BW + 1] = 0.f;
        }
        // ---- bottom row of step t-1 -> edge row for the stripe below (warp 1)
        if (pub && warp == (nt > 32 ? 1 : 0) && has_below && t >= 1) {
            const int jb = t - 1 - (RW - 1);
            if (jb >= 0 && jb <= Ly) {
                const int sl = (t - 1) % 3;
                float *dst = edge_mine + (int64_t)jb * ES;
                for (int s = lane; s < NS; s += 32) dst[s] = B[(sl * NS + s) * BW + RW];
                if (lane == 0) {
                    reinterpret_cast<int *>(dst)[NS] = E[((t - 1) & 3) * BW + RW];
                    reinterpret_cast<int *>(dst)[NS + 1] = MX[((t - 1) & 3) * BW + RW];
                }
                __threadfence();
                __syncwarp();
                if (lane == 0 && (((jb + 1) % WPUB) == 0 || jb == Ly)) st_release(prog_mine, jb + 1);
            }
        }
        // ---- compute my 4 x 4 tile
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
                        if (mb > 0 && e > EXP_NONE) EI = e + exp_of_max(mb);
                    }
                    if (row >= 1) {
                        const int mb = MX[((t - 1) & 3) * BW + r];
                        const int e = E[((t - 1) & 3) * BW + r];
                        if (mb > 0 && e > EXP_NONE) ED = e + exp_of_max(mb);
                    }
                    if (row >= 1 && j >= 1) {
                        const int mb = MX[((t - 2) & 3) * BW + r];
                        const int e = E[((t - 2) & 3) * BW + r];
                        if (mb > 0 && e > EXP_NONE) EM = e + exp_of_max(mb);
                    }
                }
                const int Eout = max(max(EI, ED), EM);
                Eo[i] = Eout;
                int Emine = qt == T_I ? EI : (qt == T_D ? ED : EM);
                const int Eraw = qt == T_I ? E[((t - 1) & 3) * BW + r + 1]
                                           : (qt == T_D ? E[((t - 1) & 3) * BW + r] : E[((t - 2) & 3) * BW + r]);
                sc[i] = (Emine > EXP_NONE && Eout > EXP_NONE) ? pow2d(Eraw - Eout) : 0.f;
            }
            const float *base = qt == T_I ? A + ((t - 1) & 1) * NS * RW + r0
                                          : (qt == T_D ? B + ((t + 2) % 3) * NS * BW + r0 : B + ((t + 1) % 3) * NS * BW + r0);
            const int stride = qt == T_I ? RW : BW;
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[i][u] = 0.f;
            const float4 *ch4 = reinterpret_cast<const float4 *>(chiS) + qd;
            // Above 64 slots, compensated blocked summation: 8 sources into a
            // block tile, the block tile into the accumulator with a Kahan
            // correction, so small terms are not lost against a large running
            // sum (sequential float32 sums of ~160 positive terms drop small
            // addends with a bias that the posteriors inherit: counts off by
            // ~1e-5 at 162 states).  At 64 slots or fewer the plain sequential
            // sum is kept: its forward and backward errors cancel in the
            // posteriors, which blocking would undo.
            const bool blocked = NS > 64;
            float cmp[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int u = 0; u < 4; ++u) cmp[i][u] = 0.f;
            auto block = [&](int s0, int nb) {
                float bt[4][4];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int u = 0; u < 4; ++u) bt[i][u] = blocked ? 0.f : acc[i][u];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    if (q < nb) {
                        const float4 pv = *reinterpret_cast<const float4 *>(base + (s0 + q) * stride);
                        const float4 cv = ch4[(s0 + q) * NQd];
                        const float pa[4] = {pv.x, pv.y, pv.z, pv.w};
                        const float ca[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                        for (int i = 0; i < 4; ++i)
#pragma unroll
                            for (int u = 0; u < 4; ++u) bt[i][u] = fmaf(pa[i], ca[u], bt[i][u]);
                    }
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (blocked) {
                            const float y = bt[i][u] - cmp[i][u];
                            const float tt = acc[i][u] + y;
                            cmp[i][u] = (tt - acc[i][u]) - y;
                            acc[i][u] = tt;
                        } else {
                            acc[i][u] = bt[i][u];
                        }
                    }
            };
            if (TC) {
                // the warp's 32 rows x 16 destinations (quads 4 warp .. 4 warp + 3)
                // as 2 x 2 tiles of m16 n8 over k-steps of 8 sources, 3xTF32
                const int g = lane >> 2, cq = lane & 3, n0 = 16 * warp;
                const float *bw = base - r0;   // the warp's rows from 0
                float c[2][2][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                        for (int e = 0; e < 4; ++e) c[mt][nt][e] = 0.f;
                for (int s0 = 0; s0 < NS; s0 += 8) {
                    const int sa0 = s0 + cq, sa1 = s0 + cq + 4;
                    const bool in0 = sa0 < NS, in1 = sa1 < NS;
                    uint32_t ahi[2][4], alo[2][4], bhi[2][2], blo[2][2];
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) {
                        const int m0 = 16 * mt + g;
                        const float a0 = in0 ? bw[sa0 * stride + m0] : 0.f;
                        const float a1 = in0 ? bw[sa0 * stride + m0 + 8] : 0.f;
                        const float a2 = in1 ? bw[sa1 * stride + m0] : 0.f;
                        const float a3 = in1 ? bw[sa1 * stride + m0 + 8] : 0.f;
                        tf32_split(a0, ahi[mt][0], alo[mt][0]);
                        tf32_split(a1, ahi[mt][1], alo[mt][1]);
                        tf32_split(a2, ahi[mt][2], alo[mt][2]);
                        tf32_split(a3, ahi[mt][3], alo[mt][3]);
                    }
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt) {
                        const int n = n0 + 8 * nt + g;
                        const float b0 = in0 ? chiS[sa0 * KS + n] : 0.f;
                        const float b1 = in1 ? chiS[sa1 * KS + n] : 0.f;
                        tf32_split(b0, bhi[nt][0], blo[nt][0]);
                        tf32_split(b1, bhi[nt][1], blo[nt][1]);
                    }
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                        for (int nt = 0; nt < 2; ++nt) {   // small terms first
                            mma_tf32(c[mt][nt], alo[mt], bhi[nt]);
                            mma_tf32(c[mt][nt], ahi[mt], blo[nt]);
                            mma_tf32(c[mt][nt], ahi[mt], bhi[nt]);
                        }
                }
                // back to this thread's 4 x 4 tile through the warp's own output
                // rows of ring A's slot for this step (free until the outputs
                // land there): [destination][row]
                float *stg = A + ((t & 1) * NS + n0) * RW;
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt) {
                        const int d = 8 * nt + 2 * cq, rw = 16 * mt + g;
                        stg[d * RW + rw] = c[mt][nt][0];
                        stg[(d + 1) * RW + rw] = c[mt][nt][1];
                        stg[d * RW + rw + 8] = c[mt][nt][2];
                        stg[(d + 1) * RW + rw + 8] = c[mt][nt][3];
                    }
                __syncwarp();
                const int ql = qd - 4 * warp;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 v = *reinterpret_cast<const float4 *>(stg + (4 * ql + u) * RW + r0);
                    acc[0][u] = v.x; acc[1][u] = v.y; acc[2][u] = v.z; acc[3][u] = v.w;
                }
                __syncwarp();
            } else {
                int s8 = 0;
                for (; s8 + 8 <= NS; s8 += 8) block(s8, 8);
                if (s8 < NS) block(s8, NS - s8);
            }
            // emissions, scale, outputs
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
                    if (valid[i] && sc[i] > 0.f) v = acc[i][u] * sc[i] * emit_g(P, eMg, eIg, eDg, 4 * qd + u, xr[i], yj);
                    if (4 * qd + u == P.s_slot) v = origin ? 1.f : 0.f;   // F[0,0,start] = 1
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
                if (valid[i] && P.lat) {
                    const int64_t cell = latc + (int64_t)t * RW + r;
                    float *rec = P.lat + cell * ES;
                    *reinterpret_cast<float4 *>(rec + 4 * qd) = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
                    if (qd == 0) {
                        for (int s2 = KS; s2 < NS; ++s2) rec[s2] = (origin && s2 == P.s_slot) ? 1.f : 0.f;
                        reinterpret_cast<int *>(rec)[NS] = origin ? 0 : Eo[i];
                    }
                }
                if (pub && valid[i] && row == Lx && j == Ly && si + 1 == m.n_stripes) {   // P(x,y): my quad's share
                    double a = 0.0;
#pragma unroll
                    for (int u = 0; u < 4; ++u) a += (double)acc[i][u] * (double)sm[L.chiE + 4 * qd + u];
                    llp[qd] = a;
                    if (qd == 0) llE = origin ? 0 : Eo[i];
                }
            }
            if (si == 0 && t == 0 && qd == 0 && rg == 0 && P.s_slot >= KS) {   // origin: F[0,0,start] = 1
                A[(0 * NS + P.s_slot) * RW + 0] = 1.f;
                B[(0 * NS + P.s_slot) * BW + 1] = 1.f;
                atomicMax(MX + 0 * BW + 1, __float_as_int(1.f));
            }
        }
        // ---- halo column t+1 for the next step (warp 0)
        if (warp == 0 && t + 1 <= T_last && !fetch_halo(t + 1)) misc[(k + 1) & 1] = 1;
    }
    __syncthreads();
    if (!pub) return;   // recomputed: the lattice records are all this stripe writes
    if (!aborted && has_below) {   // the last bottom-row cell(s) still to publish
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
    // the terminal cell's exponent was kept by the qd == 0 thread of its row group
    if (!aborted && si + 1 == m.n_stripes) {
        int *Eterm = misc + 4;
        const int rT = Lx - i0;
        if (active && qd == 0 && rg == (rT >> 2)) *Eterm = llE;
        __syncthreads();
        if (tid == 0) {
            double acc = 0.0;
            for (int q = 0; q < NQd; ++q) acc += llp[q];
            if (Lx == 0 && Ly == 0 && P.s_slot >= KS) acc += (double)sm[L.chiE + P.s_slot];   // origin = terminal
            const int Et = *Eterm;
            double ll = NEG_INF_LL;
            if (acc > 0.0 && isfinite(acc) && Et > EXP_NONE) ll = log(acc) + (double)Et * LN2;
            else atomicOr(P.status + p, PHMM_ST_ZERO_LL);
            P.ll[p] = ll;
        }
    }
    // stripe complete (lattice and, for the last stripe, the log-likelihood):
    // the count pass may start on it
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(prog_mine, Ly + 2);
}

// ---------------------------------------------------------------- backward recursion
// b[row][s] = sum_k chi[s][k] w_succ(type k)[row][k] for the destination
// slots s < KS (the count pass needs b only there); w = e b is what the
// successor rings and the edge rows carry.  Edge records of the stripe
// below are its top row, and progress counts published columns from the
// right (Ly + 1 - column).
__device__ void bwd_rec_stripe_wd(const KParams &P, int p, int si, const SmemWd &L, float *sm, unsigned char *smb) {
    const int NS = P.NS, KS = P.kend[2], NQd = KS / 4, N = P.N;
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
    const int64_t latc = P.stripe_lat ? P.stripe_lat[m.stripe_base + si] : m.lat_base + (int64_t)si * (RW + Ly) * RW;
    const bool pub = !P.recompute;   // a recomputed stripe publishes nothing (its edge rows exist)
    float *chiB = sm + L.chi, *A = sm + L.A, *B = sm + L.B;
    int *E = reinterpret_cast<int *>(sm) + L.E;
    int *MX = reinterpret_cast<int *>(sm) + L.MX;
    int *misc = reinterpret_cast<int *>(sm) + L.misc;
    unsigned char *ys = smb + L.ys;
    const int BW = RW + 4;
    {
        const float *chi = P.chi + (int64_t)p * P.chi_stride;
        for (int idx = tid; idx < KS * KS; idx += nt) {   // chiB[k][s]
            const int k = idx / KS, s = idx % KS;
            const int os = P.slot_orig[s], ok = P.slot_orig[k];
            const int kt = P.slot_type[k];
            float v = 0.f;
            if (os >= 0 && ok >= 0 && (kt == T_M || kt == T_I || kt == T_D)) v = __ldg(chi + os * N + ok);
            chiB[idx] = v;
        }
        for (int s = tid; s < NS; s += nt) {
            const int os = P.slot_orig[s];
            sm[L.chiE + s] = os >= 0 ? __ldg(chi + os * N + P.e_idx) : 0.f;
        }
        for (int idx = tid; idx < 2 * KS * RW; idx += nt) A[idx] = 0.f;
        for (int idx = tid; idx < 3 * KS * BW; idx += nt) B[idx] = 0.f;
        for (int idx = tid; idx < 4 * BW; idx += nt) { E[idx] = EXP_NONE; MX[idx] = 0; }
        for (int j = tid; j <= Ly; j += nt) {
            int c = 0;
            if (j >= 1) c = min((int)P.res[m.y_off + j - 1], 20);
            ys[j] = (unsigned char)c;
        }
        if (tid == 0) { misc[0] = 0; misc[1] = 0; }
    }
    const float *eMg = P.eM + (int64_t)p * P.eM_stride;
    const float *eIg = P.eI + (int64_t)p * P.eID_stride;
    const float *eDg = P.eD + (int64_t)p * P.eID_stride;
    int xr[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int row = i0 + r0 + i;
        xr[i] = (row >= 1 && row <= Lx) ? min((int)P.res[m.x_off + row - 1], 20) : 0;
    }
    const int kb0 = P.kbeg[0], ke0 = P.kend[0], kb1 = P.kbeg[1], ke1 = P.kend[1], kb2 = P.kbeg[2], ke2 = P.kend[2];
    const int T_last = (nrows - 1) + Ly;
    // halo: row i0+RW (the stripe below's top row) at column c sits at step c + RW:
    // B slot (c + RW) % 3, index RW + 3; exponent / maximum slot (c + RW) & 3, index RW
    auto fetch_halo = [&](int col) -> bool {
        if (!has_below || col < 0 || col > Ly) return true;
        int ok = 1;
        if (lane == 0 && pub) ok = wait_geq(prog_below, Ly + 1 - col, P.spin_limit) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) return false;
        const int bs = (col + RW) % 3, es = (col + RW) & 3;
        const float *src = edge_below + (int64_t)col * ES;
        for (int k = lane; k < KS; k += 32) B[(bs * KS + k) * BW + RW + 3] = __ldcg(src + k);
        if (lane == 0) {
            E[es * BW + RW] = __ldcg(reinterpret_cast<const int *>(src) + NS);
            MX[es * BW + RW] = __ldcg(reinterpret_cast<const int *>(src) + NS + 1);
        }
        return true;
    };
    // top row of step t (column t) -> edge row for the stripe above
    auto publish_top = [&](int t) {
        if (!pub || !has_above || t < 0 || t > Ly) return;
        float *dst = edge_mine + (int64_t)t * ES;
        for (int k = lane; k < KS; k += 32) dst[k] = A[((t & 1) * KS + k) * RW + 0];
        if (lane == 0) {
            reinterpret_cast<int *>(dst)[NS] = E[(t & 3) * BW + 0];
            reinterpret_cast<int *>(dst)[NS + 1] = MX[(t & 3) * BW + 0];
        }
        __threadfence();
        __syncwarp();
        if (lane == 0 && ((t % WPUB) == 0)) st_release(prog_mine, Ly + 1 - t);
    };
    __syncthreads();
    if (warp == 0 && !fetch_halo(T_last - (RW - 1))) misc[0] = 1;
    bool aborted = false;
    int k = 0;
    for (int t = T_last; t >= 0; --t, ++k) {
        __syncthreads();
        if (misc[k & 1]) { aborted = true; break; }
        if (tid == 0) misc[(k + 1) & 1] = 0;
        for (int r = tid; r < RW; r += nt) MX[((t - 1) & 3) * BW + r] = 0;   // maxima of step t-1
        if (warp == (nt > 32 ? 1 : 0)) publish_top(t + 1);
        if (active) {
            // per row: successor exponent of each type and the output exponent
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
                        if (mb > 0 && e > EXP_NONE) { EsI[i] = e; vI = e + exp_of_max(mb); }
                    }
                    if (row + 1 <= Lx) {
                        const int mb = MX[((t + 1) & 3) * BW + r + 1], e = E[((t + 1) & 3) * BW + r + 1];
                        if (mb > 0 && e > EXP_NONE) { EsD[i] = e; vD = e + exp_of_max(mb); }
                    }
                    if (row + 1 <= Lx && j + 1 <= Ly) {
                        const int mb = MX[((t + 2) & 3) * BW + r + 1], e = E[((t + 2) & 3) * BW + r + 1];
                        if (mb > 0 && e > EXP_NONE) { EsM[i] = e; vM = e + exp_of_max(mb); }
                    }
                }
                Eo[i] = term[i] ? 0 : max(max(vI, vD), vM);
            }
            // one accumulator over the destinations in slot order (M, I, D), each
            // successor value pre-scaled by its type's power of two: the same
            // rounding sequence as the forward's contraction, so the float32
            // drift of the two recursions stays consistent for the posteriors
            float sM[4], sI[4], sD[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                sM[i] = (EsM[i] > EXP_NONE) ? pow2d(EsM[i] - Eo[i]) : 0.f;
                sI[i] = (EsI[i] > EXP_NONE) ? pow2d(EsI[i] - Eo[i]) : 0.f;
                sD[i] = (EsD[i] > EXP_NONE) ? pow2d(EsD[i] - Eo[i]) : 0.f;
            }
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[i][u] = 0.f;
            const float4 *cb4 = reinterpret_cast<const float4 *>(chiB) + qs;   // chiB[k][4qs..]
            const int NQk = KS / 4;
            // compensated blocked summation above 64 slots, as in the forward
            // (8 destinations per block tile); the plain sequential sum below
            const bool blocked = P.NS > 64;
            float cmp[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int u = 0; u < 4; ++u) cmp[i][u] = 0.f;
            auto contract = [&](const float *base, int stride, int k0, int k1, const float (&sc)[4]) {
                for (int kb = k0; kb < k1; kb += 8) {
                    const int nb = min(8, k1 - kb);
                    float bt[4][4];
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int u = 0; u < 4; ++u) bt[i][u] = blocked ? 0.f : acc[i][u];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        if (q < nb) {
                            const int kk = kb + q;
                            const float4 w = *reinterpret_cast<const float4 *>(base + kk * stride);
                            const float4 c = cb4[kk * NQk];
                            const float wa[4] = {w.x * sc[0], w.y * sc[1], w.z * sc[2], w.w * sc[3]};
                            const float ca[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
                            for (int i = 0; i < 4; ++i)
#pragma unroll
                                for (int u = 0; u < 4; ++u) bt[i][u] = fmaf(wa[i], ca[u], bt[i][u]);
                        }
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            if (blocked) {
                                const float y = bt[i][u] - cmp[i][u];
                                const float tt = acc[i][u] + y;
                                cmp[i][u] = (tt - acc[i][u]) - y;
                                acc[i][u] = tt;
                            } else {
                                acc[i][u] = bt[i][u];
                            }
                        }
                }
            };
            contract(B + ((t + 2) % 3) * KS * BW + r0 + 4, BW, kb0, ke0, sM);   // M: (row+1, t+2)
            contract(A + ((t + 1) & 1) * KS * RW + r0, RW, kb1, ke1, sI);       // I: (row, t+1)
            contract(B + ((t + 1) % 3) * KS * BW + r0 + 4, BW, kb2, ke2, sD);   // D: (row+1, t+1)
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
                        mxr[i] = fmaxf(mxr[i], b * emit_g(P, eMg, eIg, eDg, 4 * qs + u, xr[i], yj));
                    }
                    bv[i][u] = b;
                }
            }
            // w = e b into the rings; b and its exponent into the lattice
            const int sa = t & 1, sb = t % 3;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = r0 + i, j = t - r;
                const int yj = valid[i] ? ys[j] : 0;
                float wv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    wv[u] = valid[i] ? bv[i][u] * emit_g(P, eMg, eIg, eDg, 4 * qs + u, xr[i], yj) : 0.f;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    A[(sa * KS + 4 * qs + u) * RW + r] = wv[u];
                    B[(sb * KS + 4 * qs + u) * BW + r + 3] = wv[u];
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
        if (warp == 0 && !fetch_halo(t - RW)) misc[(k + 1) & 1] = 1;
    }
    __syncthreads();
    if (!aborted && warp == (nt > 32 ? 1 : 0)) publish_top(0);
    __syncthreads();
    if (!pub) return;   // recomputed: the lattice records are all this stripe writes
    if (tid == 0) {
        if (has_above) { __threadfence(); st_release(prog_mine, Ly + 1); }
        if (aborted) atomicOr(P.status + p, PHMM_ST_TIMEOUT);
    }
    __threadfence();   // stripe complete: the count pass may start on it
    __syncthreads();
    if (tid == 0) st_release(prog_mine, Ly + 2);
}

template <bool TC>
__global__ void __launch_bounds__(512) fwdbwd_wide_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemWd Lf = make_smem_wd(P.NS, P.kend[2], P.max_ly, false);
    const SmemWd Lb = make_smem_wd(P.NS, P.kend[2], P.max_ly, true);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        if (w.y & blk::BWD_ITEM) bwd_rec_stripe_wd(P, w.x, w.y & ~blk::BWD_ITEM, Lb, sm, smem_raw);
        else fwd_stripe_wd<TC>(P, w.x, w.y, Lf, sm, smem_raw);
    }
}

// ---------------------------------------------------------------- counts from both lattices
// One item = one stripe of one pair and one half (SPL = 2) of the source
// slots; 512 threads.  Per anti-diagonal step: phase A (16 threads per cell)
// forms f~ of the item's source slots and the successor operands
//   u[k] = w~_succ(k)[k] 2^(E_succ + E_f - lambda)   (w~ = e b~)
// for every destination slot; phase B accumulates the 32-cell outer products
// in 4 x 4 tiles (Kahan).  The lattice loads of the next step are issued
// before phase B.  Half 0 also forms the posteriors f~ b~ 2^(E_f + E_b -
// lambda) for the emission counts (shared-memory tables by slot and
// character, float64 reductions at the end of the stripe).
constexpr int CT = 512;          // count CTA
constexpr int SPL = 2;           // source-slot halves per stripe
constexpr int CTPT = 2;          // outer-product tiles per thread (ceil(NQ/2) * NQd <= CT * CTPT)

struct SmemWc {
    int fst, ust, tM, tI, tD;   // float offsets
    int sg;                     // int offset: emission group of each destination slot [KS]
    int bytes;
};

__host__ __device__ inline SmemWc make_smem_wc(int NS, int KS, int wM, int wI, int wD) {
    SmemWc L;
    const int SQ = ((NS / 4) + SPL - 1) / SPL;   // source quads per half
    int o = 0;
    L.fst = o; o += RW * (4 * SQ + 4);
    L.ust = o; o += RW * (KS + 4);
    L.tM = o; o += (wM * 441 + 3) & ~3;
    L.tI = o; o += (wI * 21 + 3) & ~3;
    L.tD = o; o += (wD * 21 + 3) & ~3;
    L.sg = o; o += (KS + 3) & ~3;
    L.bytes = o * 4;
    return L;
}

__device__ void count_stripe_wd(const KParams &P, int p, int si, int sp, const SmemWc &L, float *sm) {
    const int NS = P.NS, KS = P.kend[2], NQd = KS / 4, NQ = NS / 4, N = P.N, G = P.G;
    const int SQ = (NQ + SPL - 1) / SPL;
    const int sq0 = sp * SQ, sq1 = min(NQ, sq0 + SQ), nsq = sq1 - sq0;
    const int FW = 4 * SQ + 4, UW = KS + 4;
    const PairMeta m = P.meta[p];
    const int Lx = m.Lx, Ly = m.Ly;
    const int tid = threadIdx.x;
    const int i0 = si * RW;
    const int nrows = min(RW, Lx + 1 - i0);
    const bool has_below = si + 1 < m.n_stripes;
    const int ES = ls_of(NS);
    const int64_t latc = P.stripe_lat ? P.stripe_lat[m.stripe_base + si] : m.lat_base + (int64_t)si * (RW + Ly) * RW;
    const int64_t latb = m.lat_base + (int64_t)(si + 1) * (RW + Ly) * RW;
    // with checkpoints the stripe below's lattice is not kept: its row 0 is its
    // backward edge row, whose records hold w = e b (the emission already applied)
    const float *bedge_below = P.bedge + (m.edge_base + (int64_t)(si + 1) * (Ly + 1)) * ES;
    const int T_last = (nrows - 1) + Ly;
    if (nsq <= 0) return;
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
    const bool emis = sp == 0;
    float *fst = sm + L.fst, *ust = sm + L.ust, *tM = sm + L.tM, *tI = sm + L.tI, *tD = sm + L.tD;
    if (emis) {
        for (int idx = tid; idx < wM * 441; idx += CT) tM[idx] = 0.f;
        for (int idx = tid; idx < wI * 21; idx += CT) tI[idx] = 0.f;
        for (int idx = tid; idx < wD * 21; idx += CT) tD[idx] = 0.f;
    }
    const float *eMg = P.eM + (int64_t)p * P.eM_stride;
    const float *eIg = P.eI + (int64_t)p * P.eID_stride;
    const float *eDg = P.eD + (int64_t)p * P.eID_stride;
    // phase A role: cell row c, 16 threads per cell
    const int c = tid >> 4, sub = tid & 15;
    const int row = i0 + c;
    const int xc = (row >= 1 && row <= Lx) ? min((int)P.res[m.x_off + row - 1], 20) : 0;
    const int xn = (row + 1 <= Lx) ? min((int)P.res[m.x_off + row], 20) : 0;
    // phase B role: tiles (source quad, destination quad)
    const int ntile = nsq * NQd;
    float csum[CTPT][16], ccomp[CTPT][16];
#pragma unroll
    for (int a = 0; a < CTPT; ++a)
#pragma unroll
        for (int u = 0; u < 16; ++u) { csum[a][u] = 0.f; ccomp[a][u] = 0.f; }
    constexpr int KQ = 3;   // destination quads per phase-A thread: ceil(NQd / 16) <= KQ
    constexpr int FQ = 2;   // source quads per phase-A thread: ceil(SQ / 16) <= FQ
    // per item, my destination quads' types and emission-table offsets (the
    // successor's characters: x of row + 1 for M and D, y of column + 1 for M
    // and I), so no step indexes the parameter block with a per-thread index
    int qtr[KQ];
#pragma unroll
    for (int a = 0; a < KQ; ++a) {
        const int q = sub + 16 * a;
        qtr[a] = q < NQd ? P.quad_type[q] : T_NONE;
    }
    int *sg = reinterpret_cast<int *>(sm) + L.sg;   // slot groups, read from shared memory per lookup
    for (int k = tid; k < KS; k += CT) sg[k] = P.slot_group[k];
    __syncthreads();
    // prefetched lattice data of one step
    int Ef = EXP_NONE, Eb = EXP_NONE;
    int Es[KQ];
    bool sw[KQ];   // the successor record holds w = e b (a backward edge row), not b
    float4 sv[KQ], fv[FQ], bo[KQ];
    auto issue = [&](int t) {
        const int j = t - c;
        const bool valid = t >= 0 && c < nrows && j >= 0 && j <= Ly;
        const int64_t cell = latc + (int64_t)t * RW + c;
        Ef = EXP_NONE; Eb = EXP_NONE;
#pragma unroll
        for (int a = 0; a < FQ; ++a) fv[a] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int a = 0; a < KQ; ++a) {
            Es[a] = EXP_NONE; sv[a] = make_float4(0.f, 0.f, 0.f, 0.f); bo[a] = sv[a]; sw[a] = false;
        }
        if (!valid) return;
        Ef = __ldcg(reinterpret_cast<const int *>(P.lat + cell * ES) + NS);
        Eb = __ldcg(reinterpret_cast<const int *>(P.blat + cell * ES) + NS);
#pragma unroll
        for (int a = 0; a < FQ; ++a) {
            const int q = sq0 + sub + 16 * a;
            if (q < sq1) fv[a] = __ldcg(reinterpret_cast<const float4 *>(P.lat + cell * ES) + q);
        }
        const bool hI = j + 1 <= Ly, hD = row + 1 <= Lx, hM = hI && hD;
        const bool below_ok = c + 1 < nrows || has_below;
#pragma unroll
        for (int a = 0; a < KQ; ++a) {
            const int q = sub + 16 * a;
            if (q >= NQd) continue;
            if (emis) bo[a] = __ldcg(reinterpret_cast<const float4 *>(P.blat + cell * ES) + q);
            const int qt = qtr[a];
            const float *rec = nullptr;
            if (qt == T_I && hI) rec = P.blat + (latc + (int64_t)(t + 1) * RW + c) * ES;
            else if (qt == T_D && hD && below_ok)
                rec = c + 1 < nrows ? P.blat + (latc + (int64_t)(t + 1) * RW + c + 1) * ES
                                    : (P.ckpt ? bedge_below + (int64_t)j * ES : P.blat + (latb + (int64_t)j * RW) * ES);
            else if (qt == T_M && hM && below_ok)
                rec = c + 1 < nrows ? P.blat + (latc + (int64_t)(t + 2) * RW + c + 1) * ES
                                    : (P.ckpt ? bedge_below + (int64_t)(j + 1) * ES
                                              : P.blat + (latb + (int64_t)(j + 1) * RW) * ES);
            if (rec) {
                Es[a] = __ldcg(reinterpret_cast<const int *>(rec) + NS);
                sv[a] = __ldcg(reinterpret_cast<const float4 *>(rec) + q);
                sw[a] = P.ckpt && c + 1 >= nrows && qt != T_I;
            }
        }
    };
    issue(T_last);
    for (int t = T_last; t >= 0; --t) {
        // ================= phase A
        {
            const int j = t - c;
            const bool valid = c < nrows && j >= 0 && j <= Ly;
            const bool live = valid && Ef > EXP_NONE;
            const int yj = (valid && j >= 1) ? min((int)P.res[m.y_off + j - 1], 20) : 0;
            const int yn = (valid && j + 1 <= Ly) ? min((int)P.res[m.y_off + j], 20) : 0;
            const bool term = valid && row == Lx && j == Ly;
#pragma unroll
            for (int a = 0; a < FQ; ++a) {
                const int q = sq0 + sub + 16 * a;
                if (q < sq1) {
                    const float4 f = live ? fv[a] : make_float4(0.f, 0.f, 0.f, 0.f);
                    *reinterpret_cast<float4 *>(fst + c * FW + 4 * (q - sq0)) = f;
                }
            }
#pragma unroll
            for (int a = 0; a < KQ; ++a) {
                const int q = sub + 16 * a;
                if (q >= NQd) continue;
                float4 uu = make_float4(0.f, 0.f, 0.f, 0.f);
                const int qt = qtr[a];
                if (live && Es[a] > EXP_NONE && !term) {
                    int du = Es[a] + Ef - Ep;
                    if (du > 126) { du = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                    const float us = fminf(warp2::scale_pow2(rfrac, max(du, -200)), 3e38f);
                    // I: x of my row, y of column + 1; D: x of row + 1; M: both of the successor
                    // the successor's characters: M (x of row + 1, y of column + 1), I (y), D (x)
                    const float *et = qt == T_M ? eMg : (qt == T_I ? eIg : eDg);
                    const int add = qt == T_M ? xn * 21 + yn : (qt == T_I ? yn : xn);
                    const int gm = qt == T_M ? 441 : 21;
                    float e[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) e[u] = sw[a] ? 1.f : __ldg(et + sg[4 * q + u] * gm + add);
                    uu = make_float4(sv[a].x * e[0] * us, sv[a].y * e[1] * us, sv[a].z * e[2] * us, sv[a].w * e[3] * us);
                }
                *reinterpret_cast<float4 *>(ust + c * UW + 4 * q) = uu;
                // posteriors of my destination quad -> emission counts (half 0)
                if (emis && live && Eb > EXP_NONE) {
                    int dp = Ef + Eb - Ep;
                    if (dp > 126) { dp = 126; atomicOr(P.status + p, PHMM_ST_SCALE_CLAMP); }
                    const float ps = warp2::scale_pow2(rfrac, max(dp, -200));
                    const float4 f4 = __ldcg(reinterpret_cast<const float4 *>(P.lat + (latc + (int64_t)t * RW + c) * ES) + q);
                    const float pk[4] = {f4.x * bo[a].x * ps, f4.y * bo[a].y * ps, f4.z * bo[a].z * ps, f4.w * bo[a].w * ps};
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int s = 4 * q + u;
                        const int st = qt;
                        if (pk[u] == 0.f) continue;
                        if (st == T_M) atomicAdd(tM + (s - mb) * 441 + xc * 21 + yj, pk[u]);
                        else if (st == T_I) atomicAdd(tI + (s - ib) * 21 + yj, pk[u]);
                        else if (st == T_D) atomicAdd(tD + (s - db) * 21 + xc, pk[u]);
                    }
                }
            }
            // expected End transitions: n[s][End] = f(term)[s] chi[s][End] / P
            if (emis && term && live) {
                const float *chi = P.chi + (int64_t)p * P.chi_stride;
                const double fs = exp2((double)Ef - lam);
                for (int s = sub; s < NS; s += 16) {
                    const int os = P.slot_orig[s];
                    if (os < 0) continue;
                    const float f = __ldcg(P.lat + (latc + (int64_t)t * RW + c) * ES + s);
                    const double v = (double)f * (double)__ldg(chi + os * N + P.e_idx) * fs;
                    if (v != 0.0) atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + P.e_idx, v);
                }
            }
        }
        issue(t - 1);
        __syncthreads();
        // ================= phase B: 4 x 4 tiles over the step's 32 cells
#pragma unroll
        for (int a = 0; a < CTPT; ++a) {
            const int tile = tid + a * CT;
            if (tile >= ntile) continue;
            const int bs = tile / NQd, bk = tile % NQd;
            float pz[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) pz[u] = 0.f;
#pragma unroll 4
            for (int rr = 0; rr < RW; ++rr) {
                const float4 fv4 = *reinterpret_cast<const float4 *>(fst + rr * FW + 4 * bs);
                const float4 uv4 = *reinterpret_cast<const float4 *>(ust + rr * UW + 4 * bk);
                const float fa[4] = {fv4.x, fv4.y, fv4.z, fv4.w};
                const float ua[4] = {uv4.x, uv4.y, uv4.z, uv4.w};
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
    for (int a = 0; a < CTPT; ++a) {
        const int tile = tid + a * CT;
        if (tile >= ntile) continue;
        const int bs = tile / NQd, bk = tile % NQd;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int s = 4 * (sq0 + bs) + (u >> 2), kk = 4 * bk + (u & 3);
            const int os = P.slot_orig[s], ok = P.slot_orig[kk];
            const int kt = P.slot_type[kk];
            const float val = csum[a][u] - ccomp[a][u];
            if (os < 0 || ok < 0 || !(kt == T_M || kt == T_I || kt == T_D) || val == 0.f) continue;
            atomicAdd(P.n_trans + ((int64_t)p * N + os) * N + ok, (double)val * (double)__ldg(chi + os * N + ok));
        }
    }
    if (emis) {
        for (int idx = tid; idx < wM * 441; idx += CT) {
            const float v = tM[idx];
            const int s = mb + idx / 441;
            if (v != 0.f && P.slot_type[s] == T_M)
                atomicAdd(P.cntM + ((int64_t)p * G + P.slot_group[s]) * 441 + idx % 441, (double)v);
        }
        for (int idx = tid; idx < wI * 21; idx += CT) {
            const float v = tI[idx];
            const int s = ib + idx / 21;
            if (v != 0.f && P.slot_type[s] == T_I)
                atomicAdd(P.cntI + ((int64_t)p * G + P.slot_group[s]) * 21 + idx % 21, (double)v);
        }
        for (int idx = tid; idx < wD * 21; idx += CT) {
            const float v = tD[idx];
            const int s = db + idx / 21;
            if (v != 0.f && P.slot_type[s] == T_D)
                atomicAdd(P.cntD + ((int64_t)p * G + P.slot_group[s]) * 21 + idx % 21, (double)v);
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(CT, 1) count_wide_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemWc L = make_smem_wc(P.NS, P.kend[2], P.kend[0] - P.kbeg[0], P.kend[1] - P.kbeg[1],
                                  P.kend[2] - P.kbeg[2]);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        count_stripe_wd(P, w.x, w.y >> 4, w.y & 15, L, sm);
    }
}

template <bool TC>
__global__ void __launch_bounds__(512) forward_wide_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    float *sm = reinterpret_cast<float *>(smem_raw);
    const SmemWd L = make_smem_wd(P.NS, P.kend[2], P.max_ly, false);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items) break;
        const int2 w = P.items[it];
        fwd_stripe_wd<TC>(P, w.x, w.y, L, sm, smem_raw);
    }
}

}  // namespace wide
