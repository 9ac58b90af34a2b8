// viterbi.cu -- batched 2D pair-HMM Viterbi with traceback (dp/hmm.py:1976-2040).
//
// One CTA per pair sweeps the anti-diagonals of the (Lx+1) x (Ly+1) lattice in
// float64 log space, as the reference does: V[i][j][k] = max_s (V[pred(k)][s]
// + logchi[s][k]) + logemit_k(x_i, y_j), pred by the type of k (M: (i-1,j-1),
// I: (i,j-1), D: (i-1,j)); the first maximal source wins, as argmax does.
// The three live diagonals sit in the caller's workspace, the backpointers
// (one byte per cell and state) too; thread 0 then walks the path back from
// the best terminal state.  Scores that the reference keeps at NEG_INF
// (-1e30, summed like any other number) are reproduced bit for bit, so the
// path matches the reference's whenever the maxima are not exact ties
// broken differently by rounding.
#include "pairhmm.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

extern "C" __attribute__((visibility("hidden"))) void phmm_internal_set_error(const char *msg);

namespace vit {

constexpr int NT = 256;
constexpr int MAXN = 64;
constexpr double NEG = -1e30;   // the reference's NEG_INF (dp/hmm.py:108)
constexpr int TS = 0, TM = 1, TI = 2, TD = 3;

struct Meta {
    int64_t x_off, y_off, tb_off, diag_off, path_off, mask_off;
    int32_t Lx, Ly;
};

// Backpointer of a state the envelope left out (hmm_beam.py:455-476 stores
// the triple (0, 0, S) there): the traceback jumps to the origin.
constexpr uint8_t BP_ORIGIN = 255;

struct Desc {
    int N, G, e_idx, s_idx;
    int8_t type[MAXN];
    int8_t group[MAXN];
};

__global__ void __launch_bounds__(NT)
viterbi_kernel(const __grid_constant__ Desc d, const Meta *__restrict__ meta, const uint8_t *__restrict__ res,
               const double *__restrict__ lchi_all, int chi_pp, const double *__restrict__ lM,
               const double *__restrict__ lI, const double *__restrict__ lD, int emit_pp,
               double *__restrict__ diag, uint8_t *__restrict__ tb, double *__restrict__ ll_out,
               int32_t *__restrict__ path, int32_t *__restrict__ path_len, int32_t *__restrict__ status,
               const uint8_t *__restrict__ env) {
    extern __shared__ double lchi[];   // [N][N]
    const int p = blockIdx.x, tid = threadIdx.x;
    const Meta m = meta[p];
    const int N = d.N, G = d.G;
    const double *lc = lchi_all + (chi_pp ? (int64_t)p * N * N : 0);
    for (int idx = tid; idx < N * N; idx += NT) lchi[idx] = lc[idx];
    const double *eM = lM + (emit_pp ? (int64_t)p * G * 441 : 0);
    const double *eI = lI + (emit_pp ? (int64_t)p * G * 21 : 0);
    const double *eD = lD + (emit_pp ? (int64_t)p * G * 21 : 0);
    const int Lx = m.Lx, Ly = m.Ly;
    const int64_t W = (int64_t)(Lx + 1) * N;   // one diagonal, indexed by i
    double *dg = diag + m.diag_off;
    uint8_t *bp = tb + m.tb_off;
    __syncthreads();
    for (int dd = 0; dd <= Lx + Ly; ++dd) {
        double *cur = dg + (dd % 3) * W;
        const double *d1 = dg + ((dd + 2) % 3) * W;   // diagonal dd-1
        const double *d2 = dg + ((dd + 1) % 3) * W;   // diagonal dd-2
        const int i_lo = max(0, dd - Ly), i_hi = min(dd, Lx);
        const int ncell = i_hi - i_lo + 1;
        for (int item = tid; item < ncell * N; item += NT) {
            const int i = i_lo + item / N, k = item % N, j = dd - i;
            const int64_t cell = (int64_t)i * (Ly + 1) + j;
            if (dd == 0) {
                cur[i * N + k] = k == d.s_idx ? 0.0 : NEG;
                bp[cell * N + k] = 0;
                continue;
            }
            const int st = d.type[k];
            const double *pred = nullptr;
            int pi_ = -1, pj_ = -1;
            if (st == TM && i > 0 && j > 0) { pred = d2 + (i - 1) * N; pi_ = i - 1; pj_ = j - 1; }
            else if (st == TI && j > 0) { pred = d1 + i * N; pi_ = i; pj_ = j - 1; }
            else if (st == TD && i > 0) { pred = d1 + (i - 1) * N; pi_ = i - 1; pj_ = j; }
            if (env) {   // envelope (beam_viterbi_2d): the cell and its predecessor must lie inside
                const uint8_t *ep = env + m.mask_off;
                if (!ep[cell] || (pred && !ep[(int64_t)pi_ * (Ly + 1) + pj_])) {
                    cur[i * N + k] = NEG;
                    bp[cell * N + k] = BP_ORIGIN;
                    continue;
                }
            }
            if (!pred) {
                cur[i * N + k] = NEG;
                bp[cell * N + k] = 0;
                continue;
            }
            int best = 0;
            double bv = pred[0] + lchi[k];
            for (int s = 1; s < N; ++s) {
                const double v = pred[s] + lchi[s * N + k];
                if (v > bv) { bv = v; best = s; }
            }
            // characters x_{i-1}, y_{j-1} (the reference reads x[max(i-1, 0)]: only
            // i > 0 matters for M and D states, only j > 0 for M and I)
            const int xa = i > 0 ? min((int)res[m.x_off + i - 1], 20) : 0;
            const int yb = j > 0 ? min((int)res[m.y_off + j - 1], 20) : 0;
            const int g = d.group[k];
            double e = 0.0;
            if (st == TM) e = eM[g * 441 + xa * 21 + yb];
            else if (st == TI) e = eI[g * 21 + yb];
            else e = eD[g * 21 + xa];
            cur[i * N + k] = bv + e;
            bp[cell * N + k] = (uint8_t)best;
        }
        __syncthreads();
    }
    if (tid == 0) {
        const double *last = dg + ((Lx + Ly) % 3) * W + (int64_t)Lx * N;
        int best = 0;
        double bv = last[0] + lchi[d.e_idx];
        for (int s = 1; s < N; ++s) {
            const double v = last[s] + lchi[s * N + d.e_idx];
            if (v > bv) { bv = v; best = s; }
        }
        ll_out[p] = bv;
        if (!(bv > -1e29)) atomicOr(status + p, PHMM_ST_ZERO_LL);
        int32_t *pp = path + m.path_off * 3;
        int n = 0, ci = Lx, cj = Ly, ck = best;
        while ((ci > 0 || cj > 0) && n < Lx + Ly) {
            pp[3 * n] = ci; pp[3 * n + 1] = cj; pp[3 * n + 2] = ck;
            ++n;
            const int st = d.type[ck];
            const int nk = bp[((int64_t)ci * (Ly + 1) + cj) * N + ck];
            if (nk == BP_ORIGIN) { ci = 0; cj = 0; ck = d.s_idx; break; }
            // a state with no predecessor cell here (S/E, or M/I/D on the lattice
            // edge) kept the reference's zero pointers: the walk ends at the origin
            if (st == TM && ci > 0 && cj > 0) { --ci; --cj; }
            else if (st == TI && cj > 0) { --cj; }
            else if (st == TD && ci > 0) { --ci; }
            else { ci = 0; cj = 0; }
            ck = nk;
        }
        pp[3 * n] = 0; pp[3 * n + 1] = 0; pp[3 * n + 2] = d.s_idx;
        ++n;
        for (int a = 0, b = n - 1; a < b; ++a, --b)
            for (int c = 0; c < 3; ++c) {
                const int32_t t = pp[3 * a + c];
                pp[3 * a + c] = pp[3 * b + c];
                pp[3 * b + c] = t;
            }
        path_len[p] = n;
    }
}

}  // namespace vit

static int vit_fail(int code, const char *msg) {
    phmm_internal_set_error(msg);
    return code;
}

static size_t vit_align(size_t v) { return (v + 255) & ~(size_t)255; }

struct VitLayout {
    std::vector<vit::Meta> meta;
    size_t o_diag, o_tb, total;
};

static int vit_layout(const phmm_batch *b, int N, VitLayout &L) {
    const int P = b->n_pairs;
    L.meta.resize(P);
    int64_t tb = 0, dg = 0, pth = 0, mk = 0;
    for (int p = 0; p < P; ++p) {
        const int Lx = b->Lx_host[p], Ly = b->Ly_host[p];
        if (Lx < 0 || Ly < 0) return vit_fail(PHMM_E_ARG, "phmm_viterbi: negative length");
        L.meta[p] = vit::Meta{b->x_off_host[p], b->y_off_host[p], tb, dg, pth, mk, Lx, Ly};
        mk += (int64_t)(Lx + 1) * (Ly + 1);
        tb += (int64_t)(Lx + 1) * (Ly + 1) * N;
        dg += 3 * (int64_t)(Lx + 1) * N;
        pth += Lx + Ly + 1;
    }
    L.o_diag = vit_align(sizeof(vit::Meta) * (size_t)P);
    L.o_tb = vit_align(L.o_diag + sizeof(double) * (size_t)dg);
    L.total = vit_align(L.o_tb + (size_t)tb);
    return PHMM_OK;
}

extern "C" int phmm_viterbi_workspace_bytes(const phmm_model_desc *model, const phmm_batch *batch, size_t *bytes) {
    if (!model || !batch || !bytes) return vit_fail(PHMM_E_ARG, "phmm_viterbi_workspace_bytes: null argument");
    *bytes = 0;
    if (batch->n_pairs <= 0) return PHMM_OK;
    if (!batch->Lx_host || !batch->Ly_host || !batch->x_off_host || !batch->y_off_host)
        return vit_fail(PHMM_E_ARG, "phmm_viterbi: null host length or offset array");
    VitLayout L;
    int rc = vit_layout(batch, model->n_states, L);
    if (rc) return rc;
    *bytes = L.total;
    return PHMM_OK;
}

extern "C" int phmm_viterbi(const phmm_model_desc *model, const phmm_batch *batch, const double *log_chi,
                            const double *log_emit_M, const double *log_emit_I, const double *log_emit_D,
                            void *workspace, size_t workspace_bytes, double *ll_out, int32_t *path,
                            int32_t *path_len, int32_t *status_out, void *stream) {
    using namespace vit;
    if (!model || !model->state_types || !model->state_group || !batch)
        return vit_fail(PHMM_E_ARG, "phmm_viterbi: bad model description or batch");
    const int N = model->n_states, G = model->n_groups, P = batch->n_pairs;
    if (N < 2 || N > MAXN) return vit_fail(PHMM_E_ARG, "phmm_viterbi: n_states must be in 2..64");
    if (G < 1) return vit_fail(PHMM_E_ARG, "phmm_viterbi: n_groups must be positive");
    if (P < 0) return vit_fail(PHMM_E_ARG, "phmm_viterbi: negative n_pairs");
    if (P == 0) return PHMM_OK;
    if (!batch->Lx_host || !batch->Ly_host || !batch->x_off_host || !batch->y_off_host || !batch->residues ||
        !log_chi || !log_emit_M || !log_emit_I || !log_emit_D || !workspace || !ll_out || !path || !path_len ||
        !status_out)
        return vit_fail(PHMM_E_ARG, "phmm_viterbi: null pointer");
    if ((uintptr_t)workspace & 255) return vit_fail(PHMM_E_ARG, "phmm_viterbi: workspace must be 256-byte aligned");
    Desc d;
    std::memset(&d, 0, sizeof(d));
    d.N = N;
    d.G = G;
    d.e_idx = -1;
    d.s_idx = 0;
    for (int s = 0; s < N; ++s) {
        d.type[s] = model->state_types[s];
        d.group[s] = (int8_t)std::max(0, std::min(G - 1, (int)model->state_group[s]));
        if (d.type[s] == 4 && d.e_idx < 0) d.e_idx = s;
    }
    if (d.type[0] != TS || d.e_idx < 0) return vit_fail(PHMM_E_ARG, "phmm_viterbi: state 0 must be S and one state E");
    VitLayout L;
    int rc = vit_layout(batch, N, L);
    if (rc) return rc;
    if (workspace_bytes < L.total) return vit_fail(PHMM_E_ARG, "phmm_viterbi: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    cudaError_t e = cudaMemcpyAsync(ws, L.meta.data(), sizeof(Meta) * P, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status_out, 0, sizeof(int32_t) * P, st);
    if (e != cudaSuccess) return vit_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    const size_t smem = sizeof(double) * N * N;
    e = cudaFuncSetAttribute(viterbi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return vit_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    viterbi_kernel<<<P, NT, smem, st>>>(d, (const Meta *)ws, batch->residues, log_chi, batch->chi_per_pair,
                                       log_emit_M, log_emit_I, log_emit_D, batch->emit_per_pair,
                                       (double *)(ws + L.o_diag), (uint8_t *)(ws + L.o_tb), ll_out, path, path_len,
                                       status_out, batch->cell_mask);
    e = cudaGetLastError();
    if (e != cudaSuccess) return vit_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}
