// fb1d.cu -- batched 1D alignment-conditioned forward-backward.
//
// Along a fixed alignment the pair HMM is an ordinary HMM over the alignment
// columns (dp/hmm.py:127-250, 471-607): column l emits through the states of
// its type only (dp/hmm.py:854-1082), alpha_l = (alpha_{l-1} chi) .* e_l.
// One CTA per pair walks its columns: thread k owns destination k, chi is
// staged in shared memory with an odd row stride (row and column walks are
// both conflict-free), every alpha / beta vector is rescaled by a power of
// two after its step (exact, the exponents kept as integers), and the
// expected transition counts accumulate during the backward walk in
// Kahan-compensated float32 in shared memory, one entry per thread slot.
// Emission tables come as linear per-column rows [sum L][N]; a second
// kernel builds them from an alignment and the per-group tables the 2D path
// uses.
#include "pairhmm.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

extern "C" __attribute__((visibility("hidden"))) void phmm_internal_set_error(const char *msg);

namespace fb1 {

constexpr int NT = 128;          // threads per pair
constexpr int MAXN = 64;         // states (chi and the count accumulators in shared memory)
constexpr int EXPN = -(1 << 28); // exponent of an all-zero vector
constexpr double LN2 = 0.69314718055994530942;

struct Meta {
    int64_t off;   // first column
    int32_t L;
    int32_t pad;
};

__device__ __forceinline__ int exp2_of(float m) {   // m * 2^-e in [0.5, 1) for m > 0
    int e;
    frexpf(m, &e);
    return e;
}

__device__ float block_max(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float m = red[0];
    for (int w = 1; w < NT / 32; ++w) m = fmaxf(m, red[w]);
    return m;
}

__device__ double block_sum_d(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    return s;
}

// shared layout: chi [N][NP] (NP = N | 1), a/b/w vectors, count sums and compensations
__global__ void __launch_bounds__(NT)
fb1d_kernel(const Meta *__restrict__ meta, int N, const float *__restrict__ chi_all, int chi_per_pair,
            const float *__restrict__ emit, int init_state, int final_state, float *__restrict__ alpha,
            int *__restrict__ aexp, double *__restrict__ ll_out, double *__restrict__ n_out,
            float *__restrict__ post, int32_t *__restrict__ status) {
    extern __shared__ float smf[];
    __shared__ float redf[NT / 32];
    __shared__ double redd[NT / 32];
    const int p = blockIdx.x, tid = threadIdx.x;
    const Meta m = meta[p];
    const int NP = N | 1;
    float *chi = smf;                 // [N][NP]
    float *va = chi + N * NP;         // [N] current vector
    float *vw = va + MAXN;            // [N] work vector
    float *cs = vw + MAXN;            // [N*N] count sums
    float *cc = cs + MAXN * MAXN;     // [N*N] count compensations
    const float *chig = chi_all + (chi_per_pair ? (int64_t)p * N * N : 0);
    for (int idx = tid; idx < N * N; idx += NT) {
        chi[(idx / N) * NP + idx % N] = chig[idx];
        cs[idx] = 0.f;
        cc[idx] = 0.f;
    }
    __syncthreads();
    const int L = m.L;
    double *nt = n_out + (int64_t)p * N * N;
    if (L == 0) {   // empty alignment: S -> E directly
        const float c = chi[init_state * NP + final_state];
        if (tid == 0) {
            ll_out[p] = c > 0.f ? log((double)c) : -1e30;
            if (!(c > 0.f)) atomicOr(status + p, PHMM_ST_ZERO_LL);
        }
        for (int idx = tid; idx < N * N; idx += NT) nt[idx] = (idx == init_state * N + final_state) ? 1.0 : 0.0;
        return;
    }
    const float *em = emit + m.off * N;
    float *al = alpha + m.off * N;
    int *ae = aexp + m.off;
    // ---- forward
    int cum = 0;
    for (int l = 0; l < L; ++l) {
        float mx = 0.f;
        for (int k = tid; k < N; k += NT) {
            float s = 0.f;
            if (l == 0) {
                s = chi[init_state * NP + k];
            } else {
                for (int j = 0; j < N; ++j) s = fmaf(va[j], chi[j * NP + k], s);
            }
            const float v = s * em[(int64_t)l * N + k];
            vw[k] = v;
            mx = fmaxf(mx, v);
        }
        mx = block_max(mx, redf);   // (barriers: every vw written, every va read)
        const int e = mx > 0.f ? exp2_of(mx) : 0;
        for (int k = tid; k < N; k += NT) {
            const float v = mx > 0.f ? ldexpf(vw[k], -e) : 0.f;
            va[k] = v;
            al[(int64_t)l * N + k] = v;
        }
        cum = (mx > 0.f && cum > EXPN) ? cum + e : EXPN;
        if (tid == 0) ae[l] = cum;
        __syncthreads();
    }
    double pz = 0.0;
    for (int k = tid; k < N; k += NT) pz += (double)va[k] * (double)chi[k * NP + final_state];
    pz = block_sum_d(pz, redd);
    const bool ok = pz > 0.0 && cum > EXPN;
    const double lp2 = ok ? log2(pz) + (double)cum : 0.0;   // log2 P
    if (tid == 0) {
        ll_out[p] = ok ? lp2 * LN2 : -1e30;
        if (!ok) atomicOr(status + p, PHMM_ST_ZERO_LL);
    }
    if (!ok) {
        for (int idx = tid; idx < N * N; idx += NT) nt[idx] = 0.0;
        return;
    }
    // ---- backward, with the counts
    auto add = [&](int idx, float v) {   // Kahan
        const float y = v - cc[idx];
        const float t = cs[idx] + y;
        cc[idx] = (t - cs[idx]) - y;
        cs[idx] = t;
    };
    // terminal: n[s][final] += a_{L-1}[s] chi[s][final] / P; b_{L-1}[s] = chi[s][final]
    {
        const float f = (float)exp2((double)ae[L - 1] - lp2);
        for (int s = tid; s < N; s += NT) add(s * N + final_state, al[(int64_t)(L - 1) * N + s] * chi[s * NP + final_state] * f);
    }
    float mx = 0.f;
    for (int s = tid; s < N; s += NT) {
        vw[s] = chi[s * NP + final_state];
        mx = fmaxf(mx, vw[s]);
    }
    mx = block_max(mx, redf);
    int eb = mx > 0.f ? exp2_of(mx) : 0;
    for (int s = tid; s < N; s += NT) va[s] = mx > 0.f ? ldexpf(vw[s], -eb) : 0.f;
    int cumb = mx > 0.f ? eb : EXPN;
    __syncthreads();
    if (post) {
        const float f = (float)exp2((double)ae[L - 1] + (double)cumb - lp2);
        for (int k = tid; k < N; k += NT)
            post[(m.off + L - 1) * N + k] = al[(int64_t)(L - 1) * N + k] * va[k] * f;
    }
    for (int l = L - 2; l >= -1; --l) {
        // w[k] = e_{l+1}[k] b_{l+1}[k]
        for (int k = tid; k < N; k += NT) vw[k] = em[(int64_t)(l + 1) * N + k] * va[k];
        __syncthreads();
        if (l < 0) break;   // vw now holds e_0 .* b_0 for the initial counts
        // interior counts: n[s][k] += a_l[s] chi[s][k] w[k] 2^(A_l + B_{l+1} - log2 P)
        const float f = (float)exp2((double)ae[l] + (double)cumb - lp2);
        const float *alr = al + (int64_t)l * N;
        for (int idx = tid; idx < N * N; idx += NT) {
            const int s = idx / N, k = idx % N;
            const float v = alr[s] * chi[s * NP + k] * vw[k];
            if (v != 0.f) add(idx, v * f);
        }
        // b_l[s] = sum_k chi[s][k] w[k]
        float mxb = 0.f;
        float bnew[(MAXN + NT - 1) / NT];
        for (int s = tid, q = 0; s < N; s += NT, ++q) {
            float acc = 0.f;
            for (int k = 0; k < N; ++k) acc = fmaf(chi[s * NP + k], vw[k], acc);
            bnew[q] = acc;
            mxb = fmaxf(mxb, acc);
        }
        mxb = block_max(mxb, redf);
        eb = mxb > 0.f ? exp2_of(mxb) : 0;
        for (int s = tid, q = 0; s < N; s += NT, ++q) va[s] = mxb > 0.f ? ldexpf(bnew[q], -eb) : 0.f;
        cumb = (mxb > 0.f && cumb > EXPN) ? cumb + eb : EXPN;
        __syncthreads();
        if (post) {
            const float g = (float)exp2((double)ae[l] + (double)cumb - lp2);
            for (int k = tid; k < N; k += NT) post[(m.off + l) * N + k] = alr[k] * va[k] * g;
        }
    }
    // initial: n[init][k] += chi[init][k] e_0[k] b_0[k] / P  (vw = e_0 .* b_0 at exponent cumb)
    {
        const float f = (float)exp2((double)cumb - lp2);
        for (int k = tid; k < N; k += NT) add(init_state * N + k, chi[init_state * NP + k] * vw[k] * f);
    }
    __syncthreads();
    for (int idx = tid; idx < N * N; idx += NT) nt[idx] = (double)cs[idx] - (double)cc[idx];
}

// Per-column emissions of an alignment: column l of type c (1 M, 2 I, 3 D)
// emits through the states of type c with the per-group tables of the 2D
// path (M: table_M[g][anc][desc]; I: table_I[g][desc]; D: table_D[g][anc]);
// other states (and S, E) get 0.
struct EmitDesc {
    int N;
    int8_t type[MAXN];
    int8_t group[MAXN];
};

__global__ void __launch_bounds__(256)
emit1d_kernel(const __grid_constant__ EmitDesc ed, const Meta *__restrict__ meta, const uint8_t *__restrict__ cols,
              const uint8_t *__restrict__ anc, const uint8_t *__restrict__ desc, const float *__restrict__ tM,
              const float *__restrict__ tI, const float *__restrict__ tD, int per_pair, int G,
              float *__restrict__ emit, int32_t *__restrict__ status) {
    const int p = blockIdx.x;
    const Meta m = meta[p];
    const int N = ed.N;
    const float *M_ = tM + (per_pair ? (int64_t)p * G * 441 : 0);
    const float *I_ = tI + (per_pair ? (int64_t)p * G * 21 : 0);
    const float *D_ = tD + (per_pair ? (int64_t)p * G * 21 : 0);
    for (int64_t idx = threadIdx.x; idx < (int64_t)m.L * N; idx += blockDim.x) {
        const int64_t l = idx / N;
        const int s = (int)(idx % N);
        const int c = cols[m.off + l];
        int a = anc[m.off + l], b = desc[m.off + l];
        if (a > 20 || b > 20) {
            atomicOr(status + p, PHMM_ST_BAD_RESIDUE);
            a = a > 20 ? 20 : a;
            b = b > 20 ? 20 : b;
        }
        float v = 0.f;
        if (c == ed.type[s]) {
            const int g = ed.group[s];
            if (c == 1) v = M_[g * 441 + a * 21 + b];
            else if (c == 2) v = I_[g * 21 + b];
            else if (c == 3) v = D_[g * 21 + a];
        }
        emit[(m.off + l) * N + s] = v;
    }
}

}  // namespace fb1

static int fb1_fail(int code, const char *msg) {
    phmm_internal_set_error(msg);
    return code;
}

static size_t fb1_align(size_t v) { return (v + 255) & ~(size_t)255; }

static int fb1_layout(int P, const int32_t *L_host, const int64_t *off_host, int N, size_t *cols_out,
                      size_t *o_alpha, size_t *o_aexp, size_t *total) {
    size_t cols = 0;
    for (int p = 0; p < P; ++p) {
        if (L_host[p] < 0 || off_host[p] < 0) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: negative length or offset");
        cols = std::max(cols, (size_t)(off_host[p] + L_host[p]));
    }
    const size_t o_meta = 0;
    *o_alpha = fb1_align(o_meta + sizeof(fb1::Meta) * (size_t)P);
    *o_aexp = fb1_align(*o_alpha + sizeof(float) * cols * N);
    *total = fb1_align(*o_aexp + sizeof(int) * cols);
    *cols_out = cols;
    return PHMM_OK;
}

extern "C" int phmm_fb1d_workspace_bytes(const phmm_fb1d_batch *b, size_t *bytes) {
    if (!b || !bytes) return fb1_fail(PHMM_E_ARG, "phmm_fb1d_workspace_bytes: null argument");
    *bytes = 0;
    if (b->n_pairs <= 0) return PHMM_OK;
    if (!b->L_host || !b->off_host) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: null host length or offset array");
    size_t cols, oa, oe, total;
    int rc = fb1_layout(b->n_pairs, b->L_host, b->off_host, b->n_states, &cols, &oa, &oe, &total);
    if (rc) return rc;
    *bytes = total;
    return PHMM_OK;
}

extern "C" int phmm_fb1d(const phmm_fb1d_batch *b, void *workspace, size_t workspace_bytes, double *ll_out,
                         double *n_trans, float *posteriors, int32_t *status_out, void *stream) {
    using namespace fb1;
    if (!b) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: null batch");
    const int P = b->n_pairs, N = b->n_states;
    if (P < 0) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: negative n_pairs");
    if (P == 0) return PHMM_OK;
    if (N < 2 || N > MAXN) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: n_states must be in 2..64");
    if (b->init_state < 0 || b->init_state >= N || b->final_state < 0 || b->final_state >= N)
        return fb1_fail(PHMM_E_ARG, "phmm_fb1d: bad init or final state");
    if (!b->L_host || !b->off_host || !b->emit || !b->chi || !ll_out || !n_trans || !status_out || !workspace)
        return fb1_fail(PHMM_E_ARG, "phmm_fb1d: null pointer");
    if ((uintptr_t)workspace & 255) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: workspace must be 256-byte aligned");
    size_t cols, oa, oe, total;
    int rc = fb1_layout(P, b->L_host, b->off_host, N, &cols, &oa, &oe, &total);
    if (rc) return rc;
    if (workspace_bytes < total) return fb1_fail(PHMM_E_ARG, "phmm_fb1d: workspace too small");
    std::vector<Meta> meta(P);
    for (int p = 0; p < P; ++p) meta[p] = Meta{b->off_host[p], b->L_host[p], 0};
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    cudaError_t e = cudaMemcpyAsync(ws, meta.data(), sizeof(Meta) * P, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status_out, 0, sizeof(int32_t) * P, st);
    if (e != cudaSuccess) return fb1_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    const int NP = N | 1;
    const size_t smem = sizeof(float) * ((size_t)N * NP + 2 * MAXN + 2 * MAXN * MAXN);
    e = cudaFuncSetAttribute(fb1d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fb1_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    fb1d_kernel<<<P, NT, smem, st>>>((const Meta *)ws, N, b->chi, b->chi_per_pair, b->emit, b->init_state,
                                    b->final_state, (float *)(ws + oa), (int *)(ws + oe), ll_out, n_trans,
                                    posteriors, status_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fb1_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}

extern "C" int phmm_fb1d_emissions(const phmm_model_desc *model, int32_t n_pairs, const int32_t *L_host,
                                   const int64_t *off_host, const uint8_t *cols, const uint8_t *anc,
                                   const uint8_t *desc, const float *emit_M, const float *emit_I,
                                   const float *emit_D, int32_t emit_per_pair, void *workspace,
                                   size_t workspace_bytes, float *emit, int32_t *status_out, void *stream) {
    using namespace fb1;
    if (!model || !model->state_types || !model->state_group)
        return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: bad model description");
    const int N = model->n_states, G = model->n_groups;
    if (N < 2 || N > MAXN) return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: n_states must be in 2..64");
    if (n_pairs < 0) return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: negative n_pairs");
    if (n_pairs == 0) return PHMM_OK;
    if (!L_host || !off_host || !cols || !anc || !desc || !emit_M || !emit_I || !emit_D || !emit || !workspace ||
        !status_out)
        return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: null pointer");
    if (workspace_bytes < sizeof(Meta) * (size_t)n_pairs)
        return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: workspace too small");
    EmitDesc ed;
    std::memset(&ed, 0, sizeof(ed));
    ed.N = N;
    for (int s = 0; s < N; ++s) {
        ed.type[s] = model->state_types[s];
        ed.group[s] = (int8_t)model->state_group[s];
        if (model->state_group[s] < 0 || model->state_group[s] >= G)
            return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: state group out of range");
    }
    std::vector<Meta> meta(n_pairs);
    for (int p = 0; p < n_pairs; ++p) {
        if (L_host[p] < 0 || off_host[p] < 0) return fb1_fail(PHMM_E_ARG, "phmm_fb1d_emissions: negative length");
        meta[p] = Meta{off_host[p], L_host[p], 0};
    }
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(workspace, meta.data(), sizeof(Meta) * n_pairs, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status_out, 0, sizeof(int32_t) * n_pairs, st);
    if (e != cudaSuccess) return fb1_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    emit1d_kernel<<<n_pairs, 256, 0, st>>>(ed, (const Meta *)workspace, cols, anc, desc, emit_M, emit_I, emit_D,
                                          emit_per_pair, G, emit, status_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fb1_fail(PHMM_E_CUDA, cudaGetErrorString(e));
    return PHMM_OK;
}
