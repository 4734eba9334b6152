/*
 * gckpp_gb300_mlp.h -- learned step-size / stiffness proposer of the GB300
 * chemistry solve.
 *
 * No counterpart in the reference: GEOS-Chem starts each cell's integration
 * from the previous step's Hnew (KPPHvalue) or from DeltaMin.  This proposer
 * is a small MLP (56 -> 128 -> 128 -> 5, GELU) with BF16 weights and FP32
 * activations and accumulation; it maps a cell's state to a proposed initial
 * step size (log H0) and one of 4 stiffness bins, used to seed RCNTRL(3) and
 * to order the persistent solver's work queue.  The error-controlled
 * Rosenbrock integration still decides every step.
 *
 * All pointers are device pointers; every call is asynchronous on `stream`
 * (a cudaStream_t, NULL = default stream).  Return 0, -101 for a bad
 * argument, -102 for a CUDA error.
 *
 * Layouts: features x [M][56] float; weights W1 [128][56], W2 [128][128],
 * W3 [5][128] as bf16 (row-major, out x in); biases float; activations
 * [M][128] float; head output [M][5] float (log H0, 4 bin logits).
 */
#ifndef GCKPP_GB300_MLP_H
#define GCKPP_GB300_MLP_H

#ifdef __cplusplus
extern "C" {
#endif

int gc_mlp_dims(int* nfeat, int* hidden, int* nout, int* nj, int* nspc);

/* Normalised features from cell state (cell-interleaved met/photol/c as in
 * gckpp_gb300.h; suncos [ncell] or NULL): log T, log P, log H2O mixing
 * ratio, cos SZA, log J of the PHOTOL rows jslot[20], log mixing ratio of the
 * species rows spc[32]; then (f - mean) * inv_std. */
int gc_mlp_features(int ncell, const double* met, long long ldm, const double* photol, long long ldp,
                    const double* c, long long ldc, const double* suncos, const int* jslot, const int* spc,
                    const double* mean, const double* inv_std, float* x, void* stream);

/* Forward pass; z1/z2 (pre-activations) may be NULL when not training. */
int gc_mlp_forward(int M, const float* x, const void* w1, const float* b1, const void* w2, const float* b2,
                   const void* w3, const float* b3, float* z1, float* h1, float* z2, float* h2, float* out,
                   void* stream);

/* Loss = mean squared error of out[:,0] against y_h + w_ce * mean softmax
 * cross-entropy of out[:,1:5] against y_bin; accumulates into *loss and
 * writes dLoss/dout. */
int gc_mlp_loss(int M, const float* out, const float* y_h, const int* y_bin, float w_ce, float* dout, float* loss,
                void* stream);

/* Backward pass: accumulates (+=) weight and bias gradients; scratch holds
 * M*(5 + 4*128) floats. */
int gc_mlp_backward(int M, const float* x, const void* w1, const void* w2, const void* w3, const float* z1,
                    const float* h1, const float* z2, const float* h2, const float* dout, float* g_w1, float* g_b1,
                    float* g_w2, float* g_b2, float* g_w3, float* g_b3, float* scratch, void* stream);

/* Adam step on n fp32 master weights (w_bf16 receives the rounded copy, may
 * be NULL for biases); zeroes the gradient. */
int gc_mlp_adam(int n, float* w, void* w_bf16, float* g, float* m1, float* m2, float lr, float b1, float b2,
                float eps, int step, void* stream);

/* h0 = clamp(scale * exp(out[:,0]), hmin, hmax); bin = argmax(out[:,1:5]).
 * With keep != 0, entries of h0 that are already positive (a cell's
 * KPPHvalue from its previous step) are left as they are. */
int gc_mlp_propose(int M, const float* out, double scale, double hmin, double hmax, double* h0, int* bin,
                   int keep, void* stream);

/* Stable counting sort of cells by bin, heaviest bin first: order[M] lists
 * the cells of bin 3, then 2, 1, 0, each in ascending cell order; counts[4]
 * receives the cells per bin.  scratch holds gc_mlp_bin_order_scratch(M)
 * ints.  Three kernel launches, no atomics on the order: the same order on
 * every run. */
int gc_mlp_bin_order_scratch(int M);
int gc_mlp_bin_order(int M, const int* bin, int* counts, int* scratch, int* order, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GCKPP_GB300_MLP_H */
