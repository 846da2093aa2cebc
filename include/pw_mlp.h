/*
 * pw_mlp.h -- C ABI of the learned proposal (part of libpwcollide.so).
 *
 * The reference has no collision surrogate: its learned part (src/hg,
 * src/GP/pipeline/train.py) predicts surface heat maps.  This network is the
 * engine's own: it scores SE(3) states by their probability of being
 * collision free so that samplers spend exact checks (pw_states_valid,
 * pw_segments_first_contact) where free space is likely.  The exact queries
 * stay the arbiter: a score is never a verdict.
 *
 * Network: features f(q) = [x, y, z, R(q)[:,0], R(q)[:,1]] (9 values, padded
 * to 16 with zeros), 4 hidden layers of width 256 with SiLU, one sigmoid
 * output.  Weights and activations are BF16, accumulation FP32; the master
 * weights and the Adam moments are FP32.  Loss: mean binary cross-entropy,
 * label 1 = collision free.
 *
 * Parameter block (FP32, pw_mlp_num_params values), in this order:
 *   W1 [256 x 16] (columns 9..15 unused, kept 0), b1 [256],
 *   W2 [256 x 256], b2, W3 [256 x 256], b3, W4 [256 x 256], b4,
 *   w5 [256], b5 [1]
 * Weight matrices are row-major [out][in].
 *
 * Device pointers and streams as in pw_collide.h.  One network object serves
 * one call at a time (calls share its scratch buffers).
 */
#ifndef PW_MLP_H
#define PW_MLP_H

#include <stdint.h>

#include "pw_collide.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pw_mlp pw_mlp;

/* Creates a network on `device` with He-uniform weights drawn from `seed`. */
PW_API int pw_mlp_create(pw_mlp **out, int device, uint64_t seed);
PW_API int pw_mlp_destroy(pw_mlp *m);
PW_API int64_t pw_mlp_num_params(const pw_mlp *m);

/* host: copy the FP32 parameter block out / in (set refreshes the BF16 copies). */
PW_API int pw_mlp_get_params(const pw_mlp *m, float *host_out);
PW_API int pw_mlp_set_params(pw_mlp *m, const float *host_in);
/* host: the gradient block of the last pw_mlp_gradients / pw_mlp_train_step. */
PW_API int pw_mlp_get_grads(const pw_mlp *m, float *host_out);
/* host: the Adam state (first and second moments, num_params floats each, and the
 * step count), so that a checkpoint taken between steps resumes with the same
 * next update. Either moment pointer may be NULL to skip it; set validates step >= 0. */
PW_API int pw_mlp_get_adam(const pw_mlp *m, float *m1_out, float *m2_out, int64_t *step_out);
PW_API int pw_mlp_set_adam(pw_mlp *m, const float *m1_in, const float *m2_in, int64_t step);

/* P(collision free) of n states (device float64 [n x 7] -> device float32 [n]):
 * one fused, persistent kernel on the tcgen05 tensor cores (weights streamed by
 * bulk copies, accumulators in tensor memory).  Its waits are bounded;
 * pw_mlp_check reports whether one gave up.  Asynchronous on stream, except that
 * the first call after the weights changed (a training step, pw_mlp_set_params)
 * synchronises the stream once to copy the epilogue constants (biases, head) to
 * the host: each launch passes them in its parameters. */
PW_API int pw_mlp_predict(pw_mlp *m, const double *states, int64_t n, float *prob, void *stream);

/* The logit of the same network (the score before the sigmoid): a ranking
 * score that does not saturate, for pw_select_top.  Same kernel as pw_mlp_predict. */
PW_API int pw_mlp_score(pw_mlp *m, const double *states, int64_t n, float *logit, void *stream);

/* The same prediction through the mma.sync GEMM kernels that training uses
 * (a cross-check of pw_mlp_predict; layer by layer, activations through HBM). */
PW_API int pw_mlp_predict_mma(pw_mlp *m, const double *states, int64_t n, float *prob, void *stream);

/* host: synchronises the device; PW_ERR_INTERNAL if a bounded device wait of an
 * earlier pw_mlp_predict gave up (its probabilities are then invalid). */
PW_API int pw_mlp_check(pw_mlp *m);

/* host, test of the bounded waits: the next pw_mlp_predict / pw_mlp_score
 * launch issues no weight copies, so its MMA issuer's wait for a weight stage
 * runs out after the limit (about 2 s).  Every role then stops, the kernel
 * frees its tensor memory and returns; pw_mlp_check reports PW_ERR_INTERNAL
 * and the following launches run normally.  Nothing faults or hangs. */
PW_API int pw_mlp_withhold_next_weights(pw_mlp *m);

/* host: the states whose score is at or above the k-th largest score (any
 * finite floats, e.g. pw_mlp_score output), gathered into out_states (device,
 * [capacity x 7], in no particular order); *out_count = how many (k plus ties
 * at the threshold).  PW_ERR_CAPACITY if that exceeds capacity.  Synchronises
 * the stream. */
PW_API int pw_select_top(const float *score, const double *states, int64_t n, int64_t k, double *out_states,
                         int64_t capacity, int64_t *out_count, void *stream);

/* Gradients of the mean binary cross-entropy over one batch (device states,
 * device uint8 labels, 1 = free) into the gradient block; no update.
 * loss_out (host, may be NULL) receives the loss and then the call
 * synchronises the stream. n <= 2^24. */
PW_API int pw_mlp_gradients(pw_mlp *m, const double *states, const uint8_t *labels, int64_t n, float *loss_out,
                            void *stream);

/* Kernels of the training step: 0 (default) = tcgen05 GEMMs (TMA-loaded
 * operands, accumulators in tensor memory); 1 = the mma.sync GEMMs (a
 * cross-check of the same step). */
PW_API int pw_mlp_set_training_kernels(pw_mlp *m, int use_mma);

/* pw_mlp_gradients followed by one Adam step (beta1 0.9, beta2 0.999, eps 1e-8). */
PW_API int pw_mlp_train_step(pw_mlp *m, const double *states, const uint8_t *labels, int64_t n, float lr,
                             float *loss_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PW_MLP_H */
