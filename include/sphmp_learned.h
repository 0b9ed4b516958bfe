/*
 * sphmp_learned.h — the learned large-step corrector: one step of factor x dt
 * followed by a per-particle MLP correction, so that one large step stands in
 * for `factor` plain steps.
 *
 * The network: 48 neighbour-aggregated features -> 128 -> 128 -> 128 -> 4,
 * SiLU, bf16 weights and activations, FP32 accumulation on the tensor cores
 * (tcgen05), trained on the GPU with its own backward kernels and Adam. Its
 * outputs are a correction of the particle's velocity over the step, applied to
 * the position (3, m/s: the position moves by output x factor x dt; a step of
 * 8 dt overshoots 8 steps of dt in position by 28 a dt^2 while its velocity
 * agrees to second order) and a relative density correction (the stored
 * density of the step's result is multiplied by 1 + output).
 *
 * The reference has no counterpart: this is a method on top of the reference's
 * step (the large step is the reference's own step with dt scaled).
 *
 * Pointers named *_dev are device pointers (cudaMalloc or torch memory on the
 * context's device); all others are host pointers. Streams are opaque cudaStream_t.
 */
#ifndef SPHMP_LEARNED_H
#define SPHMP_LEARNED_H

#include "sphmp.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SPHMP_LC_FEATURES 48
#define SPHMP_LC_HIDDEN 128
#define SPHMP_LC_OUTPUTS 4
/* flat FP32 parameters: W1 [128][48], b1 [128], W2 [128][128], b2, W3 [128][128], b3, W4 [4][128], b4 [4] */
#define SPHMP_LC_PARAMS 39812

typedef struct sphmp_corrector sphmp_corrector;

/* A network with room for training batches of up to max_batch rows (a multiple of
   128; 0 for inference only), zero parameters, identity normalisation. */
sphmp_status sphmp_corrector_create(int32_t max_batch, void* stream, sphmp_corrector** out);
void sphmp_corrector_destroy(sphmp_corrector* cor);
sphmp_status sphmp_corrector_set_params(sphmp_corrector* cor, const float* params);  /* SPHMP_LC_PARAMS floats; resets Adam */
sphmp_status sphmp_corrector_get_params(sphmp_corrector* cor, float* params);
/* network input = (feature - feat_shift) * feat_scale (48 each); physical correction =
   network output * out_scale (4) */
sphmp_status sphmp_corrector_set_normalisation(sphmp_corrector* cor, const float* feat_shift, const float* feat_scale,
                                               const float* out_scale);
/* network outputs y_dev [n][4] (before out_scale) of raw features x_dev [n][48] */
sphmp_status sphmp_corrector_forward(sphmp_corrector* cor, const float* x_dev, int32_t n, float* y_dev);
/* gradients of loss = mean over the batch of |y - t|^2 (t_dev [batch][4], network
   units) into grads (SPHMP_LC_PARAMS floats, host), loss into *loss; batch a
   multiple of 128, at most max_batch; no update */
sphmp_status sphmp_corrector_gradients(sphmp_corrector* cor, const float* x_dev, const float* t_dev, int32_t batch,
                                       float* grads, float* loss);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on one batch; *loss (may be NULL)
   is the batch loss before the update (reading it synchronises) */
sphmp_status sphmp_corrector_train_step(sphmp_corrector* cor, const float* x_dev, const float* t_dev, int32_t batch,
                                        float lr, float* loss);
sphmp_status sphmp_corrector_sync(sphmp_corrector* cor); /* waits; SPHMP_ERR_TIMEOUT if a tensor-core wait ran out */

/* D[s][m][n] = sum over the split's K range of A[m][k] B[n][k]: bf16 K-major
   operands (row strides lda, ldb elements, multiples of 8), FP32 out; n a multiple
   of 16 up to 128, k a multiple of 8; splits >= 1 partial products. A utility
   (tests, callers' own networks): it allocates a status word and synchronises. */
sphmp_status sphmp_gemm_bf16_tn(const void* a_dev, int32_t lda, const void* b_dev, int32_t ldb, float* d_dev,
                                int32_t m, int32_t n, int32_t k, int32_t splits, void* stream);

/* nsteps fused steps of factor x dt; with a corrector, each is followed by the
   network's correction (features taken after the step's density pass). */
sphmp_status sphmp_step_large(sphmp_ctx* ctx, sphmp_corrector* cor, int32_t factor, int32_t nsteps);
/* Of the last corrected large step, per row of the internal order (count rows):
   features feat_dev [count][48], bornid_dev [count] (-1 for rows without
   features: boundary and out-of-grid particles), applied corrections
   corr_dev [count][4] (physical units). Any pointer may be NULL. */
sphmp_status sphmp_learned_features(sphmp_ctx* ctx, float* feat_dev, int32_t* bornid_dev, float* corr_dev,
                                    int32_t* count);
/* Replace dst's particles by src's, on the device (the effect of saving src and
   loading it into dst); both contexts on one device with the same phase count. */
sphmp_status sphmp_copy_state(sphmp_ctx* dst, sphmp_ctx* src);

/* Differences of b's state against a's over the fluid particles in the grid in
   both, matched by bornid (bornids below the larger capacity): out[0] rms of
   rho_b / rho_a - 1 over the stored densities, out[1] its largest magnitude,
   out[2] rms volume-fraction difference (root of the mean over particles of the
   sum over phases of the squared difference), out[3] rms |v_b - v_a| over rms
   |v_a|, out[4] the particles compared, out[5] (when nout >= 6) rms |x_b - x_a|
   in metres. nout >= 5. */
sphmp_status sphmp_compare_states(sphmp_ctx* a, sphmp_ctx* b, double* out, int32_t nout);

typedef struct sphmp_rollout_stats {
    int32_t large_steps;     /* large steps kept */
    int32_t plain_steps;     /* plain steps run on the state (fallbacks, fallback windows, remainder) */
    int32_t audits;          /* audited large steps */
    int32_t fallbacks;       /* audits whose error exceeded the tolerance */
    double density_err_max;  /* largest rms density error of an audit */
    double alpha_err_max;    /* largest rms volume-fraction error of an audit */
} sphmp_rollout_stats;

/* Advance ctx by `steps` plain steps' worth of simulated time in large steps of
   factor x dt, corrected by `cor` (NULL: uncorrected). The first and then every
   audit_every-th large step is audited: `audit` (a second context with the same
   parameters and capacity, given the state by a device-side clone, so that it
   continues exactly as ctx would) runs `factor` plain steps from it, the
   densities of both results are recomputed at their positions, and if the rms
   density error or the rms volume-fraction error of the large step exceeds
   `tol` (0.01 for 1 %), the plain result replaces it and the next
   audit_every x factor steps run plain, after which the first large step is
   audited again. Time that does not fill a large step runs plain.
   Synchronises; stats may be NULL. */
sphmp_status sphmp_rollout(sphmp_ctx* ctx, sphmp_ctx* audit, sphmp_corrector* cor, int32_t factor, int32_t steps,
                           int32_t audit_every, double tol, sphmp_rollout_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* SPHMP_LEARNED_H */
