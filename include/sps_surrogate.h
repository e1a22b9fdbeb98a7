/*
 * sps_surrogate.h -- the learned constitutive surrogate of libsps_gb300.so.
 *
 * None of these functions has a counterpart in the reference: the reference evaluates
 * the Drucker-Prager flow rule (drucker_prager, code/3_SPH_material_2018.f90:1958-2083,
 * called from plastic_terms :1884) exactly on every stress-point.  Here a small MLP
 * (14 inputs, three hidden layers of 128 SiLU units, 4 outputs; BF16 weights and
 * activations with FP32 accumulation) may stand in for the plastic source G of loading
 * stress-points in the FP32 form of the step.
 *
 *   1. sps_capture / sps_capture_read   collect (input, target) tuples from the exact
 *                                       flow rule while a context steps;
 *   2. sps_mlp_*                         train the network on the GPU (forward, backward
 *                                       and Adam kernels of this library);
 *   3. sps_surrogate_install / _stats    let a context use the network, with a fallback
 *                                       to the exact flow rule per stress-point.
 *
 * Tuple = 14 inputs then 4 targets (18 floats), all scale-free:
 *   inputs  0-3  stress direction sigma / |sigma|, (sxx, syy, sxy, szz)
 *           4-7  strain-rate direction (e11, e22, e12, 0) / |e|,
 *                |e| = sqrt(e11^2 + e22^2 + 2 e12^2), e12 = (du/dy + dv/dx) / 2
 *           8    spin (du/dy - dv/dx) / 2 / |e|
 *           9-13 tan(phi), c / |sigma|, nu, log10(E) - 7, rho / 2000 - 1
 *   targets 0-3  the plastic source Gs = -G of drucker_prager divided by G_mod |e|,
 *                G_mod = E / (2 (1 + nu))
 * Parameters (SPS_MLP_NPARAM floats, FP32 master copy): for each layer the weights
 * W[k][n] row-major (k = input, n = output) followed by the bias b[n]; layer 1 has 16
 * input rows (rows 14, 15 unused), layer 4 has 8 output columns (columns 4-7 unused).
 */
#ifndef SPS_SURROGATE_H
#define SPS_SURROGATE_H

#include <stdint.h>

#include "sps.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SPS_MLP_NIN 14
#define SPS_MLP_NOUT 4
#define SPS_MLP_TUPLE 18
#define SPS_MLP_NPARAM 36232

/* ---- training data ------------------------------------------------------------------ */

/* Start (cap > 0) or stop (cap == 0) collecting tuples in the context: every stage of
   every later sps_step appends one tuple per loading stress-point (the exact flow rule's
   inputs and output) until cap tuples are held; later ones are counted but dropped.
   Starting again discards what was held. */
int sps_capture(sps_ctx* ctx, int64_t cap);

/* Copy the held tuples out: *n holds the capacity of `tuples` (in tuples) on entry and
   the number copied on return; *seen (may be NULL) the number offered since the start,
   including dropped ones. */
int sps_capture_read(sps_ctx* ctx, float* tuples, int64_t* n, int64_t* seen);

/* ---- training ----------------------------------------------------------------------- */

typedef struct sps_mlp sps_mlp;

typedef struct sps_mlp_config {
  int32_t quantize; /* 1: the forward pass rounds weights and activations to BF16, as the
                       tensor-core inference does (gradients pass the rounding straight
                       through); 0: plain FP32 */
  int32_t batch;    /* minibatch size, a multiple of 64, at most 65536 */
  float lr, beta1, beta2, eps; /* Adam */
  uint64_t seed;    /* weight initialisation and minibatch shuffling */
} sps_mlp_config;

/* Allocate a network (Glorot-uniform weights from seed, zero biases) on the current
   device. */
int sps_mlp_create(const sps_mlp_config* cfg, sps_mlp** out);
int sps_mlp_get_params(sps_mlp* m, float* params);
int sps_mlp_set_params(sps_mlp* m, const float* params);

/* Copy n training tuples (n x 18 floats) to the device (replaces earlier data). */
int sps_mlp_set_data(sps_mlp* m, const float* tuples, int64_t n);

/* Train `epochs` passes over the data in shuffled minibatches of cfg.batch (the tail that
   does not fill a minibatch is skipped in that epoch), one Adam step per minibatch with
   learning rate lr (lr <= 0: cfg.lr).  loss[e] (may be NULL) receives the mean squared
   error of epoch e. */
int sps_mlp_train(sps_mlp* m, int32_t epochs, float lr, float* loss);

/* Loss (mean over n rows and 4 outputs of the squared error) and its gradient with
   respect to the parameters, for the n tuples given (n x 18), with the current
   parameters; no update.  n <= cfg.batch. */
int sps_mlp_grad(sps_mlp* m, const float* tuples, int32_t n, float* grad, float* loss);

/* Network outputs for n inputs (n x 14 floats) through the tensor-core inference code
   of the step (BF16 mma with FP32 accumulation): y is n x 4. */
int sps_mlp_predict(sps_mlp* m, const float* x, int32_t n, float* y);

/* Which inference code sps_mlp_predict runs: 1 (the default) the 5th-generation tensor-core
   path the step uses (128-row tiles, tcgen05.mma with tensor-memory accumulators), 0 the
   warp-level mma.sync path. */
int sps_mlp_set_inference(sps_mlp* m, int32_t tensor_memory);

int sps_mlp_last_error(sps_mlp* m, char* buf, int32_t len);
void sps_mlp_destroy(sps_mlp* m);

/* ---- use in the step ---------------------------------------------------------------- */

typedef struct sps_surrogate_opts {
  double tol;        /* accept a prediction when the yield-function drift it causes over
                        one step, dt |grad f : (D:e + Gs)| / sqrt(J2), is at most tol
                        (the exact flow rule makes it zero up to rounding) */
  float env_lo[SPS_MLP_NIN], env_hi[SPS_MLP_NIN]; /* training envelope of the inputs */
  float out_max;     /* largest |target| component seen in training */
} sps_surrogate_opts;

/* Let the context's FP32 form use the network's current parameters for the plastic
   source of loading stress-points whose inputs lie inside the envelope and whose
   prediction passes the drift test; every other stress-point uses the exact flow rule.
   m == NULL uninstalls.  SPS_ERR_UNSUPPORTED for the FP64 plain form. */
int sps_surrogate_install(sps_ctx* ctx, sps_mlp* m, const sps_surrogate_opts* opts);

/* The gate that keeps the network from costing time where it does not pay (no reference
   counterpart): a step runs the network only while it answers at least min_answered of
   that step's loading evaluations (a step without loading evaluations counts as below:
   the network had nothing to answer); after a step below that, the exact rule alone runs for
   a period of steps and then the network is tried for one step again, the period
   doubling up to max_period steps while these tries keep failing and returning to 1 after
   one that passes.  The decision is taken on the device at the end of every step.
   min_answered <= 0 keeps the network on in every step.  Defaults at install: 0.5 and 1024
   (a network that keeps failing is then tried about once in a thousand steps).
   Setting it restarts the gate (on, period 1). */
int sps_surrogate_gate(sps_ctx* ctx, double min_answered, int32_t max_period);

/* steps[0] = steps run with the network since install, steps[1] = steps run without it
   (gate closed). */
int sps_surrogate_gate_stats(sps_ctx* ctx, int64_t* steps);

/* counts[0] = loading stress-point evaluations since install (or the last reset) in the
   steps that ran the network,
   counts[1] = those answered by the network, counts[2] = outside the envelope,
   counts[3] = rejected by the drift test.  reset != 0 zeroes them after reading. */
int sps_surrogate_stats(sps_ctx* ctx, int64_t* counts, int32_t reset);

#ifdef __cplusplus
}
#endif

#endif
