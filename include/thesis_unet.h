/*
 * thesis_unet.h -- learned warm start for the steady lattice-Boltzmann solve.
 *
 * A small convolutional U-Net maps a 2D channel geometry (node-flag mask,
 * Reynolds number, inlet profile) to its steady velocity and density; the
 * prediction seeds equilibrium populations (lbm_init) that the plain solver
 * then iterates to the residual tolerance, and the plain cold start stays
 * the fallback and the yardstick of the converged field.  The reference solver
 * has no learned part; this is the project's extension of its steady-state
 * loop (Iterate.cu:385-625: residual-driven iteration to a stop condition).
 *
 * Network (L pooling levels, widths c_l = min(base * 2^l, 64), base 16 or
 * 32): two 3x3
 * convolutions + ReLU per encoder level, 2x2 average pooling, a bottleneck of
 * two convolutions at level L, nearest upsampling with skip concatenation and
 * two convolutions per decoder level, and a 3x3 output convolution with 16
 * channels of which the first out_channels are used (4L + 3 convolutions).
 * Activations are NHWC BF16 with channels padded to multiples of 16, weights
 * BF16 copies of FP32 master weights, accumulation FP32 on the tensor cores:
 * hand-written tcgen05.mma kernels with the accumulators in tensor memory and
 * the input rows staged by tensor copies (cp.async.bulk.tensor) for every
 * forward, data-gradient and weight-gradient convolution (THESIS_UNET_TC=0
 * selects the mma.sync.m16n8k16 kernels instead); Adam in FP32.
 *
 * Conventions as in thesis_lbm.h: status codes (LBM_OK ...), caller-owned
 * host buffers, device buffers owned by the handle, one handle per thread.
 */
#ifndef THESIS_UNET_H
#define THESIS_UNET_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lbm_unet_s *lbm_unet;

typedef struct lbm_unet_config {
    int height, width;        /* image = lattice m x n */
    int in_channels;          /* input features per pixel, 1..16 */
    int out_channels;         /* predicted fields per pixel, 1..16 */
    int max_batch;            /* largest training / prediction batch;
                                 max_batch x height x width < 2^27 */
    unsigned long long seed;  /* weight initialisation (He normal) */
    int levels;               /* pooling levels L, 3..5 (0 selects 3); height and
                                 width must be multiples of 2^L */
    int base_channels;        /* width of level 0: 16 or 32 (0 selects 16) */
    int max_channels;         /* widest level: 64 (0 selects 64) */
} lbm_unet_config;

int lbm_unet_create(const lbm_unet_config *cfg, lbm_unet *out);

/* Number of FP32 parameters, and get / set them (layer by layer: weights
 * [3][3][cout][cin_padded], then bias [cout]). */
long long lbm_unet_param_count(lbm_unet u);
int lbm_unet_get_params(lbm_unet u, float *params);
int lbm_unet_set_params(lbm_unet u, const float *params);

/* Keep a training set on the device: count samples of inputs
 * [count][height][width][in_channels], targets [...][out_channels] and
 * per-pixel loss weights [count][height][width] (0 for solid nodes). */
int lbm_unet_set_dataset(lbm_unet u, int count, const float *inputs, const float *targets,
                         const float *weights);

/* Weighted mean squared error sum_p w_p sum_c (y_pc - t_pc)^2 /
 * (out_channels sum_p w_p) over the dataset samples idx[0..batch) and its
 * gradient; train_step applies one Adam update (beta1 0.9, beta2 0.999,
 * eps 1e-8) with learning rate lr, gradients fills grad (param order) and
 * leaves the parameters unchanged.  loss may be NULL. */
int lbm_unet_train_step(lbm_unet u, int batch, const int *idx, float lr, double *loss);
int lbm_unet_gradients(lbm_unet u, int batch, const int *idx, float *grad, double *loss);

/* Predict count samples (count <= max_batch): inputs as in set_dataset,
 * outputs [count][height][width][out_channels]. */
int lbm_unet_predict(lbm_unet u, int count, const float *inputs, float *outputs);

/* Milliseconds the last predict / train_step spent on the device (CUDA
 * events around its launches). */
double lbm_unet_last_ms(lbm_unet u);

const char *lbm_unet_last_error(void);
void lbm_unet_destroy(lbm_unet u);

#ifdef __cplusplus
}
#endif

#endif /* THESIS_UNET_H */
