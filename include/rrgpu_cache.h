/* rrgpu_cache.h -- C ABI of the learned radiance cache used by the lightmap
 * gather.  The cache has no counterpart in the reference: it replaces the
 * bounces past the first of the plain gather (rrgpu_gather.h), whose output
 * stays its fallback and the yardstick of its error.
 *
 * Network: 64 encoded inputs (a frequency or multiresolution hash encoding
 * of the position in the scene box, normal, albedo), four hidden layers of
 * 64 ReLU units, 3 outputs
 * (outgoing RGB radiance), BF16 weights and activations, FP32 accumulation
 * and FP32 Adam masters; layout and loss in oracle/rr_mlp.c.
 *
 * Records (48 bytes): float p[3], n[3], albedo[3], t[3]; t = training target
 * (outgoing radiance), or for inference t[0] > 0 marks a valid record.
 */
#ifndef RRGPU_CACHE_H
#define RRGPU_CACHE_H
#include "rrgpu.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct rrg_cache rrg_cache;

/* Position encodings (oracle/rr_mlp.c specifies both). */
enum {
	RRG_CACHE_FREQUENCY = 0,   /* 8 octaves of sin/cos per axis */
	RRG_CACHE_HASHGRID = 1     /* 16-level multiresolution hash grid (2 features
	                              per level, trilinear) + 4 octaves of sin/cos */
};

typedef struct rrg_cache_params {
	uint32_t size;          /* sizeof(rrg_cache_params) */
	uint32_t encoding;      /* RRG_CACHE_* */
	float lo[3], hi[3];     /* scene box of the position encoding */
	uint64_t seed;          /* weight and table initialisation */
	uint32_t log2_table;    /* hash grid: entries per level = 2^log2_table (10..24), 0 = 19 */
	float min_res, max_res; /* hash grid: coarsest / finest grid resolution, 0 = 16 / 1024 */
	uint32_t reserved[4];
} rrg_cache_params;

/* lo/hi: scene box used by the position encoding; seed: weight init.
 * Frequency encoding; rrg_cache_create_ex chooses the encoding. */
RRG_API int rrg_cache_create(const float* lo, const float* hi, uint64_t seed, rrg_cache** out);
RRG_API int rrg_cache_create_ex(const rrg_cache_params* params, rrg_cache** out);
/* Hash grid: number of table floats (16 x 2^log2_table x 2; 0 for the
 * frequency encoding), table copies and the 16 level resolutions. */
RRG_API uint64_t rrg_cache_table_floats(const rrg_cache* c);
RRG_API int rrg_cache_get_table(rrg_cache* c, float* host);
RRG_API int rrg_cache_set_table(rrg_cache* c, const float* host);
RRG_API int rrg_cache_get_resolutions(const rrg_cache* c, float* res16);
RRG_API void rrg_cache_destroy(rrg_cache* c);
/* 17,408 FP32 parameters: W1..W4 (64x64), W5 (64x16), row = input. */
RRG_API int rrg_cache_set_weights(rrg_cache* c, const float* w_host);
RRG_API int rrg_cache_get_weights(rrg_cache* c, float* w_host);
RRG_API int rrg_cache_set_adam(rrg_cache* c, float lr, float beta1, float beta2, float eps);
/* One forward/backward over B host records (B a multiple of 128), in
 * order, without an update: the gradient of the mean loss (17,408 floats),
 * the loss and the predictions (B x 3), for checks against the oracle. */
RRG_API int rrg_cache_gradient(rrg_cache* c, const void* recs_host, uint32_t B, float* grad_host, float* loss_host,
                               float* pred_host);
/* Same, plus the gradient of the hash table (rrg_cache_table_floats floats;
 * NULL to skip, which the frequency encoding requires). */
RRG_API int rrg_cache_gradient_ex(rrg_cache* c, const void* recs_host, uint32_t B, float* grad_host,
                                  float* table_grad_host, float* loss_host, float* pred_host);
/* `steps` Adam steps on batches of `batch` records drawn from nrec device
 * records; last_loss (may be NULL) receives the last batch's loss. */
RRG_API int rrg_cache_train(rrg_cache* c, const void* recs_dev, uint32_t nrec, uint32_t batch, uint32_t steps,
                            float* last_loss, void* stream);
/* out_dev: float4 per record (RGB >= 0, validity). */
RRG_API int rrg_cache_infer(rrg_cache* c, const void* recs_dev, uint64_t n, float* out_dev, void* stream);
RRG_API uint64_t rrg_cache_steps(const rrg_cache* c);
/* Error estimate for the fallback: the cache's mean prediction and the mean
 * target of nrec device records are compared per cell of a res^3 grid over
 * the box; a cell is reliable when it holds >= min_count records and
 * |mean pred - mean target| <= max(rel_threshold * mean target, 3 standard
 * errors of the mean target) (the targets are single-path estimates, so
 * their noise bounds what the test can resolve).  nreliable
 * (may be NULL) receives the number of reliable cells. */
RRG_API int rrg_cache_build_error_grid(rrg_cache* c, const void* recs_dev, uint64_t nrec, uint32_t res,
                                       float rel_threshold, uint32_t min_count, uint32_t* nreliable, void* stream);
/* Same, with the tolerance also at least the standard deviation of the
 * cell's targets over sqrt(plain_samples): a cell whose bias is below the
 * noise of the plain gather's plain_samples-sample mean is kept, because
 * falling back would add more error than it removes (0 = off). */
RRG_API int rrg_cache_build_error_grid_ex(rrg_cache* c, const void* recs_dev, uint64_t nrec, uint32_t res,
                                          float rel_threshold, uint32_t min_count, float plain_samples,
                                          uint32_t* nreliable, void* stream);

#ifdef __cplusplus
}
#endif
#endif
