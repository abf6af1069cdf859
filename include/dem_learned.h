/*
 * dem_learned.h -- the learned part: per-pair feature-contact counts predicted
 * by a small MLP, used to size the polyhedron feature buffers and to order the
 * candidate pairs into warp bins.  No reference counterpart.  The exact
 * enumeration still decides every interaction: a pair whose features do not fit the predicted
 * record is enumerated again exactly, so the interaction list is unchanged.
 *
 * Network: 16 -> 64 (ReLU) -> 64 (ReLU) -> 4, BF16 weights and inputs, FP32
 * accumulation, outputs z with rates exp(z) for the VV, VE, VF, EE counts
 * (Poisson loss, log link), trained with Adam by the library's own kernels.
 *
 * Inputs of a candidate pair (A owner, B partner), in this order:
 *   [0..3)   position of B's centre in A's body frame / (r_A + r_B)
 *   [3..7)   relative orientation q_A^-1 q_B (w >= 0)
 *   [7..13)  one-hot of the unordered shape-type pair (types mod 3)
 *   [13..16) OBB(A) and OBB(B) overlap, each enlarged by 0, skin/4, skin/2 (the
 *            last is the candidate test); all inputs in FP32
 * Labels (uint8 x 4): exact VV, VE (+swap), VF (+swap), EE counts (saturated at 255).
 */
#ifndef DEM_LEARNED_H
#define DEM_LEARNED_H
#include <stdint.h>

#include "dem_hotpath.h"

#ifdef __cplusplus
extern "C" {
#endif

#define DEM_MLP_IN 16
#define DEM_MLP_HID 64
#define DEM_MLP_OUT 4
#define DEM_MLP_NPARAM (64 * 16 + 64 + 64 * 64 + 64 + 4 * 64 + 4)

/* Inputs and exact labels of the candidate pairs (particle-particle units that
 * pass the OBB test) of the current neighbour list: requires a polyhedron
 * context whose last rebuild used fp32_broad_phase.  dev_x: capacity x 16
 * floats, dev_y: capacity x 4 bytes (device); *count = pairs written (at most
 * capacity) and *available = pairs of the list.                            */
int dem_mlp_harvest(dem_ctx* ctx, float* dev_x, uint8_t* dev_y, uint64_t capacity, uint64_t* count,
                    uint64_t* available);
/* He-uniform initial weights (seeded); output biases log(label_means) (4 values, may be NULL). */
int dem_mlp_init(dem_ctx* ctx, uint64_t seed, const float* label_means);
int dem_mlp_set_params(dem_ctx* ctx, const float* host_params); /* DEM_MLP_NPARAM FP32 */
int dem_mlp_get_params(dem_ctx* ctx, float* host_params);
/* rates exp(z), n x 4 floats (device in / device out) */
int dem_mlp_forward(dem_ctx* ctx, const float* dev_x, uint64_t n, float* dev_rates);
/* mean Poisson loss and its gradient (DEM_MLP_NPARAM floats, host) over n samples */
int dem_mlp_loss_grad(dem_ctx* ctx, const float* dev_x, const uint8_t* dev_y, uint64_t n, float* host_grad,
                      double* loss);
/* epochs of Adam (lr) over shuffled full batches; loss_per_epoch: epochs doubles (may be NULL) */
int dem_mlp_train(dem_ctx* ctx, const float* dev_x, const uint8_t* dev_y, uint64_t n, int epochs, uint64_t batch,
                  float lr, uint64_t seed, double* loss_per_epoch);

/* Last polyhedron rebuild with learned sizing: candidate units, units whose
 * features overflowed their predicted record (enumerated again exactly), and
 * record entries allocated (the fixed-size alternative holds 16 per unit). */
int dem_learned_stats(dem_ctx* ctx, uint64_t* units, uint64_t* overflow, uint64_t* record_entries);

#ifdef __cplusplus
}
#endif
#endif
