/*
 * dob_oracle.h — TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
 *
 * CPU restatement of the drop-of-blood MAC fluid step, used only by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * The product (libdropfluid.so) never links or calls it.
 *
 * The API mirrors include/dropfluid.h so a test can drive both with the same
 * calls.  fp64 != 0 runs the whole step in double precision with no storage
 * rounding (the "FP64 oracle" every result's error is reported against).
 */
#ifndef DOB_ORACLE_H
#define DOB_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/dropfluid.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

orc_sim* orc_create(const dob_config* cfg, int fp64);
void orc_destroy(orc_sim* s);
int orc_reset(orc_sim* s);
int orc_set_uniforms(orc_sim* s, const float u[128]);
int orc_inject_sphere(orc_sim* s, const float center[3], float radius, float dye,
                      const float vel[3], float noise_sigma, uint64_t seed);
int orc_inject_sphere_soft(orc_sim* s, const float center[3], float radius, float edge, float dye,
                           const float vel[3], float noise_sigma, uint64_t seed);
int orc_set_parcels(orc_sim* s, const float* p, uint32_t n, uint32_t offset);
int orc_get_parcels(orc_sim* s, float* p, uint32_t n, uint32_t offset);
int orc_set_high_water(orc_sim* s, uint32_t hw);
int orc_set_field(orc_sim* s, int field, const void* host, size_t bytes);
int orc_get_field(orc_sim* s, int field, void* host, size_t bytes);
/* stats (may be NULL): [0] rhs_l2 [1] residual_l2 [2] max_div [3] vcycles [4] outer_iters */
int orc_step(orc_sim* s, int nsteps, double* stats);
int orc_run_stage(orc_sim* s, int stage);
void orc_set_threads(int n);
int orc_get_threads(void);
/* Discrete adjoint of the closed-box step (same conventions as
   dob_adjoint_stage / dob_tape_forward / dob_tape_backward; the oracle's
   tape keeps every step, no checkpoints). */
int orc_wave_step(orc_sim* s);
int orc_light_volume(orc_sim* s);
/* the plume render (dob_render_plume): light volume, then 8 binary16 values
   per pixel; lut: 256 x 64 x 4 floats */
int orc_render_plume(orc_sim* s, const float* lut, int width, int height, uint16_t* out);
int orc_wave_fft2(float* data, int inverse);
int orc_adjoint_stage(orc_sim* s, int stage);
int orc_tape_forward(orc_sim* s, int nsteps);
int orc_tape_backward(orc_sim* s, const float* dye_grad, size_t bytes);
int orc_sphere_impulse(orc_sim* s, const float center[3], float radius, const float vel[3], double* out);
int orc_sphere_soft_grad(orc_sim* s, const float center[3], float radius, float edge, float dye,
                         const float vel[3], float noise_sigma, uint64_t seed, double out[4]);
/* double-precision access to the velocity, centre, pressure, rhs, dye,
   predictor and adjoint fields (n = element count incl. channels; not
   ADJ_CENTER), for finite differences below float32 resolution */
int orc_get_field64(orc_sim* s, int field, double* host, size_t n);
/* Dense (pseudo-)inverse of a coarsest-grid operator (n = nx*ny*nz <= 4096
   cells, out n*n doubles, natural cell order): method 0 Gauss-Jordan,
   1 the separable form the simulation uses. */
int orc_coarse_inverse(int nx, int ny, int nz, double h2, int ref, int method, double* out);
int orc_set_field64(orc_sim* s, int field, const double* host, size_t n);
/* Host evaluation of the library's elementary functions (same ids as
   dob_eval_math). */
int orc_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n);

#ifdef __cplusplus
}
#endif

#endif
