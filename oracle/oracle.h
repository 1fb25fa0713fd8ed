/*
 * CPU oracle for the sphere-tracing hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A C++ restatement of the reference renderer's depth path
 * (crates/forgedthoughts/src/renderer.rs), templated on the arithmetic type:
 * precision 32 follows the reference's f32 arithmetic step for step, precision
 * 64 is the FP64 oracle march.  It consumes the same flat scene IR the GPU
 * library consumes (include/forgedthoughts_gb300.h).
 *
 * Only the tests, the smoke check and the benchmark's CPU-baseline leg may
 * load this library; the product never links or calls it.
 */
#ifndef FT_ORACLE_H
#define FT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "forgedthoughts_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Depth preview over rows row_begin, row_begin + row_step, ... < row_end.
 * Output layouts match ft_render_depth; rows not rendered are left untouched.
 * `threads` <= 0 uses std::thread::hardware_concurrency().  `evals_out`
 * (nullable) receives the number of distance evaluations performed.
 * Returns 0 on success, a non-zero ft_status otherwise. */
int oracle_render_depth(const ft_scene_desc* desc, const ft_render_options* options,
                        int accel, uint32_t aa_samples, int precision, int threads,
                        uint32_t row_begin, uint32_t row_end, uint32_t row_step,
                        float* t_out, uint8_t* mask_out, uint32_t* material_out,
                        float* normal_out, uint8_t* rgb8_out, uint64_t* evals_out);

/* Whitted trace (trace_ray_recursive, crates/forgedthoughts/src/renderer/ray.rs:3-222)
 * over the same rows; rgb_out receives width*height*3 linear floats (the AA
 * average), rgb8_out the Reinhard + gamma bytes (renderer.rs:5229-5239). */
int oracle_render_trace(const ft_scene_desc* desc, const ft_render_options* options,
                        int accel, uint32_t aa_samples, uint32_t max_depth, int precision,
                        int threads, uint32_t row_begin, uint32_t row_end, uint32_t row_step,
                        float* rgb_out, uint8_t* rgb8_out, uint64_t* evals_out);

/* oracle_render_depth / oracle_render_trace over every row_step-th row and
 * col_step-th column from (col_begin, row_begin); outputs are full-frame
 * arrays of which only the sampled pixels are written.  jitter_seed >= 0
 * takes the jittered AA offsets (XorShift64, seed_pixel_sample ^ seed,
 * R:4735-4774) instead of the sqrt(aa) grid. */
int oracle_render_depth_strided(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                uint32_t aa_samples, int precision, int threads, uint32_t row_begin,
                                uint32_t row_end, uint32_t row_step, uint32_t col_begin, uint32_t col_step,
                                int64_t jitter_seed, float* t_out, uint8_t* mask_out, uint32_t* material_out,
                                float* normal_out, uint8_t* rgb8_out, uint64_t* evals_out);
int oracle_render_trace_strided(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                uint32_t aa_samples, uint32_t max_depth, int precision, int threads,
                                uint32_t row_begin, uint32_t row_end, uint32_t row_step, uint32_t col_begin,
                                uint32_t col_step, int64_t jitter_seed, float* rgb_out, uint8_t* rgb8_out,
                                uint64_t* evals_out);

/* Strided pixel sample of a full frame (every row_step-th row from
 * row_begin, every col_step-th column from col_begin) in f32, outputs
 * discarded: mode 0 the depth march, else the Whitted trace of max_depth.
 * The timed CPU baseline. */
int oracle_render_sample(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                         uint32_t aa_samples, uint32_t max_depth, int mode, int threads,
                         uint32_t row_begin, uint32_t row_step, uint32_t col_begin, uint32_t col_step,
                         uint64_t* evals_out);

/* Accelerator distance query (`Accelerator::distance_info`) at n points
 * (xyz triples).  Outputs are nullable. */
int oracle_distance(const ft_scene_desc* desc, int accel, int precision,
                    const float* points, size_t n, double* distance_out,
                    uint32_t* object_out, uint32_t* material_out);

/* Evaluate hook program `program` of the scene on n argument sets.  args
 * holds, per call, the parameters packed as 3 floats each (scalars use the
 * first lane).  out receives 3 floats per call. */
int oracle_eval_program(const ft_scene_desc* desc, int program, int precision,
                        const float* args, size_t n, double* out);

/* Multi-view depth / mask / soft silhouette (the definitions of
 * ft_render_views), Bvh accelerator, outputs view-major and nullable; depth
 * and silhouette as doubles so finite differences of the FP64 march keep
 * its precision. */
int oracle_render_views(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                        const ft_render_options* options, float tau, int precision, int threads,
                        double* t_out, uint8_t* mask_out, double* sil_out);

/* oracle_render_views over the pixels (offset + i * stride, offset + j * stride)
 * of every view; only those pixels of the full outputs are written. */
int oracle_render_views_strided(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                                const ft_render_options* options, float tau, int precision, int threads,
                                uint32_t stride, uint32_t offset, double* t_out, uint8_t* mask_out,
                                double* sil_out);

/* oracle_render_backward over the pixels (offset + i * stride, offset + j *
 * stride) of every view. */
int oracle_render_backward_strided(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                                   const ft_render_options* options, float tau, const ft_param* params,
                                   uint32_t n_params, const float* dl_dt, const float* dl_dsil, int precision,
                                   int threads, uint32_t stride, uint32_t offset, double* grad_out);

/* The adjoint of oracle_render_views (the definitions of ft_render_backward):
 * grad_out[k] = sum over rays of dl_dt dt/dparam_k + dl_dsil dsil/dparam_k. */
int oracle_render_backward(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                           const ft_render_options* options, float tau, const ft_param* params,
                           uint32_t n_params, const float* dl_dt, const float* dl_dsil, int precision,
                           int threads, double* grad_out);

const char* oracle_last_error(void);

/* The Whitted trace's medium functions in f32, for their known-answer tests.
 * A medium is {ior, absorption r, g, b, density}.
 * oracle_medium_transmittance: medium_transmittance (renderer.rs:5109-5119).
 * oracle_transition_medium: transition_medium (renderer.rs:5147-5166) for an
 * unblended material crossed at a front (1) or back (0) face. */
void oracle_medium_transmittance(const float medium[5], float distance, float out_rgb[3]);
void oracle_transition_medium(const ft_material* material, int front_face, const float current[5], float out[5]);

#ifdef __cplusplus
}
#endif

#endif /* FT_ORACLE_H */
