/*
 * sgba_synth.h -- seeded synthetic bundle-adjustment problems.
 *
 * Stand-ins for the reference's example-problem generators
 * (crates/sophus_opt/src/example_problems/ba_problem.rs:154-346,
 *  crates/sophus_opt/src/example_problems/cam_calib.rs:63-149): the same role
 * (a deterministic scene + noisy observations + perturbed initial values),
 * with the scene shapes of the benchmark configurations.  Random numbers come
 * from SplitMix64 streams with Box-Muller normals, so the same seed gives the
 * same problem on every host.
 */
#ifndef SGBA_SYNTH_H
#define SGBA_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SGBA_SYNTH_CIRCLE = 0,   /* cameras on a circle around a cube of points  */
  SGBA_SYNTH_SPHERE = 1,   /* Fibonacci-sphere cameras, random track subsets */
  SGBA_SYNTH_LOOP = 2,     /* outward-facing loop, consecutive-camera tracks */
  SGBA_SYNTH_WINDOW = 3,   /* one local window: circle scene scaled in size */
};

typedef struct {
  int32_t n_cam;
  int32_t n_pt;
  int64_t n_obs;
  double intrinsics[4];   /* fx fy cx cy */
  double huber_delta;
  double initial_lm_damping;
  int32_t num_iterations;
  double *poses;          /* n_cam*7 initial world_from_camera (qw qx qy qz tx ty tz) */
  double *poses_true;     /* n_cam*7 ground truth */
  uint8_t *pose_const;    /* n_cam; camera 0 is 1 */
  double *points;         /* n_pt*3 initial */
  double *points_true;    /* n_pt*3 ground truth */
  int32_t *obs_cam;       /* n_obs */
  int32_t *obs_pt;        /* n_obs */
  double *obs_uv;         /* n_obs*2 noisy pixel measurements */
} sgba_synth_problem;

/* Generate a scene.  n_cam / n_pt <= 0 select the configuration defaults:
 *   CIRCLE 10/500, SPHERE 100/20000, LOOP 1500/300000; WINDOW draws its own
 *   sizes (cameras U{5..40}, points U{200..4000}) from the seed.
 * Returns 0 or a negative error; *out must be released with sgba_synth_free. */
int sgba_synth_generate(int32_t kind, int32_t n_cam, int32_t n_pt, uint64_t seed,
                        sgba_synth_problem **out);
void sgba_synth_free(sgba_synth_problem *p);

#ifdef __cplusplus
}
#endif
#endif
