/*
 * dpg_prim_io.h -- motion-primitive files and the loader's semantics.
 *
 * Replaces the reading half of load_motion_primitives_new
 * (src/ompl/robots.cpp:3061-3174): Trajectories::load_file_msgpack of the
 * reference's msgpack document
 *     {"data": [{"states": [[...], ...], "actions": [[...], ...], ...}, ...]}
 * (numbers float32, float64 or integers; other keys of a motion skipped),
 * truncation to max_motions, and the 1e-7 noise on the first and last state
 * of every motion plus the quadrotor quaternion renormalisation
 * (robots.cpp:3111-3136).  The reference draws that noise from Eigen's
 * Random (the C library's rand()); here it is a seeded SplitMix64 stream,
 * uniform in [-noise, noise], so tables are reproducible.
 *
 * Arrays: len[P]; states[sum len][nx]; actions[sum (len - 1)][nu]; FP64,
 * row-major, caller-owned.  Motions keep their file order (Motion::idx =
 * position, robots.cpp:3169-3171).  Host code only: no device is needed.
 */
#ifndef DPG_PRIM_IO_H
#define DPG_PRIM_IO_H

#include <stdint.h>

#include "dpg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Sizes of the first max_motions motions of a file (max_motions <= 0: all):
 * motions, total states, total actions, state and control width.
 * DPG_ERR_ARG: unreadable file, not the format, ragged rows, or a motion
 * whose action count is not its state count - 1. */
int dpg_primitives_file_info(const char *path, int32_t max_motions, int32_t *P, int64_t *S, int64_t *A,
                             int32_t *nx, int32_t *nu);

/* Reads those motions into caller arrays sized by dpg_primitives_file_info. */
int dpg_primitives_file_read(const char *path, int32_t max_motions, int32_t *len, double *states,
                             double *actions);

/* Writes P motions in the same format ({"data": [{"actions", "states"}]}).
 * compact != 0: a number that is exactly a float32 is written as float32,
 * any other as float64 (the bundled files' encoding); compact == 0: every
 * number as float64.  Both are lossless. */
int dpg_primitives_file_write(const char *path, int32_t P, const int32_t *len, const double *states,
                              const double *actions, int32_t nx, int32_t nu, int32_t compact);

/* The loader's post-processing, in place: uniform noise in [-noise, noise]
 * (the reference uses 1e-7) on every component of the first and the last
 * state of each motion, then, for DPG_ROBOT_QUAD3D, every state's
 * quaternion (components 3..6, x y z w) normalised. */
int dpg_primitives_prepare(int32_t kind, int32_t P, const int32_t *len, double *states, int32_t nx, double noise,
                           uint64_t seed);

#ifdef __cplusplus
}
#endif

#endif /* DPG_PRIM_IO_H */
