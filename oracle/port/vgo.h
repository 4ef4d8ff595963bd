/* vgo: the CPU oracle of vamp_gb300.
 *
 * A plain-C restatement of the reference's collision-checking hot path, used only by the tests,
 * by __graft_entry__.smoke() and by bench.py's CPU baseline.  It is never linked into the
 * shipped library.  Each function cites the reference code it restates (paths relative to the
 * reference's src/impl/vamp/).
 *
 * Lane groups.  The reference checks configurations in SIMD blocks of `lanes` states (8 with
 * AVX2, 4 with NEON).  Several decisions inside fkcc are taken for the whole block (a coarse
 * sphere hit in any lane runs the fine tests for all lanes; the primitive loop stops only when
 * every lane allows it), so the oracle evaluates whole blocks, lane count as a parameter.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vgo_env vgo_env;
typedef struct vgo_robot vgo_robot;

/* ---------------------------------------------------------------- environment (environment.hh) */
vgo_env *vgo_env_create(void);
void vgo_env_destroy(vgo_env *e);
/* sphere x y z r (shapes.hh:217-251) */
void vgo_env_add_sphere(vgo_env *e, const float *f);
/* capsule x1 y1 z1 xv yv zv r rdv; z-aligned if xv == yv == 0 (bindings/environment.cc:132-145) */
void vgo_env_add_capsule(vgo_env *e, const float *f);
/* cuboid centre, axis_1, axis_2, axis_3, half extents; z-aligned if axis_3_z == 1
 * (bindings/environment.cc:118-131) */
void vgo_env_add_cuboid(vgo_env *e, const float *f);
/* pointcloud as a CAPT (capt.hh:294-365); returns 0 on success */
int vgo_env_add_pointcloud(vgo_env *e, const float *xyz, size_t n, float r_min, float r_max, float r_point);
void vgo_env_set_sqrt_mode(vgo_env *e, int mode); /* VGO_SQRT_X86 (default) or VGO_SQRT_EXACT */
/* Attachment (collision/attachments.hh; bindings/environment.cc:163-165,200-230): spheres [k][4]
 * in a frame at the relative transform tf (4x4, row-major) from the end effector; checked by
 * fkcc_attach.  Returns 0 on success (k <= VGO_MAX_ATTACH). */
#define VGO_MAX_ATTACH 64
/* heightfield (collision/shapes.hh:250-311; factory heightfield::flat, factory.hh:365-386):
 * centre offsets, scales (stored inverted), xd x yd samples; returns 0 on success */
#define VGO_MAX_HEIGHTFIELDS 8
int vgo_env_add_heightfield(vgo_env *e, const float *centre, const float *scale, int xd, int yd, const float *data);
int vgo_env_attach(vgo_env *e, const float *tf16, const float *spheres, int k);
void vgo_env_detach(vgo_env *e);
/* end-effector transform of one configuration: R row-major (9), then t (3) (Robot::eefk) */
void vgo_robot_ee_pose(const vgo_robot *r, const float *q, float *T);
/* kind 0..4: spheres, capsules, z-capsules, cuboids, z-cuboids; sorted by min_distance */
size_t vgo_env_count(const vgo_env *e, int kind);
/* fields of the idx-th object of a kind followed by its min_distance; returns the float count */
int vgo_env_get(const vgo_env *e, int kind, size_t idx, float *out);

/* ------------------------------------------------------------------------- robots (robots/<robot>.hh) */
const vgo_robot *vgo_robot_get(const char *name);
int vgo_robot_dim(const vgo_robot *r);
int vgo_robot_slots(const vgo_robot *r);
int vgo_robot_fine(const vgo_robot *r);
int vgo_robot_resolution(const vgo_robot *r);
void vgo_robot_limits(const vgo_robot *r, float *s_m, float *s_a);
/* all sphere slots (fine, then coarse) for one configuration, FP32 and FP64 */
void vgo_robot_spheres_f32(const vgo_robot *r, const float *q, float *out);
void vgo_robot_spheres_f64(const vgo_robot *r, const double *q, double *out);

/* objects added so far (insertion ids run 0 .. total-1 over all kinds) */
int vgo_env_total(const vgo_env *e);
/* fine self pairs over all self checks */
int vgo_robot_self_pairs(const vgo_robot *r);
/* Robot::fkcc_debug for one configuration: env_words [fine][words] (bit = insertion id of an
 * object the sphere collides with), pairs [self pairs] (1 = the fine pair collides) */
void vgo_debug(const vgo_robot *r, const vgo_env *e, const float *q, uint32_t *env_words, int words, uint8_t *pairs);
/* filter_self_from_pointcloud (bindings/robot_helper.hh:307-345): kept points to out (capacity
 * n), returns their number */
size_t vgo_filter_self(const vgo_robot *r, const vgo_env *e, const float *xyz, size_t n, float point_radius,
                       const float *q, float *out);
/* ------------------------------------------------------------------------------------- queries */
/* sphere_environment_in_collision over one block of `lanes` spheres (validity.hh:47-150) */
int vgo_sphere_env(const vgo_env *e, int lanes, const float *x, const float *y, const float *z, const float *r);
/* Robot::fkcc over one block; q is [lanes][dim].  Returns 1 if the block is valid. */
int vgo_fkcc(const vgo_robot *r, const vgo_env *e, int lanes, const float *q);
/* validate_motion<Robot, lanes, resolution> (planning/validate.hh:24-77).  Returns 1 if valid.
 * *blocks receives the number of fkcc calls made (may be NULL). */
int vgo_validate_motion(
    const vgo_robot *r, const vgo_env *e, int lanes, const float *a, const float *b, int resolution, int *blocks);
/* validate_vector<Robot, lanes, resolution> (planning/validate.hh:23-63): start, vector, and the
 * length that sets the block count.  Returns 1 if valid; *blocks as for vgo_validate_motion. */
int vgo_validate_vector(const vgo_robot *r, const vgo_env *e, int lanes, const float *start, const float *vector,
                        float distance, int resolution, int *blocks);
/* a batch of validate_vector on nthreads host threads (start, vector [n][dim], distance [n]) */
void vgo_validate_vectors(const vgo_robot *r, const vgo_env *e, int lanes, const float *start, const float *vector,
                          const float *distance, size_t n, int resolution, uint8_t *out, int32_t *blocks, int nthreads);
/* states visited by validate_motion, in visiting order: up to cap blocks of [lanes][dim] */
long vgo_motion_blocks(const vgo_robot *r, int lanes, const float *a, const float *b, int resolution, float *out, size_t cap);
/* number of blocks validate_motion would check if no block collides: max(ceil(L / lanes * res), 1) */
long vgo_motion_block_count(const vgo_robot *r, int lanes, const float *a, const float *b, int resolution);

/* batches, split over nthreads host threads.  out[i] = 1 if valid. */
void vgo_validate_states(const vgo_robot *r, const vgo_env *e, const float *q, size_t n, uint8_t *out, int nthreads);
void vgo_validate_motions(
    const vgo_robot *r,
    const vgo_env *e,
    int lanes,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    int nthreads);

/* FP64 signed distance to contact of one configuration: the minimum over the fine spheres of
 * (distance to each primitive - radius) and over the scheduled self pairs of (centre distance -
 * radii).  Negative inside.  Used to classify verdict differences near contact. */
double vgo_contact_distance_f64(const vgo_robot *r, const vgo_env *e, const double *q);

/* ------------------------------------------------------------------------ probes and counters */
/* The reference's 8-lane SIMD sqrt on x86 (v * rsqrt(v), vector/avx.hh:412-415) for one lane. */
float vgo_sqrt_x86(float v);
/* The lane sin/cos the FK uses. */
void vgo_sincos(float x, float *s, float *c);
/* CAPT of the idx-th pointcloud of an environment (NULL if none) */
const struct vgo_capt *vgo_env_capt(const vgo_env *e, int idx);

/* Work counters of the calling thread (reset with vgo_counters_reset): primitive tests executed
 * per kind (0..4), pointcloud queries, self-collision sphere pairs tested, sphere queries, fkcc
 * blocks evaluated, and lanes evaluated.  Counted per lane, as SIMD lanes do the work. */
typedef struct
{
    uint64_t tests[5];
    uint64_t capt_queries;
    uint64_t self_pairs;
    uint64_t sphere_queries;
    uint64_t blocks;
    uint64_t lanes;
} vgo_counters;
void vgo_counters_reset(void);
void vgo_counters_get(vgo_counters *out);
/* counted batch: single-threaded validate_motions that sums the counters over the batch */
void vgo_validate_motions_counted(
    const vgo_robot *r, const vgo_env *e, int lanes, const float *a, const float *b, size_t n, int resolution,
    uint8_t *out, vgo_counters *counters);

#ifdef __cplusplus
}
#endif
