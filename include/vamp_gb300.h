/* vamp_gb300: GPU (sm_103a) collision checking behind a plain C ABI.
 *
 * This is the drop-in boundary for VAMP's data-parallel hot path: batched robot forward
 * kinematics fused with sphere-vs-environment collision checking.  Every entry point takes
 * plain pointers and sizes; none allocates on behalf of the caller except where stated.
 * All functions return VG_OK (0) or a negative VG_ERR_* code; vg_last_error() describes the
 * last failure of the calling thread.  There is no CPU fallback: without a usable GPU the
 * check functions fail with VG_ERR_CUDA.
 *
 * Semantics.  Verdicts follow the reference's compiled code: an edge is checked in blocks of
 * `lanes` states exactly as planning::validate_motion<Robot, lanes, resolution> visits them, and
 * decisions the reference takes per SIMD block (coarse-sphere gating, the early exit of the
 * primitive loop) are taken per block here too.  vg_env_set_mode() selects which reference
 * build is reproduced: lanes 8 with the x86 rsqrt-based bound (AVX2, the default) or lanes 4
 * with an exact square root (NEON).
 *
 * Threading.  Calls that share a vg_env must not overlap (they share its scratch counter and
 * staging buffers); use one environment per concurrent stream.  Environments are not
 * thread-safe without external locking, like the reference's (planning is single-threaded).
 *
 * Reference paths below are relative to the reference's src/impl/vamp/ unless noted.
 */
#ifndef VAMP_GB300_H
#define VAMP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VG_OK 0
#define VG_ERR_ARG (-1)     /* invalid argument (null pointer, bad size, unknown robot) */
#define VG_ERR_CUDA (-2)    /* CUDA runtime failure or no usable device */
#define VG_ERR_NOMEM (-3)   /* host or device allocation failed */
#define VG_ERR_STATE (-4)   /* operation not valid in the object's current state */
#define VG_ERR_LIMIT (-5)   /* input exceeds a documented size limit */

#define VG_SQRT_X86 0   /* sqrt(v) = v * rsqrt(v) as the AVX2 build computes it (vector/avx.hh:412-415) */
#define VG_SQRT_EXACT 1 /* correctly rounded sqrt as the NEON build computes it (vector/neon.hh:520-523) */

typedef struct vg_env vg_env;
typedef struct vg_mlp vg_mlp;
typedef struct vg_batch vg_batch;

/* Message for the calling thread's last error ("" if none). */
const char *vg_last_error(void);
const char *vg_version(void);

/* ------------------------------------------------------------------------------- robots
 * Robots: "panda", "ur5", "fetch", "baxter".  Replaces the per-robot constants of
 * robots/<robot>.hh:11-18 (dimension, n_spheres, min_radius, max_radius, resolution). */
int vg_robot_info(const char *robot, int *dim, int *n_spheres, float *r_min, float *r_max, int *resolution);
/* Joint scaling q = u * s_m + s_a (robots/panda.hh:50-80, scale_configuration).  dim floats each. */
int vg_robot_limits(const char *robot, float *s_m, float *s_a);

/* --------------------------------------------------------------------------- environment
 * Replaces collision::Environment<float> and its Python constructors
 * (collision/environment.hh:15-85, bindings/environment.cc:109-165). */
vg_env *vg_env_create(void);
void vg_env_destroy(vg_env *env);
/* Sphere x y z r (collision/shapes.hh:217-251). */
int vg_env_add_sphere(vg_env *env, const float *xyzr);
/* Capsule x1 y1 z1 xv yv zv r rdv with rdv = 1 / (v . v) (collision/shapes.hh:122-214);
 * stored as z-aligned when xv == yv == 0, as Environment.add_capsule does
 * (bindings/environment.cc:132-145). */
int vg_env_add_capsule(vg_env *env, const float *fields8);
/* Cuboid: centre xyz, axis_1 xyz, axis_2 xyz, axis_3 xyz, half extents (collision/shapes.hh:29-120);
 * stored as z-aligned when axis_3_z == 1 (bindings/environment.cc:118-131). */
int vg_env_add_cuboid(vg_env *env, const float *fields15);
/* One primitive in the kind list the caller chose (0 spheres, 1 capsules, 2 z-aligned capsules,
 * 3 cuboids, 4 z-aligned cuboids; fields as vg_env_add_sphere / _capsule / _cuboid) with the
 * min_distance the caller computed: the form a converted collision::Environment<FloatVector<rake>>
 * needs (collision/environment.hh:15-85), whose objects already sit in their kind lists
 * (Shape::min_distance, collision/shapes.hh:9-12).  Kept sorted by min_distance, as
 * Environment::sort (collision/environment.hh:43-69) leaves them. */
int vg_env_add_primitive(vg_env *env, int kind, const float *fields, float min_distance);
/* A pointcloud tree as the reference built it (collision/capt.hh:584-617), in the layout
 * vg_env_pointcloud_layout returns: tests[2^nlog2 - 1], aabbs[2^nlog2][6], aff_starts[2^nlog2 + 1]
 * (non-decreasing, in 8-point blocks, the last equal to n_blocks), aff[n_blocks][3][8], top[6],
 * and the tree's r_min, r_max, r_point.  For converting a collision::CAPT without rebuilding it. */
int vg_env_add_pointcloud_layout(vg_env *env, int nlog2, const float *tests, const float *aabbs, const uint32_t *aff_starts,
                                 const float *aff, size_t n_blocks, const float *top, float r_min, float r_max,
                                 float r_point);
/* A pointcloud, checked as a CAPT built exactly as the reference builds it
 * (collision/capt.hh:294-365; Environment.add_pointcloud, bindings/environment.cc:150-161):
 * xyz is [n][3], n >= 2; queries pad sphere radii by r_point; the tree affords points for radii
 * up to r_max.  At most 4 pointclouds per environment. */
int vg_env_add_pointcloud(vg_env *env, const float *xyz, size_t n, float r_min, float r_max, float r_point);
/* The same tree as vg_env_add_pointcloud, built on the current GPU (no counterpart in the
 * reference, whose CAPT is built on the host: collision/capt.hh:294-365): xyz is a device array
 * [n][3] on that GPU; the call returns once the tree is built (synchronous on `stream`, a
 * cudaStream_t or NULL).  The layout is bit-identical to the host build's.  Points must be
 * finite (as for the host build, whose median sort is undefined for NaN). */
int vg_env_add_pointcloud_device(vg_env *env, const float *xyz, size_t n, float r_min, float r_max, float r_point,
                                 void *stream);
/* The reference's pointcloud filter on the current GPU (collision/filter.hh:176-320,
 * filter_pointcloud; Python binding bindings/environment.cc:167-197): keeps a subset of xyz[n][3]
 * in which no two consecutive points of six Morton-order passes lie within min_dist, and, when
 * cull != 0, only points closer than max_range to origin[3] and inside the box workcell_min[3]
 * .. workcell_max[3] (plus the reference's extra copy of point 0 when any point was culled).
 * origin and the workcell are host arrays.  Equal Morton codes keep their previous order (the
 * reference sorts with the unstable pdqsort; with a stable sort its results are these).  The
 * kept points go to out (capacity n points), their number to *n_out.
 *   _device: xyz and out on the current GPU; synchronous on `stream` (a cudaStream_t or NULL).
 *   host form: xyz and out in host memory; *elapsed_ns (if non-NULL) gets the call's wall time,
 *   as the reference's binding returns it.
 * Coordinates must be finite.  Runs of more than 32,768 consecutive points within min_dist of one
 * another cost time in proportion to their length (the tile skipping handles the rest). */
int vg_filter_pointcloud_device(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                                const float *workcell_min, const float *workcell_max, int cull, float *out, size_t *n_out,
                                void *stream);
int vg_filter_pointcloud(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                         const float *workcell_min, const float *workcell_max, int cull, float *out, size_t *n_out,
                         uint64_t *elapsed_ns);
/* filter_self_from_pointcloud (bindings/robot_helper.hh:307-345): the points of xyz[n][3], as
 * spheres of point_radius, that collide with no fine sphere of the robot at configuration
 * q[dim] (a host array) and with no object of env, in input order, to out (capacity n); their
 * number to *n_out.  _device: xyz and out on the GPU, synchronous on `stream`; host form: host
 * buffers. */
int vg_filter_self_from_pointcloud_device(const char *robot, vg_env *env, const float *xyz, size_t n, float point_radius,
                                          const float *q, float *out, size_t *n_out, void *stream);
int vg_filter_self_from_pointcloud(const char *robot, vg_env *env, const float *xyz, size_t n, float point_radius,
                                   const float *q, float *out, size_t *n_out);
/* The tree of the index-th pointcloud (collision/capt.hh:584-617): sizes = {nlog2, tests,
 * leaves, 8-point blocks}; then, if non-NULL, tests[tests], aabbs[leaves][6], aff_starts[leaves
 * + 1], aff[blocks][3][8] (x, y, z planes of each block), top[6].  Call with NULL arrays for the
 * sizes. */
int vg_env_pointcloud_layout(const vg_env *env, int index, uint64_t *sizes, float *tests, float *aabbs,
                             uint32_t *aff_starts, float *aff, float *top);
/* A heightfield (collision/shapes.hh:250-311; factory heightfield::flat, collision/factory.hh:
 * 365-386; Environment.add_heightfield, bindings/environment.cc:146-149): xd x yd samples
 * (data[y * xd + x]), placed at centre[3], cells scale[0] x scale[1], heights data / scale[2] +
 * centre[2].  Checked by sphere_heightfield (collision/sphere_heightfield.hh:9-30) in every
 * environment query.  At most 8 per environment and 2^24 samples each. */
int vg_env_add_heightfield(vg_env *env, const float *centre, const float *scale, size_t xd, size_t yd, const float *data);
/* An attachment (collision/attachments.hh:11-56; Environment.attach / detach,
 * bindings/environment.cc:162-165; vamp.Attachment, :200-230): k spheres {x, y, z, r} in a frame
 * at the row-major 4x4 transform tf16 from the robot's end effector.  The environment copies
 * them; while attached, every check runs Robot::fkcc_attach (robots/panda.hh:10265-15445, chosen
 * by planning/validate.hh:43,58), which also tests the posed spheres against the environment and
 * the robot links the reference lists.  At most VG_MAX_ATTACH_SPHERES spheres. */
#define VG_MAX_ATTACH_SPHERES 64
int vg_env_attach(vg_env *env, const float *tf16, const float *spheres, size_t k);
/* A heightfield from the fields a collision::HeightField stores (collision/shapes.hh:250-311):
 * offsets x y z and the (already inverted) scales xs ys zs, then the xd x yd samples. */
int vg_env_add_heightfield_fields(vg_env *env, const float *fields6, size_t xd, size_t yd, const float *data);
int vg_env_detach(vg_env *env);
/* Robot::eefk (robots/panda.hh:15447-15552; binding robot_helper.hh:302-305,580): the end
 * effector's transform, row-major 4x4, for configurations q[n][dim].  _device: q and out on the
 * current GPU (stream-ordered); host form: host buffers (synchronous). */
int vg_eefk_device(const char *robot, const float *q, size_t n, float *out, void *stream);
int vg_eefk(const char *robot, const float *q, size_t n, float *out);
/* Which reference build to reproduce: lanes 8 + VG_SQRT_X86 (default) or lanes 4 + VG_SQRT_EXACT. */
int vg_env_set_mode(vg_env *env, int lanes, int sqrt_mode);
/* How vg_validate_motions schedules edges on the GPU (verdicts are the same either way):
 * 1 = a warp checks consecutive blocks of one edge, 0 = each lane-block checks its own edge, 2 = as
 * 1 with the kernel built for fewer resident blocks and more registers per thread, 3 = as 2 with
 * the segments an edge's last blocks leave free starting on the next edge, -1 (default) = each
 * robot's own (2 for the Panda, UR5 and Fetch, 1 for Baxter).  An autotuner pick
 * (vg_autotune_motions) takes precedence until this is called again.
 * No reference counterpart: the reference validates one edge at a time on one core. */
int vg_env_set_schedule(vg_env *env, int schedule);
/* Number of objects of a kind (0 spheres, 1 capsules, 2 z-capsules, 3 cuboids, 4 z-cuboids)
 * and the fields of one, in checking order, followed by its min_distance. */
int vg_env_count(const vg_env *env, int kind, size_t *count);
int vg_env_get(const vg_env *env, int kind, size_t index, float *out);

/* ----------------------------------------------------------------------- checks (device)
 * Inputs and outputs in device memory; asynchronous on `stream` (a cudaStream_t, or NULL for
 * the default stream).  Configurations are row-major [n][dim] float32. */

/* Per-configuration validity: out[i] = 1 if configuration i is collision free.
 * Replaces Robot::fkcc on a broadcast block, i.e. the Python binding's validate()
 * (bindings/robot_helper.hh:256-267; robots/panda.hh:5227 fkcc). */
int vg_validate_states_device(const char *robot, vg_env *env, const float *q, size_t n, uint8_t *out, void *stream);

/* planning::validate_vector<Robot, lanes, resolution> (planning/validate.hh:23-63), as the
 * reference's planners call it (rrtc.hh:136,176; aorrtc.hh:191,227,280): edge e starts at
 * start[e][dim], moves by vector[e][dim], and is checked in max(ceil(distance[e] / lanes *
 * resolution), 1) blocks, distance[e] being the length the caller gives.  _device: device
 * pointers, stream-ordered, optional blocks[n]; host form: host buffers, synchronous. */
int vg_validate_vectors_device(const char *robot, vg_env *env, const float *start, const float *vector,
                               const float *distance, size_t n, int resolution, uint8_t *out, int32_t *blocks,
                               void *stream);
int vg_validate_vectors(const char *robot, vg_env *env, const float *start, const float *vector, const float *distance,
                        size_t n, int resolution, uint8_t *out);
/* Per-edge validity of the straight-line motions a[i] -> b[i]: out[i] = 1 if valid.
 * Replaces planning::validate_motion<Robot, lanes, resolution> (planning/validate.hh:24-77).
 * blocks (optional, may be NULL) receives the number of lane-blocks checked per edge. */
int vg_validate_motions_device(
    const char *robot,
    vg_env *env,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    void *stream);

/* Allocation-free form of vg_validate_motions_device, for callers that must not allocate GPU
 * memory while they run (a real-time planner that reserves all memory up front so no call can
 * block on the allocator or run out of memory mid-plan; a framework that owns device memory
 * through its own pool).  No counterpart in the reference, which runs on the CPU.  Same verdicts
 * and block counts; allocates nothing.  Its only scratch, the edge kernel's work counter, is a
 * fixed 256-byte device array inside the library that every GPU loading the library keeps until
 * exit.  Requirements: env already uploaded to the current device by an earlier ordinary check
 * call and unchanged since (VG_ERR_STATE otherwise); n <= 2^31 - 1 (VG_ERR_LIMIT).  The first
 * call on each device looks up the array's device address: make it before any stream capture.
 * Under CUDA's lazy module loading the driver loads a kernel the first time it runs, which may
 * allocate: let the earlier ordinary call be a vg_validate_motions_device with the same robot,
 * environment settings and schedule (so the same kernel is already loaded), or run with
 * CUDA_MODULE_LOADING=EAGER.
 * All calls share the array (the counter is cleared on `stream` before each launch): calls whose
 * kernels overlap on the GPU race, so issue them on one stream or wait between them. */
int vg_validate_motions_device_noalloc(
    const char *robot,
    const vg_env *env,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    void *stream);

/* Sphere centres and radii of every sphere slot (fine spheres, then each checked link's coarse
 * sphere), out is [n][slots][4].  Replaces Robot::sphere_fk (robots/panda.hh:117-462). */
int vg_sphere_fk_device(const char *robot, const float *q, size_t n, float *out, void *stream);
/* Robot::fkcc<rake> (robots/panda.hh:5226-5229; ur5.hh:3218, fetch.hh:17185, baxter.hh:12710) on
 * caller-given ConfigurationBlocks: q is [n_blocks][lanes][dim] with lanes the environment's
 * (vg_env_set_mode: 8 or 4); out[b] = 1 when block b is valid, with the reference's block
 * semantics (a coarse sphere that hits in any lane gates the fine tests of every lane).  Device
 * form: device buffers on the current GPU, stream-ordered; host form: host buffers,
 * synchronous. */
int vg_fkcc_blocks_device(const char *robot, vg_env *env, const float *q, size_t n_blocks, uint8_t *out, void *stream);
int vg_fkcc_blocks(const char *robot, vg_env *env, const float *q, size_t n_blocks, uint8_t *out);

/* ------------------------------------------------------------------------- checks (host)
 * Same as the device forms with host buffers: copies in, checks, copies out, and waits.
 * Pinned buffers (vg_host_alloc) make the copies fastest.  Staging memory is owned by env.
 * vg_validate_motions and vg_validate_vectors check a batch of at most 4,096 blocks in all (a
 * planner's single edge, say) block by block: the blocks are built on the host with the edge
 * kernels' arithmetic and checked at once by the blocks kernel, an edge being valid when all its
 * blocks are; larger batches go to the edge kernels.  The verdicts are the same either way. */
int vg_validate_states(const char *robot, vg_env *env, const float *q, size_t n, uint8_t *out);
int vg_validate_motions(
    const char *robot, vg_env *env, const float *a, const float *b, size_t n, int resolution, uint8_t *out);
int vg_sphere_fk(const char *robot, const float *q, size_t n, float *out);

/* ------------------------------------------------------------------------- debug reports
 * Replaces Robot::fkcc_debug (robots/panda.hh:468), the per-sphere collision listing behind the
 * Python binding's debug() (bindings/robot_helper.hh:249-253, 585-589), for a batch of
 * configurations.  For each configuration: env_bits [fine][words], a bit per environment object
 * a fine sphere collides with (sphere_environment_get_collisions' rule, collision/validity.hh:
 * 152-249; pointclouds are not part of it), the bit index being the object's insertion order
 * among the environment's primitives (the reference reports object names); pairs [self_pairs],
 * 1 for each fine self pair that collides, pairs in the order of the robot's self checks (the
 * reference's order; it reports the colliding pairs' sphere indices).  Sizes from
 * vg_debug_sizes.  The device form is synchronous (it allocates and frees its scratch). */
int vg_debug_sizes(const char *robot, const vg_env *env, int *fine, int *words, int *self_pairs);
int vg_debug_device(const char *robot, vg_env *env, const float *q, size_t n, uint32_t *env_bits, uint8_t *pairs,
                    void *stream);
int vg_debug(const char *robot, vg_env *env, const float *q, size_t n, uint32_t *env_bits, uint8_t *pairs);

/* ------------------------------------------------------------------- tensor-core GEMM
 * D[M][N] (fp32) = A[M][K] * B[N][K]^T with A, B row-major bf16 (device pointers), on the 5th-
 * generation tensor cores (tcgen05, FP32 accumulation in tensor memory).  M % 128 == 0,
 * 16 <= N <= 256 with N % 16 == 0, K % 16 == 0.  *err (device int) is set to 1 if a kernel gave
 * up waiting for its MMAs.  The building block of the learned block ordering's MLP; no
 * counterpart in the reference (which has no learned component). */
int vg_gemm_bf16_device(const void *a, const void *b, float *d, int M, int N, int K, int *err, void *stream);

/* ------------------------------------------------------------- learned block ordering
 * None of these has a counterpart in the reference, which checks an edge's blocks in one fixed
 * order (planning/validate.hh:40-66).  They change which blocks of an edge are checked first,
 * never a verdict.
 *
 * A collision predictor for one robot: features sin(q_d), cos(q_d) (zero-padded to 16 or 32
 * columns) -> 256 -> 256 -> 1 with ReLU, BF16 weights and activations, FP32 accumulation, FP32
 * master weights.  Parameters, in order: W1 [256][kin], b1 [256], W2 [256][256], b2 [256],
 * w3 [256], b3 [1] with kin = 16 for dim <= 8, 32 for dim <= 16 (dim up to 16). */
vg_mlp *vg_mlp_create(int dim, uint64_t seed);
void vg_mlp_destroy(vg_mlp *m);
size_t vg_mlp_param_count(int dim);
int vg_mlp_get_params(const vg_mlp *m, float *out); /* host buffer of vg_mlp_param_count floats */
int vg_mlp_set_params(vg_mlp *m, const float *in);

/* Adam training (lr, beta 0.9 / 0.999) on n labelled configurations (device q [n][dim],
 * valid [n]: 1 = collision free, the exact checker's verdicts) for `epochs` passes in
 * minibatches of `batch` rows (a multiple of 128); the mean binary cross-entropy of each epoch
 * goes to losses[epochs] (host, may be NULL).  Synchronous. */
int vg_mlp_train_device(vg_mlp *m, const float *q, const uint8_t *valid, size_t n, int epochs, int batch, float lr,
                        float *losses, void *stream);

/* One forward and backward pass on n <= 65536 labelled configurations without an update:
 * gradients (host, vg_mlp_param_count floats, parameter order) of the mean loss, the loss, and
 * the BF16 features the GEMMs saw (host [n][kin] as floats, may be NULL).  For gradient checks. */
int vg_mlp_gradients(vg_mlp *m, const float *q, const uint8_t *valid, size_t n, float *grads, float *loss,
                     float *features);

/* Collision probability per configuration (device q [n][dim] -> p [n]): the training forward
 * (separate GEMM launches) and the fused inference kernel (weights resident in shared memory). */
int vg_mlp_predict_device(vg_mlp *m, const float *q, size_t n, float *p, void *stream);
int vg_mlp_infer_device(vg_mlp *m, const float *q, size_t n, float *p, void *stream);

/* Logits of `probes` (1..32) states per edge, the state at fraction (p + 0.5) / probes from a to
 * b: scores [n][probes]. */
int vg_mlp_score_edges_device(vg_mlp *m, const float *a, const float *b, size_t n, int probes, float *scores,
                              void *stream);

/* VG_OK, or VG_ERR_CUDA if a tensor-core kernel of m gave up waiting for its MMAs since the last
 * report (synchronous).  A kernel that gives up sets the flag, waits (with the default limit) for
 * the MMAs it issued, frees its tensor memory and returns; later kernels of m then do nothing
 * until this call reports the flag, which clears it. */
int vg_mlp_error(vg_mlp *m);
/* How many times m's tensor-core kernels poll an MMA-completion barrier before they give up
 * (negative: the default, 2^22; 0: give up at once, which the failure tests use).  The wait for
 * MMAs still in flight before tensor memory is released always uses the default. */
int vg_mlp_set_wait_limit(vg_mlp *m, long long polls);

/* validate_motion verdicts (those of vg_validate_motions_device, bit for bit) with each edge's
 * blocks checked in the order the scores rank them: block 0 first, then blocks by the largest
 * score over their states (probe scores interpolated along the edge); blocks past the 64th follow
 * in the reference's order.  scores [n][probes] (device), any collision score.  `blocks` gets the
 * number of blocks checked.  Always the same-edge schedule. */
int vg_validate_motions_scored_device(
    const char *robot,
    vg_env *env,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    const float *scores,
    int probes,
    uint8_t *out,
    int32_t *blocks,
    void *stream);

/* Scores with m (vg_mlp_score_edges_device into m's scratch) and checks in learned order
 * (vg_validate_motions_scored_device).  Calls sharing m must not overlap. */
int vg_validate_motions_learned_device(
    const char *robot,
    vg_env *env,
    vg_mlp *m,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    int probes,
    uint8_t *out,
    int32_t *blocks,
    void *stream);

/* ------------------------------------------------------------- autotuning and batches
 * Neither has a counterpart in the reference, which checks one edge per call on the calling
 * thread (planning/validate.hh:24-77; callers rrtc.hh:136,176, prm.hh:122,138, fcit.hh:238,333).
 *
 * vg_autotune_motions times the edge-check schedules on the given edges (device buffers, a
 * sample of the caller's workload) and keeps the fastest for this robot in env, where later edge
 * checks of that robot use it: a segment per edge (*schedule_out 0), a warp per edge (1), a
 * warp per edge built for fewer resident blocks and more registers (2), or the same with the
 * segments an edge's last blocks leave free starting on the next edge (3); and the resident
 * blocks per SM (*blocks_per_sm_out, 0 = as many as fit); *ms_out is its time on the
 * sample.  Verdicts do not depend on the pick.  vg_env_set_schedule clears the picks.
 * Synchronous. */
int vg_autotune_motions(const char *robot, vg_env *env, const float *a, const float *b, size_t n, int resolution,
                        int *schedule_out, int *blocks_per_sm_out, float *ms_out, void *stream);

/* A batch of edge checks (several robots, environments and edge sets; device buffers) run as
 * one CUDA graph: vg_batch_launch captures the checks on its first call (and after a change to
 * the batch or to one of its environments), one graph branch per check, and replays the graph
 * on later calls, so a caller that refills the same buffers pays one launch per batch.  With
 * mlp non-NULL a check scores `probes` states per edge with it and checks in learned order
 * (vg_validate_motions_learned_device).  Verdicts equal vg_validate_motions_device's.  Calls on
 * one batch must not overlap; the buffers must stay valid while the batch exists.  At most 64
 * checks per batch. */
vg_batch *vg_batch_create(void);
void vg_batch_destroy(vg_batch *b);
int vg_batch_add_motions(vg_batch *b, const char *robot, vg_env *env, const float *a, const float *goal, size_t n,
                         int resolution, vg_mlp *mlp, int probes, uint8_t *out, int32_t *blocks);
int vg_batch_launch(vg_batch *b, void *stream);

/* Page-locked host memory for the host-buffer calls. */
void *vg_host_alloc(size_t bytes);
void vg_host_free(void *p);

#ifdef __cplusplus
}
#endif

#endif /* VAMP_GB300_H */
