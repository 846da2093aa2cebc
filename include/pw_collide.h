/*
 * pw_collide.h -- C ABI of the GB300 collision-query engine (libpwcollide.so).
 *
 * Drop-in boundary for the collision-query path of pyosr's UnitWorld
 * (lib/pyosr/module.cc:127-250, class UnitWorld; C++ in lib/osr/unit_world.cc).
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns an
 * int status (PW_OK or a PW_ERR_* code; the message is in pw_last_error()),
 * and never throws.  Batched queries take DEVICE pointers and a cudaStream_t
 * passed as `void *` (NULL = legacy default stream) and are asynchronous on
 * that stream.  Functions marked "host" take host memory and are synchronous.
 *
 * States are 7 doubles [x, y, z, w, qx, qy, qz] (lib/osr/osr_state.h:20-33),
 * row-major, one state per row.
 *
 * One world serves one query at a time: queries share the world's scratch
 * buffers, so concurrent queries on one world must be ordered on one stream.
 */
#ifndef PW_COLLIDE_H
#define PW_COLLIDE_H

#include <stdint.h>

#if defined(__GNUC__)
#define PW_API __attribute__((visibility("default")))
#else
#define PW_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PW_OK 0
#define PW_ERR_INVALID_ARG 1   /* bad pointer, size or value */
#define PW_ERR_CUDA 2          /* a CUDA runtime call failed */
#define PW_ERR_NO_MODEL 3      /* query before load/scale/angle set-up (isDisentangled throws here too) */
#define PW_ERR_OUT_OF_MEMORY 4
#define PW_ERR_CAPACITY 5      /* caller buffer too small; the required size is reported */
#define PW_ERR_INTERNAL 6      /* a device-side consistency check failed */

#define PW_GEO_ENV 0           /* UnitWorld::GEO_ENV, lib/osr/unit_world.h:26 */
#define PW_GEO_ROB 1           /* UnitWorld::GEO_ROB, lib/osr/unit_world.h:27 */

#define PW_SEG_TRANSIT 0       /* transit_state_to(_with_contact): step = verify_delta */
#define PW_SEG_TRANSITION 1    /* is_valid_transition: step = min(dist / 2, verify_delta) */

/* Node boxes of the BVH traversals (pw_world_set_node_boxes). */
#define PW_BOXES_ALIGNED 0     /* boxes aligned with each mesh's own frame */
#define PW_BOXES_ORIENTED 1    /* boxes along the principal axes of each node's vertices (default) */

/* Hierarchy of the BVHs (pw_world_set_bvh). */
#define PW_BVH_TOPDOWN 0       /* top-down (default): surface-area splits for meshes up to 65536 triangles, mean splits above */
#define PW_BVH_MORTON 1        /* Karras's LBVH over Morton codes */
#define PW_BVH_SAH 2           /* top-down, surface-area splits at any size */

/* Round phases of segment queries (pw_world_set_segment_phases). */
#define PW_PHASES_AUTO 0       /* phases when a call has at least 2^22 32-step chunks (default) */
#define PW_PHASES_OFF 1        /* every round in one phase */
#define PW_PHASES_ON 2         /* always eight phases */

/* First-contact codes written by pw_segments_first_contact (>= 0: step index). */
#define PW_STEP_FREE (-1)      /* every step free: the reference's `done` is true */
#define PW_STEP_NONE (-2)      /* verify_delta >= dist: no step checked, `done` false (unit_world.cc:445-447) */
#define PW_STEP_INVALID (-3)   /* not answered: a device-side capacity or step-bound check failed */

/* Bits of pw_query_stats.device_errors. */
#define PW_DEVERR_STEP_BOUND 1 /* a segment had more steps than its bound (never expected) */
#define PW_DEVERR_CKPT_CAP 2   /* graph mode: reserved checkpoint slots too few for a segment */
#define PW_DEVERR_ROUND_CAP 4  /* graph mode: the longest segment has more chunks than reserved */
#define PW_DEVERR_NONFINITE 8  /* a state had a NaN / infinite component; its verdict is 0 (not free) */
#define PW_DEVERR_WAIT 16      /* a bounded wait for a bulk copy ran out (never expected); the call's
                                  verdicts are not valid */

typedef struct pw_world pw_world;

typedef struct pw_world_info {
	double scene_scale;          /* UnitWorld::getSceneScale, 1 / max(span_env, span_rob) as float */
	double robot_center[3];      /* Scene::getCenter of the robot (possibly enforced) */
	double robot_ompl_center[3]; /* Scene::getOMPLCenter: float mean of the robot vertices */
	double scene_matrix[16];     /* getSceneMatrix, row-major 4x4 */
	double robot_matrix[16];     /* getRobotMatrix, row-major 4x4 */
	int64_t env_vertices, env_faces, robot_vertices, robot_faces;
	int32_t env_bvh_depth, robot_bvh_depth;
	int32_t ready;               /* 1 once angle_model has built both CD models */
	int32_t device;
} pw_world_info;

/* After pw_states_disentangled: retests = states the FP32 box test left to the
 * FP64 one (the others are 0).
 * After a contact enumeration (pw_intersecting_segments, _batch): queries = states,
 * retests = candidate triangle pairs tested in FP64, retest_hits = rows,
 * work_items = kernels of this library launched, reference_checks = states. */
typedef struct pw_query_stats {
	int64_t queries;             /* states or (segment, step) pairs examined */
	int64_t node_tests;          /* BVH node-pair box tests */
	int64_t leaf_tests;          /* FP32 triangle-pair tests */
	int64_t retests;             /* triangle pairs re-tested in FP64 */
	int64_t retest_hits;         /* FP64 re-tests that found contact */
	int64_t inline_retests;      /* FP64 re-tests done in the traversal kernel (queue full) */
	int64_t work_items;          /* work items the persistent kernel executed */
	int64_t reference_checks;    /* isValid calls the sequential reference loop makes for the same batch */
	int64_t detailed_chunks;     /* 32-step segment chunks that needed a transform per step */
	double traverse_ms;          /* device time of the traversal kernel (CUDA events on the query stream) */
	double retest_ms;            /* device time of the FP64 re-test kernel */
	int64_t device_errors;       /* PW_DEVERR_* bits: a device-side capacity or consistency check
	                                failed (the affected segments carry PW_STEP_INVALID), or a
	                                state was not finite */
	int64_t kernel_launches;     /* kernels of this library the query launched (CUB's sorts and scans
	                                not counted); pw_world_segments_contact_states adds its one to the
	                                segment query it follows */
} pw_query_stats;

/* Thread-local message for the last failing call on this thread. */
PW_API const char *pw_last_error(void);

/* World life cycle.  Replaces UnitWorld::UnitWorld / ~UnitWorld (unit_world.cc:64-74). */
PW_API int pw_world_create(pw_world **out, int device);
PW_API int pw_world_destroy(pw_world *w);

/* host: UnitWorld::loadModelFromFile / loadRobotFromFile (unit_world.cc:94-110) for an
 * already-parsed triangle mesh: nv float32 vertices (x, y, z) and nf uint32 index triples. */
PW_API int pw_world_load_env(pw_world *w, const float *V, int64_t nv, const uint32_t *F, int64_t nf);
PW_API int pw_world_load_robot(pw_world *w, const float *V, int64_t nv, const uint32_t *F, int64_t nf);

/* host: UnitWorld::enforceRobotCenter (unit_world.cc:114-118). */
PW_API int pw_world_enforce_robot_center(pw_world *w, const double center[3]);

/* host: UnitWorld::scaleToUnit (unit_world.cc:123-131). */
PW_API int pw_world_scale_to_unit(pw_world *w);

/* host: UnitWorld::angleModel (unit_world.cc:137-161): builds the CD vertices of both
 * meshes and their BVHs on the device.  Both angles must be 0, as in the reference. */
PW_API int pw_world_angle_model(pw_world *w, float latitude, float longitude);

/* host: UnitWorld::setPerturbation / getPerturbation (unit_world.cc:164-175). */
PW_API int pw_world_set_perturbation(pw_world *w, const double q[7]);
PW_API int pw_world_get_perturbation(const pw_world *w, double q[7]);

/* host: scene_scale, centres, scene_matrix / robot_matrix (module.cc:245-250). */
PW_API int pw_world_info_get(const pw_world *w, pw_world_info *out);

/* host: CD-model geometry, CDModel::vertices / faces (cdmodel.cc:232-242).
 * geo = PW_GEO_ENV (in the perturbation frame) or PW_GEO_ROB (robot local frame). */
PW_API int pw_world_cd_vertices(const pw_world *w, int geo, double *out);
PW_API int pw_world_cd_faces(const pw_world *w, int geo, int32_t *out);

/* device, async: UnitWorld::isValid (unit_world.cc:215-247) for n states.
 * valid[i] = 1 when the robot at states[i] touches no env triangle.  A state
 * with a non-finite component gets 0 and sets PW_DEVERR_NONFINITE (the
 * reference hands such a transform to FCL, whose answer is unspecified). */
PW_API int pw_states_valid(pw_world *w, const double *states, int64_t n, uint8_t *valid, void *stream);

/* device, async: the verdicts of pw_states_valid without allocating any device memory.
 * No counterpart in the reference.  For callers that may not allocate once running (a
 * host framework whose pool allocator owns the device heap, or a loop that cannot take
 * cudaMalloc's implicit synchronisation): the scratch lives in a fixed array inside the
 * library (about 16 MiB per GPU that loads it, held until exit).  At most 1048576 states
 * per call; larger batches are rejected with PW_ERR_INVALID_ARG.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and should come
 * before any stream capture.  All calls share the array, so calls whose work overlaps on
 * the GPU (different streams, different worlds on the same device) race; order them on
 * one stream.  It uses the world's launch configuration (pw_world_set_launch_config) as
 * pw_states_valid does.  When more pairs need the FP64 re-test than its queue holds
 * (1048576), the rest are re-tested inline by the traversal, with the same verdicts.
 * pw_world_last_stats does not report on this entry point. */
PW_API int pw_states_valid_noalloc(pw_world *w, const double *states, int64_t n, uint8_t *valid, void *stream);

/* device, async: UnitWorld::isDisentangled (unit_world.cc:249-264) for n states. */
PW_API int pw_states_disentangled(pw_world *w, const double *states, int64_t n, uint8_t *disentangled, void *stream);

/* device, async: UnitWorld::transitStateToWithContact (unit_world.cc:405-474) in PW_SEG_TRANSIT
 * mode, or isValidTransition (unit_world.cc:477-486) in PW_SEG_TRANSITION mode, for n segments
 * from[i] -> to[i].  first_step[i] = index of the first colliding step (0 = the first state
 * checked, at delta = verify_delta), PW_STEP_FREE or PW_STEP_NONE.  verify_delta must be > 0
 * and dist / verify_delta below 2^30 (the reference loop never ends for verify_delta <= 0). */
PW_API int pw_segments_first_contact(pw_world *w, const double *from, const double *to, int64_t n,
                              double verify_delta, int mode, int32_t *first_step, void *stream);

/* host in, host out, synchronous: UnitWorld::intersectingSegments (unit_world.cc:959-1012).
 * Writes up to `capacity` rows sorted by (env face, robot face): segment begins/ends (3 doubles
 * each), lengths, face pairs (env, robot) and coplanar flags; *count = total pairs found.
 * Returns PW_ERR_CAPACITY (with *count set) when capacity < *count. */
PW_API int pw_intersecting_segments(pw_world *w, const double q[7], int64_t capacity, double *begins,
                             double *ends, double *mags, int32_t *face_pairs, int32_t *coplanar,
                             int64_t *count);

/* host in, host out, synchronous: pw_intersecting_segments for n unit states at once
 * (one warp per state on the device, rows sorted on the device).  The rows of
 * state i are rows offsets[i] .. offsets[i + 1] - 1 (offsets has n + 1 entries), each
 * state's rows sorted by (env face, robot face); *total = rows of all states.
 * Returns PW_ERR_CAPACITY (with offsets and *total set, rows not all written) when
 * capacity < *total. */
PW_API int pw_intersecting_segments_batch(pw_world *w, const double *q, int64_t n, int64_t capacity, double *begins,
                                   double *ends, double *mags, int32_t *face_pairs, int32_t *coplanar,
                                   int64_t *offsets, int64_t *total);

/* Graph mode (on != 0): pw_segments_first_contact makes no host synchronisation
 * and no device allocation, so a caller can capture it into a CUDA graph and
 * replay it.  It then runs within the scratch sized by pw_segments_reserve or
 * by the last call made with graph mode off; segments that do not fit get
 * PW_STEP_INVALID and pw_world_last_stats reports device_errors.  Off by default. */
PW_API int pw_world_set_graph_mode(pw_world *w, int on);

/* host: an identifier of the world's current query scratch (its buffers'
 * addresses and sizes).  A call made outside graph mode may grow, and so move,
 * the scratch: a CUDA graph captured earlier is valid only while the epoch it
 * was captured under is unchanged. */
PW_API int pw_world_scratch_epoch(pw_world *w, uint64_t *out);

/* host: size the segment-query scratch for up to n segments with, in total, up
 * to total_chunks 32-step chunks and at most max_chunks chunks in one segment. */
PW_API int pw_segments_reserve(pw_world *w, int64_t n, int64_t total_chunks, int64_t max_chunks);

/* Launch configuration of the persistent traversal kernels (kernel 0: states,
 * 1: segments): width = queries a warp takes per grab (1..32, states only),
 * soft_cap = traversal stack entries before the warp narrows to depth-first
 * (>= 64, clamped to the stack), blocks = resident blocks per SM (clamped to
 * occupancy).  0 keeps the default.  Verdicts do not depend on it. */
PW_API int pw_world_set_launch_config(pw_world *w, int kernel, int width, int soft_cap, int blocks);
PW_API int pw_world_get_launch_config(pw_world *w, int kernel, int *width, int *soft_cap, int *blocks);

/* The node boxes a traversal kernel tests (kernel 0 = states, 1 = segments, -1 =
 * both): PW_BOXES_ORIENTED (default) or PW_BOXES_ALIGNED.  Both kinds are built
 * with every mesh; verdicts are identical, only the number of box and triangle
 * tests differs, and which is faster depends on the meshes and the workload (the
 * autotuner picks per kernel).  FCL's OBBRSS nodes (cdmodel.cc:17-18) are
 * oriented boxes; the LBVH here fits both kinds to the same hierarchy.  Not
 * allowed in graph mode (captured launches hold the kernel). */
PW_API int pw_world_set_node_boxes(pw_world *w, int kernel, int kind);
PW_API int pw_world_get_node_boxes(pw_world *w, int kernel, int *kind);

/* host: the hierarchy the next BVH build (pw_world_angle_model) uses.  Top-down:
 * each range of triangles split in the frame of its vertices' principal axes,
 * either at the mean of the centroids' projections on the first axis (the
 * OBBTree split, as FCL's OBBRSS build splits along a node's box axis) or at
 * the plane of least binned surface-area cost (16 bins on each axis); Morton:
 * Karras's LBVH.  All carry both node-box kinds; verdicts do not depend on the
 * choice. */
PW_API int pw_world_set_bvh(pw_world *w, int kind);
PW_API int pw_world_get_bvh(const pw_world *w, int *kind);

/* Round phases of pw_segments_first_contact.  The work of a segment query is its
 * 32-step chunks in chunk-major order (chunk j of every segment before chunk j + 1),
 * so that a contact found in one chunk prunes the segment's later chunks.  In
 * phases (rounds 0, 1, 2-3, 4-7, ..., 64 and above) the FP32 anchor frames of a
 * phase are computed only for chunks ahead of the contacts earlier phases found,
 * at the cost of one launch pair and one tail per phase: it pays for large
 * batches of long segments.  Results do not depend on the mode.  Not allowed in
 * graph mode (captured launches hold the phases). */
PW_API int pw_world_set_segment_phases(pw_world *w, int mode);
PW_API int pw_world_get_segment_phases(pw_world *w, int *mode);

/* The result tuple of transit_state_to_with_contact (unit_world.cc:405-474) for n
 * segments, from the codes pw_segments_first_contact(PW_SEG_TRANSIT) wrote for
 * the same segments and verify_delta (device arrays): last_free [n x 7],
 * contact [n x 7] (first colliding state, or the last state when done), done
 * [n] (1 = every step free), last_tau [n], tau [n].  *err_flag (device int,
 * zeroed by the caller) becomes non-zero if a code was PW_STEP_INVALID.
 * Used by touch sampling (src/GP/pipeline/touchq_util.py:8-27). */
PW_API int pw_segments_contact_states(const double *from, const double *to, const int32_t *first_step, int64_t n,
                                      double verify_delta, double *last_free, double *contact, uint8_t *done,
                                      float *last_tau, float *tau, int *err_flag, void *stream);

/* pw_segments_contact_states for the batch of this world's last
 * pw_segments_first_contact(PW_SEG_TRANSIT) call (same from, to, n and
 * verify_delta): starts each state from that call's 32-step checkpoints
 * instead of re-running the delta loop.  Any other batch takes the
 * pw_segments_contact_states path; the results are the same. */
PW_API int pw_world_segments_contact_states(pw_world *w, const double *from, const double *to,
                                            const int32_t *first_step, int64_t n, double verify_delta,
                                            double *last_free, double *contact, uint8_t *done, float *last_tau,
                                            float *tau, int *err_flag, void *stream);

/* Plate crossings of expansions (narrow-passage search): for candidate i (ends
 * [n x 7], device) from root i / per_root (roots, device), out[i] = 1 if some
 * probe point (robot-local unit frame, probes [nprobe <= 64 x 3], device) is on
 * different sides of the plane z = plane_z at the root and at the end, with
 * the straight-line crossing inside |x|, |y| <= extent.  Geometry only, FP32
 * (a candidate filter, not a verdict); no reference counterpart (the reference
 * has no narrow-passage expansion). */
PW_API int pw_expansion_crossings(const double *roots, const double *ends, int64_t n, int per_root,
                                  const double *probes, int nprobe, double plane_z, double extent, uint8_t *out,
                                  void *stream);

/* per_root perturbed copies of each of nroots states (device, [nroots x 7] ->
 * out [nroots * per_root x 7]): translation + N(0, sigma_t^2 I) and a rotation
 * vector ~ N(0, sigma_rot^2 I) applied on the left (as osr::apply,
 * osr_state.cc:244-259).  Counter-based random numbers: the same seed gives
 * the same candidates.  For narrow-passage expansion; no reference counterpart. */
PW_API int pw_expand_states(const double *roots, int64_t nroots, int per_root, double sigma_t, double sigma_rot,
                            uint64_t seed, double *out, void *stream);

/* device in, device out, async: the candidate states of
 * UnitWorld::enumFreeConfiguration / sampleFreeConfiguration
 * (lib/osr/unit_world.cc:1294-1389) for npairs surface pairs (points and
 * normals [npairs x 3]) and nspins spins each: the robot surface point plus
 * margin x normal placed on the environment's, normals opposed (shortest arc),
 * then spun about the environment normal.  half_cos / half_sin: cosine and sine
 * of half of each spin's angle, [nspins] shared by every pair (per_pair_angles
 * 0) or [npairs x nspins] (1).  out: [npairs x nspins x 7] unit states, FP64
 * with every operation rounded on its own in a fixed order (the oracle's
 * or_keyconf_states gives the same bits). */
PW_API int pw_keyconf_states(const double *rob_points, const double *rob_normals, const double *env_points,
                             const double *env_normals, int64_t npairs, double margin, const double *half_cos,
                             const double *half_sin, int64_t nspins, int per_pair_angles, double *out,
                             void *stream);

/* device in, device out, async: the random segments of touchq_util.calc_touch
 * (src/GP/pipeline/touchq_util.py:8-27) for nkeys keys [nkeys x 7], per_key
 * each: row i * per_key + j goes from key i (copied to from) to the key
 * translated by a random point of the unit sphere and rotated on the left by a
 * rotation vector uniform in the ball of radius 2 pi (osr::apply,
 * osr_state.cc:244-259), normalised.  Counter-based random numbers: the same
 * seed gives the same targets. */
PW_API int pw_touch_targets(const double *keys, int64_t nkeys, int per_key, uint64_t seed, double *from,
                            double *to, void *stream);

/* host: state-frame conversions (unit_world.cc:526-539, 689-711, 713-737). */
PW_API int pw_world_translate_to_unit(const pw_world *w, const double *in, int64_t n, double *out);
PW_API int pw_world_translate_from_unit(const pw_world *w, const double *in, int64_t n, double *out);
PW_API int pw_world_translate_ompl_to_unit(const pw_world *w, const double *in, int64_t n, double *out);
PW_API int pw_world_translate_unit_to_ompl(const pw_world *w, const double *in, int64_t n, double *out,
                                    int to_angle_axis);

/* device in, synchronous: OmplDriver::validateMotionPairs (lib/pyse3ompl/ompldriver.cc:597-621)
 * with OMPL's discrete motion validator, for n OMPL-frame motions from[i] -> to[i]
 * (x, y, z, qx, qy, qz, qw).  The state space is OMPL.app's SE(3) with the translation bounded
 * by lo / hi and the longest valid segment a fraction cdres of each component's extent
 * (setStateValidityCheckingResolution, ompldriver.cc:676-677).  valid[i] = 1 when to[i] and
 * every state interpolate(from[i], to[i], k / nd), k = 1 .. nd - 1, are collision free;
 * from[i] itself is not checked, as in OMPL.  A motion with a non-finite component gets 0.
 * The states are checked in passes, each over the motions still valid: the targets, then
 * dyadic levels (with m = nd - 1 and T = floor(log2 m), level l holds the odd multiples of
 * 2^(T - l) in 1 .. m), up to the first level no valid motion has; *states_checked (may be
 * NULL) = the states the passes checked, and pw_world_last_stats' kernel_launches counts the
 * whole call's kernels.  Rejects cdres outside (0, 1), bounds with lo > hi or no extent, and
 * motions of more than 2^31 - 1 segments. */
PW_API int pw_ompl_check_motions(pw_world *w, const double *from, const double *to, int64_t n,
                                 const double lo[3], const double hi[3], double cdres, uint8_t *valid,
                                 int64_t *states_checked, void *stream);

/* device in, synchronous: every state pw_ompl_check_motions may check, in the unit frame.
 * Motion i's states are rows offsets[i] .. offsets[i + 1] - 1 of `states`: first to[i], then the
 * interpolated states k = 1 .. nd - 1 (the check's passes skip those of motions found colliding
 * earlier).  offsets (device, n + 1 entries) may be NULL.  *total = the number of states;
 * PW_ERR_CAPACITY when it exceeds capacity, with *total and offsets written and `states`
 * untouched.  No counterpart in the reference: it exposes what the check looks at. */
PW_API int pw_ompl_motion_states(pw_world *w, const double *from, const double *to, int64_t n,
                                 const double lo[3], const double hi[3], double cdres, int64_t capacity,
                                 double *states, int64_t *offsets, int64_t *total, void *stream);

/* host: statistics of the last query on this world (synchronises its stream). */
PW_API int pw_world_last_stats(pw_world *w, pw_query_stats *out);

/* host: SE(3) state math with the engine's deterministic FP64 routines.
 * distance (osr_state.cc:130-154) and interpolate (osr_state.cc:27-44). */
PW_API int pw_state_distance(const double a[7], const double b[7], double *out);
PW_API int pw_state_interpolate(const double a[7], const double b[7], double tau, double out[7]);

/* host: the k-th state the reference stepping loop checks on a segment and its tau
 * (unit_world.cc:445-470); *num_steps = number of steps of the whole segment. */
PW_API int pw_segment_step_state(const double from[7], const double to[7], double verify_delta, int64_t k,
                          double out[7], double *tau, int64_t *num_steps);

#ifdef __cplusplus
}
#endif

#endif /* PW_COLLIDE_H */
