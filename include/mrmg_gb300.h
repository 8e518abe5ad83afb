/*
 * mrmg_gb300.h -- C ABI of the GB300 collision / distance / nearest-neighbour
 * backend for multi-robot multi-goal planners.
 *
 * Conventions
 *  - Every array argument named d_* is a DEVICE pointer (for example a torch
 *    tensor's data_ptr()), caller-owned, contiguous, row-major.  Host arrays
 *    (scene tables) are named h_* and are copied by the library.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default
 *    stream.  Calls on one scene handle must be serialised on one stream
 *    (the handle owns the call's scratch counters).
 *  - Verdict outputs are uint8: 1 = collision free, 0 = in collision (the
 *    Python bool of the reference).
 *  - Every function returns an int status: MRMG_OK (0) or a negative code;
 *    mrmg_last_error() gives a message for the calling thread.
 *  - Unless MRMG_FLAG_ASYNC is given, a call synchronises its stream before
 *    returning, so that device-side input errors are reported as its status.
 *
 * Reference paths are inside src/multi_robot_multi_goal_planning/ of
 * vhartman/multirobot-pathplanning-benchmark.
 */
#ifndef MRMG_GB300_H
#define MRMG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mrmg_scene mrmg_scene;

enum {
  MRMG_OK = 0,
  MRMG_ERR_ARG = -1,          /* bad argument or bad input value (ValueError)   */
  MRMG_ERR_CUDA = -2,         /* CUDA runtime error                             */
  MRMG_ERR_TIMEOUT = -3,      /* a bounded device wait ran out                  */
  MRMG_ERR_UNSUPPORTED = -4,  /* shape outside the compiled kernel variants     */
  MRMG_ERR_N_START = -5,      /* N_start > N (the reference asserts)            */
  MRMG_ERR_HOST = -6          /* host memory allocation failed (MemoryError);
                                 no C++ exception leaves an entry point         */
};

enum { MRMG_F32 = 0, MRMG_F64 = 1 };

/* distance metrics of batch_config_dist (problems/core/configuration.py:332-349) */
enum {
  MRMG_METRIC_EUCLIDEAN = 0,
  MRMG_METRIC_SUM_EUCLIDEAN = 1,
  MRMG_METRIC_MAX_EUCLIDEAN = 2,
  MRMG_METRIC_MAX = 3
};

/* per-agent cost metric and reduction of batch_config_cost
 * (problems/core/configuration.py:437-510) */
enum { MRMG_COST_EUCLIDEAN = 0, MRMG_COST_MAX = 1 };
enum { MRMG_REDUCE_MAX = 0, MRMG_REDUCE_SUM = 1 };

/* call flags
 *  MRMG_FLAG_ASYNC      return after enqueueing; the status of the device-side
 *                       input checks is then not reported (graph capture)
 *  MRMG_FLAG_FULL_EVAL  arm scenes: evaluate every interpolated configuration
 *                       and every sphere pair without stopping at the first
 *                       collision (same verdicts; used to measure the
 *                       kernel's throughput against its roofline)
 *  MRMG_FLAG_BATCH_FORM abstract scenes, mrmg_is_collision_free_batch: decide
 *                       Sphere obstacles with the arithmetic of
 *                       Sphere.batch_collides_with_sphere (abstract_env.py:
 *                       51-55: np.linalg.norm(..., axis=1) = rounded squares,
 *                       numpy's sum, sqrt) instead of the single form's
 *                       (:44-47: the norm of one vector, a fused dot
 *                       product); the two differ on ties within an ulp of the
 *                       contact distance.  _batch_is_collision_free
 *                       (abstract_env.py:278-299) is the AND of the verdicts
 *                       of this form.  Rectangle obstacles and agent pairs
 *                       use the same arithmetic in both forms; arm scenes
 *                       have no Sphere obstacles and ignore the flag. */
enum { MRMG_FLAG_ASYNC = 1, MRMG_FLAG_FULL_EVAL = 2, MRMG_FLAG_BATCH_FORM = 4 };

const char *mrmg_version(void);
const char *mrmg_last_error(void);

/* ------------------------------------------------------------------------ */
/* Scenes                                                                    */
/* ------------------------------------------------------------------------ */

/* Abstract point-agent scene: spherical agents whose position is their slice
 * of the configuration, among axis-aligned boxes and sphere obstacles.
 * Replaces AbstractEnvironment's scene state (problems/abstract_env.py:112-131,
 * Sphere :41-58, Rectangle :61-109).
 *   h_agent_offsets[A]      start of agent i's slice in q (all agents have `dim` coords)
 *   h_agent_radius[A]       agent_radii
 *   h_pair_threshold[A*A]   agent_radii[i] + agent_radii[j]      (:266)
 *   h_agent_radius_sq[A]    agent_radii[i] ** 2                  (:84)
 *   h_box_lo/h_box_hi[nb*dim] Rectangle min_bounds / max_bounds  (:66-67)
 *   h_sphere_pos[ns*dim], h_sphere_radius[ns]
 *   h_sphere_threshold[ns*A] sphere.radius + agent_radii[i]      (:47)
 * dim must be 1..15, A <= 16. */
int mrmg_abstract_scene_create(int32_t n_agents, int32_t dim, int32_t q_dim,
                               const int64_t *h_agent_offsets, const double *h_agent_radius,
                               const double *h_pair_threshold, const double *h_agent_radius_sq,
                               int32_t n_boxes, const double *h_box_lo, const double *h_box_hi,
                               int32_t n_spheres, const double *h_sphere_pos,
                               const double *h_sphere_radius, const double *h_sphere_threshold,
                               mrmg_scene **out);

/* Sphere-arm scene: R serial DH arms (base kind 0 = fixed pose, 1 = planar
 * x,y,theta base followed by a fixed mount) carrying collision spheres, among
 * axis-aligned boxes.  New: the reference delegates robot geometry to external
 * engines (rai_base_env.py:442-477, pinocchio_env.py:410-500); the per-pair
 * tests restate Rectangle.collides_with_sphere (abstract_env.py:69-84) and the
 * agent-agent rule (abstract_env.py:261-268) for every pair of spheres on
 * different robots.
 *   h_q_offset[R]        first configuration index of robot r
 *   h_base_kind[R]       0 fixed, 1 planar (consumes x, y, theta before the arm joints)
 *   h_base_pose[R*12]    rotation (row-major 3x3) then translation: fixed base pose,
 *                        or the mount transform applied after the planar base
 *   h_n_links[R]         DH links (<= 8); joint k of robot r is q[offset(+3) + k]
 *   h_dh[R*8*4]          per link: a, d, cos(alpha), sin(alpha)  (standard DH,
 *                        T_k = T_{k-1} Rz(theta) Tz(d) Tx(a) Rx(alpha))
 *   h_sphere_robot[S], h_sphere_link[S] (0 = base frame, k = after link k)
 *   h_sphere_local[S*3]  centre in that frame; h_sphere_radius[S]
 *   h_box_lo/h_box_hi[B*3]
 *   band                 FP32 re-check band in metres (<= 0: derived from the
 *                        kinematic reach: 16 (L + 1) 2^-24 times the reach plus
 *                        4 2^-24 times the largest box coordinate)
 * R <= 16, D <= 96, S <= 1024, B <= 1024. */
int mrmg_arm_scene_create(int32_t n_robots, int32_t q_dim, const int32_t *h_q_offset,
                          const int32_t *h_base_kind, const double *h_base_pose,
                          const int32_t *h_n_links, const double *h_dh, int32_t n_spheres,
                          const int32_t *h_sphere_robot, const int32_t *h_sphere_link,
                          const double *h_sphere_local, const double *h_sphere_radius,
                          int32_t n_boxes, const double *h_box_lo, const double *h_box_hi,
                          double band, mrmg_scene **out);

/* Fixed joint-angle offsets of an arm scene: revolute joint j turns by
 * q[j] + h_offsets[j] (h_offsets[q_dim]; NULL clears them).  General serial
 * chains (URDF <origin> + <axis>, MJCF body frames) are brought to the
 * standard DH form of mrmg_arm_scene_create by an importer, and the DH angle
 * of a joint differs from the file's joint value by a constant: this offset.
 * Planar-base translations take no offset; |offset| <= 64.  The FP32 path adds
 * the offset in double-float before the angle reduction, the FP64 path with
 * one IEEE addition.  Synchronises the device (not capturable).  New: the
 * reference delegates kinematics to its engines (mujoco_env.py:380-409,
 * pinocchio_env.py:410-500). */
int mrmg_arm_scene_set_joint_offsets(mrmg_scene *scene, const double *h_offsets);

/* Per-mode scene tables (objects placed or attached by mode: the rai scenes'
 * set_to_mode, rai_base_env.py:704-840, and VAMP's
 * attached objects, mr_vamp_env.py:506-650).  The box pool is the scene's
 * boxes; mode m keeps boxes h_mode_boxes[h_mode_box_off[m] ..
 * h_mode_box_off[m+1]).  h_sphere_attach[S] (may be NULL) tags spheres that
 * belong to an attached object (id >= 0; -1 = part of the robot, always
 * present): mode m keeps the tagged spheres whose id is listed in
 * h_mode_attach[h_mode_attach_off[m] .. h_mode_attach_off[m+1]).  Each mode
 * gets its own device tables; set once per scene. */
int mrmg_arm_scene_set_modes(mrmg_scene *sc, int32_t n_modes, const int32_t *h_sphere_attach,
                             const int64_t *h_mode_box_off, const int32_t *h_mode_boxes,
                             const int64_t *h_mode_attach_off, const int32_t *h_mode_attach);

/* Selects the tables later calls on this scene use: mode m, or -1 for the
 * scene as created (every box and sphere).  A host-side switch; launches
 * already captured in a CUDA graph keep the tables of their capture. */
int mrmg_scene_set_mode(mrmg_scene *sc, int32_t mode);

int mrmg_scene_destroy(mrmg_scene *scene);

/* Scene facts: [0] kind (0 abstract, 1 arm), [1] q_dim, [2] spheres per group,
 * [3] groups, [4] inter-robot group pairs, [5] CTAs of the persistent grid,
 * [6] warps per CTA.  out_band gets the FP32 re-check band. */
int mrmg_scene_info(const mrmg_scene *scene, int64_t *out7, double *out_band);

/* *out = 1 when the current device reads pageable host memory coherently
 * (cudaDevAttrPageableMemoryAccess; GB300 over its host link), so kernels may
 * read callers' host arrays in place; 0 otherwise or when the environment
 * variable MRMG_STAGE_HOST_INPUTS=1 asks for staged copies. */
int mrmg_host_access(int32_t *out);

/* The serving batcher's input gather (serving.py): one launch copies every
 * planner instance's request arrays from host memory into a step's device
 * buffers -- configurations into rows [0, ccap) of both d_q1 and d_q2 (the
 * edge q -> q), edge starts and ends into rows [ccap, ccap + ecap), edge step
 * counts into d_N[ccap + ...], and step counts 3 for the configurations and
 * 2 for unused slots.  h_table (device-readable: pinned, or pageable where
 * mrmg_host_access says so) is int64 {n_src, n_configs, n_edges, 0}
 * followed by n_src rows of {source address, rows, first destination row,
 * kind (0 configurations, 1 starts, 2 ends, 3 step counts) | 0 << 32}; the
 * sources are C-contiguous FP32 [rows, q_dim] or int64 [rows] arrays the
 * device can read (pageable host memory where mrmg_host_access = 1).  The
 * table is read on the device when the launch runs (a CUDA graph may
 * capture the launch and rewrite the table between replays); rows outside
 * the capacities or n_src > max_src set E_BAD_INPUT in *d_err instead of
 * copying.  Asynchronous.  No reference counterpart. */
int mrmg_serving_gather(const void *h_table, int32_t max_src, int32_t q_dim, int64_t ccap, int64_t ecap,
                        float *d_q1, float *d_q2, int64_t *d_N, int32_t *d_err, void *stream);

/* The collision kernels stage a scene's FP32 tables (boxes, spheres, frames,
 * group pairs) into shared memory with one bulk asynchronous copy (the TMA
 * engine) of a table image built at scene creation, awaited on an mbarrier
 * with a bounded wait.  A copy that does not complete within the wait is
 * replaced by plain loads (the verdicts do not change) and counted here, for
 * the current device, since the library was loaded.  No reference
 * counterpart. */
int mrmg_table_stage_timeouts(uint32_t *out);

/* Launch shape of the persistent kernels (0 = automatic).  Used by the
 * autotuner; the verdicts never depend on it. */
int mrmg_scene_set_launch(mrmg_scene *scene, int32_t ctas, int32_t warps_per_cta);

/* Work-shape tuning of an arm scene's collision kernels; the verdicts never
 * depend on it, and launches already captured in a CUDA graph keep the
 * tuning of their capture.  box_block (1..32, 0 = default 8): boxes whose
 * near (sphere group, box) pairs are compacted and tested together -- the
 * obstacle tile; box_head (0..64, taken as given; 8 at creation): boxes
 * tested one by one, with an exit at the first hit, before the blocks on an
 * edge's first position; cfg_chunk (1..32, 0 = default 4): configurations a
 * warp takes from the work queue at a time; phase_b1 (1..64, 0 = default
 * 3): positions per surviving edge
 * in the first phase-B launch.  MRMG_ERR_UNSUPPORTED when box_block needs
 * more shared memory than a CTA has.  Synchronises the device. */
int mrmg_scene_set_tuning(mrmg_scene *scene, int32_t box_block, int32_t box_head, int32_t cfg_chunk,
                          int32_t phase_b1);

/* The current tuning: out4 = box_block, box_head, cfg_chunk, phase_b1. */
int mrmg_scene_get_tuning(const mrmg_scene *scene, int32_t *out4);

/* Test-order autotuning for an arm scene: for the sample configurations
 * d_q[n] (for example uniform in the joint limits) record which boxes each
 * one touches, then order the boxes by greedy set cover so that a colliding
 * configuration meets a touching box as early as possible.  Verdicts do not
 * depend on the order.  h_order_out[B] (optional) receives the new order as
 * indices into the current one.  Not capturable (it synchronises). */
int mrmg_arm_scene_tune_order(mrmg_scene *scene, const void *d_q, int32_t dtype, int64_t n,
                              int32_t *h_order_out, void *stream);

/* ------------------------------------------------------------------------ */
/* Collision checks                                                          */
/* ------------------------------------------------------------------------ */

/* Per-configuration verdicts for d_q[n, q_dim] (dtype MRMG_F32 or MRMG_F64).
 * Batched form of BaseProblem.is_collision_free (planning_env.py:1724-1734;
 * abstract_env.py:255-276); _batch_is_collision_free (abstract_env.py:278-299)
 * is the AND of these verdicts computed with MRMG_FLAG_BATCH_FORM. */
int mrmg_is_collision_free_batch(mrmg_scene *scene, const void *d_q, int32_t dtype, int64_t n,
                                 uint8_t *d_out, void *stream, int32_t flags);

/* is_collision_free_for_robot (rai_base_env.py:515-615, pinocchio_env.py:
 * 502-, called by the per-robot rejection sampler,
 * planners/collision_free_sampler.py:115-135) for a set of robots of an arm
 * scene, per configuration: a configuration is free for the set unless a
 * sphere of a robot in the set touches a box or a sphere of another robot in
 * the set (collisions with robots outside the set are ignored, as the
 * reference ignores collisions that involve another robot).  Bit r of
 * robot_mask selects robot r.  Exact, like is_collision_free.  The rai
 * engine's tolerance (a colliding configuration counts as free while the
 * scene's total penetration stays within collision_tolerance) is applied
 * above this call with mrmg_arm_total_penetration (env.py,
 * Gb300ArmEnvironment(penetration_tolerance=...)). */
int mrmg_is_collision_free_batch_robots(mrmg_scene *scene, const void *d_q, int32_t dtype, int64_t n,
                                        uint32_t robot_mask, uint8_t *d_out, void *stream, int32_t flags);

/* Per-edge verdicts for the linear edges d_q1[n] -> d_q2[n], interpolated at
 * `resolution` exactly as BaseProblem.is_edge_collision_free
 * (planning_env.py:1746-1763; abstract_env.py:301-354):
 *   N = max(2, int(max_k |q1_k - q2_k| / resolution) + 1) unless d_N gives it,
 *   indices generate_binary_search_indices(N)[N_start : min(N, N_max)]
 *   (planning_env.py:34-51), endpoints 0 and N-1 skipped unless
 *   include_endpoints, q = q1 + ((q2 - q1) / (N - 1)) * i in FP64.
 * d_N may be NULL; N_max < 0 means None.  N_start > N gives MRMG_ERR_N_START.
 * Buffers (device memory, not checked by the library): d_q1 and d_q2 hold
 * n * q_dim values of `dtype`, d_N (when given) n int64 step counts, d_out n
 * bytes.  The same holds for every batched call: d_q[n, q_dim] in, d_out[n]
 * out. */
int mrmg_is_edge_collision_free_batch(mrmg_scene *scene, const void *d_q1, const void *d_q2,
                                      int32_t dtype, int64_t n, double resolution,
                                      int32_t include_endpoints, const int64_t *d_N,
                                      int64_t N_start, int64_t N_max, uint8_t *d_out,
                                      void *stream, int32_t flags);

/* Host-pointer forms of the two checks, for the planners' one-call-at-a-time
 * pattern: is_collision_free (planning_env.py:1724-1734; callers
 * planners/rrtstar_base.py:626-629 via the samplers,
 * collision_free_sampler.py:110) and is_edge_collision_free
 * (planning_env.py:1746-1763; callers rrtstar_base.py:626-629,
 * prm_graph.py:675).  Inputs and verdicts are HOST memory: the library
 * copies the inputs into a pinned staging buffer of the scene, moves them to
 * the device in one copy together with the zeroed counters, checks them and
 * returns the verdicts (1 = free) and the status in one copy back; the call
 * is synchronous on the scene's own stream.  Arm scenes with up to 4,096
 * configurations or 256 edges (65,536 edge positions) run one kernel launch
 * in which every configuration or edge position is a warp's work item and a
 * configuration left pending by the FP32 pass is decided in FP64 at once;
 * other batches run the batched kernels on the staged inputs.  Verdicts and
 * status codes are those of mrmg_is_collision_free_batch /
 * mrmg_is_edge_collision_free_batch (robot_mask: 0 = every robot, else as
 * mrmg_is_collision_free_batch_robots; arm scenes only).  Buffers: h_q /
 * h_q1 / h_q2 hold n * q_dim values of `dtype`, h_N (optional) n int64, h_out
 * n bytes.  Calls on one scene must not overlap (one staging buffer per
 * scene); the staging buffer grows with the largest batch seen.  Where the
 * device reads pageable host memory coherently (cudaDevAttrPageableMemoryAccess,
 * e.g. a Grace CPU over NVLink-C2C), the kernels read the caller's input
 * arrays in place instead of a staged copy; the environment variable
 * MRMG_STAGE_HOST_INPUTS=1, read when a scene is created, forces staging. */
int mrmg_is_collision_free_host(mrmg_scene *scene, const void *h_q, int32_t dtype, int64_t n,
                                uint32_t robot_mask, uint8_t *h_out, int32_t flags);
int mrmg_is_edge_collision_free_host(mrmg_scene *scene, const void *h_q1, const void *h_q2, int32_t dtype,
                                     int64_t n, double resolution, int32_t include_endpoints,
                                     const int64_t *h_N, int64_t N_start, int64_t N_max, uint8_t *h_out,
                                     int32_t flags);

/* Edge check that allocates nothing.  No counterpart in the reference.
 * Same arguments, semantics and verdicts as mrmg_is_edge_collision_free_batch,
 * for callers that cannot allocate device memory while they check edges:
 * planner steps recorded into a CUDA graph (cudaMalloc is not a capturable
 * operation), real-time loops that forbid allocation after start-up, and
 * processes whose memory pool already owns the device.  The regular entry
 * point may grow the scene's scratch with cudaMalloc; this one uses a fixed
 * static device array instead and never allocates or frees.
 *   Limit: at most MRMG_NOALLOC_MAX_EDGES edges per call; larger batches
 *   return MRMG_ERR_ARG.  The array (256 B + 40 B per edge = 640 KiB) is
 *   held by every GPU that loads the library until the process exits.
 *   The first call on a device looks up the array's device address
 *   (cudaGetSymbolAddress); make that first call before any stream capture.
 *   The address is cached with the id of the device's CUDA context; a call
 *   in a new context (after cudaDeviceReset) looks it up again, and that
 *   call too should come before any stream capture.
 *   All calls share the array: calls that overlap on the GPU (other streams,
 *   threads or scenes) race and must be serialised by the caller.  A call
 *   also copies its counters into the scene's own counter words, so the
 *   word of mrmg_scene_error_word and mrmg_last_call_stats describe it (also
 *   when it was recorded into a graph with MRMG_FLAG_ASYNC), and its status
 *   lands in the scene's pinned host mirror: two calls on one scene that
 *   overlap on the GPU race there as well, whichever entry points they use.
 *   Flags: as the regular entry point (MRMG_FLAG_ASYNC, MRMG_FLAG_FULL_EVAL). */
#define MRMG_NOALLOC_MAX_EDGES 16384
int mrmg_is_edge_collision_free_batch_noalloc(mrmg_scene *scene, const void *d_q1, const void *d_q2,
                                              int32_t dtype, int64_t n, double resolution,
                                              int32_t include_endpoints, const int64_t *d_N,
                                              int64_t N_start, int64_t N_max, uint8_t *d_out,
                                              void *stream, int32_t flags);

/* Total penetration depth of each configuration of an arm scene, d_out[n]
 * (FP64, metres), as the rai engine's getCollisionsTotalPenetration that
 * is_collision_free and is_collision_free_for_robot compare with
 * collision_tolerance (rai_base_env.py:488-615): the sum over every
 * sphere-box pair of the radius minus the signed distance of the centre to
 * the box (outside the box the Euclidean distance, inside minus the distance
 * to the nearest face) and over every pair of spheres on different robots of
 * the two radii minus the centre distance, where positive; FP64 sphere
 * centres; each overlap rounded to a multiple of 2^-40 m and summed exactly,
 * so the total is independent of the order of the sum.  Robots' own
 * sphere pairs are not counted (the sphere model has no self-collision).
 * Synchronous. */
int mrmg_arm_total_penetration(mrmg_scene *scene, const void *d_q, int32_t dtype, int64_t n, double *d_out,
                               void *stream);

/* Sphere centres of an arm scene for d_q[n, q_dim]: d_c32[n, S, 3] from the
 * FP32 bulk path and d_c64[n, S, 3] from the exact FP64 path (either may be
 * NULL).  Used to verify the FP32 error bound against the re-check band. */
int mrmg_arm_sphere_centers(mrmg_scene *scene, const void *d_q, int32_t dtype, int64_t n,
                            float *d_c32, double *d_c64, void *stream);

/* Smoothed path-penetration cost of an arm scene and its gradient through
 * forward kinematics.  No counterpart in the reference: it feeds gradient
 * path repair and shortcutting (robot_mode_shortcut,
 * planners/shortcutting.py:87-244).  d_paths is [n_paths, n_waypoints,
 * q_dim] FP32.  h_params = {margin, scale, beta, smooth_weight}; per path
 *   cost = sum_t sum_pairs softplus(beta (margin - d)) / (beta scale)
 *        + smooth_weight * sum_t |w[t+1] - w[t]|^2
 * over every sphere-box pair (d = signed box distance of the centre minus the
 * radius) and every pair of spheres on different robots (d = centre distance
 * minus both radii).  Outputs (each may be NULL, not all): d_cost[n_paths]
 * (FP64), d_wp_cost[n_paths, n_waypoints] (the pair terms of waypoint t plus
 * its smoothness term towards t+1), d_grad[n_paths, n_waypoints, q_dim] =
 * d_grad_cost[p] * dcost_p/dw (d_grad_cost NULL means 1).  warps_per_cta 0 =
 * automatic (16).  The gradient runs as one launch, or -- when one CTA's
 * shared memory cannot hold every sphere's gradient for 32 waypoints (about
 * 270 spheres) -- as one launch per group of consecutive robots, each
 * writing its robots' joints (the cost then has its own launch).
 * Synchronises unless MRMG_FLAG_ASYNC. */
int mrmg_path_penetration(mrmg_scene *scene, const float *d_paths, int64_t n_paths,
                          int32_t n_waypoints, const double *h_params, const float *d_grad_cost,
                          double *d_cost, float *d_wp_cost, float *d_grad, int32_t warps_per_cta,
                          void *stream, int32_t flags);

/* Penetration-kernel facts: [0] spheres, [1] boxes, [2] shared memory per CTA
 * of the cost-only kernel, [3] of a single-launch gradient kernel covering
 * every robot (bytes, 16 warps; above the device's limit the gradient runs
 * per group of robots). */
int mrmg_penetration_info(const mrmg_scene *scene, int64_t *out4);

/* Graph-capture support.  A call made with MRMG_FLAG_ASYNC inside a stream
 * capture reports no status; its device-side error bits live in the word
 * returned here (valid until the next call on the scene), which a captured
 * graph can copy after each call.  mrmg_status_from_error_bits turns such
 * bits into the status the synchronous call would have returned.
 * mrmg_scene_reserve sizes the scene's scratch for batches of n items ahead
 * of a capture (allocation is not capturable). */
int mrmg_scene_error_word(mrmg_scene *scene, void **d_err);
int mrmg_scene_reserve(mrmg_scene *scene, int64_t n, void *stream);
int mrmg_status_from_error_bits(int32_t bits);

/* Statistics of the scene's last completed call: [0] items re-checked in
 * FP64 (pass two), [1] device error bits, [2] configurations evaluated by the
 * edge kernel's first pass, [3] reserved. */
int mrmg_last_call_stats(const mrmg_scene *scene, int64_t *out4);

/* Slot layout of an arm scene: out[slot] = input sphere index or -1 for a
 * padding slot (rows of mrmg_arm_sphere_centers are per slot).  Returns the
 * slot count, or a negative status. */
int mrmg_arm_slot_map(const mrmg_scene *scene, int32_t *out, int64_t cap);

/* Device-side generate_binary_search_indices(N) (planning_env.py:34-51),
 * written to d_out[N] (int64): chunked = 0 uses the closed-form position map
 * the parallel edge phases use, 1 the level-by-level iterator of the
 * sequential walks.  Exposes the edge kernels' index order. */
int mrmg_binary_search_indices(int64_t N, int64_t *d_out, int32_t chunked, void *stream);

/* ------------------------------------------------------------------------ */
/* Distances and costs (FP64, bit-identical to the reference)                */
/* ------------------------------------------------------------------------ */

/* d_out[q, m] = batch_config_dist(queries[q], nodes, metric)[m]
 * (problems/core/configuration.py:342-349 -> NpConfiguration._batch_dist
 * :303-329): diff = query - node, then
 *   euclidean      sqrt of the sequential sum of d*d over [0, slices[A-1].end)
 *   sum_euclidean  sum of the per-agent euclidean norms
 *   max_euclidean  max of the per-agent euclidean norms (strict '>')
 *   max            max |d| over all D coordinates
 * h_slices[A*2] are the agents' (start, end) (NpConfiguration._array_slice).
 * With Q = 1 this is batch_config_dist itself. */
int mrmg_config_dist_matrix(const double *d_queries, int64_t Q, const double *d_nodes, int64_t M,
                            int32_t D, const int64_t *h_slices, int32_t A, int32_t metric,
                            double *d_out, void *stream, int32_t flags);

/* batch_config_cost (problems/core/configuration.py:437-510): per-agent
 * euclidean norm or max |d| of the row difference, then max + w * sum
 * (reduction MRMG_REDUCE_MAX) or the sum.
 *   mode 0: d_starts is one row, diff = starts - ends[m]   (Configuration x array)
 *   mode 1: diff = starts[m] - ends[m]                      (array x array + slice)
 *   mode 2: diff = starts[m + 1] - starts[m], d_ends unused (path form, :460-472) */
int mrmg_batch_config_cost(const double *d_starts, const double *d_ends, int64_t M, int32_t D,
                           const int64_t *h_slices, int32_t A, int32_t cost_metric,
                           int32_t reduction, double w, int32_t mode, double *d_out, void *stream,
                           int32_t flags);

/* ------------------------------------------------------------------------ */
/* Per-mode nearest neighbours                                               */
/* ------------------------------------------------------------------------ */

/* Exact k nearest neighbours of every query within its mode: the k smallest
 * batch_config_dist(query, nodes of the mode, metric) values
 * (problems/core/configuration.py:303-349) in (distance, index) order --
 * the selection of PRM get_neighbors (planners/prm/prm_graph.py:441-447,
 * argpartition + argsort; ties, unspecified there, go to the lower index) and,
 * with k = 1, RRT nearest (planners/rrtstar_base.py:1228-1254, argmin).
 *   d_query_mode[Q]: mode of each query; d_mode_offsets[n_modes + 1]: the
 *   node range of each mode in d_nodes[M, D]; indices are local to the mode.
 *   Rows beyond the mode's size get index -1 and distance +inf.  k <= 64.
 *   The device arrays are read as given: every d_query_mode value must lie
 *   in [0, n_modes) and d_mode_offsets must rise from 0 to M (the Python
 *   binding checks both on the host). */
int mrmg_knn_exact(const double *d_queries, int64_t Q, const int32_t *d_query_mode,
                   const double *d_nodes, const int64_t *d_mode_offsets, int32_t D,
                   const int64_t *h_slices, int32_t A, int32_t metric, int32_t k, int64_t *d_idx,
                   double *d_dist, void *stream, int32_t flags);

/* Per-mode node store for repeated k-NN and radius queries (the planners'
 * per-mode node arrays: PRM node_array_cache, prm_graph.py:399-402; RRT
 * batch_subtree, rrtstar_base.py:254-306).  The store copies d_nodes[M, D]
 * (FP64, grouped by mode: h_mode_offsets[n_modes + 1]) into device memory it
 * owns; the caller's array may be freed afterwards.  For euclidean (D <= 29)
 * and max_euclidean (<= 4 agents of <= 7 coordinates) it also packs
 * split-BF16 tiles for the tensor-core candidate path; other metrics use the
 * exact kernel.  M may be 0 (every mode empty). */
typedef struct mrmg_node_store mrmg_node_store;
int mrmg_node_store_create(const double *d_nodes, int64_t M, int32_t D, const int64_t *h_mode_offsets,
                           int32_t n_modes, const int64_t *h_slices, int32_t A, int32_t metric,
                           mrmg_node_store **out, void *stream);
int mrmg_node_store_destroy(mrmg_node_store *store);

/* Incremental insertion (SingleTree.add_node, rrtstar_base.py:270-276, and
 * MultimodalGraph.add_nodes, prm_graph.py:289-291): appends rows[n, D] (FP64,
 * host or device memory) to `mode`, after its existing nodes, so that the
 * mode-local index of a node is its insertion order.  A mode index past the
 * last creates the modes in between, empty (mode < MRMG_MAX_STORE_MODES).
 * Only the tiles the new rows touch are packed; a full mode segment doubles
 * its capacity.  Synchronises. */
#define MRMG_MAX_STORE_MODES (1 << 20)
int mrmg_node_store_append(mrmg_node_store *store, int32_t mode, const double *rows, int64_t n, void *stream);

/* Removal as SingleTree.remove_node (rrtstar_base.py:278-289): the mode's
 * last node moves into slot idx and the mode shrinks by one.  Synchronises. */
int mrmg_node_store_remove(mrmg_node_store *store, int32_t mode, int64_t idx, void *stream);

/* Query path of the store (all give identical results): 0 = automatic (the
 * node-parallel path for batches of less than about 4M node-row x
 * coordinate work, else the tensor-core path where the metric and shape
 * allow it), 1 = the tensor-core path wherever it applies, 2 = the
 * node-parallel path (work items are (query, 256-node chunk) pairs; for
 * euclidean and max_euclidean with k <= 31 an FP32 candidate pass on the
 * store's FP32 node copy, certified and re-ranked in FP64, else the FP64
 * distance of every node). */
int mrmg_node_store_set_path(mrmg_node_store *store, int32_t path);

/* out3: [0] number of modes, [1] nodes in `mode`, [2] tensor-core path. */
int mrmg_node_store_info(const mrmg_node_store *store, int32_t mode, int64_t *out3);

/* (Queries of mrmg_knn and mrmg_near may be in device or host memory; host
 * rows are copied to a staging buffer of the store.)
 * k nearest neighbours of d_queries[Q, D] within their modes h_query_mode[Q]
 * (host array): same result as mrmg_knn_exact -- on the tensor-core path the
 * tcgen05 distance GEMM selects candidates, a certificate proves they contain
 * the true k nearest (else the query reruns exactly) and FP64 re-ranks them.
 * out_stats2 (optional): [0] tensor-core path used, [1] queries rerun exactly.
 * Synchronises its stream. */
int mrmg_knn(mrmg_node_store *store, const double *d_queries, int64_t Q, const int32_t *h_query_mode,
             int32_t k, int64_t *d_idx, double *d_dist, int64_t *out_stats2, void *stream);

/* Radius neighbours (RRT* near, planners/rrtstar_base.py:1296-1337, with
 * find_nearest_indices, rrtstar_base.py:439-453): for each query q, every
 * node j of its mode h_query_mode[q] whose batch_config_dist value satisfies
 * dist <= h_radius[q] + add_eps (the sum in FP64: the reference adds 1e-10),
 * in ascending j (np.nonzero order).  Result in CSR form: d_offsets[Q + 1]
 * (always written), mode-local d_idx[] and FP64 d_dist[] (may be NULL: no
 * distances) at positions offsets[q] .. offsets[q+1]; positions >= cap are
 * not written.
 * *out_total = offsets[Q].  When it exceeds cap, mrmg_near_fetch writes the
 * whole result into larger buffers without recomputing it (the store keeps
 * it until its next radius query; d_queries must stay unchanged until then).
 * On the tensor-core store the candidate bitmap comes from the tcgen05
 * distance tiles with the error bound added to the radius, then every
 * candidate is re-checked in FP64; other metrics check every node in FP64.
 * Synchronises its stream. */
int mrmg_near(mrmg_node_store *store, const double *d_queries, int64_t Q, const int32_t *h_query_mode,
              const double *h_radius, double add_eps, int64_t *d_offsets, int64_t *d_idx, double *d_dist,
              int64_t cap, int64_t *out_total, void *stream);
int mrmg_near_fetch(mrmg_node_store *store, int64_t *d_idx, double *d_dist, int64_t cap, void *stream);

/* Tensor-core self-test (no counterpart in the reference): C[128 x n] =
 * A[128 x 64] * B[n x 64]^T for row-major BF16 A, B through the same shared-
 * memory descriptors, instruction descriptor and tensor-memory path as the
 * nearest-neighbour kernel; n in 32..256, multiple of 32. */
int mrmg_selftest_umma(const void *d_a, const void *d_b, int32_t n, float *d_c, void *stream);

/* ------------------------------------------------------------------------ */
/* Calibration                                                               */
/* ------------------------------------------------------------------------ */

/* Measured fused-multiply-add throughput of the device (precision 0 = FP32,
 * 1 = FP64) in TFLOP/s, or (precision 2) the special-function-unit rate of
 * ex2.approx in T operations/s: the roofline denominators of the collision
 * (FP32 pipe), distance (FP64 pipe) and penetration-cost (MUFU) kernels.  No
 * counterpart in the reference. */
int mrmg_microbench_fma(int32_t precision, int64_t iters, double *out_tflops, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MRMG_GB300_H */
