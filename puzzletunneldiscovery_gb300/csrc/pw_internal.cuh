// pw_internal.cuh -- data layout shared by the world set-up and the query kernels.
#pragma once

#include "pw_trace.h"
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "pw_collide.h"
#include "pw_frames.cuh"

// One mesh on the device.  Triangles and BVH leaves share "slot" order (the
// Morton order of the build); FP64 data stays in the original face order.
//   nodeA[i] = (centre.xyz, left child)   nodeB[i] = (half-extent.xyz, right child)
//   internal nodes 0 .. ntri-2 (root 0), leaves ntri-1 .. 2*ntri-2 (slot = i - leaf_base).
//   triA/B/C[slot] = FP32 vertex 0, edge 1-0, edge 2-0, each rounded once from FP64
//   (w of triA = original face id).
// Boxes are conservative: they contain the FP64 vertices exactly.
//   Oriented boxes on the same hierarchy (obbA = (centre.xyz, left child),
//   obbB = (half-extent.xyz, right child), obbR0..2 = the box's axes as rows, FP32
//   roundings of an orthonormal FP64 frame): axes from the principal directions
//   of the node's vertices, extents measured in FP64 around the FP32 centre and
//   rounded up, so the box spanned by the exact FP64 frame contains the vertices.
struct MeshDev {
	int32_t ntri = 0;
	int32_t nvert = 0;
	int32_t leaf_base = 0;
	int32_t depth = 0;
	float4 *nodeA = nullptr, *nodeB = nullptr;
	float4 *obbA = nullptr, *obbB = nullptr, *obbR0 = nullptr, *obbR1 = nullptr, *obbR2 = nullptr;
	float4 *triA = nullptr, *triB = nullptr, *triC = nullptr;
	double *V64 = nullptr;   // nvert x 3 (env: perturbation frame; robot: local frame)
	int32_t *F = nullptr;    // ntri x 3
	float r1 = 0.f;          // L1 bound of any point of any node box (robot: local frame)
	double r2 = 0.0;         // max Euclidean norm of a vertex (robot: local frame)
	float emax = 0.f;        // max |coordinate| of any vertex or oriented node box corner
};

// Node pairs a single-query traversal starts from: a partition of the root
// pair (env root, robot root) into up to 32 pairs, so that a warp's first round
// has work for its lanes.
constexpr int MAX_SEEDS = 32;

struct WorldDev {
	MeshDev env, rob;
	float del_env;           // FP32 rounding bound of an env vertex coordinate
	int32_t nseeds = 0;
	const uint2 *seeds = nullptr;   // nseeds (env node, robot node) pairs, device memory
};

// Round phases of a segment query: phase p holds the rounds (32-step chunk
// indices) SEG_PHASE_START[p] .. SEG_PHASE_START[p + 1] - 1; each phase computes
// the anchor frames of its chunks that are still needed, then traverses them.
constexpr int SEG_PHASES = 8;

// Per-query device counters; zeroed before every query.
struct QueryCounters {
	unsigned long long work;        // next work item of the persistent kernels
	unsigned long long phase_work[SEG_PHASES];   // next work item of each segment round phase
	unsigned long long retest_count;
	unsigned long long stat[10];    // see STAT_* below
	unsigned long long ref_checks;  // isValid calls of the sequential reference loop
	unsigned int error;             // device-side consistency failure (PW_ERR_INTERNAL)
	unsigned int pad;
};
enum {
	STAT_QUERIES = 0,
	STAT_NODE_TESTS = 1,
	STAT_LEAF_TESTS = 2,
	STAT_RETESTS = 3,
	STAT_RETEST_HITS = 4,
	STAT_INLINE = 5,
	STAT_ITEMS = 6,
	STAT_TOTAL_ITEMS = 7,
	STAT_DETAILED = 8,   // segment chunks that needed per-step transforms
};

// A triangle pair whose FP32 verdict fell inside the error band.
struct RetestEntry {
	uint32_t query;   // state index or segment index
	uint32_t step;    // segment step (0 for states)
	uint32_t env_tri; // original face ids
	uint32_t rob_tri;
};

// Per-segment constants of the stepping loop, built on the device.
struct SegParams {
	double qa[4], qb[4];      // normalised rotations
	double d, theta, stheta;  // slerp constants
	double inv_stheta;        // 1 / stheta (0 on the linear branch): the filter frames' slerp weights
	double dist, inv_dist, step;
	double skip_scale;        // bound on the motion of any robot point from one step to the next
	int32_t linear;
	int32_t nsteps;           // steps the reference loop takes (0: none)
	int64_t ckpt_base;        // first checkpoint slot
};

struct DeviceBuffer {
	void *ptr = nullptr;
	size_t bytes = 0;
	cudaError_t reserve(size_t need);
	void release();
	~DeviceBuffer() { release(); }
};

// Page-locked host memory (staging of device-to-host copies).
struct PinnedBuffer {
	void *ptr = nullptr;
	size_t bytes = 0;
	cudaError_t reserve(size_t need);
	void release();
	~PinnedBuffer() { release(); }
};

struct pw_world {
	int device = 0;
	bool has_env = false, has_rob = false, scaled = false, ready = false;
	std::vector<float> Ve, Vr;
	std::vector<uint32_t> Fe, Fr;
	float scale = 1.0f;
	float center[3] = { 0, 0, 0 };
	float ompl_center[3] = { 0, 0, 0 };
	double pert[7] = { 0, 0, 0, 1, 0, 0, 0 };
	double pertR[9], pert_t[3];
	std::vector<double> env_local, env_world, rob_local;
	double env_box_c[3], env_box_h[3], rob_box_c[3], rob_box_h[3];
	WorldDev dev;
	// owned device allocations of the meshes
	std::vector<void *> mesh_allocs;
	// query scratch
	DeviceBuffer counters;     // QueryCounters
	DeviceBuffer retest;       // RetestEntry[retest_cap]
	uint64_t retest_cap = 0;
	DeviceBuffer seg_params, seg_ckpt, seg_anchor, seg_keys, seg_order, seg_keys2, seg_order2, round_off, cub_tmp, misc;
	DeviceBuffer isect;        // contact enumeration (candidates, rows, sort keys, output columns)
	PinnedBuffer isect_stage;  // two halves: one chunk's output columns on their way to the caller
	DeviceBuffer dis_queue;    // states the FP32 isDisentangled test left undecided
	DeviceBuffer seeds;        // the traversals' seed pairs (WorldDev::seeds)
	cudaStream_t last_stream = nullptr;
	cudaEvent_t ev[4] = { nullptr, nullptr, nullptr, nullptr }; // traversal start/end, re-test start/end
	bool timed = false;
	int64_t last_states = -1;   // size of the last state batch (-1: the last query was segments)
	int64_t last_launches = 0;  // kernels of this library the last query launched (pw_query_stats)
	int num_sms = 0;
	int dis_per_sm[2] = { 0, 0 };   // resident blocks per SM of the isDisentangled kernels (0: not yet asked)
	// graph mode: segment queries make no host synchronisation and no allocation;
	// they run within the scratch sizes that pw_segments_reserve or the last
	// segment query made outside graph mode left
	bool graph_mode = false;
	// launch configuration (pw_world_set_launch_config; 0 = default)
	int launch_width[2] = { 0, 0 };     // queries a warp takes per grab (states kernel only)
	int launch_soft_cap[2] = { 0, 0 };  // traversal stack soft cap
	int launch_blocks[2] = { 0, 0 };    // resident blocks per SM of the persistent kernel
	int grid_cache[4] = { 0, 0, 0, 0 }; // grid of the persistent kernels under that configuration, per box kind
	int node_boxes[2] = { PW_BOXES_ORIENTED, PW_BOXES_ORIENTED }; // per kernel (pw_world_set_node_boxes)
	int seg_phases = PW_PHASES_AUTO;   // round phases of segment queries (pw_world_set_segment_phases)
	int bvh_kind = PW_BVH_TOPDOWN;     // hierarchy of the next build (pw_world_set_bvh)
	// the last segment query's inputs: its parameters and checkpoints stay in the
	// scratch, so the transit tuples of the same batch can start from them
	const double *last_seg_from = nullptr, *last_seg_to = nullptr;
	int64_t last_seg_n = -1;
	double last_seg_delta = 0.0;
	int last_seg_mode = -1;
};

// error plumbing (pw_world.cu)
int pw_fail(int code, const std::string &msg);
int pw_cuda_fail(cudaError_t e, const char *what);
#define PW_CUDA(call)                                         \
	do {                                                      \
		cudaError_t e__ = (call);                             \
		if (e__ != cudaSuccess) return pw_cuda_fail(e__, #call); \
	} while (0)

int pw_build_mesh_device(pw_world *w, MeshDev &m, const std::vector<double> &V64, const std::vector<uint32_t> &F);

// The frame conversions of a world (pw_world.cu).
pwfr::Frame world_frame(const pw_world *w);
void pw_free_mesh_device(pw_world *w);
