// pw_world.cu -- world life cycle, the unit-world recipe and the GPU LBVH build.
//
// The unit-world recipe restates lib/osr/unit_world.cc:94-161 (load,
// scaleToUnit, angleModel), lib/osr/scene.cc:141-145,211-229 (vertex mean,
// moveToCenter, scale), lib/osr/bbox.h:21-51 (bounding box seeded at the
// origin) and lib/osr/cdmodel.cc:120-160 (the float xform applied in double).
// The BVH replaces FCL's BVHModel<OBBRSS> (cdmodel.cc:17-18,85-114) with a
// linear BVH built on the device: 30-bit Morton codes of triangle centroids,
// a radix sort, Karras' 2012 parallel hierarchy construction and a bottom-up
// refit of conservative FP32 boxes.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "pw_internal.cuh"
#include "pw_math.cuh"

static thread_local std::string g_last_error;

int pw_fail(int code, const std::string &msg)
{
	g_last_error = msg;
	return code;
}

int pw_cuda_fail(cudaError_t e, const char *what)
{
	g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
	if (e == cudaErrorMemoryAllocation)
		return PW_ERR_OUT_OF_MEMORY;
	return PW_ERR_CUDA;
}

cudaError_t DeviceBuffer::reserve(size_t need)
{
	if (need <= bytes && ptr)
		return cudaSuccess;
	release();
	size_t n = need < 256 ? 256 : need;
	cudaError_t e = cudaMalloc(&ptr, n);
	if (e != cudaSuccess) {
		ptr = nullptr;
		bytes = 0;
		return e;
	}
	bytes = n;
	return cudaSuccess;
}

void DeviceBuffer::release()
{
	if (ptr)
		cudaFree(ptr);
	ptr = nullptr;
	bytes = 0;
}

cudaError_t PinnedBuffer::reserve(size_t need)
{
	if (need <= bytes && ptr)
		return cudaSuccess;
	release();
	size_t n = need < 4096 ? 4096 : need;
	cudaError_t e = cudaMallocHost(&ptr, n);
	if (e != cudaSuccess) {
		ptr = nullptr;
		bytes = 0;
		return e;
	}
	bytes = n;
	return cudaSuccess;
}

void PinnedBuffer::release()
{
	if (ptr)
		cudaFreeHost(ptr);
	ptr = nullptr;
	bytes = 0;
}

extern "C" const char *pw_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------------------ life cycle

extern "C" int pw_world_create(pw_world **out, int device)
{
	if (!out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_create: out is NULL");
	int ndev = 0;
	PW_CUDA(cudaGetDeviceCount(&ndev));
	if (device < 0 || device >= ndev)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_create: no such CUDA device");
	PW_CUDA(cudaSetDevice(device));
	pw_world *w = new pw_world();
	w->device = device;
	pwm::state_transform(w->pert, w->pertR, w->pert_t);
	cudaDeviceGetAttribute(&w->num_sms, cudaDevAttrMultiProcessorCount, device);
	*out = w;
	return PW_OK;
}

void pw_free_mesh_device(pw_world *w)
{
	for (void *p : w->mesh_allocs)
		cudaFree(p);
	w->mesh_allocs.clear();
	w->dev.env = MeshDev();
	w->dev.rob = MeshDev();
}

extern "C" int pw_world_destroy(pw_world *w)
{
	if (!w)
		return PW_OK;
	cudaSetDevice(w->device);
	pw_free_mesh_device(w);
	for (cudaEvent_t &e : w->ev)
		if (e)
			cudaEventDestroy(e);
	delete w;
	return PW_OK;
}

static int check_mesh(const float *V, int64_t nv, const uint32_t *F, int64_t nf, const char *who)
{
	if (nv < 0 || nf < 0 || (nv > 0 && !V) || (nf > 0 && !F))
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": bad mesh pointers or sizes");
	if (nv > (int64_t(1) << 30) || nf > (int64_t(1) << 29))
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": mesh too large");
	for (int64_t i = 0; i < 3 * nf; i++)
		if (F[i] >= (uint64_t)nv)
			return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": face index out of range");
	for (int64_t i = 0; i < 3 * nv; i++)
		if (!std::isfinite(V[i]))
			return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": non-finite vertex");
	return PW_OK;
}

// Float mean of the vertices, summed in order (the OMPL centre, scene.cc:40-50,141-145).
static void float_mean(const std::vector<float> &V, float out[3])
{
	float acc[3] = { 0.f, 0.f, 0.f };
	const size_t n = V.size() / 3;
	for (size_t i = 0; i < n; i++)
		for (int c = 0; c < 3; c++)
			acc[c] = acc[c] + V[3 * i + c];
	for (int c = 0; c < 3; c++)
		out[c] = n ? acc[c] / (float)n : 0.0f;
}

extern "C" int pw_world_load_env(pw_world *w, const float *V, int64_t nv, const uint32_t *F, int64_t nf)
{
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_load_env: world is NULL");
	int rc = check_mesh(V, nv, F, nf, "pw_world_load_env");
	if (rc)
		return rc;
	w->Ve.assign(V, V + 3 * nv);
	w->Fe.assign(F, F + 3 * nf);
	w->has_env = true;
	w->ready = false;
	return PW_OK;
}

extern "C" int pw_world_load_robot(pw_world *w, const float *V, int64_t nv, const uint32_t *F, int64_t nf)
{
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_load_robot: world is NULL");
	int rc = check_mesh(V, nv, F, nf, "pw_world_load_robot");
	if (rc)
		return rc;
	w->Vr.assign(V, V + 3 * nv);
	w->Fr.assign(F, F + 3 * nf);
	w->has_rob = true;
	w->ready = false;
	float_mean(w->Vr, w->ompl_center);
	for (int c = 0; c < 3; c++)
		w->center[c] = w->ompl_center[c];
	return PW_OK;
}

extern "C" int pw_world_enforce_robot_center(pw_world *w, const double c[3])
{
	if (!w || !c)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_enforce_robot_center: NULL argument");
	if (!w->has_rob)
		return pw_fail(PW_ERR_NO_MODEL, "pw_world_enforce_robot_center: robot not loaded");
	for (int k = 0; k < 3; k++)
		w->center[k] = (float)c[k];
	return PW_OK;
}

// Bounding box seeded at the origin (bbox.h:21-51): the span includes the origin.
static float span_of(const std::vector<float> &V)
{
	float lo[3] = { 0.f, 0.f, 0.f }, hi[3] = { 0.f, 0.f, 0.f };
	const size_t n = V.size() / 3;
	for (size_t i = 0; i < n; i++)
		for (int c = 0; c < 3; c++) {
			const float x = V[3 * i + c];
			hi[c] = std::max(x, hi[c]);
			lo[c] = std::min(x, lo[c]);
		}
	return std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
}

extern "C" int pw_world_scale_to_unit(pw_world *w)
{
	PW_TRACE("pw_world_scale_to_unit");
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_scale_to_unit: world is NULL");
	if (!w->has_env)
		return pw_fail(PW_ERR_NO_MODEL, "pw_world_scale_to_unit: environment not loaded");
	const float se = span_of(w->Ve);
	const float sr = w->has_rob ? span_of(w->Vr) : 1.0f;
	w->scale = (float)(1.0 / (double)std::max(se, sr));
	w->scaled = true;
	return PW_OK;
}

// Every device array of a mesh (the allocations a rebuild of the other mesh keeps).
static std::vector<const void *> mesh_arrays(const MeshDev &m)
{
	return { m.nodeA, m.nodeB, m.obbA, m.obbB, m.obbR0, m.obbR1, m.obbR2, m.triA, m.triB, m.triC, m.V64, m.F };
}

static void apply_perturbation_to_env(pw_world *w)
{
	const size_t n = w->env_local.size() / 3;
	w->env_world.resize(w->env_local.size());
	for (size_t i = 0; i < n; i++)
		pwm::xform_point(w->pertR, w->pert_t, &w->env_local[3 * i], &w->env_world[3 * i]);
}

static void local_box(const std::vector<double> &V, double c[3], double h[3])
{
	double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
	const size_t n = V.size() / 3;
	for (size_t i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			lo[k] = std::min(lo[k], V[3 * i + k]);
			hi[k] = std::max(hi[k], V[3 * i + k]);
		}
	for (int k = 0; k < 3; k++) {
		c[k] = n ? (lo[k] + hi[k]) * 0.5 : 0.0;
		h[k] = n ? (hi[k] - lo[k]) * 0.5 : 0.0;
	}
}


// The seed pairs of a world's meshes: starting from the root pair, the pair with
// the largest boxes (sum of both half-extents) is replaced by the pairs of its
// larger non-leaf side's children (the traversal's own descent rule), until 32
// pairs or only leaf pairs remain.  The pairs partition the root pair's leaf
// pairs, so a traversal from them tests what one from the root tests.
static int compute_seeds(pw_world *w)
{
	struct Node {
		float h[3];
		uint32_t left, right;
		bool leaf;
	};
	auto fetch = [&](const MeshDev &m, uint32_t id, Node &o) -> int {
		float4 a, b;
		PW_CUDA(cudaMemcpy(&a, m.nodeA + id, sizeof(float4), cudaMemcpyDeviceToHost));
		PW_CUDA(cudaMemcpy(&b, m.nodeB + id, sizeof(float4), cudaMemcpyDeviceToHost));
		o.h[0] = b.x;
		o.h[1] = b.y;
		o.h[2] = b.z;
		memcpy(&o.left, &a.w, 4);
		memcpy(&o.right, &b.w, 4);
		o.leaf = (int64_t)id >= (int64_t)m.leaf_base;
		return PW_OK;
	};
	struct Pair {
		uint32_t e, r;
		Node ne, nr;
	};
	std::vector<Pair> pairs(1);
	pairs[0].e = pairs[0].r = 0;
	int rc;
	if ((rc = fetch(w->dev.env, 0, pairs[0].ne)) || (rc = fetch(w->dev.rob, 0, pairs[0].nr)))
		return rc;
	auto size = [](const Node &n) { return n.h[0] + n.h[1] + n.h[2]; };
	while ((int)pairs.size() < MAX_SEEDS) {
		int best = -1;
		float bs = -1.f;
		for (int i = 0; i < (int)pairs.size(); i++) {
			const Pair &p = pairs[i];
			if (p.ne.leaf && p.nr.leaf)
				continue;
			const float sz = size(p.ne) + size(p.nr);
			if (sz > bs) {
				bs = sz;
				best = i;
			}
		}
		if (best < 0)
			break;
		const Pair p = pairs[best];
		const bool da = !p.ne.leaf && (p.nr.leaf || size(p.ne) >= size(p.nr));
		Pair a = p, b = p;
		if (da) {
			a.e = p.ne.left;
			b.e = p.ne.right;
			if ((rc = fetch(w->dev.env, a.e, a.ne)) || (rc = fetch(w->dev.env, b.e, b.ne)))
				return rc;
		} else {
			a.r = p.nr.left;
			b.r = p.nr.right;
			if ((rc = fetch(w->dev.rob, a.r, a.nr)) || (rc = fetch(w->dev.rob, b.r, b.nr)))
				return rc;
		}
		pairs[best] = a;
		pairs.push_back(b);
	}
	std::vector<uint2> h(pairs.size());
	for (size_t i = 0; i < pairs.size(); i++)
		h[i] = make_uint2(pairs[i].e, pairs[i].r);
	PW_CUDA(w->seeds.reserve(sizeof(uint2) * MAX_SEEDS));
	PW_CUDA(cudaMemcpy(w->seeds.ptr, h.data(), sizeof(uint2) * h.size(), cudaMemcpyHostToDevice));
	w->dev.seeds = (const uint2 *)w->seeds.ptr;
	w->dev.nseeds = (int32_t)pairs.size();
	return PW_OK;
}

extern "C" int pw_world_angle_model(pw_world *w, float latitude, float longitude)
{
	PW_TRACE("pw_world_angle_model");
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_angle_model: world is NULL");
	if (latitude != 0.0f || longitude != 0.0f)
		return pw_fail(PW_ERR_INVALID_ARG,
		               "The arguments of UnitWorld::angleModel are reserved for compatibility; both must be 0.");
	if (!w->has_env || !w->has_rob)
		return pw_fail(PW_ERR_NO_MODEL, "pw_world_angle_model: environment and robot must both be loaded");
	if (!w->scaled)
		return pw_fail(PW_ERR_NO_MODEL, "pw_world_angle_model: call scale_to_unit first");
	PW_CUDA(cudaSetDevice(w->device));
	const double s = (double)w->scale;
	// env: xform = S(s); robot: xform = S(s) T(-c), translation column fl32(s * -c)
	w->env_local.resize(w->Ve.size());
	for (size_t i = 0; i < w->Ve.size(); i++)
		w->env_local[i] = s * (double)w->Ve[i];
	float tr[3];
	for (int c = 0; c < 3; c++)
		tr[c] = w->scale * (-w->center[c]);
	w->rob_local.resize(w->Vr.size());
	for (size_t i = 0; i < w->Vr.size() / 3; i++)
		for (int c = 0; c < 3; c++)
			w->rob_local[3 * i + c] = s * (double)w->Vr[3 * i + c] + (double)tr[c];
	local_box(w->env_local, w->env_box_c, w->env_box_h);
	local_box(w->rob_local, w->rob_box_c, w->rob_box_h);
	apply_perturbation_to_env(w);
	pw_free_mesh_device(w);
	w->ready = false;
	int rc = pw_build_mesh_device(w, w->dev.env, w->env_world, w->Fe);
	if (rc)
		return rc;
	rc = pw_build_mesh_device(w, w->dev.rob, w->rob_local, w->Fr);
	if (rc)
		return rc;
	w->dev.del_env = 5.9604645e-08f * w->dev.env.emax * 1.0001f;
	if ((rc = compute_seeds(w)))
		return rc;
	w->ready = true;
	return PW_OK;
}

extern "C" int pw_world_set_bvh(pw_world *w, int kind)
{
	if (!w || (kind != PW_BVH_TOPDOWN && kind != PW_BVH_MORTON && kind != PW_BVH_SAH))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_bvh: bad argument");
	w->bvh_kind = kind;
	return PW_OK;
}

extern "C" int pw_world_get_bvh(const pw_world *w, int *kind)
{
	if (!w || !kind)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_get_bvh: bad argument");
	*kind = w->bvh_kind;
	return PW_OK;
}

extern "C" int pw_world_set_perturbation(pw_world *w, const double q[7])
{
	if (!w || !q)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_perturbation: NULL argument");
	for (int i = 0; i < 7; i++)
		if (!std::isfinite(q[i]))
			return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_perturbation: non-finite state");
	memcpy(w->pert, q, sizeof(double) * 7);
	pwm::state_transform(w->pert, w->pertR, w->pert_t);
	if (w->ready) {
		PW_CUDA(cudaSetDevice(w->device));
		apply_perturbation_to_env(w);
		// rebuild only the env mesh; keep the robot
		const std::vector<const void *> rob = mesh_arrays(w->dev.rob);
		std::vector<void *> keep;
		for (void *p : w->mesh_allocs) {
			if (std::find(rob.begin(), rob.end(), (const void *)p) != rob.end())
				keep.push_back(p);
			else
				cudaFree(p);
		}
		w->mesh_allocs = keep;
		w->ready = false;
		int rc = pw_build_mesh_device(w, w->dev.env, w->env_world, w->Fe);
		if (rc)
			return rc;
		w->dev.del_env = 5.9604645e-08f * w->dev.env.emax * 1.0001f;
		if ((rc = compute_seeds(w)))
			return rc;
		w->ready = true;
	}
	return PW_OK;
}

extern "C" int pw_world_get_perturbation(const pw_world *w, double q[7])
{
	if (!w || !q)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_get_perturbation: NULL argument");
	memcpy(q, w->pert, sizeof(double) * 7);
	return PW_OK;
}

extern "C" int pw_world_info_get(const pw_world *w, pw_world_info *o)
{
	if (!w || !o)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_info_get: NULL argument");
	memset(o, 0, sizeof(*o));
	o->scene_scale = (double)w->scale;
	for (int c = 0; c < 3; c++) {
		o->robot_center[c] = w->center[c];
		o->robot_ompl_center[c] = w->ompl_center[c];
	}
	// scene xform S(s); robot xform S(s) T(-c), both float, as row-major doubles
	for (int i = 0; i < 16; i++) {
		o->scene_matrix[i] = 0.0;
		o->robot_matrix[i] = 0.0;
	}
	for (int i = 0; i < 3; i++) {
		o->scene_matrix[5 * i] = (double)w->scale;
		o->robot_matrix[5 * i] = (double)w->scale;
		o->robot_matrix[4 * i + 3] = (double)(w->scale * (-w->center[i]));
	}
	o->scene_matrix[15] = 1.0;
	o->robot_matrix[15] = 1.0;
	o->env_vertices = (int64_t)(w->Ve.size() / 3);
	o->env_faces = (int64_t)(w->Fe.size() / 3);
	o->robot_vertices = (int64_t)(w->Vr.size() / 3);
	o->robot_faces = (int64_t)(w->Fr.size() / 3);
	o->env_bvh_depth = w->dev.env.depth;
	o->robot_bvh_depth = w->dev.rob.depth;
	o->ready = w->ready ? 1 : 0;
	o->device = w->device;
	return PW_OK;
}

extern "C" int pw_world_cd_vertices(const pw_world *w, int geo, double *out)
{
	if (!w || !out || (geo != PW_GEO_ENV && geo != PW_GEO_ROB))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_cd_vertices: bad argument");
	if (!w->ready)
		return pw_fail(PW_ERR_NO_MODEL, "pw_world_cd_vertices: world not set up");
	const std::vector<double> &V = geo == PW_GEO_ENV ? w->env_world : w->rob_local;
	memcpy(out, V.data(), sizeof(double) * V.size());
	return PW_OK;
}

extern "C" int pw_world_cd_faces(const pw_world *w, int geo, int32_t *out)
{
	if (!w || !out || (geo != PW_GEO_ENV && geo != PW_GEO_ROB))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_cd_faces: bad argument");
	const std::vector<uint32_t> &F = geo == PW_GEO_ENV ? w->Fe : w->Fr;
	for (size_t i = 0; i < F.size(); i++)
		out[i] = (int32_t)F[i];
	return PW_OK;
}

// ------------------------------------------------------------------ frames

// The conversions of one world, in the shared host / device form.
pwfr::Frame world_frame(const pw_world *w)
{
	pwfr::Frame F;
	F.scale = (double)w->scale;
	for (int c = 0; c < 7; c++) F.pert[c] = w->pert[c];
	for (int c = 0; c < 3; c++) F.dc[c] = (double)(w->ompl_center[c] - w->center[c]) * (double)w->scale;
	return F;
}

static int check_conv(const pw_world *w, const double *in, int64_t n, const double *out, const char *who)
{
	if (!w || (n > 0 && (!in || !out)) || n < 0)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": bad argument");
	if (!w->scaled)
		return pw_fail(PW_ERR_NO_MODEL, std::string(who) + ": world not scaled");
	return PW_OK;
}

extern "C" int pw_world_translate_to_unit(const pw_world *w, const double *in, int64_t n, double *out)
{
	int rc = check_conv(w, in, n, out, "pw_world_translate_to_unit");
	if (rc) return rc;
	const pwfr::Frame F = world_frame(w);
	for (int64_t i = 0; i < n; i++)
		pwfr::to_unit(F, in + 7 * i, out + 7 * i);
	return PW_OK;
}

extern "C" int pw_world_translate_from_unit(const pw_world *w, const double *in, int64_t n, double *out)
{
	int rc = check_conv(w, in, n, out, "pw_world_translate_from_unit");
	if (rc) return rc;
	const pwfr::Frame F = world_frame(w);
	for (int64_t i = 0; i < n; i++)
		pwfr::from_unit(F, in + 7 * i, out + 7 * i);
	return PW_OK;
}

// translateOMPLStateToUnitState (unit_world.cc:689-711): w-last -> w-first, to unit,
// then t' = t - R(q) * (ompl_centre - centre) * scale.
extern "C" int pw_world_translate_ompl_to_unit(const pw_world *w, const double *in, int64_t n, double *out)
{
	int rc = check_conv(w, in, n, out, "pw_world_translate_ompl_to_unit");
	if (rc) return rc;
	const pwfr::Frame F = world_frame(w);
	for (int64_t i = 0; i < n; i++)
		pwfr::ompl_to_unit(F, in + 7 * i, out + 7 * i);
	return PW_OK;
}

// translateUnitStateToOMPLState (unit_world.cc:556-590).
extern "C" int pw_world_translate_unit_to_ompl(const pw_world *w, const double *in, int64_t n, double *out,
                                               int to_angle_axis)
{
	int rc = check_conv(w, in, n, out, "pw_world_translate_unit_to_ompl");
	if (rc) return rc;
	const pwfr::Frame F = world_frame(w);
	for (int64_t i = 0; i < n; i++) {
		double t[3], rot[4], R[9], Rd[3], t2[3], c7[7], o[7];
		pwfr::decompose(in + 7 * i, t, rot);
		pwm::quat_to_matrix(rot, R);
		pwfr::mat_vec(R, F.dc, Rd);
		for (int c = 0; c < 3; c++) t2[c] = pwm::add(t[c], Rd[c]);
		pwfr::compose(t2, rot, c7);
		pwfr::from_unit(F, c7, o);
		double *dst = out + 7 * i;
		dst[0] = o[0]; dst[1] = o[1]; dst[2] = o[2];
		if (to_angle_axis) {
			// angle-axis of the w-first quaternion: angle = 2 atan2(|v|, |w|) with the axis
			// sign following w, as Eigen::AngleAxis does from a quaternion
			const double vn = std::sqrt(o[4] * o[4] + o[5] * o[5] + o[6] * o[6]);
			double ang = 2.0 * std::atan2(vn, std::fabs(o[3]));
			double ax[3] = { 1.0, 0.0, 0.0 };
			if (vn > 0.0) {
				const double sgn = o[3] < 0.0 ? -1.0 : 1.0;
				for (int c = 0; c < 3; c++) ax[c] = sgn * o[4 + c] / vn;
			}
			dst[3] = ang; dst[4] = ax[0]; dst[5] = ax[1]; dst[6] = ax[2];
		} else {
			dst[3] = o[4]; dst[4] = o[5]; dst[5] = o[6]; dst[6] = o[3];
		}
	}
	return PW_OK;
}

// ------------------------------------------------------------------ host state math

extern "C" int pw_state_distance(const double a[7], const double b[7], double *out)
{
	if (!a || !b || !out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_state_distance: NULL argument");
	*out = pwm::distance(a, b);
	return PW_OK;
}

extern "C" int pw_state_interpolate(const double a[7], const double b[7], double tau, double out[7])
{
	if (!a || !b || !out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_state_interpolate: NULL argument");
	pwm::interpolate(a, b, tau, out);
	return PW_OK;
}

extern "C" int pw_segment_step_state(const double from[7], const double to[7], double verify_delta, int64_t k,
                                     double out[7], double *tau, int64_t *num_steps)
{
	if (!from || !to || !out || !tau || !num_steps)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segment_step_state: NULL argument");
	const double dist = pwm::distance(from, to);
	if (!(verify_delta >= dist) && dist == dist && (!(verify_delta > 0.0) || dist / verify_delta > 1073741824.0))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segment_step_state: verify_delta must be > 0 and dist/verify_delta < 2^30");
	int64_t K = 0;
	if (!(verify_delta >= dist) && dist == dist) {
		double delta = verify_delta;
		while (delta <= dist) {
			delta = pwm::advance_delta(delta, dist, verify_delta);
			K++;
		}
	}
	*num_steps = K;
	if (k < 0 || k >= K)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segment_step_state: step index out of range");
	double delta = verify_delta;
	for (int64_t j = 0; j < k; j++)
		delta = pwm::advance_delta(delta, dist, verify_delta);
	const double inv = pwm::dvd(1.0, dist);
	*tau = pwm::mul(delta, inv);
	pwm::interpolate(from, to, *tau, out);
	return PW_OK;
}

// ------------------------------------------------------------------ LBVH build

// Per triangle: FP32 vertices (nearest), conservative box (directed rounding), centroid.
__global__ void k_tri_prep(const double *V, const int32_t *F, int n, float4 *ta, float4 *tb, float4 *tc,
                           float *lo, float *hi, float *cen)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n)
		return;
	double p[3][3];
	for (int k = 0; k < 3; k++)
		for (int c = 0; c < 3; c++)
			p[k][c] = V[3 * F[3 * t + k] + c];
	// vertex 0 and the two edges from it, each rounded once from FP64
	ta[t] = make_float4(__double2float_rn(p[0][0]), __double2float_rn(p[0][1]), __double2float_rn(p[0][2]),
	                    __int_as_float(t));
	tb[t] = make_float4(__double2float_rn(__dsub_rn(p[1][0], p[0][0])), __double2float_rn(__dsub_rn(p[1][1], p[0][1])),
	                    __double2float_rn(__dsub_rn(p[1][2], p[0][2])), 0.f);
	tc[t] = make_float4(__double2float_rn(__dsub_rn(p[2][0], p[0][0])), __double2float_rn(__dsub_rn(p[2][1], p[0][1])),
	                    __double2float_rn(__dsub_rn(p[2][2], p[0][2])), 0.f);
	for (int c = 0; c < 3; c++) {
		const double mn = fmin(fmin(p[0][c], p[1][c]), p[2][c]);
		const double mx = fmax(fmax(p[0][c], p[1][c]), p[2][c]);
		const float l = __double2float_rd(mn), h = __double2float_ru(mx);
		lo[3 * t + c] = l;
		hi[3 * t + c] = h;
		cen[3 * t + c] = 0.5f * (l + h);
	}
}

// Single-block min/max of the centroids: out = (min.xyz, max.xyz).
__global__ void k_bounds(const float *cen, int n, float *out)
{
	__shared__ float smin[3][256], smax[3][256];
	float mn[3] = { INFINITY, INFINITY, INFINITY }, mx[3] = { -INFINITY, -INFINITY, -INFINITY };
	for (int i = threadIdx.x; i < n; i += blockDim.x)
		for (int c = 0; c < 3; c++) {
			mn[c] = fminf(mn[c], cen[3 * i + c]);
			mx[c] = fmaxf(mx[c], cen[3 * i + c]);
		}
	for (int c = 0; c < 3; c++) {
		smin[c][threadIdx.x] = mn[c];
		smax[c][threadIdx.x] = mx[c];
	}
	__syncthreads();
	for (int s = blockDim.x / 2; s > 0; s >>= 1) {
		if (threadIdx.x < s)
			for (int c = 0; c < 3; c++) {
				smin[c][threadIdx.x] = fminf(smin[c][threadIdx.x], smin[c][threadIdx.x + s]);
				smax[c][threadIdx.x] = fmaxf(smax[c][threadIdx.x], smax[c][threadIdx.x + s]);
			}
		__syncthreads();
	}
	if (threadIdx.x == 0)
		for (int c = 0; c < 3; c++) {
			out[c] = smin[c][0];
			out[3 + c] = smax[c][0];
		}
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v)
{
	v = (v * 0x00010001u) & 0xFF0000FFu;
	v = (v * 0x00000101u) & 0x0F00F00Fu;
	v = (v * 0x00000011u) & 0xC30C30C3u;
	v = (v * 0x00000005u) & 0x49249249u;
	return v;
}

__global__ void k_morton(const float *cen, int n, const float *bounds, uint32_t *keys, uint32_t *vals)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n)
		return;
	uint32_t code = 0;
	uint32_t q[3];
	for (int c = 0; c < 3; c++) {
		const float ext = bounds[3 + c] - bounds[c];
		float f = ext > 0.f ? (cen[3 * t + c] - bounds[c]) / ext : 0.5f;
		f = fminf(fmaxf(f * 1024.f, 0.f), 1023.f);
		q[c] = (uint32_t)f;
	}
	code = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
	keys[t] = code;
	vals[t] = (uint32_t)t;
}

__device__ __forceinline__ int lcp_delta(const uint32_t *keys, int n, int i, int j)
{
	if (j < 0 || j >= n)
		return -1;
	const uint32_t a = keys[i], b = keys[j];
	if (a == b)
		return 32 + __clz((uint32_t)i ^ (uint32_t)j);
	return __clz(a ^ b);
}

// Karras 2012: internal node i covers a key range; children are internal or leaf nodes.
__global__ void k_karras(const uint32_t *keys, int n, int32_t *left, int32_t *right, int32_t *parent,
                         int32_t *rlo, int32_t *rhi)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n - 1)
		return;
	const int d = (lcp_delta(keys, n, i, i + 1) - lcp_delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
	const int dmin = lcp_delta(keys, n, i, i - d);
	int lmax = 2;
	while (lcp_delta(keys, n, i, i + lmax * d) > dmin)
		lmax *= 2;
	int l = 0;
	for (int t = lmax / 2; t >= 1; t /= 2)
		if (lcp_delta(keys, n, i, i + (l + t) * d) > dmin)
			l += t;
	const int j = i + l * d;
	const int dnode = lcp_delta(keys, n, i, j);
	int s = 0;
	int t = l;
	do {
		t = (t + 1) >> 1;
		if (lcp_delta(keys, n, i, i + (s + t) * d) > dnode)
			s += t;
	} while (t > 1);
	const int gamma = i + s * d + min(d, 0);
	const int leaf_base = n - 1;
	const int lc = (min(i, j) == gamma) ? leaf_base + gamma : gamma;
	const int rc = (max(i, j) == gamma + 1) ? leaf_base + gamma + 1 : gamma + 1;
	left[i] = lc;
	right[i] = rc;
	parent[lc] = i;
	parent[rc] = i;
	rlo[i] = min(i, j);      // the node's leaves, in slot order
	rhi[i] = max(i, j);
}

// Leaves: permute triangles into slot order and write leaf boxes, then refit
// the ancestors bottom-up (the second child to arrive computes the union).
__global__ void k_refit(const uint32_t *order, int n, const float *tlo, const float *thi, const float4 *ta,
                        const float4 *tb, const float4 *tc, float4 *sa, float4 *sb, float4 *sc, float *blo,
                        float *bhi, const int32_t *left, const int32_t *right, const int32_t *parent,
                        unsigned int *flags)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= n)
		return;
	const int leaf_base = n - 1;
	const uint32_t t = order[j];
	sa[j] = ta[t];
	sb[j] = tb[t];
	sc[j] = tc[t];
	int node = leaf_base + j;
	for (int c = 0; c < 3; c++) {
		blo[3 * node + c] = tlo[3 * t + c];
		bhi[3 * node + c] = thi[3 * t + c];
	}
	__threadfence();
	int p = node == 0 ? -1 : parent[node];
	while (p >= 0) {
		if (atomicAdd(&flags[p], 1u) == 0)
			return;
		__threadfence();
		const int l = left[p], r = right[p];
		for (int c = 0; c < 3; c++) {
			const float lo = fminf(__ldcg(&blo[3 * l + c]), __ldcg(&blo[3 * r + c]));
			const float hi = fmaxf(__ldcg(&bhi[3 * l + c]), __ldcg(&bhi[3 * r + c]));
			blo[3 * p + c] = lo;
			bhi[3 * p + c] = hi;
		}
		__threadfence();
		p = p == 0 ? -1 : parent[p];
	}
}

// Boxes to (centre, half-extent) with [c - h, c + h] containing [lo, hi]; child links.
__global__ void k_finalize(int nnodes, int n, const float *blo, const float *bhi, const int32_t *left,
                           const int32_t *right, const float4 *sa, float4 *na, float4 *nb)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nnodes)
		return;
	float c[3], h[3];
	for (int k = 0; k < 3; k++) {
		const double lo = blo[3 * i + k], hi = bhi[3 * i + k];
		const float cf = __double2float_rn(0.5 * (lo + hi));
		const double hh = fmax(hi - (double)cf, (double)cf - lo);
		c[k] = cf;
		h[k] = __double2float_ru(hh);
	}
	const int leaf_base = n - 1;
	int l = -1, r = -1;
	if (i < leaf_base) {
		l = left[i];
		r = right[i];
	} else {
		l = __float_as_int(sa[i - leaf_base].w);
	}
	na[i] = make_float4(c[0], c[1], c[2], __int_as_float(l));
	nb[i] = make_float4(h[0], h[1], h[2], __int_as_float(r));
}

// ------------------------------------------------------------------ oriented node boxes
//
// Principal axes (Gottschalk, Lin, Manocha 1996: the eigenvectors of the
// covariance of the node's vertices) on the LBVH's hierarchy.  Vertex moments
// are summed per slot and prefix-summed, so a node's covariance is the
// difference of two prefix entries; the eigenvectors come from cyclic Jacobi
// rotations (pwm::jacobi_eigen3); the extents are measured over the node's
// vertices in FP64.

// Per slot: the sums of the slot triangle's three vertices (relative to `org`)
// and of their outer products: 9 arrays of n.
__global__ void k_slot_moments(const double *V, const int32_t *F, const uint32_t *order, int n, const double *org,
                               double *mom)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= n)
		return;
	const int t = (int)order[j];
	double s[9] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 };
	for (int k = 0; k < 3; k++) {
		const double *p = V + 3 * F[3 * t + k];
		const double x = p[0] - org[0], y = p[1] - org[1], z = p[2] - org[2];
		s[0] += x; s[1] += y; s[2] += z;
		s[3] += x * x; s[4] += y * y; s[5] += z * z;
		s[6] += x * y; s[7] += x * z; s[8] += y * z;
	}
	for (int k = 0; k < 9; k++)
		mom[(size_t)k * n + j] = s[k];
}

// One warp per node (leaves included): axes from the covariance of the node's
// slot range, then two passes over its vertices -- the extents along each axis,
// the FP32 centre of that range, and the half-extents about that FP32 centre,
// measured in FP64 and rounded up with a margin for the FP64 rounding.
// Writes the oriented node arrays and the two magnitude bounds the error model
// needs: max over node boxes of |corner|_1 (rb1) and |corner|_inf (rbinf), as
// float bit patterns (non-negative floats order like their bits).
__global__ void k_obb_fit(const double *V, const int32_t *F, const uint32_t *order, int n, const double *scan,
                          const int32_t *rlo, const int32_t *rhi, const int32_t *left, const int32_t *right,
                          const float4 *slot_a, float4 *oa, float4 *ob, float4 *r0, float4 *r1, float4 *r2,
                          unsigned int *rb1, unsigned int *rbinf)
{
	const int warp = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	const int nnodes = 2 * n - 1;
	if (warp >= nnodes)
		return;
	const int leaf_base = n - 1;
	const bool leaf = warp >= leaf_base;
	const int lo = leaf ? warp - leaf_base : rlo[warp];
	const int hi = leaf ? warp - leaf_base : rhi[warp];
	// covariance from the prefix sums of the slot moments (inclusive scans)
	double m[9];
	for (int k = 0; k < 9; k++) {
		const double *sk = scan + (size_t)k * n;
		m[k] = sk[hi] - (lo > 0 ? sk[lo - 1] : 0.0);
	}
	const double cnt = 3.0 * (double)(hi - lo + 1);
	const double mu[3] = { m[0] / cnt, m[1] / cnt, m[2] / cnt };
	const double S[6] = { m[3] / cnt - mu[0] * mu[0], m[4] / cnt - mu[1] * mu[1], m[5] / cnt - mu[2] * mu[2],
	                      m[6] / cnt - mu[0] * mu[1], m[7] / cnt - mu[0] * mu[2], m[8] / cnt - mu[1] * mu[2] };
	double E[9];
	pwm::jacobi_eigen3(S, E);
	// pass 1: the projections' range along each axis
	double pmin[3] = { 1e300, 1e300, 1e300 }, pmax[3] = { -1e300, -1e300, -1e300 };
	for (int j = lo + lane; j <= hi; j += 32) {
		const int t = (int)order[j];
		for (int k = 0; k < 3; k++) {
			const double *p = V + 3 * F[3 * t + k];
			for (int a = 0; a < 3; a++) {
				const double pr = E[3 * a] * p[0] + E[3 * a + 1] * p[1] + E[3 * a + 2] * p[2];
				pmin[a] = fmin(pmin[a], pr);
				pmax[a] = fmax(pmax[a], pr);
			}
		}
	}
	for (int o = 16; o > 0; o >>= 1)
		for (int a = 0; a < 3; a++) {
			pmin[a] = fmin(pmin[a], __shfl_xor_sync(0xffffffffu, pmin[a], o));
			pmax[a] = fmax(pmax[a], __shfl_xor_sync(0xffffffffu, pmax[a], o));
		}
	float c[3];
	for (int k = 0; k < 3; k++) {
		double ck = 0.0;
		for (int a = 0; a < 3; a++)
			ck += E[3 * a + k] * 0.5 * (pmin[a] + pmax[a]);
		c[k] = __double2float_rn(ck);
	}
	// pass 2: half-extents about the FP32 centre, and the largest |x - c|_1 for the rounding margin
	double h[3] = { 0, 0, 0 }, dmax = 0.0;
	for (int j = lo + lane; j <= hi; j += 32) {
		const int t = (int)order[j];
		for (int k = 0; k < 3; k++) {
			const double *p = V + 3 * F[3 * t + k];
			const double d0 = p[0] - (double)c[0], d1 = p[1] - (double)c[1], d2 = p[2] - (double)c[2];
			dmax = fmax(dmax, fabs(d0) + fabs(d1) + fabs(d2));
			for (int a = 0; a < 3; a++)
				h[a] = fmax(h[a], fabs(E[3 * a] * d0 + E[3 * a + 1] * d1 + E[3 * a + 2] * d2));
		}
	}
	for (int o = 16; o > 0; o >>= 1) {
		dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
		for (int a = 0; a < 3; a++)
			h[a] = fmax(h[a], __shfl_xor_sync(0xffffffffu, h[a], o));
	}
	if (lane != 0)
		return;
	// the FP64 differences and dot products are off by a few ulps of |x - c|_1 (and of |x|, |c| in the subtraction)
	const double cinf = fmax(fmax(fabs((double)c[0]), fabs((double)c[1])), fabs((double)c[2]));
	const double pad = 1e-14 * (dmax + 2.0 * cinf) + 1e-300;
	float hf[3];
	for (int a = 0; a < 3; a++)
		hf[a] = __double2float_ru(h[a] * (1.0 + 1e-14) + pad);
	int l, r;
	if (!leaf) {
		l = left[warp];
		r = right[warp];
	} else {
		l = __float_as_int(slot_a[warp - leaf_base].w);
		r = -1;
	}
	float4 rows[3];
	double b1 = fabs((double)c[0]) + fabs((double)c[1]) + fabs((double)c[2]);
	double binf = cinf;
	for (int a = 0; a < 3; a++) {
		rows[a] = make_float4(__double2float_rn(E[3 * a]), __double2float_rn(E[3 * a + 1]),
		                      __double2float_rn(E[3 * a + 2]), 0.f);
		b1 += (double)hf[a] * (fabs(E[3 * a]) + fabs(E[3 * a + 1]) + fabs(E[3 * a + 2]));
		binf += (double)hf[a];
	}
	oa[warp] = make_float4(c[0], c[1], c[2], __int_as_float(l));
	ob[warp] = make_float4(hf[0], hf[1], hf[2], __int_as_float(r));
	r0[warp] = rows[0];
	r1[warp] = rows[1];
	r2[warp] = rows[2];
	atomicMax(rb1, __float_as_uint(__double2float_ru(b1 * (1.0 + 1e-12))));
	atomicMax(rbinf, __float_as_uint(__double2float_ru(binf * (1.0 + 1e-12))));
}

__global__ void k_depth(int n, const int32_t *parent, int *maxdepth)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= n)
		return;
	int node = (n - 1) + j;
	int d = 0;
	while (node != 0 && d < 4096) {
		node = parent[node];
		d++;
	}
	atomicMax(maxdepth, d);
}

// Top-down hierarchy over the triangles (the OBBTree split, Gottschalk, Lin and
// Manocha 1996): a range of triangles is split at the mean of their centroids
// projected on the principal axis of their vertices; where that leaves one side
// empty, or below depth 40, at the median of the projections instead, which
// bounds the depth.  Internal nodes are numbered in preorder (root 0) and cover
// the contiguous slot range rlo..rhi; leaf j (the triangle order[j]) is node
// n - 1 + j.  Oriented boxes fitted to these nodes are tighter than to the
// Morton-order hierarchy, whose splits are axis-aligned by construction.
static void build_topdown(const std::vector<double> &V, const std::vector<uint32_t> &F, std::vector<uint32_t> &order,
                          std::vector<int32_t> &left, std::vector<int32_t> &right, std::vector<int32_t> &parent,
                          std::vector<int32_t> &rlo, std::vector<int32_t> &rhi, bool sah)
{
	const int n = (int)(F.size() / 3);
	const int leaf_base = n - 1;
	order.resize(n);
	for (int i = 0; i < n; i++)
		order[i] = (uint32_t)i;
	left.assign(n > 1 ? n - 1 : 0, -1);
	right.assign(n > 1 ? n - 1 : 0, -1);
	rlo.assign(n > 1 ? n - 1 : 0, 0);
	rhi.assign(n > 1 ? n - 1 : 0, 0);
	parent.assign(n > 0 ? 2 * n - 1 : 0, -1);
	if (n < 2)
		return;
	std::vector<double> cen(3 * (size_t)n), proj(n);
	for (int t = 0; t < n; t++)
		for (int c = 0; c < 3; c++)
			cen[3 * t + c] = (V[3 * F[3 * t] + c] + V[3 * F[3 * t + 1] + c] + V[3 * F[3 * t + 2] + c]) / 3.0;
	struct Task {
		int a, b, id, depth;
	};
	std::vector<Task> stack;
	stack.push_back(Task{ 0, n, 0, 0 });
	int next = 1;
	while (!stack.empty()) {
		const Task k = stack.back();
		stack.pop_back();
		// principal axis of the range's vertices
		double mu[3] = { 0, 0, 0 };
		const double inv = 1.0 / (3.0 * (k.b - k.a));
		for (int i = k.a; i < k.b; i++)
			for (int v = 0; v < 3; v++)
				for (int c = 0; c < 3; c++)
					mu[c] += V[3 * F[3 * order[i] + v] + c] * inv;
		double S[6] = { 0, 0, 0, 0, 0, 0 };
		for (int i = k.a; i < k.b; i++)
			for (int v = 0; v < 3; v++) {
				const double *p = &V[3 * F[3 * order[i] + v]];
				const double d[3] = { p[0] - mu[0], p[1] - mu[1], p[2] - mu[2] };
				S[0] += d[0] * d[0]; S[1] += d[1] * d[1]; S[2] += d[2] * d[2];
				S[3] += d[0] * d[1]; S[4] += d[0] * d[2]; S[5] += d[1] * d[2];
			}
		double E[9];
		pwm::jacobi_eigen3(S, E);
		// the row of E with the largest variance
		int best = 0;
		double bv = -1.0;
		for (int r = 0; r < 3; r++) {
			const double *e = E + 3 * r;
			const double var = e[0] * (S[0] * e[0] + S[3] * e[1] + S[4] * e[2]) +
			                   e[1] * (S[3] * e[0] + S[1] * e[1] + S[5] * e[2]) +
			                   e[2] * (S[4] * e[0] + S[5] * e[1] + S[2] * e[2]);
			if (var > bv) {
				bv = var;
				best = r;
			}
		}
		const double *ax = E + 3 * best;
		if (sah && k.depth < 40 && k.b - k.a > 2) {
			// binned surface-area cost in the node's principal frame: the split plane (one of
			// 15 bin boundaries on each of the three axes) that minimises the children's
			// box areas (in that frame) weighted by their triangle counts
			constexpr int NB = 16;
			double bestc = 1e300;
			int bax = -1;
			double bcut = 0.0;
			for (int a3 = 0; a3 < 3; a3++) {
				const double *e = E + 3 * a3;
				double lo = 1e300, hi = -1e300;
				for (int i = k.a; i < k.b; i++) {
					const double *c = &cen[3 * order[i]];
					const double pr = e[0] * c[0] + e[1] * c[1] + e[2] * c[2];
					lo = std::min(lo, pr);
					hi = std::max(hi, pr);
				}
				if (!(hi > lo))
					continue;
				double bl[NB][3], bh[NB][3];
				int cnt[NB] = { 0 };
				for (int b = 0; b < NB; b++)
					for (int c = 0; c < 3; c++) {
						bl[b][c] = 1e300;
						bh[b][c] = -1e300;
					}
				for (int i = k.a; i < k.b; i++) {
					const uint32_t t = order[i];
					const double *c = &cen[3 * t];
					const double pr = e[0] * c[0] + e[1] * c[1] + e[2] * c[2];
					int b = (int)((pr - lo) / (hi - lo) * NB);
					b = b < 0 ? 0 : (b >= NB ? NB - 1 : b);
					cnt[b]++;
					for (int v = 0; v < 3; v++) {
						const double *p = &V[3 * F[3 * t + v]];
						for (int r = 0; r < 3; r++) {
							const double q = E[3 * r] * p[0] + E[3 * r + 1] * p[1] + E[3 * r + 2] * p[2];
							bl[b][r] = std::min(bl[b][r], q);
							bh[b][r] = std::max(bh[b][r], q);
						}
					}
				}
				auto area = [](const double *l, const double *h) {
					const double x = h[0] - l[0], y = h[1] - l[1], z = h[2] - l[2];
					return x * y + y * z + z * x;
				};
				// prefix (left) boxes and counts; suffix (right) sweep
				double pl[NB][3], ph[NB][3];
				int pc[NB];
				for (int b = 0; b < NB; b++) {
					for (int c = 0; c < 3; c++) {
						pl[b][c] = b ? std::min(pl[b - 1][c], bl[b][c]) : bl[b][c];
						ph[b][c] = b ? std::max(ph[b - 1][c], bh[b][c]) : bh[b][c];
					}
					pc[b] = (b ? pc[b - 1] : 0) + cnt[b];
				}
				double sl[3] = { 1e300, 1e300, 1e300 }, sh[3] = { -1e300, -1e300, -1e300 };
				int sc = 0;
				for (int b = NB - 1; b >= 1; b--) {
					for (int c = 0; c < 3; c++) {
						sl[c] = std::min(sl[c], bl[b][c]);
						sh[c] = std::max(sh[c], bh[b][c]);
					}
					sc += cnt[b];
					const int nl = pc[b - 1];
					if (nl == 0 || sc == 0)
						continue;
					const double cost = area(pl[b - 1], ph[b - 1]) * nl + area(sl, sh) * sc;
					if (cost < bestc) {
						bestc = cost;
						bax = a3;
						bcut = lo + (hi - lo) * b / NB;
					}
				}
			}
			if (bax >= 0) {
				const double *e = E + 3 * bax;
				int i = k.a, j = k.b - 1;
				while (i <= j) {
					const double *c = &cen[3 * order[i]];
					const double pr = e[0] * c[0] + e[1] * c[1] + e[2] * c[2];
					if (pr < bcut)
						i++;
					else
						std::swap(order[i], order[j--]);
				}
				const int mid = i;
				if (mid > k.a && mid < k.b) {
					const int lc = mid - k.a == 1 ? leaf_base + k.a : next++;
					if (mid - k.a > 1)
						stack.push_back(Task{ k.a, mid, lc, k.depth + 1 });
					const int rc = k.b - mid == 1 ? leaf_base + mid : next++;
					if (k.b - mid > 1)
						stack.push_back(Task{ mid, k.b, rc, k.depth + 1 });
					left[k.id] = lc;
					right[k.id] = rc;
					parent[lc] = k.id;
					parent[rc] = k.id;
					rlo[k.id] = k.a;
					rhi[k.id] = k.b - 1;
					continue;
				}
			}
		}
		double mean = 0.0;
		for (int i = k.a; i < k.b; i++) {
			const double *c = &cen[3 * order[i]];
			proj[order[i]] = ax[0] * c[0] + ax[1] * c[1] + ax[2] * c[2];
			mean += proj[order[i]];
		}
		mean /= (double)(k.b - k.a);
		int mid = k.a;
		if (k.depth < 40) {
			int i = k.a, j = k.b - 1;
			while (i <= j) {
				if (proj[order[i]] < mean)
					i++;
				else
					std::swap(order[i], order[j--]);
			}
			mid = i;
		}
		if (mid == k.a || mid == k.b) {
			mid = (k.a + k.b) / 2;
			std::nth_element(order.begin() + k.a, order.begin() + mid, order.begin() + k.b,
			                 [&](uint32_t x, uint32_t y) { return proj[x] < proj[y] || (proj[x] == proj[y] && x < y); });
		}
		const int lc = mid - k.a == 1 ? leaf_base + k.a : next++;
		if (mid - k.a > 1)
			stack.push_back(Task{ k.a, mid, lc, k.depth + 1 });
		const int rc = k.b - mid == 1 ? leaf_base + mid : next++;
		if (k.b - mid > 1)
			stack.push_back(Task{ mid, k.b, rc, k.depth + 1 });
		left[k.id] = lc;
		right[k.id] = rc;
		parent[lc] = k.id;
		parent[rc] = k.id;
		rlo[k.id] = k.a;
		rhi[k.id] = k.b - 1;
	}
}

// The largest mesh whose default (top-down) hierarchy takes surface-area splits.
constexpr int SAH_MAX_TRIANGLES = 1 << 16;

template <typename T>
static cudaError_t walloc(pw_world *w, T **p, size_t count)
{
	cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
	if (e == cudaSuccess)
		w->mesh_allocs.push_back((void *)*p);
	return e;
}

int pw_build_mesh_device(pw_world *w, MeshDev &m, const std::vector<double> &V64, const std::vector<uint32_t> &F)
{
	m = MeshDev();
	const int n = (int)(F.size() / 3);
	const int nv = (int)(V64.size() / 3);
	m.ntri = n;
	m.nvert = nv;
	m.leaf_base = n > 0 ? n - 1 : 0;
	// host-side magnitudes
	double emax = 0.0, r2 = 0.0;
	for (double x : V64)
		emax = std::max(emax, std::fabs(x));
	for (size_t i = 0; i + 2 < V64.size(); i += 3)
		r2 = std::max(r2, std::sqrt(V64[i] * V64[i] + V64[i + 1] * V64[i + 1] + V64[i + 2] * V64[i + 2]));
	m.emax = (float)emax * 1.0001f + 1e-30f;
	m.r2 = r2 * (1.0 + 1e-12) + 1e-300;
	PW_CUDA(walloc(w, &m.V64, V64.size()));
	PW_CUDA(walloc(w, &m.F, F.size()));
	PW_CUDA(cudaMemcpy(m.V64, V64.data(), sizeof(double) * V64.size(), cudaMemcpyHostToDevice));
	PW_CUDA(cudaMemcpy(m.F, F.data(), sizeof(int32_t) * F.size(), cudaMemcpyHostToDevice));
	if (n == 0)
		return PW_OK;
	const int nnodes = 2 * n - 1;
	PW_CUDA(walloc(w, &m.nodeA, nnodes));
	PW_CUDA(walloc(w, &m.nodeB, nnodes));
	PW_CUDA(walloc(w, &m.obbA, nnodes));
	PW_CUDA(walloc(w, &m.obbB, nnodes));
	PW_CUDA(walloc(w, &m.obbR0, nnodes));
	PW_CUDA(walloc(w, &m.obbR1, nnodes));
	PW_CUDA(walloc(w, &m.obbR2, nnodes));
	PW_CUDA(walloc(w, &m.triA, n));
	PW_CUDA(walloc(w, &m.triB, n));
	PW_CUDA(walloc(w, &m.triC, n));

	// temporaries
	float4 *ta, *tb, *tc;
	float *tlo, *thi, *cen, *bounds, *blo, *bhi;
	uint32_t *keys, *vals, *keys2, *vals2;
	int32_t *left, *right, *parent, *rlo, *rhi;
	unsigned int *flags, *obb_bounds;
	int *maxdepth;
	double *mom, *mscan, *org;
	std::vector<void *> tmp;
	auto tal = [&](void **p, size_t bytes) -> cudaError_t {
		cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
		if (e == cudaSuccess)
			tmp.push_back(*p);
		return e;
	};
	auto cleanup = [&]() {
		for (void *p : tmp)
			cudaFree(p);
		tmp.clear();
	};
#define TAL(ptr, bytes)                                     \
	do {                                                    \
		cudaError_t e__ = tal((void **)&(ptr), (bytes));    \
		if (e__ != cudaSuccess) {                           \
			cleanup();                                      \
			return pw_cuda_fail(e__, "BVH temporaries");    \
		}                                                   \
	} while (0)
	TAL(ta, sizeof(float4) * n);
	TAL(tb, sizeof(float4) * n);
	TAL(tc, sizeof(float4) * n);
	TAL(tlo, sizeof(float) * 3 * n);
	TAL(thi, sizeof(float) * 3 * n);
	TAL(cen, sizeof(float) * 3 * n);
	TAL(bounds, sizeof(float) * 6);
	TAL(blo, sizeof(float) * 3 * nnodes);
	TAL(bhi, sizeof(float) * 3 * nnodes);
	TAL(keys, sizeof(uint32_t) * n);
	TAL(vals, sizeof(uint32_t) * n);
	TAL(keys2, sizeof(uint32_t) * n);
	TAL(vals2, sizeof(uint32_t) * n);
	TAL(left, sizeof(int32_t) * nnodes);
	TAL(right, sizeof(int32_t) * nnodes);
	TAL(parent, sizeof(int32_t) * nnodes);
	TAL(flags, sizeof(unsigned int) * nnodes);
	TAL(maxdepth, sizeof(int));
	TAL(rlo, sizeof(int32_t) * nnodes);
	TAL(rhi, sizeof(int32_t) * nnodes);
	TAL(obb_bounds, sizeof(unsigned int) * 2);
	TAL(mom, sizeof(double) * 9 * (size_t)n);
	TAL(mscan, sizeof(double) * 9 * (size_t)n);
	TAL(org, sizeof(double) * 3);
	const int B = 256;
	const int G = (n + B - 1) / B;
	cudaMemset(flags, 0, sizeof(unsigned int) * nnodes);
	cudaMemset(maxdepth, 0, sizeof(int));
	cudaMemset(parent, 0xff, sizeof(int32_t) * nnodes);
	k_tri_prep<<<G, B>>>(m.V64, m.F, n, ta, tb, tc, tlo, thi, cen);
	cudaError_t se = cudaSuccess;
	if (w->bvh_kind != PW_BVH_MORTON) {
		// the hierarchy built on the host (build_topdown), uploaded in the Karras layout
		std::vector<uint32_t> h_order;
		std::vector<int32_t> h_left, h_right, h_parent, h_rlo, h_rhi;
		// surface-area splits where the mesh is small enough for their build cost (measured:
		// the 4096-triangle tori's segment step 131.5 ms against 138.7 with mean splits;
		// the 320k-triangle plate 179.3 against 176.5 ms, and 0.9 against 0.27 s to build)
		const bool sah = w->bvh_kind == PW_BVH_SAH || (w->bvh_kind == PW_BVH_TOPDOWN && n <= SAH_MAX_TRIANGLES);
		build_topdown(V64, F, h_order, h_left, h_right, h_parent, h_rlo, h_rhi, sah);
		cudaMemcpy(vals2, h_order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
		cudaMemcpy(parent, h_parent.data(), sizeof(int32_t) * nnodes, cudaMemcpyHostToDevice);
		if (n > 1) {
			cudaMemcpy(left, h_left.data(), sizeof(int32_t) * (n - 1), cudaMemcpyHostToDevice);
			cudaMemcpy(right, h_right.data(), sizeof(int32_t) * (n - 1), cudaMemcpyHostToDevice);
			cudaMemcpy(rlo, h_rlo.data(), sizeof(int32_t) * (n - 1), cudaMemcpyHostToDevice);
			cudaMemcpy(rhi, h_rhi.data(), sizeof(int32_t) * (n - 1), cudaMemcpyHostToDevice);
		}
	} else {
		k_bounds<<<1, 256>>>(cen, n, bounds);
		k_morton<<<G, B>>>(cen, n, bounds, keys, vals);
		size_t tmp_bytes = 0;
		se = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, vals2, n, 0, 30);
		if (se != cudaSuccess) {
			cleanup();
			return pw_cuda_fail(se, "BVH sort (size query)");
		}
		void *cub_tmp = nullptr;
		TAL(cub_tmp, tmp_bytes);
		se = cub::DeviceRadixSort::SortPairs(cub_tmp, tmp_bytes, keys, keys2, vals, vals2, n, 0, 30);
		if (se != cudaSuccess) {
			cleanup();
			return pw_cuda_fail(se, "BVH sort");
		}
		if (n > 1)
			k_karras<<<(n - 1 + B - 1) / B, B>>>(keys2, n, left, right, parent, rlo, rhi);
	}
	k_refit<<<G, B>>>(vals2, n, tlo, thi, ta, tb, tc, m.triA, m.triB, m.triC, blo, bhi, left, right, parent, flags);
	k_finalize<<<(nnodes + B - 1) / B, B>>>(nnodes, n, blo, bhi, left, right, m.triA, m.nodeA, m.nodeB);
	// oriented boxes on the same hierarchy: slot moments about the vertices' box centre,
	// their prefix sums, then one warp per node
	{
		double vlo[3] = { 1e300, 1e300, 1e300 }, vhi[3] = { -1e300, -1e300, -1e300 };
		for (size_t i = 0; i + 2 < V64.size(); i += 3)
			for (int c = 0; c < 3; c++) {
				vlo[c] = std::min(vlo[c], V64[i + c]);
				vhi[c] = std::max(vhi[c], V64[i + c]);
			}
		const double o[3] = { 0.5 * (vlo[0] + vhi[0]), 0.5 * (vlo[1] + vhi[1]), 0.5 * (vlo[2] + vhi[2]) };
		cudaMemcpy(org, o, sizeof(o), cudaMemcpyHostToDevice);
	}
	cudaMemset(obb_bounds, 0, sizeof(unsigned int) * 2);
	k_slot_moments<<<G, B>>>(m.V64, m.F, vals2, n, org, mom);
	{
		size_t sbytes = 0;
		se = cub::DeviceScan::InclusiveSum(nullptr, sbytes, mom, mscan, n);
		void *scan_tmp = nullptr;
		if (se == cudaSuccess)
			TAL(scan_tmp, sbytes);
		for (int k = 0; k < 9 && se == cudaSuccess; k++)
			se = cub::DeviceScan::InclusiveSum(scan_tmp, sbytes, mom + (size_t)k * n, mscan + (size_t)k * n, n);
		if (se != cudaSuccess) {
			cleanup();
			return pw_cuda_fail(se, "BVH moment scan");
		}
	}
	k_obb_fit<<<(unsigned)(((int64_t)nnodes * 32 + B - 1) / B), B>>>(m.V64, m.F, vals2, n, mscan, rlo, rhi, left, right,
	                                                                 m.triA, m.obbA, m.obbB, m.obbR0, m.obbR1, m.obbR2,
	                                                                 obb_bounds, obb_bounds + 1);
	k_depth<<<G, B>>>(n, parent, maxdepth);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess)
		e = cudaDeviceSynchronize();
	if (e != cudaSuccess) {
		cleanup();
		return pw_cuda_fail(e, "BVH build");
	}
	int depth = 0;
	float rootlo[3], roothi[3];
	cudaMemcpy(&depth, maxdepth, sizeof(int), cudaMemcpyDeviceToHost);
	cudaMemcpy(rootlo, blo, sizeof(float) * 3, cudaMemcpyDeviceToHost);
	cudaMemcpy(roothi, bhi, sizeof(float) * 3, cudaMemcpyDeviceToHost);
	unsigned int ob[2] = { 0, 0 };
	cudaMemcpy(ob, obb_bounds, sizeof(ob), cudaMemcpyDeviceToHost);
	float ob1, obinf;
	memcpy(&ob1, &ob[0], 4);
	memcpy(&obinf, &ob[1], 4);
	m.depth = depth;
	// r1 and emax bound the points of both kinds of node box (the oriented boxes'
	// corners can reach past the vertices' coordinates)
	double r1 = 0.0;
	for (int c = 0; c < 3; c++)
		r1 += std::max(std::fabs((double)rootlo[c]), std::fabs((double)roothi[c]));
	r1 = std::max(r1, (double)ob1);
	m.r1 = (float)r1 * 1.0001f + 1e-30f;
	m.emax = std::max(m.emax, obinf * 1.0001f);
	cleanup();
#undef TAL
	if (depth >= 4096)
		return pw_fail(PW_ERR_INTERNAL, "BVH build: hierarchy deeper than 4096 levels");
	return PW_OK;
}
