// Immediate-mode PGS on the GB300: one frame of PxConstructSolverBodies /
// PxConstructStaticSolverBody, PxBatchConstraints, PxCreateContactConstraints,
// PxSolveConstraints and PxIntegrateSolverBodies
// (physx/include/PxImmediateMode.h; NpImmediateMode.cpp:55-78,269,292,552).
//
// One scene per call, kernels launched per stage: bodies (thread per body),
// rows (thread per constraint: the per-pair rows, or one lane of a 4-wide
// header's block rows), then for every iteration one launch per wave of
// consecutive headers whose constraints touch distinct dynamic bodies (the
// reference solves headers one after the other; inside a wave the order does
// not change any value), and one integration launch.
#include "common.cuh"
#include "pgs.cuh"
#include "batching.h"
#include <vector>

namespace gbpx
{
namespace pgs
{
__global__ void constructBodiesKernel(const RigidBody* __restrict__ rigid, uint32_t nbDyn, const float* __restrict__ staticPose, uint32_t nbStatic,
                                      float gx, float gy, float gz, float dt, BodyData* __restrict__ data, BodyVel* __restrict__ vel)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nbDyn + nbStatic) return;
	if(i < nbDyn)
		constructDynamicBody(rigid[i], v3(gx, gy, gz), dt, data[i]);
	else
	{
		const float* s = staticPose + 7 * size_t(i - nbDyn);
		Tr p;
		p.q.x = s[0]; p.q.y = s[1]; p.q.z = s[2]; p.q.w = s[3];
		p.p = v3(s[4], s[5], s[6]);
		constructStaticBody(p, data[i]);
	}
	// PxSolveConstraints starts from zeroed solver bodies
	BodyVel z;
	z.lin = zero3(); z.ang = zero3(); z.pad0 = z.pad1 = 0.0f;
	vel[i] = z;
}

// lane flags of a constraint in the ordered list
constexpr uint8_t LANE_BLOCK = 1, LANE_BLOCK_DYNAMIC = 2, LANE_STORE_B = 4, LANE_DYNAMIC_B = 8;

__global__ void prepKernel(const uint32_t* __restrict__ ordered, uint32_t n, const uint32_t* __restrict__ pairA, const uint32_t* __restrict__ pairB,
                           const uint32_t* __restrict__ cStart, const uint32_t* __restrict__ cCount, const float* __restrict__ contacts,
                           const float* __restrict__ material, const BodyData* __restrict__ data, const uint8_t* __restrict__ laneFlags,
                           PrepParams pp, Record* __restrict__ recs)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const uint32_t ci = ordered[k];
	const uint32_t a = pairA[ci], b = pairB[ci];
	Contact cs[MAX_CONTACTS];
	const uint32_t cnt = cCount[ci] < uint32_t(MAX_CONTACTS) ? cCount[ci] : uint32_t(MAX_CONTACTS);
	for(uint32_t c = 0; c < cnt; c++)
	{
		const float* s = contacts + 8 * size_t(cStart[ci] + c);
		cs[c].n = v3(s[0], s[1], s[2]);
		cs[c].sep = s[3];
		cs[c].p = v3(s[4], s[5], s[6]);
		cs[c].staticFriction = material[3 * ci + 0];
		cs[c].dynamicFriction = material[3 * ci + 1];
		cs[c].restitution = material[3 * ci + 2];
	}
	const uint8_t f = laneFlags[k];
	if(f & LANE_BLOCK)
		prepBlockLane(cs, int(cnt), int(a), int(b), data[a], data[b], pp, (f & LANE_BLOCK_DYNAMIC) != 0, (f & LANE_STORE_B) != 0, recs[k]);
	else
		prepPair(cs, int(cnt), int(a), int(b), data[a], data[b], pp, (f & LANE_DYNAMIC_B) != 0, recs[k]);
}

// records [begin, end) touch distinct dynamic bodies; a static body B keeps
// its zero solver body (the reference's writes leave it at +0)
__global__ void solveWaveKernel(Record* __restrict__ recs, uint32_t begin, uint32_t end, BodyVel* __restrict__ vel, uint32_t nbDyn, int doFriction,
                                int conclude)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	Record& r = recs[k];
	if(r.nbPatches == 0) return;
	BodyVel b0 = vel[r.bodyA];
	BodyVel b1 = vel[r.bodyB];
	bool writeB;
	if(r.flags & REC_BLOCK)
	{
		solveBlockLane(r, b0, b1, doFriction != 0, conclude != 0);
		writeB = (r.flags & REC_BLOCK_DYNAMIC) && (r.flags & REC_STORE_B);
	}
	else
	{
		solvePair(r, b0, b1, doFriction != 0, conclude != 0);
		writeB = (r.flags & REC_DYNAMIC_B) != 0;
	}
	vel[r.bodyA] = b0;
	if(writeB && uint32_t(r.bodyB) < nbDyn) vel[r.bodyB] = b1;
}

// the motion velocities PxSolveConstraints saves after the position iterations
__global__ void saveMotionKernel(const BodyVel* __restrict__ vel, uint32_t nbDyn, BodyVel* __restrict__ motion)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < nbDyn) motion[i] = vel[i];
}

// PxIntegrateSolverBodies: velocities (linear, angular) and pose per dynamic body
__global__ void integrateKernel(BodyData* __restrict__ data, const BodyVel* __restrict__ vel, const BodyVel* __restrict__ motion, uint32_t nbDyn,
                                float dt, float* __restrict__ outVel, float* __restrict__ outPose)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nbDyn) return;
	BodyData d = data[i];
	integrateBody(motion[i].lin, motion[i].ang, vel[i], d, dt);
	data[i] = d;
	float* o = outVel + 6 * size_t(i);
	o[0] = d.lin.x; o[1] = d.lin.y; o[2] = d.lin.z;
	o[3] = d.ang.x; o[4] = d.ang.y; o[5] = d.ang.z;
	float* q = outPose + 7 * size_t(i);
	q[0] = d.pose.q.x; q[1] = d.pose.q.y; q[2] = d.pose.q.z; q[3] = d.pose.q.w;
	q[4] = d.pose.p.x; q[5] = d.pose.p.y; q[6] = d.pose.p.z;
}

// the normal impulses the last velocity iteration leaves, per contact of the
// caller's array in the constraint's row order (writeBackContact's order)
__global__ void forcesKernel(const Record* __restrict__ recs, const uint32_t* __restrict__ ordered, uint32_t n, const uint32_t* __restrict__ cStart,
                             float* __restrict__ outForces)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const Record& r = recs[k];
	const uint32_t base = cStart[ordered[k]];
	int p = 0;
	for(int i = 0; i < r.nbPatches; i++)
		for(int j = 0; j < r.patch[i].nbPoints; j++, p++) outForces[base + p] = r.point[p].force;
}
} // namespace pgs

struct PgsWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<pgs::RigidBody> rigid;
	DevBuf<float> statics, contacts, material, outVel, outPose, outForces;
	DevBuf<uint32_t> pairA, pairB, cStart, cCount, ordered;
	DevBuf<uint8_t> laneFlags;
	DevBuf<pgs::BodyData> data;
	DevBuf<pgs::BodyVel> vel, motion;
	DevBuf<pgs::Record> recs;
	int init() { GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); return GBPX_OK; }
};

static PgsWorkspace* pgsWorkspace()
{
	static PgsWorkspace* ws = nullptr;
	if(!ws)
	{
		ws = new PgsWorkspace;
		if(ws->init()) { delete ws; ws = nullptr; }
	}
	return ws;
}
} // namespace gbpx

using namespace gbpx;

// One PGS frame from given contacts.  Inputs as gbpx_tgs_solve; batch != 0:
// PxBatchConstraints's headers, else one header per constraint in the
// caller's order.  Outputs: per dynamic body the linear and angular velocity
// (6 floats) and the pose (7 floats) after PxIntegrateSolverBodies; the
// headers (start, stride, constraintType as PxCreateContactConstraints sets
// it), the constraint order, per contact the normal impulse written back by
// the last velocity iteration (in the constraint's row order, as
// PxSolverContactDesc::contactForces receives it) and the header count.
GBPX_API int gbpx_pgs_solve(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA,
                            const uint32_t* pairB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                            const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel,
                            float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, int batch, float* outVel,
                            float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outHeaderType, uint32_t* outOrder,
                            float* outForces, uint32_t* outNbHeaders)
{
	gbpx::Zone zone("gbpx::pgsSolve");
	(void)correlationDistance;   // fresh friction data: nothing to correlate with
	if(!nbDyn || !rigid || !gravity || !outVel || !outPose || !outNbHeaders || !(dt > 0.0f) || !nbPos || !nbVel) return GBPX_ERR_INVALID;
	if(nbConstraints && (!pairA || !pairB || !contactStart || !contactCount || !contacts || !material || !outHeaderStart || !outHeaderStride ||
	                     !outHeaderType || !outOrder))
		return GBPX_ERR_INVALID;
	for(uint32_t i = 0; i < nbConstraints; i++)
		if(pairA[i] >= nbDyn || pairB[i] >= nbDyn + nbStatic || !contactCount[i] || contactCount[i] > uint32_t(pgs::MAX_CONTACTS))
			return GBPX_ERR_INVALID;   // body A dynamic, 1..4 contacts (PxSolveConstraints has no method for an empty constraint)
	PgsWorkspace* ws = pgsWorkspace();
	if(!ws) return GBPX_ERR_CUDA;

	// headers and order
	std::vector<uint32_t> hStart, hStride, order(nbConstraints);
	if(batch && nbConstraints)
	{
		batching::Result r;
		batching::partition(pairA, pairB, nbConstraints, nbDyn, r);
		hStart.assign(r.headerStart.begin(), r.headerStart.end());
		hStride.assign(r.headerStride.begin(), r.headerStride.end());
		for(uint32_t i = 0; i < nbConstraints; i++) order[i] = r.order[i];
	}
	else
	{
		for(uint32_t i = 0; i < nbConstraints; i++) { hStart.push_back(i); hStride.push_back(1); order[i] = i; }
	}
	const size_t nbHeaders = hStart.size();
	// header types and lane flags: a header of stride 4 holding at most 64
	// contacts takes the block path (NpImmediateMode.cpp:312-330), typed by
	// whether some body B is dynamic; otherwise the first constraint's type,
	// static contacts turning dynamic when another constraint of the header is
	std::vector<uint8_t> laneFlags(nbConstraints ? nbConstraints : 1, 0);
	std::vector<uint32_t> hType(nbHeaders, 0);
	for(size_t h = 0; h < nbHeaders; h++)
	{
		const uint32_t s0 = hStart[h], st = hStride[h];
		uint32_t total = 0;
		bool dyn = false;
		for(uint32_t l = 0; l < st; l++)
		{
			total += contactCount[order[s0 + l]];
			dyn = dyn || pairB[order[s0 + l]] < nbDyn;
		}
		if(st == 4 && total <= 64)
		{
			hType[h] = dyn ? 6u : 7u;   // DY_SC_TYPE_BLOCK_RB_CONTACT / _BLOCK_STATIC_RB_CONTACT
			for(uint32_t l = 0; l < 4; l++)
				laneFlags[s0 + l] = uint8_t(pgs::LANE_BLOCK | (dyn ? pgs::LANE_BLOCK_DYNAMIC : 0) | (pairB[order[s0 + l]] != 0 ? pgs::LANE_STORE_B : 0));
		}
		else
		{
			uint32_t type = pairB[order[s0]] >= nbDyn ? 5u : 1u;   // DY_SC_TYPE_STATIC_CONTACT / _RB_CONTACT
			if(type == 5u)
				for(uint32_t l = 1; l < st; l++)
					if(pairB[order[s0 + l]] < nbDyn) { type = 1u; break; }
			hType[h] = type;
			for(uint32_t l = 0; l < st; l++) laneFlags[s0 + l] = type == 1u ? pgs::LANE_DYNAMIC_B : 0;
		}
	}
	// waves: runs of consecutive headers whose constraints touch distinct dynamic bodies
	std::vector<uint32_t> waveEnds;
	{
		std::vector<uint32_t> stamp(nbDyn, 0xffffffffu);
		uint32_t wave = 0;
		for(size_t h = 0; h < nbHeaders; h++)
		{
			bool clash = false;
			for(uint32_t l = 0; l < hStride[h] && !clash; l++)
			{
				const uint32_t ci = order[hStart[h] + l];
				clash = stamp[pairA[ci]] == wave || (pairB[ci] < nbDyn && stamp[pairB[ci]] == wave);
			}
			if(clash)
			{
				waveEnds.push_back(hStart[h]);
				wave++;
			}
			for(uint32_t l = 0; l < hStride[h]; l++)
			{
				const uint32_t ci = order[hStart[h] + l];
				stamp[pairA[ci]] = wave;
				if(pairB[ci] < nbDyn) stamp[pairB[ci]] = wave;
			}
		}
		if(nbConstraints) waveEnds.push_back(nbConstraints);
	}

	uint32_t nbContacts = 0;
	for(uint32_t i = 0; i < nbConstraints; i++) nbContacts = std::max(nbContacts, contactStart[i] + contactCount[i]);
	const uint32_t nbTotal = nbDyn + nbStatic;
	const uint32_t nc = nbConstraints ? nbConstraints : 1;
	if(ws->rigid.reserve(nbDyn) || ws->statics.reserve(7 * size_t(nbStatic) + 1) || ws->pairA.reserve(nc) || ws->pairB.reserve(nc) ||
	   ws->cStart.reserve(nc) || ws->cCount.reserve(nc) || ws->ordered.reserve(nc) || ws->contacts.reserve(8 * size_t(nbContacts) + 8) ||
	   ws->material.reserve(3 * size_t(nc)) || ws->data.reserve(nbTotal) || ws->vel.reserve(nbTotal) || ws->motion.reserve(nbDyn) ||
	   ws->recs.reserve(nc) || ws->outVel.reserve(6 * size_t(nbDyn)) || ws->outPose.reserve(7 * size_t(nbDyn)) ||
	   ws->outForces.reserve(size_t(nbContacts) + 1) || ws->laneFlags.reserve(nc))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rigid.ptr, rigid, size_t(nbDyn) * sizeof(pgs::RigidBody), cudaMemcpyHostToDevice, s));
	if(nbStatic) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->statics.ptr, staticPose, size_t(nbStatic) * 28, cudaMemcpyHostToDevice, s));
	if(nbConstraints)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->pairA.ptr, pairA, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->pairB.ptr, pairB, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->cStart.ptr, contactStart, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->cCount.ptr, contactCount, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->ordered.ptr, order.data(), size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->material.ptr, material, size_t(nbConstraints) * 12, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->laneFlags.ptr, laneFlags.data(), size_t(nbConstraints), cudaMemcpyHostToDevice, s));
		if(nbContacts) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->contacts.ptr, contacts, size_t(nbContacts) * 32, cudaMemcpyHostToDevice, s));
	}
	pgs::constructBodiesKernel<<<divUp(nbTotal, 128), 128, 0, s>>>(ws->rigid.ptr, nbDyn, ws->statics.ptr, nbStatic, gravity[0], gravity[1],
	                                                               gravity[2], dt, ws->data.ptr, ws->vel.ptr);
	pgs::PrepParams pp;
	pp.invDt = 1.0f / dt;
	pp.bounceThreshold = bounceThreshold;
	pp.frictionOffsetThreshold = frictionOffsetThreshold;
	if(nbConstraints)
		pgs::prepKernel<<<divUp(nbConstraints, 128), 128, 0, s>>>(ws->ordered.ptr, nbConstraints, ws->pairA.ptr, ws->pairB.ptr, ws->cStart.ptr,
		                                                          ws->cCount.ptr, ws->contacts.ptr, ws->material.ptr, ws->data.ptr,
		                                                          ws->laneFlags.ptr, pp, ws->recs.ptr);
	auto iterate = [&](int doFriction, int conclude) {
		for(size_t w = 0; w < waveEnds.size(); w++)
		{
			const uint32_t b = w ? waveEnds[w - 1] : 0u, e = waveEnds[w];
			if(e > b)
				pgs::solveWaveKernel<<<divUp(e - b, 64), 64, 0, s>>>(ws->recs.ptr, b, e, ws->vel.ptr, nbDyn, doFriction, conclude);
		}
	};
	// PxSolveConstraints: position iterations (friction in the last three), the
	// last one concluding; the motion velocities saved; velocity iterations
	for(uint32_t i = nbPos; i > 1; --i) iterate(i <= 3 ? 1 : 0, 0);
	iterate(1, 1);
	pgs::saveMotionKernel<<<divUp(nbDyn, 128), 128, 0, s>>>(ws->vel.ptr, nbDyn, ws->motion.ptr);
	for(uint32_t i = nbVel; i > 0; --i) iterate(1, 0);
	pgs::integrateKernel<<<divUp(nbDyn, 128), 128, 0, s>>>(ws->data.ptr, ws->vel.ptr, ws->motion.ptr, nbDyn, dt, ws->outVel.ptr, ws->outPose.ptr);
	if(nbConstraints && outForces && nbContacts) GBPX_CUDA_TRY(cudaMemsetAsync(ws->outForces.ptr, 0, size_t(nbContacts) * 4, s));
	if(nbConstraints && outForces)
		pgs::forcesKernel<<<divUp(nbConstraints, 128), 128, 0, s>>>(ws->recs.ptr, ws->ordered.ptr, nbConstraints, ws->cStart.ptr, ws->outForces.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outVel, ws->outVel.ptr, size_t(nbDyn) * 24, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outPose, ws->outPose.ptr, size_t(nbDyn) * 28, cudaMemcpyDeviceToHost, s));
	if(nbConstraints && outForces && nbContacts)
		GBPX_CUDA_TRY(cudaMemcpyAsync(outForces, ws->outForces.ptr, size_t(nbContacts) * 4, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	for(size_t h = 0; h < nbHeaders; h++)
	{
		outHeaderStart[h] = hStart[h];
		outHeaderStride[h] = hStride[h];
		outHeaderType[h] = hType[h];
	}
	for(uint32_t i = 0; i < nbConstraints; i++) outOrder[i] = order[i];
	*outNbHeaders = uint32_t(nbHeaders);
	return GBPX_OK;
}

// ---------------------------------------------------------------- split-phase PGS on reference layouts
// The stages of the reference's immediate-mode PGS as separate calls, on solver
// bodies in the reference's layouts (PxSolverBodyData 112 B: linearVelocity,
// invMass, angularVelocity, reportThreshold, sqrtInvInertia, penBiasClamp,
// nodeIndex, maxContactImpulse, body2World; PxSolverBody 32 B: linearVelocity,
// progress counters, angularState, solverProgress), for callers that drive the
// stages themselves (the physx::immediate drop-in).
namespace gbpx
{
namespace pgs
{
__device__ __forceinline__ BodyData loadDataRef(const float* r)
{
	BodyData d;
	d.lin = v3(r[0], r[1], r[2]); d.invMass = r[3];
	d.ang = v3(r[4], r[5], r[6]);
	d.sqrtInvInertia.c0 = v3(r[8], r[9], r[10]);
	d.sqrtInvInertia.c1 = v3(r[11], r[12], r[13]);
	d.sqrtInvInertia.c2 = v3(r[14], r[15], r[16]);
	d.penBiasClamp = r[17];
	d.maxContactImpulse = r[19];
	d.pose.q.x = r[20]; d.pose.q.y = r[21]; d.pose.q.z = r[22]; d.pose.q.w = r[23];
	d.pose.p = v3(r[24], r[25], r[26]);
	return d;
}
// reportThreshold = PX_MAX_F32, nodeIndex = PX_INVALID_NODE, as the immediate-mode
// constructors pass them (NpImmediateMode.cpp:64,75)
__device__ __forceinline__ void storeDataRef(const BodyData& d, float* r)
{
	r[0] = d.lin.x; r[1] = d.lin.y; r[2] = d.lin.z; r[3] = d.invMass;
	r[4] = d.ang.x; r[5] = d.ang.y; r[6] = d.ang.z; r[7] = FLT_MAX;
	r[8] = d.sqrtInvInertia.c0.x; r[9] = d.sqrtInvInertia.c0.y; r[10] = d.sqrtInvInertia.c0.z;
	r[11] = d.sqrtInvInertia.c1.x; r[12] = d.sqrtInvInertia.c1.y; r[13] = d.sqrtInvInertia.c1.z;
	r[14] = d.sqrtInvInertia.c2.x; r[15] = d.sqrtInvInertia.c2.y; r[16] = d.sqrtInvInertia.c2.z;
	r[17] = d.penBiasClamp;
	r[18] = __uint_as_float(0xffffffffu);
	r[19] = d.maxContactImpulse;
	r[20] = d.pose.q.x; r[21] = d.pose.q.y; r[22] = d.pose.q.z; r[23] = d.pose.q.w;
	r[24] = d.pose.p.x; r[25] = d.pose.p.y; r[26] = d.pose.p.z;
	r[27] = 0.0f;
}

__global__ void constructRefKernel(const RigidBody* __restrict__ rigid, const float* __restrict__ poses, uint32_t n, float gx, float gy, float gz,
                                   float dt, float* __restrict__ out)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	BodyData d;
	if(rigid)
		constructDynamicBody(rigid[i], v3(gx, gy, gz), dt, d);
	else
	{
		const float* s = poses + 7 * size_t(i);
		Tr p;
		p.q.x = s[0]; p.q.y = s[1]; p.q.z = s[2]; p.q.w = s[3];
		p.p = v3(s[4], s[5], s[6]);
		constructStaticBody(p, d);
	}
	storeDataRef(d, out + 28 * size_t(i));
}

// rows of constraint k from its bodies' PxSolverBodyData, its frames (the
// PxSolverContactDesc's bodyFrame0/1) and its PxContactPoints (80 B each:
// friction and restitution read from the points)
__global__ void prepRefKernel(uint32_t n, const float* __restrict__ data0, const float* __restrict__ data1, const float* __restrict__ frame0,
                              const float* __restrict__ frame1, const uint32_t* __restrict__ cStart, const uint32_t* __restrict__ cCount,
                              const float* __restrict__ points, const uint8_t* __restrict__ laneFlags, PrepParams pp, Record* __restrict__ recs)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	Contact cs[MAX_CONTACTS];
	const uint32_t cnt = cCount[k] < uint32_t(MAX_CONTACTS) ? cCount[k] : uint32_t(MAX_CONTACTS);
	for(uint32_t c = 0; c < cnt; c++)
	{
		const float* s = points + 20 * size_t(cStart[k] + c);
		cs[c].n = v3(s[0], s[1], s[2]);
		cs[c].sep = s[3];
		cs[c].p = v3(s[4], s[5], s[6]);
		cs[c].staticFriction = s[11];
		cs[c].dynamicFriction = s[14];
		cs[c].restitution = s[15];
	}
	BodyData d0 = loadDataRef(data0 + 28 * size_t(k)), d1 = loadDataRef(data1 + 28 * size_t(k));
	const float* a = frame0 + 7 * size_t(k);
	const float* b = frame1 + 7 * size_t(k);
	d0.pose.q.x = a[0]; d0.pose.q.y = a[1]; d0.pose.q.z = a[2]; d0.pose.q.w = a[3]; d0.pose.p = v3(a[4], a[5], a[6]);
	d1.pose.q.x = b[0]; d1.pose.q.y = b[1]; d1.pose.q.z = b[2]; d1.pose.q.w = b[3]; d1.pose.p = v3(b[4], b[5], b[6]);
	const uint8_t f = laneFlags[k];
	if(f & LANE_BLOCK)
		prepBlockLane(cs, int(cnt), 0, 1, d0, d1, pp, (f & LANE_BLOCK_DYNAMIC) != 0, (f & LANE_STORE_B) != 0, recs[k]);
	else
		prepPair(cs, int(cnt), 0, 1, d0, d1, pp, (f & LANE_DYNAMIC_B) != 0, recs[k]);
}

// PxSolverBody (32 B) <-> BodyVel: linearVelocity at 0, angularState at 16
__global__ void loadVelKernel(const float* __restrict__ ref, uint32_t n, BodyVel* __restrict__ vel)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const float* r = ref + 8 * size_t(i);
	BodyVel v;
	v.lin = v3(r[0], r[1], r[2]); v.pad0 = 0.0f;
	v.ang = v3(r[4], r[5], r[6]); v.pad1 = 0.0f;
	vel[i] = v;
}
__global__ void storeVelKernel(const BodyVel* __restrict__ vel, uint32_t n, float* __restrict__ ref, float* __restrict__ motionLin,
                               float* __restrict__ motionAng, const BodyVel* __restrict__ motion)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	float* r = ref + 8 * size_t(i);
	r[0] = vel[i].lin.x; r[1] = vel[i].lin.y; r[2] = vel[i].lin.z;
	r[4] = vel[i].ang.x; r[5] = vel[i].ang.y; r[6] = vel[i].ang.z;
	float* ml = motionLin + 3 * size_t(i);
	float* ma = motionAng + 3 * size_t(i);
	ml[0] = motion[i].lin.x; ml[1] = motion[i].lin.y; ml[2] = motion[i].lin.z;
	ma[0] = motion[i].ang.x; ma[1] = motion[i].ang.y; ma[2] = motion[i].ang.z;
}

// one wave of records whose bodies are bodyA[k], bodyB[k] (indices into vel;
// >= nbBodies: a body outside the caller's solver-body array, read as zero and
// never written)
__global__ void solveWaveRefKernel(Record* __restrict__ recs, const uint32_t* __restrict__ bodyA, const uint32_t* __restrict__ bodyB, uint32_t begin,
                                   uint32_t end, BodyVel* __restrict__ vel, uint32_t nbBodies, int doFriction, int conclude)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	Record& r = recs[k];
	if(r.nbPatches == 0) return;
	const uint32_t a = bodyA[k], b = bodyB[k];
	BodyVel zero;
	zero.lin = zero3(); zero.ang = zero3(); zero.pad0 = zero.pad1 = 0.0f;
	BodyVel b0 = a < nbBodies ? vel[a] : zero;
	BodyVel b1 = b < nbBodies ? vel[b] : zero;
	bool writeB;
	if(r.flags & REC_BLOCK)
	{
		solveBlockLane(r, b0, b1, doFriction != 0, conclude != 0);
		writeB = (r.flags & REC_BLOCK_DYNAMIC) && (r.flags & REC_STORE_B);
	}
	else
	{
		solvePair(r, b0, b1, doFriction != 0, conclude != 0);
		writeB = (r.flags & REC_DYNAMIC_B) != 0;
	}
	if(a < nbBodies) vel[a] = b0;
	if(writeB && b < nbBodies) vel[b] = b1;
}

__global__ void integrateRefKernel(float* __restrict__ data, const float* __restrict__ bodies, float* __restrict__ motionLin,
                                   float* __restrict__ motionAng, uint32_t n, float dt)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	float* r = data + 28 * size_t(i);
	BodyData d = loadDataRef(r);
	const float* sb = bodies + 8 * size_t(i);
	BodyVel v;
	v.lin = v3(sb[0], sb[1], sb[2]);
	v.ang = v3(sb[4], sb[5], sb[6]);
	float* ml = motionLin + 3 * size_t(i);
	float* ma = motionAng + 3 * size_t(i);
	const V3 mLin = v3(ml[0], ml[1], ml[2]), mAng = v3(ma[0], ma[1], ma[2]);
	// integrateCore also returns the motion velocities it integrated with
	const V3 linearMotionVel = add(d.lin, mLin);
	const V3 angularMotionVelIn = add(d.ang, m33MulVS(d.sqrtInvInertia, mAng));
	integrateBody(mLin, mAng, v, d, dt);
	V3 angularMotionVel = angularMotionVelIn;
	const float w = sqrtf(lenSqS(angularMotionVel));
	if(w > 1e+7f) angularMotionVel = scale(normalizeS(angularMotionVel), 1e+7f);
	ml[0] = linearMotionVel.x; ml[1] = linearMotionVel.y; ml[2] = linearMotionVel.z;
	ma[0] = angularMotionVel.x; ma[1] = angularMotionVel.y; ma[2] = angularMotionVel.z;
	const float keep7 = r[7], keep18 = r[18];   // reportThreshold, nodeIndex as the caller left them
	storeDataRef(d, r);
	r[7] = keep7;
	r[18] = keep18;
}
} // namespace pgs

struct PgsStageWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<pgs::RigidBody> rigid;
	DevBuf<float> poses, data, data0, data1, frame0, frame1, points, bodies, motionLin, motionAng;
	DevBuf<uint32_t> cStart, cCount, bodyA, bodyB;
	DevBuf<uint8_t> laneFlags;
	DevBuf<pgs::BodyVel> vel, motion;
	DevBuf<pgs::Record> recs;
	int init() { GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); return GBPX_OK; }
};

static PgsStageWorkspace* pgsStageWorkspace()
{
	static PgsStageWorkspace* ws = nullptr;
	if(!ws)
	{
		ws = new PgsStageWorkspace;
		if(ws->init()) { delete ws; ws = nullptr; }
	}
	return ws;
}
} // namespace gbpx

// Bytes of one PGS constraint record (gbpx_create_contact_constraints_pgs).
GBPX_API uint32_t gbpx_pgs_record_bytes(void) { return uint32_t(sizeof(pgs::Record)); }

// PxConstructSolverBodies (rigid != NULL: nb PxRigidBodyData) or
// PxConstructStaticSolverBody (rigid == NULL: nb poses, 7 floats each) into nb
// PxSolverBodyData records (112 B).
GBPX_API int gbpx_construct_solver_bodies_pgs(const void* rigid, const float* poses, uint32_t nb, const float* gravity, float dt, void* outData)
{
	gbpx::Zone zone("gbpx::constructSolverBodies");
	if(!nb) return GBPX_OK;
	if((!rigid && !poses) || !outData || (rigid && !gravity)) return GBPX_ERR_INVALID;
	PgsStageWorkspace* ws = pgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	if(ws->rigid.reserve(nb) || ws->poses.reserve(7 * size_t(nb)) || ws->data.reserve(28 * size_t(nb))) return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	if(rigid) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rigid.ptr, rigid, size_t(nb) * sizeof(pgs::RigidBody), cudaMemcpyHostToDevice, s));
	else GBPX_CUDA_TRY(cudaMemcpyAsync(ws->poses.ptr, poses, size_t(nb) * 28, cudaMemcpyHostToDevice, s));
	const float g0 = rigid ? gravity[0] : 0.0f, g1 = rigid ? gravity[1] : 0.0f, g2 = rigid ? gravity[2] : 0.0f;
	pgs::constructRefKernel<<<divUp(nb, 128), 128, 0, s>>>(rigid ? ws->rigid.ptr : nullptr, ws->poses.ptr, nb, g0, g1, g2, dt, ws->data.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outData, ws->data.ptr, size_t(nb) * 112, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// PxCreateContactConstraints, one contact descriptor per constraint: the two
// bodies' PxSolverBodyData (data0/data1, 112 B each), the body frames
// (PxTransform), contactPoints[contactStart[k] .. +contactCount[k]]
// (PxContactPoint, 80 B, 1..4 per constraint).  laneFlags[k]: bit 0 one of the
// four constraints of a header of stride 4 on the reference's 4-wide block
// path, bit 1 that header has a dynamic body B, bit 2 the block solve stores
// body B (its bodyBDataIndex is not 0), bit 3 the per-pair solve treats body B
// as dynamic (the header is DY_SC_TYPE_RB_CONTACT).  Records (gbpx_pgs_record_bytes()
// each) go to outRecords.
GBPX_API int gbpx_create_contact_constraints_pgs(uint32_t n, const void* data0, const void* data1, const float* frame0, const float* frame1,
                                                 const uint32_t* contactStart, const uint32_t* contactCount, const void* contactPoints,
                                                 uint32_t nbPoints, const uint8_t* laneFlags, float invDt, float bounceThreshold,
                                                 float frictionOffsetThreshold, void* outRecords)
{
	gbpx::Zone zone("gbpx::createContactConstraints");
	if(!n) return GBPX_OK;
	if(!data0 || !data1 || !frame0 || !frame1 || !contactStart || !contactCount || !laneFlags || !outRecords || (nbPoints && !contactPoints) ||
	   !(invDt > 0.0f))
		return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < n; k++)
		if(!contactCount[k] || contactCount[k] > uint32_t(pgs::MAX_CONTACTS) || contactStart[k] + contactCount[k] > nbPoints) return GBPX_ERR_INVALID;
	PgsStageWorkspace* ws = pgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	const size_t m = n;
	if(ws->data0.reserve(28 * m) || ws->data1.reserve(28 * m) || ws->frame0.reserve(7 * m) || ws->frame1.reserve(7 * m) || ws->cStart.reserve(m) ||
	   ws->cCount.reserve(m) || ws->points.reserve(20 * size_t(nbPoints) + 20) || ws->laneFlags.reserve(m) || ws->recs.reserve(m))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->data0.ptr, data0, m * 112, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->data1.ptr, data1, m * 112, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->frame0.ptr, frame0, m * 28, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->frame1.ptr, frame1, m * 28, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->cStart.ptr, contactStart, m * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->cCount.ptr, contactCount, m * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->laneFlags.ptr, laneFlags, m, cudaMemcpyHostToDevice, s));
	if(nbPoints) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->points.ptr, contactPoints, size_t(nbPoints) * 80, cudaMemcpyHostToDevice, s));
	pgs::PrepParams pp;
	pp.invDt = invDt;
	pp.bounceThreshold = bounceThreshold;
	pp.frictionOffsetThreshold = frictionOffsetThreshold;
	pgs::prepRefKernel<<<divUp(n, 128), 128, 0, s>>>(n, ws->data0.ptr, ws->data1.ptr, ws->frame0.ptr, ws->frame1.ptr, ws->cStart.ptr, ws->cCount.ptr,
	                                                 ws->points.ptr, ws->laneFlags.ptr, pp, ws->recs.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outRecords, ws->recs.ptr, m * sizeof(pgs::Record), cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// PxSolveConstraints: records (n of gbpx_pgs_record_bytes(), in solve order,
// updated in place with the impulses), record k joining bodies bodyA[k],
// bodyB[k] (indices into bodies; >= nbBodies: read as a zero solver body, not
// written).  Wave w solves records [waveEnds[w-1], waveEnds[w]), which touch
// distinct bodies below nbBodies.  bodies: nbBodies PxSolverBody records (32 B,
// zeroed by the caller), updated in place; outMotionLin / outMotionAng
// (nbBodies x 3 floats): the velocities after the position iterations.
GBPX_API int gbpx_solve_constraints_pgs(void* records, const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, const uint32_t* waveEnds,
                                        uint32_t nbWaves, void* bodies, uint32_t nbBodies, uint32_t nbPos, uint32_t nbVel, float* outMotionLin,
                                        float* outMotionAng)
{
	gbpx::Zone zone("gbpx::solveConstraints");
	if(!nbPos || !nbVel || (nbBodies && (!bodies || !outMotionLin || !outMotionAng))) return GBPX_ERR_INVALID;
	if(n && (!records || !bodyA || !bodyB || !waveEnds || !nbWaves || waveEnds[nbWaves - 1] != n)) return GBPX_ERR_INVALID;
	for(uint32_t w = 0; w < nbWaves; w++)
		if(waveEnds[w] > n || (w && waveEnds[w] < waveEnds[w - 1])) return GBPX_ERR_INVALID;
	PgsStageWorkspace* ws = pgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	const size_t m = n ? n : 1, nb = nbBodies ? nbBodies : 1;
	if(ws->recs.reserve(m) || ws->bodyA.reserve(m) || ws->bodyB.reserve(m) || ws->bodies.reserve(8 * nb) || ws->vel.reserve(nb) ||
	   ws->motion.reserve(nb) || ws->motionLin.reserve(3 * nb) || ws->motionAng.reserve(3 * nb))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	if(n)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->recs.ptr, records, size_t(n) * sizeof(pgs::Record), cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->bodyA.ptr, bodyA, size_t(n) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->bodyB.ptr, bodyB, size_t(n) * 4, cudaMemcpyHostToDevice, s));
	}
	if(nbBodies)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->bodies.ptr, bodies, size_t(nbBodies) * 32, cudaMemcpyHostToDevice, s));
		pgs::loadVelKernel<<<divUp(nbBodies, 128), 128, 0, s>>>(ws->bodies.ptr, nbBodies, ws->vel.ptr);
	}
	auto iterate = [&](int doFriction, int conclude) {
		for(uint32_t w = 0; w < nbWaves; w++)
		{
			const uint32_t b = w ? waveEnds[w - 1] : 0u, e = waveEnds[w];
			if(e > b)
				pgs::solveWaveRefKernel<<<divUp(e - b, 64), 64, 0, s>>>(ws->recs.ptr, ws->bodyA.ptr, ws->bodyB.ptr, b, e, ws->vel.ptr, nbBodies, doFriction,
				                                                         conclude);
		}
	};
	for(uint32_t i = nbPos; i > 1; --i) iterate(i <= 3 ? 1 : 0, 0);
	iterate(1, 1);
	if(nbBodies) pgs::saveMotionKernel<<<divUp(nbBodies, 128), 128, 0, s>>>(ws->vel.ptr, nbBodies, ws->motion.ptr);
	for(uint32_t i = nbVel; i > 0; --i) iterate(1, 0);
	if(nbBodies)
		pgs::storeVelKernel<<<divUp(nbBodies, 128), 128, 0, s>>>(ws->vel.ptr, nbBodies, ws->bodies.ptr, ws->motionLin.ptr, ws->motionAng.ptr,
		                                                          ws->motion.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	if(n) GBPX_CUDA_TRY(cudaMemcpyAsync(records, ws->recs.ptr, size_t(n) * sizeof(pgs::Record), cudaMemcpyDeviceToHost, s));
	if(nbBodies)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(bodies, ws->bodies.ptr, size_t(nbBodies) * 32, cudaMemcpyDeviceToHost, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(outMotionLin, ws->motionLin.ptr, size_t(nbBodies) * 12, cudaMemcpyDeviceToHost, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(outMotionAng, ws->motionAng.ptr, size_t(nbBodies) * 12, cudaMemcpyDeviceToHost, s));
	}
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// PxIntegrateSolverBodies: n PxSolverBodyData records (updated in place: pose,
// velocities), PxSolverBody records and the motion velocities of
// gbpx_solve_constraints_pgs (replaced by the velocities integrated with).
GBPX_API int gbpx_integrate_solver_bodies_pgs(void* data, const void* bodies, float* motionLin, float* motionAng, uint32_t n, float dt)
{
	gbpx::Zone zone("gbpx::integrateSolverBodies");
	if(!n) return GBPX_OK;
	if(!data || !bodies || !motionLin || !motionAng) return GBPX_ERR_INVALID;
	PgsStageWorkspace* ws = pgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	if(ws->data.reserve(28 * size_t(n)) || ws->bodies.reserve(8 * size_t(n)) || ws->motionLin.reserve(3 * size_t(n)) || ws->motionAng.reserve(3 * size_t(n)))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->data.ptr, data, size_t(n) * 112, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->bodies.ptr, bodies, size_t(n) * 32, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->motionLin.ptr, motionLin, size_t(n) * 12, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->motionAng.ptr, motionAng, size_t(n) * 12, cudaMemcpyHostToDevice, s));
	pgs::integrateRefKernel<<<divUp(n, 128), 128, 0, s>>>(ws->data.ptr, ws->bodies.ptr, ws->motionLin.ptr, ws->motionAng.ptr, n, dt);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(data, ws->data.ptr, size_t(n) * 112, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(motionLin, ws->motionLin.ptr, size_t(n) * 12, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(motionAng, ws->motionAng.ptr, size_t(n) * 12, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}
