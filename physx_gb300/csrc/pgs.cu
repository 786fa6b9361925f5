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
