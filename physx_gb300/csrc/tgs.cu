// Immediate-mode TGS on the GB300: PxConstructSolverBodiesTGS,
// PxBatchConstraintsTGS, PxCreateContactConstraintsTGS, PxSolveConstraintsTGS
// and PxIntegrateSolverBodiesTGS (physx/include/PxImmediateMode.h:592-729).
//
// One scene per call, kernels launched per stage: bodies (thread per body),
// rows (thread per constraint), then for every iteration one launch per
// partition (thread per constraint; constraints of a partition touch disjoint
// dynamic bodies) followed by an integration launch.  This is the plain
// one-scene-per-launch-sequence GPU step; the batched multi-scene step lives
// in world.cu and reuses the same device functions.
#include "common.cuh"
#include "solver.cuh"
#include "batching.h"
#include <vector>

namespace gbpx
{
namespace tgs
{
__global__ void constructBodiesKernel(const RigidBody* __restrict__ rigid, uint32_t nbDyn, const float* __restrict__ staticPose, uint32_t nbStatic,
                                      float gx, float gy, float gz, float dt, BodyVel* __restrict__ vel, BodyTx* __restrict__ tx,
                                      BodyData* __restrict__ data, Tr* __restrict__ pose)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < nbDyn)
	{
		Tr p;
		constructDynamicBody(rigid[i], v3(gx, gy, gz), dt, vel[i], tx[i], data[i], p);
		pose[i] = p;
	}
	else if(i < nbDyn + nbStatic)
	{
		const float* s = staticPose + 7 * size_t(i - nbDyn);
		Tr p;
		p.q.x = s[0]; p.q.y = s[1]; p.q.z = s[2]; p.q.w = s[3];
		p.p = v3(s[4], s[5], s[6]);
		constructStaticBody(p, vel[i], tx[i], data[i]);
		pose[i] = p;
	}
}

// Rows for constraint k of the ordered list (ordered[k] = caller's constraint index).
__global__ void prepKernel(const uint32_t* __restrict__ ordered, uint32_t n, const uint32_t* __restrict__ pairA, const uint32_t* __restrict__ pairB,
                           const uint32_t* __restrict__ cStart, const uint32_t* __restrict__ cCount, const float* __restrict__ contacts,
                           const float* __restrict__ material, const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx,
                           const BodyData* __restrict__ data, const Tr* __restrict__ pose, PrepParams pp, ConstraintRecord* __restrict__ recs)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const uint32_t ci = ordered[k];
	const uint32_t a = pairA[ci], b = pairB[ci];
	Contact cs[MAX_CONTACTS];
	const uint32_t cnt = cCount[ci] < MAX_CONTACTS ? cCount[ci] : MAX_CONTACTS;
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
	prepConstraint(cs, int(cnt), int(a), int(b), vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a], pose[b], pp, recs[k]);
}

__global__ void solvePartitionKernel(ConstraintRecord* __restrict__ recs, uint32_t begin, uint32_t end, BodyVel* __restrict__ vel, uint32_t nbDyn,
                                     float minPen, float elapsed)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	ConstraintRecord& r = recs[k];
	if(r.nbPatches == 0) return;
	BodyVel b0 = vel[r.bodyA];
	BodyVel b1 = vel[r.bodyB];
	const bool dynB = uint32_t(r.bodyB) < nbDyn;
	solveConstraint(r, b0, b1, dynB, minPen, elapsed);
	vel[r.bodyA].lin = b0.lin;
	vel[r.bodyA].ang = b0.ang;
	if(dynB)
	{
		vel[r.bodyB].lin = b1.lin;
		vel[r.bodyB].ang = b1.ang;
	}
}

__global__ void integrateKernel(BodyVel* __restrict__ vel, BodyTx* __restrict__ tx, uint32_t nbDyn, float dt)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < nbDyn) integrateStep(vel[i], tx[i], dt);
}

__global__ void finalizeKernel(const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx, const Tr* __restrict__ pose, uint32_t nbDyn,
                               float* __restrict__ outVel, float* __restrict__ outPose)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nbDyn) return;
	Tr p = pose[i];
	V3 w;
	finalizeBody(vel[i], tx[i], p, w);
	float* o = outVel + 6 * size_t(i);
	o[0] = vel[i].lin.x; o[1] = vel[i].lin.y; o[2] = vel[i].lin.z;
	o[3] = w.x; o[4] = w.y; o[5] = w.z;
	float* q = outPose + 7 * size_t(i);
	q[0] = p.q.x; q[1] = p.q.y; q[2] = p.q.z; q[3] = p.q.w;
	q[4] = p.p.x; q[5] = p.p.y; q[6] = p.p.z;
}

// Solver bodies in the reference's byte layouts (PxTGSSolverBodyVel 64 B,
// PxTGSSolverBodyTxInertia 64 B, PxTGSSolverBodyData 48 B).
__global__ void exportBodiesKernel(const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx, const BodyData* __restrict__ data, uint32_t n,
                                   float* __restrict__ outVel, float* __restrict__ outTx, float* __restrict__ outData)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	float* v = outVel + 16 * size_t(i);
	v[0] = vel[i].lin.x; v[1] = vel[i].lin.y; v[2] = vel[i].lin.z; v[3] = 0.0f;
	v[4] = vel[i].ang.x; v[5] = vel[i].ang.y; v[6] = vel[i].ang.z; v[7] = 0.0f;
	v[8] = vel[i].dAng.x; v[9] = vel[i].dAng.y; v[10] = vel[i].dAng.z; v[11] = vel[i].maxAngVel;
	v[12] = vel[i].dLin.x; v[13] = vel[i].dLin.y; v[14] = vel[i].dLin.z;
	uint32_t lockAndKin = vel[i].kinematic ? (1u << 16) : 0u;   // lockFlags (u16) = 0, isKinematic (u8), pad (u8)
	memcpy(&v[15], &lockAndKin, 4);
	float* t = outTx + 16 * size_t(i);
	t[0] = tx[i].dq.x; t[1] = tx[i].dq.y; t[2] = tx[i].dq.z; t[3] = tx[i].dq.w;
	t[4] = tx[i].p.x; t[5] = tx[i].p.y; t[6] = tx[i].p.z;
	const M33& m = tx[i].sqrtInvInertia;
	t[7] = m.c0.x; t[8] = m.c0.y; t[9] = m.c0.z; t[10] = m.c1.x; t[11] = m.c1.y; t[12] = m.c1.z; t[13] = m.c2.x; t[14] = m.c2.y; t[15] = m.c2.z;
	float* d = outData + 12 * size_t(i);
	d[0] = data[i].origLin.x; d[1] = data[i].origLin.y; d[2] = data[i].origLin.z; d[3] = data[i].maxContactImpulse;
	d[4] = data[i].origAng.x; d[5] = data[i].origAng.y; d[6] = data[i].origAng.z; d[7] = data[i].penBiasClamp;
	d[8] = data[i].invMass;
	const uint32_t invalidNode = 0x7fffffffu;   // nodeIndex: immediate mode passes PX_INVALID_NODE
	memcpy(&d[9], &invalidNode, 4);
	d[10] = FLT_MAX;                            // reportThreshold
	d[11] = 0.0f;
}
} // namespace tgs

struct TgsWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<tgs::RigidBody> rigid;
	DevBuf<float> statics, contacts, material, outVel, outPose, outTx, outData;
	DevBuf<uint32_t> pairA, pairB, cStart, cCount, ordered;
	DevBuf<tgs::BodyVel> vel;
	DevBuf<tgs::BodyTx> tx;
	DevBuf<tgs::BodyData> data;
	DevBuf<Tr> pose;
	DevBuf<tgs::ConstraintRecord> recs;
	int init() { GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); return GBPX_OK; }
};

static TgsWorkspace* tgsWorkspace()
{
	static TgsWorkspace* ws = nullptr;
	if(!ws)
	{
		ws = new TgsWorkspace;
		if(ws->init()) { delete ws; ws = nullptr; }
	}
	return ws;
}
} // namespace gbpx

using namespace gbpx;

// PxBatchConstraintsTGS: constraint i joins bodies bodyA[i], bodyB[i]; indices
// >= nbDyn are static/kinematic.  Writes headers (start, stride) and the
// order of the caller's constraint indices; returns the header count.
GBPX_API uint32_t gbpx_batch_constraints_tgs(const uint32_t* bodyA, const uint32_t* bodyB, uint32_t nbConstraints, uint32_t nbDyn,
                                             uint32_t nbStatic, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder)
{
	(void)nbStatic;
	if(!nbConstraints) return 0;
	if(!bodyA || !bodyB || !outHeaderStart || !outHeaderStride || !outOrder) return 0;
	batching::Result r;
	batching::partition(bodyA, bodyB, nbConstraints, nbDyn, r);
	for(size_t h = 0; h < r.headerStart.size(); h++)
	{
		outHeaderStart[h] = r.headerStart[h];
		outHeaderStride[h] = r.headerStride[h];
	}
	for(uint32_t i = 0; i < nbConstraints; i++) outOrder[i] = r.order[i];
	return uint32_t(r.headerStart.size());
}

// PxConstructSolverBodiesTGS for nb bodies (PxRigidBodyData in, reference
// solver-body layouts out).
GBPX_API int gbpx_construct_solver_bodies_tgs(const void* rigid, uint32_t nb, const float* gravity, float dt, void* outVel, void* outTxI,
                                              void* outData)
{
	if(!nb) return GBPX_OK;
	if(!rigid || !gravity || !outVel || !outTxI || !outData) return GBPX_ERR_INVALID;
	TgsWorkspace* ws = tgsWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	if(ws->rigid.reserve(nb) || ws->vel.reserve(nb) || ws->tx.reserve(nb) || ws->data.reserve(nb) || ws->pose.reserve(nb) ||
	   ws->outVel.reserve(16 * size_t(nb)) || ws->outTx.reserve(16 * size_t(nb)) || ws->outData.reserve(12 * size_t(nb)))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rigid.ptr, rigid, size_t(nb) * sizeof(tgs::RigidBody), cudaMemcpyHostToDevice, s));
	tgs::constructBodiesKernel<<<divUp(nb, 128), 128, 0, s>>>(ws->rigid.ptr, nb, nullptr, 0, gravity[0], gravity[1], gravity[2], dt, ws->vel.ptr,
	                                                          ws->tx.ptr, ws->data.ptr, ws->pose.ptr);
	tgs::exportBodiesKernel<<<divUp(nb, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, ws->data.ptr, nb, ws->outVel.ptr, ws->outTx.ptr, ws->outData.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outVel, ws->outVel.ptr, size_t(nb) * 64, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outTxI, ws->outTx.ptr, size_t(nb) * 64, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outData, ws->outData.ptr, size_t(nb) * 48, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// One TGS step from given contacts: construct bodies, batch, create contact
// constraints, solve (nbPos position + nbVel velocity iterations) and
// integrate.  rigid = PxRigidBodyData[nbDyn], staticPose = PxTransform[nbStatic],
// constraint i joins pairA[i], pairB[i] (statics indexed from nbDyn) with
// contacts[contactStart[i] .. +contactCount[i]] (8 floats each, <= 4 per pair)
// and material (static friction, dynamic friction, restitution).  Outputs:
// linear and world angular velocity (6 floats) and pose (7 floats) per dynamic
// body, headers, constraint order and the header count.
GBPX_API int gbpx_tgs_solve(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA,
                                 const uint32_t* pairB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                                 const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel,
                                 float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, float* outVel, float* outPose,
                                 uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder, uint32_t* outNbHeaders)
{
	(void)correlationDistance;
	if(!nbDyn || !rigid || !gravity || !outVel || !outPose || !outNbHeaders || !(dt > 0.0f) || !nbPos || !nbVel) return GBPX_ERR_INVALID;
	if(nbConstraints && (!pairA || !pairB || !contactStart || !contactCount || !contacts || !material || !outHeaderStart || !outHeaderStride || !outOrder))
		return GBPX_ERR_INVALID;
	for(uint32_t i = 0; i < nbConstraints; i++)
		if(pairA[i] >= nbDyn + nbStatic || pairB[i] >= nbDyn + nbStatic || contactCount[i] > tgs::MAX_CONTACTS ||
		   (pairA[i] >= nbDyn && pairB[i] >= nbDyn))   // a constraint needs one dynamic body
			return GBPX_ERR_INVALID;
	TgsWorkspace* ws = tgsWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	batching::Result batch;
	if(nbConstraints) batching::partition(pairA, pairB, nbConstraints, nbDyn, batch);
	uint32_t nbContacts = 0;
	for(uint32_t i = 0; i < nbConstraints; i++) nbContacts = std::max(nbContacts, contactStart[i] + contactCount[i]);
	const uint32_t nbTotal = nbDyn + nbStatic;
	const uint32_t nc = nbConstraints ? nbConstraints : 1;
	if(ws->rigid.reserve(nbDyn) || ws->statics.reserve(7 * size_t(nbStatic) + 1) || ws->pairA.reserve(nc) || ws->pairB.reserve(nc) ||
	   ws->cStart.reserve(nc) || ws->cCount.reserve(nc) || ws->ordered.reserve(nc) || ws->contacts.reserve(8 * size_t(nbContacts) + 8) ||
	   ws->material.reserve(3 * size_t(nc)) || ws->vel.reserve(nbTotal) || ws->tx.reserve(nbTotal) || ws->data.reserve(nbTotal) ||
	   ws->pose.reserve(nbTotal) || ws->recs.reserve(nc) || ws->outVel.reserve(6 * size_t(nbDyn)) || ws->outPose.reserve(7 * size_t(nbDyn)))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	if(cudaMemcpyAsync(ws->rigid.ptr, rigid, size_t(nbDyn) * sizeof(tgs::RigidBody), cudaMemcpyHostToDevice, s) != cudaSuccess) return GBPX_ERR_CUDA;
	if(nbStatic && cudaMemcpyAsync(ws->statics.ptr, staticPose, size_t(nbStatic) * 28, cudaMemcpyHostToDevice, s) != cudaSuccess) return GBPX_ERR_CUDA;
	if(nbConstraints)
	{
		if(cudaMemcpyAsync(ws->pairA.ptr, pairA, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
		   cudaMemcpyAsync(ws->pairB.ptr, pairB, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
		   cudaMemcpyAsync(ws->cStart.ptr, contactStart, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
		   cudaMemcpyAsync(ws->cCount.ptr, contactCount, size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
		   cudaMemcpyAsync(ws->ordered.ptr, batch.order.data(), size_t(nbConstraints) * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
		   cudaMemcpyAsync(ws->material.ptr, material, size_t(nbConstraints) * 12, cudaMemcpyHostToDevice, s) != cudaSuccess ||
		   (nbContacts && cudaMemcpyAsync(ws->contacts.ptr, contacts, size_t(nbContacts) * 32, cudaMemcpyHostToDevice, s) != cudaSuccess))
			return GBPX_ERR_CUDA;
	}
	tgs::constructBodiesKernel<<<divUp(nbTotal, 128), 128, 0, s>>>(ws->rigid.ptr, nbDyn, ws->statics.ptr, nbStatic, gravity[0], gravity[1],
	                                                               gravity[2], dt, ws->vel.ptr, ws->tx.ptr, ws->data.ptr, ws->pose.ptr);
	const float invDt = 1.0f / dt;
	const float stepDt = dt / float(nbPos);
	const float invStepDt = invDt * float(nbPos);
	tgs::PrepParams pp;
	pp.invStepDt = invStepDt;
	pp.invTotalDt = invDt;
	pp.totalDt = 1.0f / invDt;
	pp.stepDt = 1.0f / invStepDt;
	pp.bounceThreshold = bounceThreshold;
	pp.frictionOffsetThreshold = frictionOffsetThreshold;
	pp.biasCoefficient = 2.0f * sqrtf(invDt / invStepDt);
	if(nbConstraints)
		tgs::prepKernel<<<divUp(nbConstraints, 128), 128, 0, s>>>(ws->ordered.ptr, nbConstraints, ws->pairA.ptr, ws->pairB.ptr, ws->cStart.ptr,
		                                                          ws->cCount.ptr, ws->contacts.ptr, ws->material.ptr, ws->vel.ptr, ws->tx.ptr,
		                                                          ws->data.ptr, ws->pose.ptr, pp, ws->recs.ptr);
	float elapsed = 0.0f;
	auto sweep = [&](float minPen) {
		for(size_t p = 0; p < batch.partitionEnds.size(); p++)
		{
			const uint32_t b = p == 0 ? 0u : batch.partitionEnds[p - 1], e = batch.partitionEnds[p];
			if(e > b)
				tgs::solvePartitionKernel<<<divUp(e - b, 128), 128, 0, s>>>(ws->recs.ptr, b, e, ws->vel.ptr, nbDyn, minPen, elapsed);
		}
	};
	for(uint32_t it = 0; it < nbPos; it++)
	{
		if(nbConstraints) sweep(-FLT_MAX);
		tgs::integrateKernel<<<divUp(nbDyn, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, nbDyn, stepDt);
		elapsed += stepDt;
	}
	for(uint32_t it = 0; it < nbVel; it++)
		if(nbConstraints) sweep(0.0f);
	tgs::finalizeKernel<<<divUp(nbDyn, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, ws->pose.ptr, nbDyn, ws->outVel.ptr, ws->outPose.ptr);
	if(cudaGetLastError() != cudaSuccess) return GBPX_ERR_CUDA;
	if(cudaMemcpyAsync(outVel, ws->outVel.ptr, size_t(nbDyn) * 24, cudaMemcpyDeviceToHost, s) != cudaSuccess) return GBPX_ERR_CUDA;
	if(cudaMemcpyAsync(outPose, ws->outPose.ptr, size_t(nbDyn) * 28, cudaMemcpyDeviceToHost, s) != cudaSuccess) return GBPX_ERR_CUDA;
	if(cudaStreamSynchronize(s) != cudaSuccess) return GBPX_ERR_CUDA;
	for(size_t h = 0; h < batch.headerStart.size(); h++)
	{
		outHeaderStart[h] = batch.headerStart[h];
		outHeaderStride[h] = batch.headerStride[h];
	}
	for(uint32_t i = 0; i < nbConstraints; i++) outOrder[i] = batch.order[i];
	*outNbHeaders = uint32_t(batch.headerStart.size());
	return GBPX_OK;
}
