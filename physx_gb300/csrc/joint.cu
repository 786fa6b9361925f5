// Joints on the GB300: PxCreateJointConstraintsTGS and the joint half of
// PxSolveConstraintsTGS (physx/source/immediatemode/src/NpImmediateMode.cpp:1480,1630).
//
// Prep runs a thread per joint (sort, orthogonalise and build its rows, one
// JointRecord each); the solve runs a thread per joint for every partition of
// PxBatchConstraintsTGS (the joints of a partition touch disjoint dynamic
// bodies), then integrates; write-back is a thread per joint.  The device
// functions are in joint.cuh.
#include "common.cuh"
#include "joint.cuh"
#include "batching.h"
#include <vector>

namespace gbpx
{
namespace joint
{
// Prep of the joints in solve order: joint k = ordered[k] joins bodyA/bodyB,
// rows[rowStart .. +rowCount] (copied into scratch, the prep rewrites them).
__global__ void prepFrameKernel(const uint32_t* __restrict__ ordered, uint32_t n, const uint32_t* __restrict__ jointA,
                                const uint32_t* __restrict__ jointB, const uint32_t* __restrict__ rowStart, const uint32_t* __restrict__ rowCount,
                                const Row1D* __restrict__ rows, const float* __restrict__ params, const uint8_t* __restrict__ block,
                                const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx, const BodyData* __restrict__ data,
                                const Tr* __restrict__ pose, PrepTimes pt, JointRecord* __restrict__ recs)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const uint32_t ji = ordered[k];
	const uint32_t a = jointA[ji], b = jointB[ji];
	const int nr = int(rowCount[ji] < MAX_ROWS ? rowCount[ji] : MAX_ROWS);
	Row1D local[MAX_ROWS];
	for(int i = 0; i < nr; i++) local[i] = rows[rowStart[ji] + i];
	JointRecord& rec = recs[ji];
	rec.bodyA = a;
	rec.bodyB = b;
	prepJoint(local, nr, params + PARAM_FLOATS * size_t(ji), block[k] != 0, vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a].p, pose[b].p, pt,
	          rec);
}

// One partition of joints [begin, end) in solve order, bodies updated in place.
__global__ void solvePartitionKernel(const uint32_t* __restrict__ ordered, JointRecord* __restrict__ recs, uint32_t begin, uint32_t end,
                                     BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx, float elapsed, int conclude)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	JointRecord& j = recs[ordered[k]];
	if(j.count)
	{
		BodyVel b0 = vel[j.bodyA], b1 = vel[j.bodyB];
		solveJoint(j, b0, b1, tx[j.bodyA], tx[j.bodyB], elapsed);
		vel[j.bodyA] = b0;
		vel[j.bodyB] = b1;
	}
	if(conclude) concludeJoint(j);
}

__global__ void writeBackKernel(const JointRecord* __restrict__ recs, uint32_t n, float* __restrict__ force, uint32_t* __restrict__ broken)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	writeBackJoint(recs[k], force + 6 * size_t(k), broken + k);
}

__global__ void integrateKernel(BodyVel* __restrict__ vel, BodyTx* __restrict__ tx, uint32_t n, float dt)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) integrateStep(vel[i], tx[i], dt);
}

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

__global__ void finalizeKernel(const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx, const Tr* __restrict__ pose, uint32_t nbDyn,
                               float* __restrict__ outVel, float* __restrict__ outPose)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nbDyn) return;
	Tr p = pose[i];
	V3 w;
	finalizeBody(vel[i], tx[i], p, w);
	float* v = outVel + 6 * size_t(i);
	v[0] = vel[i].lin.x; v[1] = vel[i].lin.y; v[2] = vel[i].lin.z;
	v[3] = w.x; v[4] = w.y; v[5] = w.z;
	float* o = outPose + 7 * size_t(i);
	o[0] = p.q.x; o[1] = p.q.y; o[2] = p.q.z; o[3] = p.q.w;
	o[4] = p.p.x; o[5] = p.p.y; o[6] = p.p.z;
}

// ---- solver bodies in the reference's layouts (PxTGSSolverBodyVel 16 floats,
// PxTGSSolverBodyTxInertia 16, PxTGSSolverBodyData 12)
__device__ __forceinline__ BodyVel loadVelRef(const float* v)
{
	BodyVel o;
	o.lin = v3(v[0], v[1], v[2]);
	o.ang = v3(v[4], v[5], v[6]);
	o.dAng = v3(v[8], v[9], v[10]);
	o.maxAngVel = v[11];
	o.dLin = v3(v[12], v[13], v[14]);
	o.kinematic = reinterpret_cast<const uint8_t*>(v)[62] ? 1 : 0;
	return o;
}
__device__ __forceinline__ BodyTx loadTxRef(const float* t)
{
	BodyTx o;
	o.dq.x = t[0]; o.dq.y = t[1]; o.dq.z = t[2]; o.dq.w = t[3];
	o.p = v3(t[4], t[5], t[6]);
	o.sqrtInvInertia.c0 = v3(t[7], t[8], t[9]);
	o.sqrtInvInertia.c1 = v3(t[10], t[11], t[12]);
	o.sqrtInvInertia.c2 = v3(t[13], t[14], t[15]);
	return o;
}
__device__ __forceinline__ BodyData loadDataRef(const float* d)
{
	BodyData o;
	o.origLin = v3(d[0], d[1], d[2]);
	o.maxContactImpulse = d[3];
	o.origAng = v3(d[4], d[5], d[6]);
	o.penBiasClamp = d[7];
	o.invMass = d[8];
	return o;
}

// PxCreateJointConstraintsTGS, one descriptor per thread on copies of its two
// bodies' records (reference layouts) and frames (PxTransform).
__global__ void prepDescKernel(uint32_t n, const float* __restrict__ vel0, const float* __restrict__ vel1, const float* __restrict__ tx0,
                               const float* __restrict__ tx1, const float* __restrict__ data0, const float* __restrict__ data1,
                               const float* __restrict__ frame0, const float* __restrict__ frame1, const uint32_t* __restrict__ rowStart,
                               const uint32_t* __restrict__ rowCount, const Row1D* __restrict__ rows, const float* __restrict__ params,
                               const uint8_t* __restrict__ block, PrepTimes pt, JointRecord* __restrict__ recs)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const int nr = int(rowCount[k] < MAX_ROWS ? rowCount[k] : MAX_ROWS);
	Row1D local[MAX_ROWS];
	for(int i = 0; i < nr; i++) local[i] = rows[rowStart[k] + i];
	const float* f0 = frame0 + 7 * size_t(k);
	const float* f1 = frame1 + 7 * size_t(k);
	JointRecord& rec = recs[k];
	rec.bodyA = rec.bodyB = 0;
	prepJoint(local, nr, params + PARAM_FLOATS * size_t(k), block[k] != 0, loadVelRef(vel0 + 16 * size_t(k)), loadVelRef(vel1 + 16 * size_t(k)),
	          loadTxRef(tx0 + 16 * size_t(k)), loadTxRef(tx1 + 16 * size_t(k)), loadDataRef(data0 + 12 * size_t(k)), loadDataRef(data1 + 12 * size_t(k)),
	          v3(f0[4], f0[5], f0[6]), v3(f1[4], f1[5], f1[6]), pt, rec);
}
} // namespace joint

namespace
{
struct JointWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<tgs::RigidBody> rigid;
	DevBuf<float> statics, params, outVel, outPose, force, vel0, vel1, tx0, tx1, data0, data1, frame0, frame1;
	DevBuf<uint32_t> jointA, jointB, rowStart, rowCount, ordered, broken;
	DevBuf<uint8_t> block;
	DevBuf<joint::Row1D> rows;
	DevBuf<tgs::BodyVel> vel;
	DevBuf<tgs::BodyTx> tx;
	DevBuf<tgs::BodyData> data;
	DevBuf<Tr> pose;
	DevBuf<joint::JointRecord> recs;
	int init() { GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); return GBPX_OK; }
};
JointWorkspace* jointWorkspace()
{
	static JointWorkspace* ws = nullptr;
	if(!ws)
	{
		ws = new JointWorkspace;
		if(ws->init()) { delete ws; ws = nullptr; }
	}
	return ws;
}

// the reference's timing arguments of PxCreateJointConstraintsTGS as the
// immediate-mode snippet passes them: (stepDt, dt, 1/stepDt, 1/dt, lengthScale)
joint::PrepTimes prepTimes(float stepDt, float simDt, float recipStepDt, float recipSimDt, float lengthScale)
{
	joint::PrepTimes pt;
	pt.stepDt = stepDt;
	pt.simDt = simDt;
	pt.recipStepDt = recipStepDt;
	pt.recipSimDt = recipSimDt;
	pt.lengthScale = lengthScale;
	pt.biasCoefficient = 2.0f * sqrtf(stepDt / simDt);   // NpImmediateMode.cpp:1485
	return pt;
}

bool paramsSupported(const float* params, uint32_t n)
{
	for(uint32_t k = 0; k < n; k++)
		if(uint32_t(params[joint::PARAM_FLOATS * size_t(k) + 16]) & joint::PARAM_IMPROVED_SLERP) return false;
	return true;
}
} // namespace
} // namespace gbpx

using namespace gbpx;

GBPX_API uint32_t gbpx_joint_record_bytes(void) { return uint32_t(sizeof(joint::JointRecord)); }

// One TGS frame of joints (same arguments as the reference harness frame):
// construct bodies, PxBatchConstraintsTGS over the joints (or, batchJoints = 0,
// one header of stride 1 per joint in input order), PxCreateJointConstraintsTGS
// per header, nbPos position + nbVel velocity iterations, write-back,
// PxIntegrateSolverBodiesTGS.  rigid = PxRigidBodyData[nbDyn],
// staticPose = PxTransform[nbStatic]; joint j joins jointA[j], jointB[j]
// (statics indexed from nbDyn) with rows[rowStart[j] .. +rowCount[j]]
// (Px1DConstraint, <= 12) and 20 parameter floats (params + 20 j: invMassScales,
// cA2w, cB2w, body0WorldOffset, linBreakForce, angBreakForce,
// minResponseThreshold, flags 1 disablePreprocessing | 4 driveLimitsAreForces;
// 2 improvedSlerp is refused).  Outputs: linear and world angular velocity (6)
// and pose (7) per dynamic body, headers (start, stride, DY_SC_TYPE_RB_1D = 2 /
// DY_SC_TYPE_BLOCK_1D = 8), joint order, per joint the write-back impulse
// (linear, angular) and broken flag; the header count in *outNbHeaders.
GBPX_API int gbpx_joint_frame(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* jointA,
                              const uint32_t* jointB, uint32_t nbJoints, const uint32_t* rowStart, const uint32_t* rowCount, const void* rows,
                              const float* params, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel, uint32_t batchJoints, float* outVel,
                              float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outHeaderType, uint32_t* outOrder,
                              float* outForce, uint32_t* outBroken, uint32_t* outNbHeaders)
{
	gbpx::Zone zone("gbpx::jointFrame");
	if(!nbDyn || !rigid || !gravity || !outVel || !outPose || !outNbHeaders || !(dt > 0.0f) || !nbPos || !nbVel) return GBPX_ERR_INVALID;
	if(nbStatic && !staticPose) return GBPX_ERR_INVALID;
	if(nbJoints && (!jointA || !jointB || !rowStart || !rowCount || !rows || !params || !outHeaderStart || !outHeaderStride || !outHeaderType ||
	                !outOrder || !outForce || !outBroken))
		return GBPX_ERR_INVALID;
	uint32_t nbRows = 0;
	for(uint32_t j = 0; j < nbJoints; j++)
	{
		if(jointA[j] >= nbDyn + nbStatic || jointB[j] >= nbDyn + nbStatic || (jointA[j] >= nbDyn && jointB[j] >= nbDyn) ||
		   rowCount[j] > uint32_t(joint::MAX_ROWS))
			return GBPX_ERR_INVALID;
		nbRows = std::max(nbRows, rowStart[j] + rowCount[j]);
	}
	if(nbJoints && !paramsSupported(params, nbJoints)) return GBPX_ERR_INVALID;
	JointWorkspace* ws = jointWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	batching::Result batch;
	if(nbJoints)
	{
		if(batchJoints) batching::partition(jointA, jointB, nbJoints, nbDyn, batch);
		else
		{
			// the snippet's unbatched path: a header of stride 1 per joint, one partition each
			for(uint32_t j = 0; j < nbJoints; j++)
			{
				batch.order.push_back(j);
				batch.headerStart.push_back(j);
				batch.headerStride.push_back(1);
				batch.partitionEnds.push_back(j + 1);
			}
		}
	}
	const uint32_t nbHeaders = uint32_t(batch.headerStart.size());
	// a header of stride 4 whose joints all have rows takes the 4-wide path (NpImmediateMode.cpp:1495-1517)
	std::vector<uint8_t> block(nbJoints ? nbJoints : 1, 0);
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		const uint32_t s0 = batch.headerStart[h], st = batch.headerStride[h];
		bool b = st == 4;
		for(uint32_t l = 0; l < st && b; l++) b = rowCount[batch.order[s0 + l]] > 0;
		outHeaderStart[h] = s0;
		outHeaderStride[h] = st;
		outHeaderType[h] = b ? joint::TYPE_BLOCK_1D : joint::TYPE_RB_1D;
		for(uint32_t l = 0; l < st; l++) block[s0 + l] = b ? 1 : 0;
	}
	const uint32_t nbTotal = nbDyn + nbStatic;
	const uint32_t nj = nbJoints ? nbJoints : 1;
	if(ws->rigid.reserve(nbDyn) || ws->statics.reserve(7 * size_t(nbStatic) + 1) || ws->jointA.reserve(nj) || ws->jointB.reserve(nj) ||
	   ws->rowStart.reserve(nj) || ws->rowCount.reserve(nj) || ws->ordered.reserve(nj) || ws->block.reserve(nj) || ws->rows.reserve(nbRows + 1) ||
	   ws->params.reserve(joint::PARAM_FLOATS * size_t(nj)) || ws->vel.reserve(nbTotal) || ws->tx.reserve(nbTotal) || ws->data.reserve(nbTotal) ||
	   ws->pose.reserve(nbTotal) || ws->recs.reserve(nj) || ws->outVel.reserve(6 * size_t(nbDyn)) || ws->outPose.reserve(7 * size_t(nbDyn)) ||
	   ws->force.reserve(6 * size_t(nj)) || ws->broken.reserve(nj))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rigid.ptr, rigid, size_t(nbDyn) * sizeof(tgs::RigidBody), cudaMemcpyHostToDevice, s));
	if(nbStatic) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->statics.ptr, staticPose, size_t(nbStatic) * 28, cudaMemcpyHostToDevice, s));
	if(nbJoints)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->jointA.ptr, jointA, size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->jointB.ptr, jointB, size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rowStart.ptr, rowStart, size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rowCount.ptr, rowCount, size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->ordered.ptr, batch.order.data(), size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->block.ptr, block.data(), size_t(nbJoints), cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->params.ptr, params, size_t(nbJoints) * joint::PARAM_FLOATS * 4, cudaMemcpyHostToDevice, s));
		if(nbRows) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rows.ptr, rows, size_t(nbRows) * sizeof(joint::Row1D), cudaMemcpyHostToDevice, s));
	}
	joint::constructBodiesKernel<<<divUp(nbTotal, 128), 128, 0, s>>>(ws->rigid.ptr, nbDyn, ws->statics.ptr, nbStatic, gravity[0], gravity[1],
	                                                                 gravity[2], dt, ws->vel.ptr, ws->tx.ptr, ws->data.ptr, ws->pose.ptr);
	const float invDt = 1.0f / dt;
	const float stepDt = dt / float(nbPos);
	const float invStepDt = invDt * float(nbPos);
	if(nbJoints)
		joint::prepFrameKernel<<<divUp(nbJoints, 64), 64, 0, s>>>(ws->ordered.ptr, nbJoints, ws->jointA.ptr, ws->jointB.ptr, ws->rowStart.ptr,
		                                                          ws->rowCount.ptr, ws->rows.ptr, ws->params.ptr, ws->block.ptr, ws->vel.ptr,
		                                                          ws->tx.ptr, ws->data.ptr, ws->pose.ptr,
		                                                          prepTimes(stepDt, dt, invStepDt, invDt, 1.0f), ws->recs.ptr);
	float elapsed = 0.0f;
	auto sweep = [&](bool conclude) {
		for(size_t p = 0; p < batch.partitionEnds.size(); p++)
		{
			const uint32_t b = p == 0 ? 0u : batch.partitionEnds[p - 1], e = batch.partitionEnds[p];
			if(e > b)
				joint::solvePartitionKernel<<<divUp(e - b, 64), 64, 0, s>>>(ws->ordered.ptr, ws->recs.ptr, b, e, ws->vel.ptr, ws->tx.ptr, elapsed,
				                                                            conclude ? 1 : 0);
		}
	};
	for(uint32_t it = 0; it < nbPos; it++)
	{
		if(nbJoints) sweep(it + 1 == nbPos);
		joint::integrateKernel<<<divUp(nbDyn, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, nbDyn, stepDt);
		elapsed += stepDt;
	}
	for(uint32_t it = 0; it < nbVel; it++)
		if(nbJoints) sweep(false);
	if(nbJoints) joint::writeBackKernel<<<divUp(nbJoints, 128), 128, 0, s>>>(ws->recs.ptr, nbJoints, ws->force.ptr, ws->broken.ptr);
	joint::finalizeKernel<<<divUp(nbDyn, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, ws->pose.ptr, nbDyn, ws->outVel.ptr, ws->outPose.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outVel, ws->outVel.ptr, size_t(nbDyn) * 24, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outPose, ws->outPose.ptr, size_t(nbDyn) * 28, cudaMemcpyDeviceToHost, s));
	if(nbJoints)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(outForce, ws->force.ptr, size_t(nbJoints) * 24, cudaMemcpyDeviceToHost, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(outBroken, ws->broken.ptr, size_t(nbJoints) * 4, cudaMemcpyDeviceToHost, s));
	}
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	for(uint32_t i = 0; i < nbJoints; i++) outOrder[i] = batch.order[i];
	*outNbHeaders = nbHeaders;
	return GBPX_OK;
}

// PxCreateJointConstraintsTGS, one joint descriptor per entry: the two bodies'
// records (vel0/vel1: PxTGSSolverBodyVel 64 B, txI0/txI1: 64 B, data0/data1:
// PxTGSSolverBodyData 48 B), the body frames (PxTransform), rows[rowStart[k] ..
// +rowCount[k]] (Px1DConstraint, <= 12) and 20 parameter floats per joint (as
// gbpx_joint_frame).  block[k] = 1 for the lanes of a header of stride 4 whose
// joints all have rows (the reference's 4-wide path).  Times as the snippet
// passes them: stepDt, simDt (= total dt), their reciprocals, lengthScale.
// Writes one record of gbpx_joint_record_bytes() per joint to outRecords.
GBPX_API int gbpx_create_joint_constraints_tgs(uint32_t n, const void* vel0, const void* vel1, const void* txI0, const void* txI1, const void* data0,
                                               const void* data1, const float* frame0, const float* frame1, const uint32_t* rowStart,
                                               const uint32_t* rowCount, const void* rows, uint32_t nbRows, const float* params,
                                               const uint8_t* block, float stepDt, float simDt, float recipStepDt, float recipSimDt,
                                               float lengthScale, void* outRecords)
{
	gbpx::Zone zone("gbpx::createJointConstraintsTGS");
	if(!n) return GBPX_OK;
	if(!vel0 || !vel1 || !txI0 || !txI1 || !data0 || !data1 || !frame0 || !frame1 || !rowStart || !rowCount || !params || !block || !outRecords ||
	   (nbRows && !rows) || !(stepDt > 0.0f) || !(simDt > 0.0f))
		return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < n; k++)
		if(rowCount[k] > uint32_t(joint::MAX_ROWS) || rowStart[k] + rowCount[k] > nbRows) return GBPX_ERR_INVALID;
	if(!paramsSupported(params, n)) return GBPX_ERR_INVALID;
	JointWorkspace* ws = jointWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	const size_t m = n;
	if(ws->vel0.reserve(16 * m) || ws->vel1.reserve(16 * m) || ws->tx0.reserve(16 * m) || ws->tx1.reserve(16 * m) || ws->data0.reserve(12 * m) ||
	   ws->data1.reserve(12 * m) || ws->frame0.reserve(7 * m) || ws->frame1.reserve(7 * m) || ws->rowStart.reserve(m) || ws->rowCount.reserve(m) ||
	   ws->rows.reserve(size_t(nbRows) + 1) || ws->params.reserve(joint::PARAM_FLOATS * m) || ws->block.reserve(m) || ws->recs.reserve(m))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->vel0.ptr, vel0, m * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->vel1.ptr, vel1, m * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->tx0.ptr, txI0, m * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->tx1.ptr, txI1, m * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->data0.ptr, data0, m * 48, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->data1.ptr, data1, m * 48, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->frame0.ptr, frame0, m * 28, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->frame1.ptr, frame1, m * 28, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rowStart.ptr, rowStart, m * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rowCount.ptr, rowCount, m * 4, cudaMemcpyHostToDevice, s));
	if(nbRows) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->rows.ptr, rows, size_t(nbRows) * sizeof(joint::Row1D), cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->params.ptr, params, m * joint::PARAM_FLOATS * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->block.ptr, block, m, cudaMemcpyHostToDevice, s));
	joint::prepDescKernel<<<divUp(n, 64), 64, 0, s>>>(n, ws->vel0.ptr, ws->vel1.ptr, ws->tx0.ptr, ws->tx1.ptr, ws->data0.ptr, ws->data1.ptr,
	                                                  ws->frame0.ptr, ws->frame1.ptr, ws->rowStart.ptr, ws->rowCount.ptr, ws->rows.ptr, ws->params.ptr,
	                                                  ws->block.ptr, prepTimes(stepDt, simDt, recipStepDt, recipSimDt, lengthScale), ws->recs.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outRecords, ws->recs.ptr, m * sizeof(joint::JointRecord), cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}
