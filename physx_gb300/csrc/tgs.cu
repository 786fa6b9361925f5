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
#include "joint.cuh"
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

// Lane flags of a constraint (one byte each): LANE_BLOCK = one lane of a
// header of stride 4 (the 4-wide block path), LANE_BLOCK_DYNAMIC = that header
// has a dynamic body B, LANE_KEEP_B = body B's data index is 0.
constexpr uint8_t LANE_BLOCK = 1, LANE_BLOCK_DYNAMIC = 2, LANE_KEEP_B = 4;

__device__ __forceinline__ void prepByFlags(uint8_t flags, const Contact* cs, int cnt, int a, int b, const BodyVel& va, const BodyVel& vb,
                                            const BodyTx& ta, const BodyTx& tb, const BodyData& da, const BodyData& db, const Tr& f0, const Tr& f1,
                                            const PrepParams& pp, ConstraintRecord& rec, const FrictionState* prev = nullptr,
                                            FrictionState* written = nullptr)
{
	if(flags & LANE_BLOCK)
		prepConstraintBlock(cs, cnt, a, b, va, vb, ta, tb, da, db, f0, f1, pp, (flags & LANE_BLOCK_DYNAMIC) != 0, (flags & LANE_KEEP_B) != 0, rec,
		                    prev, written);
	else
		prepConstraint(cs, cnt, a, b, va, vb, ta, tb, da, db, f0, f1, pp, rec, prev, written);
}

// Rows for constraint k of the ordered list (ordered[k] = caller's constraint index).
__global__ void prepKernel(const uint32_t* __restrict__ ordered, uint32_t n, const uint32_t* __restrict__ pairA, const uint32_t* __restrict__ pairB,
                           const uint32_t* __restrict__ cStart, const uint32_t* __restrict__ cCount, const float* __restrict__ contacts,
                           const float* __restrict__ material, const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx,
                           const BodyData* __restrict__ data, const Tr* __restrict__ pose, const uint8_t* __restrict__ laneFlags, PrepParams pp,
                           ConstraintRecord* __restrict__ recs)
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
	prepByFlags(laneFlags[k], cs, int(cnt), int(a), int(b), vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a], pose[b], pp, recs[k]);
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
	solveRecord(r, b0, b1, dynB, minPen, elapsed);
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

// One solver body in the reference's byte layouts (PxTGSSolverBodyVel 64 B,
// PxTGSSolverBodyTxInertia 64 B, PxTGSSolverBodyData 48 B).
__device__ __forceinline__ void exportBodiesKernelBody(const BodyVel& vel, const BodyTx& tx, const BodyData& data, float* v, float* t, float* d)
{
	v[0] = vel.lin.x; v[1] = vel.lin.y; v[2] = vel.lin.z; v[3] = 0.0f;
	v[4] = vel.ang.x; v[5] = vel.ang.y; v[6] = vel.ang.z; v[7] = 0.0f;
	v[8] = vel.dAng.x; v[9] = vel.dAng.y; v[10] = vel.dAng.z; v[11] = vel.maxAngVel;
	v[12] = vel.dLin.x; v[13] = vel.dLin.y; v[14] = vel.dLin.z;
	uint32_t lockAndKin = vel.kinematic ? (1u << 16) : 0u;   // lockFlags (u16) = 0, isKinematic (u8), pad (u8)
	memcpy(&v[15], &lockAndKin, 4);
	t[0] = tx.dq.x; t[1] = tx.dq.y; t[2] = tx.dq.z; t[3] = tx.dq.w;
	t[4] = tx.p.x; t[5] = tx.p.y; t[6] = tx.p.z;
	const M33& m = tx.sqrtInvInertia;
	t[7] = m.c0.x; t[8] = m.c0.y; t[9] = m.c0.z; t[10] = m.c1.x; t[11] = m.c1.y; t[12] = m.c1.z; t[13] = m.c2.x; t[14] = m.c2.y; t[15] = m.c2.z;
	d[0] = data.origLin.x; d[1] = data.origLin.y; d[2] = data.origLin.z; d[3] = data.maxContactImpulse;
	d[4] = data.origAng.x; d[5] = data.origAng.y; d[6] = data.origAng.z; d[7] = data.penBiasClamp;
	d[8] = data.invMass;
	const uint32_t invalidNode = 0x7fffffffu;   // nodeIndex: immediate mode passes PX_INVALID_NODE
	memcpy(&d[9], &invalidNode, 4);
	d[10] = FLT_MAX;                            // reportThreshold
	d[11] = 0.0f;
}

__global__ void exportBodiesKernel(const BodyVel* __restrict__ vel, const BodyTx* __restrict__ tx, const BodyData* __restrict__ data, uint32_t n,
                                   float* __restrict__ outVel, float* __restrict__ outTx, float* __restrict__ outData)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	exportBodiesKernelBody(vel[i], tx[i], data[i], outVel + 16 * size_t(i), outTx + 16 * size_t(i), outData + 12 * size_t(i));
}
// ---- records in the reference's solver-body layouts, used in place
// (PxTGSSolverBodyVel 16 floats, PxTGSSolverBodyTxInertia 16, PxTGSSolverBodyData 12)
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

// PxConstructStaticSolverBodyTGS for n poses (zero velocity, zero inverse inertia, flagged kinematic).
__global__ void staticBodiesKernel(const float* __restrict__ poses, uint32_t n, float* __restrict__ outVel, float* __restrict__ outTx,
                                   float* __restrict__ outData)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const float* s = poses + 7 * size_t(i);
	Tr p;
	p.q.x = s[0]; p.q.y = s[1]; p.q.z = s[2]; p.q.w = s[3];
	p.p = v3(s[4], s[5], s[6]);
	BodyVel v;
	BodyTx t;
	BodyData d;
	constructStaticBody(p, v, t, d);
	exportBodiesKernelBody(v, t, d, outVel + 16 * size_t(i), outTx + 16 * size_t(i), outData + 12 * size_t(i));
}

// PxCreateContactConstraintsTGS for one descriptor per thread: both bodies'
// records, frames and the descriptor's PxContactPoints (80 bytes each:
// normal, separation, point, ..., staticFriction at 44, dynamicFriction at 56,
// restitution at 60).  Rows go to outRows[k] (bodyA/bodyB set by the solve).
__global__ void prepDescKernel(uint32_t n, const float* __restrict__ vel0, const float* __restrict__ vel1, const float* __restrict__ tx0,
                               const float* __restrict__ tx1, const float* __restrict__ data0, const float* __restrict__ data1,
                               const float* __restrict__ frame0, const float* __restrict__ frame1, const uint32_t* __restrict__ cStart,
                               const uint32_t* __restrict__ cCount, const float* __restrict__ points, const uint8_t* __restrict__ laneFlags,
                               const FrictionState* __restrict__ frictionIn, FrictionState* __restrict__ frictionOut, PrepParams pp,
                               ConstraintRecord* __restrict__ recs, uint32_t* __restrict__ recBytes)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	Contact cs[MAX_CONTACTS];
	const uint32_t cnt = cCount[k] < MAX_CONTACTS ? cCount[k] : MAX_CONTACTS;
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
	const BodyVel va = loadVelRef(vel0 + 16 * size_t(k)), vb = loadVelRef(vel1 + 16 * size_t(k));
	const BodyTx ta = loadTxRef(tx0 + 16 * size_t(k)), tb = loadTxRef(tx1 + 16 * size_t(k));
	const BodyData da = loadDataRef(data0 + 12 * size_t(k)), db = loadDataRef(data1 + 12 * size_t(k));
	Tr f0, f1;
	const float* a = frame0 + 7 * size_t(k);
	const float* b = frame1 + 7 * size_t(k);
	f0.q.x = a[0]; f0.q.y = a[1]; f0.q.z = a[2]; f0.q.w = a[3]; f0.p = v3(a[4], a[5], a[6]);
	f1.q.x = b[0]; f1.q.y = b[1]; f1.q.z = b[2]; f1.q.w = b[3]; f1.p = v3(b[4], b[5], b[6]);
	prepByFlags(laneFlags ? laneFlags[k] : uint8_t(0), cs, int(cnt), 0, 1, va, vb, ta, tb, da, db, f0, f1, pp, recs[k],
	            frictionIn && frictionIn[k].count ? frictionIn + k : nullptr, frictionOut ? frictionOut + k : nullptr);
	recBytes[k] = recs[k].bytes();
}

// One wave of independent constraints on solver bodies held in the
// reference's layouts: rows[k] joins bodyA[k], bodyB[k].
__global__ void solveWaveRefKernel(ConstraintRecord* __restrict__ recs, const uint32_t* __restrict__ bodyA, const uint32_t* __restrict__ bodyB,
                                   uint32_t begin, uint32_t end, float* __restrict__ vel, float minPen, float elapsed, uint32_t* __restrict__ broken)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	ConstraintRecord& r = recs[k];
	if(r.nbPatches == 0) return;
	float* va = vel + 16 * size_t(bodyA[k]);
	float* vb = vel + 16 * size_t(bodyB[k]);
	BodyVel b0 = loadVelRef(va), b1 = loadVelRef(vb);
	solveRecord(r, b0, b1, true, minPen, elapsed, broken ? broken + k : nullptr);
	va[0] = b0.lin.x; va[1] = b0.lin.y; va[2] = b0.lin.z; va[4] = b0.ang.x; va[5] = b0.ang.y; va[6] = b0.ang.z;
	vb[0] = b1.lin.x; vb[1] = b1.lin.y; vb[2] = b1.lin.z; vb[4] = b1.ang.x; vb[5] = b1.ang.y; vb[6] = b1.ang.z;
}

// One wave of joints on solver bodies in the reference's layouts: joint k
// joins bodyA[k], bodyB[k]; conclude after the last position iteration's solve.
__global__ void solveJointWaveRefKernel(joint::JointRecord* __restrict__ recs, const uint32_t* __restrict__ bodyA, const uint32_t* __restrict__ bodyB,
                                        uint32_t begin, uint32_t end, float* __restrict__ vel, const float* __restrict__ tx, float elapsed, int conclude)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	joint::JointRecord& j = recs[k];
	if(j.count)
	{
		float* va = vel + 16 * size_t(bodyA[k]);
		float* vb = vel + 16 * size_t(bodyB[k]);
		BodyVel b0 = loadVelRef(va), b1 = loadVelRef(vb);
		joint::solveJoint(j, b0, b1, loadTxRef(tx + 16 * size_t(bodyA[k])), loadTxRef(tx + 16 * size_t(bodyB[k])), elapsed);
		va[0] = b0.lin.x; va[1] = b0.lin.y; va[2] = b0.lin.z; va[4] = b0.ang.x; va[5] = b0.ang.y; va[6] = b0.ang.z;
		vb[0] = b1.lin.x; vb[1] = b1.lin.y; vb[2] = b1.lin.z; vb[4] = b1.ang.x; vb[5] = b1.ang.y; vb[6] = b1.ang.z;
	}
	if(conclude) joint::concludeJoint(j);
}

__global__ void jointWriteBackKernel(const joint::JointRecord* __restrict__ recs, uint32_t n, float* __restrict__ force, uint32_t* __restrict__ broken)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k < n) joint::writeBackJoint(recs[k], force + 6 * size_t(k), broken + k);
}

// integrateCoreStep on records in the reference's layouts.
__global__ void integrateRefKernel(float* __restrict__ vel, float* __restrict__ tx, uint32_t n, float dt)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	float* v = vel + 16 * size_t(i);
	float* t = tx + 16 * size_t(i);
	BodyVel bv = loadVelRef(v);
	BodyTx bt = loadTxRef(t);
	integrateStep(bv, bt, dt);
	v[8] = bv.dAng.x; v[9] = bv.dAng.y; v[10] = bv.dAng.z;
	v[12] = bv.dLin.x; v[13] = bv.dLin.y; v[14] = bv.dLin.z;
	t[0] = bt.dq.x; t[1] = bt.dq.y; t[2] = bt.dq.z; t[3] = bt.dq.w;
	t[4] = bt.p.x; t[5] = bt.p.y; t[6] = bt.p.z;
}

// PxIntegrateSolverBodiesTGS: world angular velocity into the velocity record, new poses.
__global__ void finalizeRefKernel(float* __restrict__ vel, const float* __restrict__ tx, float* __restrict__ poses, uint32_t n)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	float* v = vel + 16 * size_t(i);
	float* q = poses + 7 * size_t(i);
	Tr p;
	p.q.x = q[0]; p.q.y = q[1]; p.q.z = q[2]; p.q.w = q[3];
	p.p = v3(q[4], q[5], q[6]);
	V3 w;
	finalizeBody(loadVelRef(v), loadTxRef(tx + 16 * size_t(i)), p, w);
	v[4] = w.x; v[5] = w.y; v[6] = w.z;
	q[0] = p.q.x; q[1] = p.q.y; q[2] = p.q.z; q[3] = p.q.w;
	q[4] = p.p.x; q[5] = p.p.y; q[6] = p.p.z;
}
} // namespace tgs

struct TgsWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<tgs::RigidBody> rigid;
	DevBuf<float> statics, contacts, material, outVel, outPose, outTx, outData;
	DevBuf<uint32_t> pairA, pairB, cStart, cCount, ordered;
	DevBuf<uint8_t> laneFlags;
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

// PxBatchConstraintsTGS over a list mixing constraint types: kind[i] is
// constraint i's PxSolverConstraintDesc type (0 contact, 1 joint); a header
// only joins consecutive constraints of one type.  Otherwise as
// gbpx_batch_constraints_tgs.
GBPX_API uint32_t gbpx_batch_typed_constraints_tgs(const uint32_t* bodyA, const uint32_t* bodyB, const uint8_t* kind, uint32_t nbConstraints,
                                                   uint32_t nbDyn, uint32_t nbStatic, uint32_t* outHeaderStart, uint32_t* outHeaderStride,
                                                   uint32_t* outOrder)
{
	(void)nbStatic;
	if(!nbConstraints) return 0;
	if(!bodyA || !bodyB || !kind || !outHeaderStart || !outHeaderStride || !outOrder) return 0;
	batching::Result r;
	batching::partition(bodyA, bodyB, nbConstraints, nbDyn, r, kind);
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
	gbpx::Zone zone("gbpx::constructSolverBodiesTGS");
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
	gbpx::Zone zone("gbpx::tgsSolve");
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
	// headers of stride 4 with at most 64 contacts take the 4-wide block path
	// (PxCreateContactConstraintsTGS, NpImmediateMode.cpp:1422-1444)
	std::vector<uint8_t> laneFlags(nbConstraints ? nbConstraints : 1, 0);
	for(size_t h = 0; h < batch.headerStart.size(); h++)
	{
		if(batch.headerStride[h] != 4) continue;
		const uint32_t s0 = batch.headerStart[h];
		uint32_t total = 0;
		bool dyn = false;
		for(uint32_t l = 0; l < 4; l++)
		{
			const uint32_t ci = batch.order[s0 + l];
			total += contactCount[ci];
			dyn = dyn || pairB[ci] < nbDyn;
		}
		if(total > 64) continue;
		for(uint32_t l = 0; l < 4; l++)
			laneFlags[s0 + l] = uint8_t(tgs::LANE_BLOCK | (dyn ? tgs::LANE_BLOCK_DYNAMIC : 0) | (pairB[batch.order[s0 + l]] == 0 ? tgs::LANE_KEEP_B : 0));
	}
	uint32_t nbContacts = 0;
	for(uint32_t i = 0; i < nbConstraints; i++) nbContacts = std::max(nbContacts, contactStart[i] + contactCount[i]);
	const uint32_t nbTotal = nbDyn + nbStatic;
	const uint32_t nc = nbConstraints ? nbConstraints : 1;
	if(ws->rigid.reserve(nbDyn) || ws->statics.reserve(7 * size_t(nbStatic) + 1) || ws->pairA.reserve(nc) || ws->pairB.reserve(nc) ||
	   ws->cStart.reserve(nc) || ws->cCount.reserve(nc) || ws->ordered.reserve(nc) || ws->contacts.reserve(8 * size_t(nbContacts) + 8) ||
	   ws->material.reserve(3 * size_t(nc)) || ws->vel.reserve(nbTotal) || ws->tx.reserve(nbTotal) || ws->data.reserve(nbTotal) ||
	   ws->pose.reserve(nbTotal) || ws->recs.reserve(nc) || ws->outVel.reserve(6 * size_t(nbDyn)) || ws->outPose.reserve(7 * size_t(nbDyn)) ||
	   ws->laneFlags.reserve(nc))
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
		   cudaMemcpyAsync(ws->laneFlags.ptr, laneFlags.data(), size_t(nbConstraints), cudaMemcpyHostToDevice, s) != cudaSuccess ||
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
	pp.correlationDistance = correlationDistance;
	if(nbConstraints)
		tgs::prepKernel<<<divUp(nbConstraints, 128), 128, 0, s>>>(ws->ordered.ptr, nbConstraints, ws->pairA.ptr, ws->pairB.ptr, ws->cStart.ptr,
		                                                          ws->cCount.ptr, ws->contacts.ptr, ws->material.ptr, ws->vel.ptr, ws->tx.ptr,
		                                                          ws->data.ptr, ws->pose.ptr, ws->laneFlags.ptr, pp, ws->recs.ptr);
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

// ---------------------------------------------------------------- split-phase TGS on reference layouts
// The stages of the reference's immediate-mode TGS as separate calls, on solver
// bodies in the reference's layouts (PxTGSSolverBodyVel / TxInertia / Data),
// for callers that drive the stages themselves.

namespace gbpx
{
struct TgsStageWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<float> vel0, vel1, tx0, tx1, data0, data1, frame0, frame1, points, vel, tx, poses;
	DevBuf<uint32_t> cStart, cCount, bodyA, bodyB, recBytes, broken;
	DevBuf<uint8_t> laneFlags;
	DevBuf<tgs::FrictionState> frictionIn, frictionOut;
	DevBuf<tgs::ConstraintRecord> recs;
	DevBuf<joint::JointRecord> jointRecs;
	DevBuf<uint32_t> jointA, jointB, jointBroken;
	DevBuf<float> jointForce;
	int init() { GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); return GBPX_OK; }
};
static TgsStageWorkspace* tgsStageWorkspace()
{
	static TgsStageWorkspace* ws = nullptr;
	if(!ws)
	{
		ws = new TgsStageWorkspace;
		if(ws->init()) { delete ws; ws = nullptr; }
	}
	return ws;
}
} // namespace gbpx

// Bytes of one constraint's row block (the stride of gbpx_create_contact_constraints_tgs outputs).
GBPX_API uint32_t gbpx_constraint_row_stride(void)
{
	return uint32_t(sizeof(tgs::ConstraintRecord));
}

// PxConstructStaticSolverBodyTGS for n poses (PxTransform in, reference solver-body layouts out).
GBPX_API int gbpx_construct_static_solver_bodies_tgs(const float* poses, uint32_t n, void* outVel, void* outTxI, void* outData)
{
	gbpx::Zone zone("gbpx::constructStaticSolverBodiesTGS");
	if(!n) return GBPX_OK;
	if(!poses || !outVel || !outTxI || !outData) return GBPX_ERR_INVALID;
	TgsStageWorkspace* ws = tgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	if(ws->poses.reserve(7 * size_t(n)) || ws->vel.reserve(16 * size_t(n)) || ws->tx.reserve(16 * size_t(n)) || ws->data0.reserve(12 * size_t(n)))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->poses.ptr, poses, size_t(n) * 28, cudaMemcpyHostToDevice, s));
	tgs::staticBodiesKernel<<<divUp(n, 128), 128, 0, s>>>(ws->poses.ptr, n, ws->vel.ptr, ws->tx.ptr, ws->data0.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outVel, ws->vel.ptr, size_t(n) * 64, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outTxI, ws->tx.ptr, size_t(n) * 64, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outData, ws->data0.ptr, size_t(n) * 48, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// PxCreateContactConstraintsTGS, one contact descriptor per constraint: the two
// bodies' records (vel0/vel1: 64 B each, txI0/txI1: 64 B, data0/data1: 48 B),
// the body frames (PxTransform), and contactPoints[contactStart[k] .. +contactCount[k]]
// (PxContactPoint, 80 B, <= 4 per constraint; friction and restitution are read
// from the points).  laneFlags[k] (may be null: every constraint on the
// per-pair path): bit 0 = one of the four constraints of a header of stride 4
// that takes the reference's 4-wide block path, bit 1 = that header has a
// dynamic body B, bit 2 = the descriptor's bodyBDataIndex is 0.
// frictionIn / frictionOut (may be null): per constraint a 464-byte friction
// record (count, then <= 4 friction patches of 112 bytes), the patches it left
// last frame (frictionPtr / frictionCount) and the ones it leaves now.
// invDt = 1 / (dt / nbPositionIterations), invTotalDt = 1 / dt.
// Writes each constraint's rows to outRows + k * gbpx_constraint_row_stride()
// and their used size to outRowBytes[k].
GBPX_API int gbpx_create_contact_constraints_tgs(uint32_t n, const void* vel0, const void* vel1, const void* txI0, const void* txI1, const void* data0,
                                                 const void* data1, const float* frame0, const float* frame1, const uint32_t* contactStart,
                                                 const uint32_t* contactCount, const void* contactPoints, uint32_t nbPoints, const uint8_t* laneFlags,
                                                 const void* frictionIn, void* frictionOut, float invDt, float invTotalDt, float bounceThreshold,
                                                 float frictionOffsetThreshold, float correlationDistance, void* outRows, uint32_t* outRowBytes)
{
	gbpx::Zone zone("gbpx::createContactConstraintsTGS");
	if(!n) return GBPX_OK;
	if(!vel0 || !vel1 || !txI0 || !txI1 || !data0 || !data1 || !frame0 || !frame1 || !contactStart || !contactCount || !outRows || !outRowBytes ||
	   (nbPoints && !contactPoints) || !(invDt > 0.0f) || !(invTotalDt > 0.0f))
		return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < n; k++)
		if(contactCount[k] > tgs::MAX_CONTACTS || contactStart[k] + contactCount[k] > nbPoints) return GBPX_ERR_INVALID;
	TgsStageWorkspace* ws = tgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	const size_t m = n;
	if(ws->vel0.reserve(16 * m) || ws->vel1.reserve(16 * m) || ws->tx0.reserve(16 * m) || ws->tx1.reserve(16 * m) || ws->data0.reserve(12 * m) ||
	   ws->data1.reserve(12 * m) || ws->frame0.reserve(7 * m) || ws->frame1.reserve(7 * m) || ws->cStart.reserve(m) || ws->cCount.reserve(m) ||
	   ws->points.reserve(20 * size_t(nbPoints) + 20) || ws->recs.reserve(m) || ws->recBytes.reserve(m) || ws->laneFlags.reserve(m) ||
	   (frictionIn && ws->frictionIn.reserve(m)) || (frictionOut && ws->frictionOut.reserve(m)))
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
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->cStart.ptr, contactStart, m * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->cCount.ptr, contactCount, m * 4, cudaMemcpyHostToDevice, s));
	if(nbPoints) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->points.ptr, contactPoints, size_t(nbPoints) * 80, cudaMemcpyHostToDevice, s));
	if(laneFlags) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->laneFlags.ptr, laneFlags, m, cudaMemcpyHostToDevice, s));
	if(frictionIn) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->frictionIn.ptr, frictionIn, m * sizeof(tgs::FrictionState), cudaMemcpyHostToDevice, s));
	tgs::PrepParams pp;
	pp.invStepDt = invDt;
	pp.invTotalDt = invTotalDt;
	pp.totalDt = 1.0f / invTotalDt;
	pp.stepDt = 1.0f / invDt;
	pp.bounceThreshold = bounceThreshold;
	pp.frictionOffsetThreshold = frictionOffsetThreshold;
	pp.biasCoefficient = 2.0f * sqrtf(invTotalDt / invDt);
	pp.correlationDistance = correlationDistance;
	tgs::prepDescKernel<<<divUp(n, 128), 128, 0, s>>>(n, ws->vel0.ptr, ws->vel1.ptr, ws->tx0.ptr, ws->tx1.ptr, ws->data0.ptr, ws->data1.ptr,
	                                                  ws->frame0.ptr, ws->frame1.ptr, ws->cStart.ptr, ws->cCount.ptr, ws->points.ptr,
	                                                  laneFlags ? ws->laneFlags.ptr : nullptr, frictionIn ? ws->frictionIn.ptr : nullptr,
	                                                  frictionOut ? ws->frictionOut.ptr : nullptr, pp, ws->recs.ptr, ws->recBytes.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(outRows, ws->recs.ptr, m * sizeof(tgs::ConstraintRecord), cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(outRowBytes, ws->recBytes.ptr, m * 4, cudaMemcpyDeviceToHost, s));
	if(frictionOut) GBPX_CUDA_TRY(cudaMemcpyAsync(frictionOut, ws->frictionOut.ptr, m * sizeof(tgs::FrictionState), cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// PxSolveConstraintsTGS over contacts and joints: contact rows (n blocks of
// gbpx_constraint_row_stride() bytes, in solve order, updated in place with
// the accumulated impulses), contact k joining bodies bodyA[k], bodyB[k]; joint
// records (nbJoints of gbpx_joint_record_bytes(), from
// gbpx_create_joint_constraints_tgs, in solve order, updated in place), joint
// k joining jointA[k], jointB[k].  Wave w solves contacts [waveEnds[w-1],
// waveEnds[w]) and joints [jointWaveEnds[w-1], jointWaveEnds[w]), which touch
// distinct dynamic bodies.  bodyVel/bodyTxI: nbBodies records in the
// reference's layouts, updated in place; the first nbIntegrate bodies are
// integrated after every position iteration.  dt = time step /
// nbPositionIterations.  outBroken (may be null): per contact, bit p set when
// patch p's friction was clamped in the last iteration.  outJointForce /
// outJointBroken (may be null): per joint the write-back impulse (linear,
// angular) and broken flag.
GBPX_API int gbpx_solve_constraints_joints_tgs(void* rows, const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, const uint32_t* waveEnds,
                                               void* jointRecords, const uint32_t* jointA, const uint32_t* jointB, uint32_t nbJoints,
                                               const uint32_t* jointWaveEnds, uint32_t nbWaves, void* bodyVel, void* bodyTxI, uint32_t nbBodies,
                                               uint32_t nbIntegrate, uint32_t nbPos, uint32_t nbVel, float dt, uint32_t* outBroken, float* outJointForce,
                                               uint32_t* outJointBroken)
{
	gbpx::Zone zone("gbpx::solveConstraintsTGS");
	if(!bodyVel || !bodyTxI || !nbBodies || nbIntegrate > nbBodies || !nbPos || !(dt > 0.0f)) return GBPX_ERR_INVALID;
	if(n && (!rows || !bodyA || !bodyB || !waveEnds || !nbWaves || waveEnds[nbWaves - 1] != n)) return GBPX_ERR_INVALID;
	if(nbJoints && (!jointRecords || !jointA || !jointB || !jointWaveEnds || !nbWaves || jointWaveEnds[nbWaves - 1] != nbJoints))
		return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < n; k++)
		if(bodyA[k] >= nbBodies || bodyB[k] >= nbBodies) return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < nbJoints; k++)
		if(jointA[k] >= nbBodies || jointB[k] >= nbBodies) return GBPX_ERR_INVALID;
	for(uint32_t w = 0; w < nbWaves; w++)
		if((n && (waveEnds[w] > n || (w && waveEnds[w] < waveEnds[w - 1]))) ||
		   (nbJoints && (jointWaveEnds[w] > nbJoints || (w && jointWaveEnds[w] < jointWaveEnds[w - 1]))))
			return GBPX_ERR_INVALID;
	TgsStageWorkspace* ws = tgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	const size_t m = n ? n : 1, mj = nbJoints ? nbJoints : 1;
	if(ws->vel.reserve(16 * size_t(nbBodies)) || ws->tx.reserve(16 * size_t(nbBodies)) || ws->bodyA.reserve(m) || ws->bodyB.reserve(m) ||
	   ws->recs.reserve(m) || (outBroken && ws->broken.reserve(m)) || ws->jointRecs.reserve(mj) || ws->jointA.reserve(mj) ||
	   ws->jointB.reserve(mj) || ws->jointForce.reserve(6 * mj) || ws->jointBroken.reserve(mj))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	if(outBroken && n) GBPX_CUDA_TRY(cudaMemsetAsync(ws->broken.ptr, 0, size_t(n) * 4, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->vel.ptr, bodyVel, size_t(nbBodies) * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->tx.ptr, bodyTxI, size_t(nbBodies) * 64, cudaMemcpyHostToDevice, s));
	if(n)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->bodyA.ptr, bodyA, size_t(n) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->bodyB.ptr, bodyB, size_t(n) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->recs.ptr, rows, size_t(n) * sizeof(tgs::ConstraintRecord), cudaMemcpyHostToDevice, s));
	}
	if(nbJoints)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->jointA.ptr, jointA, size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->jointB.ptr, jointB, size_t(nbJoints) * 4, cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(ws->jointRecs.ptr, jointRecords, size_t(nbJoints) * sizeof(joint::JointRecord), cudaMemcpyHostToDevice, s));
	}
	float elapsed = 0.0f;
	auto sweep = [&](float minPen, bool last, bool conclude) {
		for(uint32_t w = 0; w < nbWaves; w++)
		{
			if(n)
			{
				const uint32_t b = w ? waveEnds[w - 1] : 0u, e = waveEnds[w];
				if(e > b)
					tgs::solveWaveRefKernel<<<divUp(e - b, 128), 128, 0, s>>>(ws->recs.ptr, ws->bodyA.ptr, ws->bodyB.ptr, b, e, ws->vel.ptr, minPen,
					                                                         elapsed, last && outBroken ? ws->broken.ptr : nullptr);
			}
			if(nbJoints)
			{
				const uint32_t b = w ? jointWaveEnds[w - 1] : 0u, e = jointWaveEnds[w];
				if(e > b)
					tgs::solveJointWaveRefKernel<<<divUp(e - b, 64), 64, 0, s>>>(ws->jointRecs.ptr, ws->jointA.ptr, ws->jointB.ptr, b, e, ws->vel.ptr,
					                                                            ws->tx.ptr, elapsed, conclude ? 1 : 0);
			}
		}
	};
	const bool any = n || nbJoints;
	for(uint32_t it = 0; it < nbPos; it++)
	{
		if(any) sweep(-FLT_MAX, !nbVel && it + 1 == nbPos, it + 1 == nbPos);
		if(nbIntegrate) tgs::integrateRefKernel<<<divUp(nbIntegrate, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, nbIntegrate, dt);
		elapsed += dt;
	}
	for(uint32_t it = 0; it < nbVel; it++)
		if(any) sweep(0.0f, it + 1 == nbVel, false);
	if(nbJoints) tgs::jointWriteBackKernel<<<divUp(nbJoints, 128), 128, 0, s>>>(ws->jointRecs.ptr, nbJoints, ws->jointForce.ptr, ws->jointBroken.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(bodyVel, ws->vel.ptr, size_t(nbBodies) * 64, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(bodyTxI, ws->tx.ptr, size_t(nbBodies) * 64, cudaMemcpyDeviceToHost, s));
	if(n) GBPX_CUDA_TRY(cudaMemcpyAsync(rows, ws->recs.ptr, size_t(n) * sizeof(tgs::ConstraintRecord), cudaMemcpyDeviceToHost, s));
	if(n && outBroken) GBPX_CUDA_TRY(cudaMemcpyAsync(outBroken, ws->broken.ptr, size_t(n) * 4, cudaMemcpyDeviceToHost, s));
	if(nbJoints)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(jointRecords, ws->jointRecs.ptr, size_t(nbJoints) * sizeof(joint::JointRecord), cudaMemcpyDeviceToHost, s));
		if(outJointForce) GBPX_CUDA_TRY(cudaMemcpyAsync(outJointForce, ws->jointForce.ptr, size_t(nbJoints) * 24, cudaMemcpyDeviceToHost, s));
		if(outJointBroken) GBPX_CUDA_TRY(cudaMemcpyAsync(outJointBroken, ws->jointBroken.ptr, size_t(nbJoints) * 4, cudaMemcpyDeviceToHost, s));
	}
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

// PxSolveConstraintsTGS over contacts only: as gbpx_solve_constraints_joints_tgs
// without joints.
GBPX_API int gbpx_solve_constraints_tgs(void* rows, const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, const uint32_t* waveEnds, uint32_t nbWaves,
                                        void* bodyVel, void* bodyTxI, uint32_t nbBodies, uint32_t nbIntegrate, uint32_t nbPos, uint32_t nbVel, float dt,
                                        uint32_t* outBroken)
{
	return gbpx_solve_constraints_joints_tgs(rows, bodyA, bodyB, n, waveEnds, nullptr, nullptr, nullptr, 0, nullptr, nbWaves, bodyVel, bodyTxI,
	                                         nbBodies, nbIntegrate, nbPos, nbVel, dt, outBroken, nullptr, nullptr);
}

// PxIntegrateSolverBodiesTGS: world angular velocity written back into the
// velocity records, poses (PxTransform) updated in place.
GBPX_API int gbpx_integrate_solver_bodies_tgs(void* bodyVel, const void* bodyTxI, float* poses, uint32_t n)
{
	gbpx::Zone zone("gbpx::integrateSolverBodiesTGS");
	if(!n) return GBPX_OK;
	if(!bodyVel || !bodyTxI || !poses) return GBPX_ERR_INVALID;
	TgsStageWorkspace* ws = tgsStageWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	if(ws->vel.reserve(16 * size_t(n)) || ws->tx.reserve(16 * size_t(n)) || ws->poses.reserve(7 * size_t(n))) return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->vel.ptr, bodyVel, size_t(n) * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->tx.ptr, bodyTxI, size_t(n) * 64, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->poses.ptr, poses, size_t(n) * 28, cudaMemcpyHostToDevice, s));
	tgs::finalizeRefKernel<<<divUp(n, 128), 128, 0, s>>>(ws->vel.ptr, ws->tx.ptr, ws->poses.ptr, n);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(bodyVel, ws->vel.ptr, size_t(n) * 64, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(poses, ws->poses.ptr, size_t(n) * 28, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	return GBPX_OK;
}

namespace gbpx
{
namespace tgs
{
__global__ void sinCosAngleKernel(const float* __restrict__ x, uint32_t n, float* __restrict__ out)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	float s, c;
	sinCosAngle(x[i], s, c);
	double ds, dc;
	sincos(double(x[i]), &ds, &dc);
	out[4 * size_t(i) + 0] = s;
	out[4 * size_t(i) + 1] = c;
	out[4 * size_t(i) + 2] = float(ds);
	out[4 * size_t(i) + 3] = float(dc);
}
} // namespace tgs
} // namespace gbpx

// The integrator's sine and cosine of n angles (host arrays): per angle the
// values the solver uses and the double-precision values rounded to float
// (out: 4 floats per angle).
GBPX_API int gbpx_eval_sincos_angle(const float* x, uint32_t n, float* out)
{
	if(!n) return GBPX_OK;
	if(!x || !out) return GBPX_ERR_INVALID;
	float *dx = nullptr, *dout = nullptr;
	cudaError_t e = cudaMalloc(&dx, size_t(n) * 4);
	if(e == cudaSuccess) e = cudaMalloc(&dout, size_t(n) * 16);
	if(e == cudaSuccess) e = cudaMemcpy(dx, x, size_t(n) * 4, cudaMemcpyHostToDevice);
	if(e == cudaSuccess)
	{
		gbpx::tgs::sinCosAngleKernel<<<(n + 255) / 256, 256>>>(dx, n, dout);
		e = cudaGetLastError();
	}
	if(e == cudaSuccess) e = cudaMemcpy(out, dout, size_t(n) * 16, cudaMemcpyDeviceToHost);
	cudaFree(dx);
	cudaFree(dout);
	return e == cudaSuccess ? GBPX_OK : GBPX_ERR_CUDA;
}
