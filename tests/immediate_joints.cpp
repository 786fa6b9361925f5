// One immediate-mode joint frame written against the reference's interface
// (physx::immediate: PxConstructSolverBodiesTGS, PxConstructStaticSolverBodyTGS,
// PxBatchConstraintsTGS, PxCreateJointConstraintsTGS, PxSolveConstraintsTGS,
// PxIntegrateSolverBodiesTGS) the way the reference's immediate-mode snippet
// builds its joints (SnippetImmediateMode.cpp:838-1061), with the joint rows
// given instead of a joint shader, or (argument "shader") returned by an
// immediate joint shader through PxCreateJointConstraintsWithImmediateShadersTGS;
// linked against libgbpx_immediate.so.  Used by tests/test_joints_gpu.py.
//
// stdin (binary): nbDyn, nbStatic, nbJoints, nbRows, batch (u32);
// PxRigidBodyData[nbDyn]; static poses (PxTransform); jointA, jointB,
// rowStart, rowCount (u32 each per joint); Px1DConstraint[nbRows]; 20 floats
// per joint (invMassScales, cA2w, cB2w, body0WorldOffset, linBreakForce,
// angBreakForce, minResponseThreshold, flags 1 disablePreprocessing |
// 4 driveLimitsAreForces, unused); dt, gravity xyz (4 floats); nbPos, nbVel (u32).
// stdout (binary): per dynamic body linear velocity, world angular velocity
// (6 floats) and pose (7 floats); the header count (u32) and per header start,
// stride, type (u32); per joint (caller's order) the write-back's linear and
// angular impulse (6 floats) and broken flag (u32).
#include "gbpx_immediate.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace gbpx_px;

namespace
{
template <typename T> void readAll(T* p, size_t n)
{
	if(n && fread(p, sizeof(T), n, stdin) != n) { fprintf(stderr, "short input\n"); exit(2); }
}
template <typename T> void writeAll(const T* p, size_t n) { if(n) fwrite(p, sizeof(T), n, stdout); }

struct Arena : PxConstraintAllocator
{
	std::vector<std::vector<uint8_t>> blocks;
	uint8_t* reserveConstraintData(const uint32_t size) override
	{
		blocks.emplace_back(size + 16);
		uint8_t* p = blocks.back().data();
		return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
	}
	uint8_t* reserveFrictionData(const uint32_t size) override { return reserveConstraintData(size); }
};

// constant block of the immediate joint shader: the joint's rows and parameters
struct JointBlock
{
	const Px1DConstraint* rows;
	uint32_t count;
	const float* p;
};
uint32_t copyRowsShader(Px1DConstraint* rows, PxVec3p& body0WorldOffset, uint32_t maxRows, PxConstraintInvMassScale& invMassScale,
                        const void* constantBlock, const PxTransform&, const PxTransform&, bool, PxVec3p& cA2w, PxVec3p& cB2w)
{
	const JointBlock& b = *static_cast<const JointBlock*>(constantBlock);
	const uint32_t n = b.count < maxRows ? b.count : maxRows;
	memcpy(rows, b.rows, sizeof(Px1DConstraint) * n);
	invMassScale = PxConstraintInvMassScale{b.p[0], b.p[1], b.p[2], b.p[3]};
	cA2w.v = PxVec3{b.p[4], b.p[5], b.p[6]};
	cB2w.v = PxVec3{b.p[7], b.p[8], b.p[9]};
	body0WorldOffset.v = PxVec3{b.p[10], b.p[11], b.p[12]};
	return n;
}

// Dy::ConstraintWriteback
struct Writeback
{
	PxVec3 linearImpulse;
	uint32_t broken;
	PxVec3 angularImpulse;
	float residual;
};
} // namespace

int main(int argc, char** argv)
{
	const bool shader = argc > 1 && strcmp(argv[1], "shader") == 0;
	uint32_t head[5];
	readAll(head, 5);
	const uint32_t nbDyn = head[0], nbStatic = head[1], nbJoints = head[2], nbRows = head[3], batch = head[4];
	std::vector<PxRigidBodyData> rigid(nbDyn);
	readAll(rigid.data(), nbDyn);
	std::vector<PxTransform> statics(nbStatic);
	readAll(statics.data(), nbStatic);
	std::vector<uint32_t> ja(nbJoints), jb(nbJoints), rs(nbJoints), rc(nbJoints);
	readAll(ja.data(), nbJoints);
	readAll(jb.data(), nbJoints);
	readAll(rs.data(), nbJoints);
	readAll(rc.data(), nbJoints);
	std::vector<Px1DConstraint> rows(nbRows ? nbRows : 1);
	readAll(rows.data(), nbRows);
	std::vector<float> params(size_t(nbJoints) * 20);
	readAll(params.data(), params.size());
	float f[4];
	readAll(f, 4);
	uint32_t iters[2];
	readAll(iters, 2);
	const float dt = f[0];
	const PxVec3 gravity{f[1], f[2], f[3]};
	const uint32_t nbPos = iters[0], nbVel = iters[1];

	// solver bodies: dynamic ones first, statics after (the snippet's layout)
	const uint32_t nbTotal = nbDyn + nbStatic;
	std::vector<PxTGSSolverBodyVel> bodies(nbTotal);
	std::vector<PxTGSSolverBodyTxInertia> txI(nbTotal);
	std::vector<PxTGSSolverBodyData> data(nbTotal);
	std::vector<PxTransform> poses(nbTotal);
	PxConstructSolverBodiesTGS(rigid.data(), bodies.data(), txI.data(), data.data(), nbDyn, gravity, dt, false);
	for(uint32_t a = 0; a < nbDyn; a++) poses[a] = rigid[a].body2World;
	for(uint32_t s = 0; s < nbStatic; s++)
	{
		poses[nbDyn + s] = statics[s];
		PxConstructStaticSolverBodyTGS(statics[s], bodies[nbDyn + s], txI[nbDyn + s], data[nbDyn + s]);
	}

	std::vector<PxSolverConstraintDesc> descs(nbJoints), ordered(nbJoints);
	std::vector<uint32_t> ids(nbJoints);
	for(uint32_t j = 0; j < nbJoints; j++)
	{
		PxSolverConstraintDesc& d = descs[j];
		memset(&d, 0, sizeof(d));
		d.tgsBodyA = &bodies[ja[j]];
		d.tgsBodyB = &bodies[jb[j]];
		d.bodyADataIndex = ja[j];
		d.bodyBDataIndex = jb[j];
		d.linkIndexA = d.linkIndexB = 0xffff;
		ids[j] = j;
		d.constraint = reinterpret_cast<uint8_t*>(&ids[j]);
		d.constraintLengthOver16 = 1;   // PxSolverConstraintDesc::eJOINT_CONSTRAINT
	}
	std::vector<PxConstraintBatchHeader> headers(nbJoints ? nbJoints : 1);
	uint32_t nbHeaders = 0;
	if(batch)
		nbHeaders = PxBatchConstraintsTGS(descs.data(), nbJoints, bodies.data(), nbDyn, headers.data(), ordered.data(), nullptr, 0);
	else
	{
		for(uint32_t j = 0; j < nbJoints; j++)
		{
			headers[j].startIndex = j;
			headers[j].stride = 1;
			headers[j].constraintType = 1;
			ordered[j] = descs[j];
		}
		nbHeaders = nbJoints;
	}
	std::vector<uint32_t> order(nbJoints);
	for(uint32_t k = 0; k < nbJoints; k++) order[k] = *reinterpret_cast<const uint32_t*>(ordered[k].constraint);

	const float invDt = 1.0f / dt;
	const float stepDt = dt / float(nbPos);
	const float invStepDt = invDt * float(nbPos);
	Arena arena;
	std::vector<Writeback> writeback(nbJoints ? nbJoints : 1);
	memset(writeback.data(), 0, sizeof(Writeback) * writeback.size());
	std::vector<Px1DConstraint> rowCopy(rows);
	// shader mode: every header's descriptors, in header order, and their shaders
	std::vector<PxTGSSolverConstraintPrepDesc> jdAll(nbJoints ? nbJoints : 1);
	std::vector<JointBlock> blocks(nbJoints ? nbJoints : 1);
	std::vector<PxImmediateConstraint> shaders(nbJoints ? nbJoints : 1);
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		PxConstraintBatchHeader& header = headers[h];
		PxTGSSolverConstraintPrepDesc jd[4];
		for(uint32_t a = 0; a < header.stride; a++)
		{
			PxSolverConstraintDesc& desc = ordered[header.startIndex + a];
			const uint32_t j = order[header.startIndex + a];
			const float* p = &params[size_t(j) * 20];
			PxTGSSolverConstraintPrepDesc& c = shader ? jdAll[header.startIndex + a] : jd[a];
			memset(&c, 0, sizeof(c));
			c.body0 = desc.tgsBodyA;
			c.body1 = desc.tgsBodyB;
			c.bodyData0 = &data[desc.bodyADataIndex];
			c.bodyData1 = &data[desc.bodyBDataIndex];
			c.body0TxI = &txI[desc.bodyADataIndex];
			c.body1TxI = &txI[desc.bodyBDataIndex];
			c.bodyFrame0 = poses[desc.bodyADataIndex];
			c.bodyFrame1 = poses[desc.bodyBDataIndex];
			c.bodyState0 = desc.bodyADataIndex < nbDyn ? eDYNAMIC_BODY : eSTATIC_BODY;
			c.bodyState1 = desc.bodyBDataIndex < nbDyn ? eDYNAMIC_BODY : eSTATIC_BODY;
			c.desc = &desc;
			c.writeback = &writeback[j];
			c.invMassScales = PxConstraintInvMassScale{p[0], p[1], p[2], p[3]};
			c.cA2w.v = PxVec3{p[4], p[5], p[6]};
			c.cB2w.v = PxVec3{p[7], p[8], p[9]};
			c.body0WorldOffset.v = PxVec3{p[10], p[11], p[12]};
			c.linBreakForce = p[13];
			c.angBreakForce = p[14];
			c.minResponseThreshold = p[15];
			const uint32_t fl = uint32_t(p[16]);
			c.disablePreprocessing = (fl & 1u) != 0;
			c.driveLimitsAreForces = (fl & 4u) != 0;
			c.rows = rowCopy.data() + rs[j];
			c.numRows = rc[j];
			if(shader)
			{
				// the shader sets the rows, mass scales, frames and offset itself
				c.rows = nullptr;
				c.numRows = 0;
				blocks[header.startIndex + a] = JointBlock{rowCopy.data() + rs[j], rc[j], p};
				shaders[header.startIndex + a] = PxImmediateConstraint{copyRowsShader, &blocks[header.startIndex + a]};
			}
		}
		if(!shader && !PxCreateJointConstraintsTGS(&header, 1, jd, arena, stepDt, dt, invStepDt, invDt, 1.0f))
		{
			fprintf(stderr, "joint prep failed\n");
			return 3;
		}
	}
	if(shader && !PxCreateJointConstraintsWithImmediateShadersTGS(headers.data(), nbHeaders, shaders.data(), jdAll.data(), arena, stepDt, dt,
	                                                             invStepDt, invDt, 1.0f))
	{
		fprintf(stderr, "joint prep failed\n");
		return 3;
	}
	PxSolveConstraintsTGS(headers.data(), nbHeaders, ordered.data(), bodies.data(), txI.data(), nbDyn, nbPos, nbVel, stepDt, invStepDt, 0, nullptr,
	                      nullptr, nullptr);
	PxIntegrateSolverBodiesTGS(bodies.data(), txI.data(), poses.data(), nbDyn, dt);
	for(uint32_t a = 0; a < nbDyn; a++)
	{
		const float v[13] = {bodies[a].linearVelocity.x, bodies[a].linearVelocity.y, bodies[a].linearVelocity.z, bodies[a].angularVelocity.x,
		                     bodies[a].angularVelocity.y, bodies[a].angularVelocity.z, poses[a].q.x, poses[a].q.y, poses[a].q.z, poses[a].q.w,
		                     poses[a].p.x, poses[a].p.y, poses[a].p.z};
		writeAll(v, 13);
	}
	writeAll(&nbHeaders, 1);
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		const uint32_t hv[3] = {headers[h].startIndex, headers[h].stride, headers[h].constraintType};
		writeAll(hv, 3);
	}
	for(uint32_t j = 0; j < nbJoints; j++)
	{
		const Writeback& w = writeback[j];
		const float fv[6] = {w.linearImpulse.x, w.linearImpulse.y, w.linearImpulse.z, w.angularImpulse.x, w.angularImpulse.y, w.angularImpulse.z};
		writeAll(fv, 6);
		const uint32_t b = (w.broken & 0x80000000u) ? 1u : 0u;
		writeAll(&b, 1);
	}
	return 0;
}
