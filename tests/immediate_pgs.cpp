// One immediate-mode PGS frame written against the reference's interface
// (physx::immediate: PxConstructSolverBodies, PxConstructStaticSolverBody,
// PxBatchConstraints, PxCreateContactConstraints, PxSolveConstraints,
// PxIntegrateSolverBodies) the way the reference's immediate-mode snippet runs
// its PGS branch (SnippetImmediateMode.cpp:495-503,749,761,886-961,1080-1099),
// from given contacts; linked against libgbpx_immediate.so.  Used by
// tests/test_immediate_dropin_gpu.py.  With the argument "nullalloc" the
// constraint allocator returns null: PxCreateContactConstraints must return
// false (exit code 3) without touching the memory.
//
// stdin (binary): nbDyn, nbStatic, nbConstraints, nbContacts, batch (u32);
// PxRigidBodyData[nbDyn]; static poses (PxTransform); pairA, pairB,
// contactStart, contactCount (u32 each per constraint); contacts (8 floats:
// normal, separation, point, 0); material (static friction, dynamic friction,
// restitution per constraint); dt, gravity xyz (4 floats); nbPos, nbVel (u32).
// stdout (binary): per dynamic body linear velocity, angular velocity (6
// floats) and pose (7 floats); the header count (u32) and per header start,
// stride, type (u32); the constraint order (u32 each); per contact the
// written-back normal impulse (float).
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
	bool null = false;
	uint8_t* reserveConstraintData(const uint32_t size) override
	{
		if(null) return nullptr;
		blocks.emplace_back(size + 16);
		uint8_t* p = blocks.back().data();
		return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
	}
	uint8_t* reserveFrictionData(const uint32_t size) override { return reserveConstraintData(size); }
};
} // namespace

int main(int argc, char** argv)
{
	const bool nullAlloc = argc > 1 && strcmp(argv[1], "nullalloc") == 0;
	uint32_t head[5];
	readAll(head, 5);
	const uint32_t nbDyn = head[0], nbStatic = head[1], nbCons = head[2], nbContacts = head[3], batch = head[4];
	std::vector<PxRigidBodyData> rigid(nbDyn);
	readAll(rigid.data(), nbDyn);
	std::vector<PxTransform> statics(nbStatic);
	readAll(statics.data(), nbStatic);
	std::vector<uint32_t> pa(nbCons), pb(nbCons), cs(nbCons), cc(nbCons);
	readAll(pa.data(), nbCons);
	readAll(pb.data(), nbCons);
	readAll(cs.data(), nbCons);
	readAll(cc.data(), nbCons);
	std::vector<float> contacts(size_t(nbContacts) * 8), material(size_t(nbCons) * 3);
	readAll(contacts.data(), contacts.size());
	readAll(material.data(), material.size());
	float f[4];
	readAll(f, 4);
	uint32_t iters[2];
	readAll(iters, 2);
	const float dt = f[0];
	const PxVec3 gravity{f[1], f[2], f[3]};

	// solver bodies: dynamic ones first, statics after (the snippet's layout)
	const uint32_t nbTotal = nbDyn + nbStatic;
	std::vector<PxSolverBody> bodies(nbTotal);
	std::vector<PxSolverBodyData> data(nbTotal);
	for(uint32_t a = 0; a < nbDyn; a++) PxConstructSolverBodies(&rigid[a], &data[a], 1, gravity, dt, false);
	for(uint32_t s = 0; s < nbStatic; s++) PxConstructStaticSolverBody(statics[s], data[nbDyn + s]);

	// the contact points the snippet's recorder fills in
	std::vector<PxContactPoint> points(nbContacts ? nbContacts : 1);
	for(uint32_t i = 0; i < nbCons; i++)
		for(uint32_t c = 0; c < cc[i]; c++)
		{
			const float* s = &contacts[8 * size_t(cs[i] + c)];
			PxContactPoint& p = points[cs[i] + c];
			memset(&p, 0, sizeof(p));
			p.normal = PxVec3{s[0], s[1], s[2]};
			p.separation = s[3];
			p.point = PxVec3{s[4], s[5], s[6]};
			p.maxImpulse = 3.402823466e+38f;
			p.staticFriction = material[3 * i];
			p.dynamicFriction = material[3 * i + 1];
			p.restitution = material[3 * i + 2];
		}
	std::vector<float> forces(nbContacts ? nbContacts : 1, 0.0f);

	std::vector<PxSolverConstraintDesc> descs(nbCons), ordered(nbCons);
	std::vector<uint32_t> ids(nbCons);
	for(uint32_t i = 0; i < nbCons; i++)
	{
		PxSolverConstraintDesc& d = descs[i];
		memset(&d, 0, sizeof(d));
		d.bodyA = &bodies[pa[i]];
		d.bodyB = &bodies[pb[i]];
		d.bodyADataIndex = pa[i];
		d.bodyBDataIndex = pb[i];
		d.linkIndexA = d.linkIndexB = 0xffff;
		ids[i] = i;
		d.constraint = reinterpret_cast<uint8_t*>(&ids[i]);
		d.constraintLengthOver16 = 0;   // PxSolverConstraintDesc::eCONTACT_CONSTRAINT
	}
	std::vector<PxConstraintBatchHeader> headers(nbCons ? nbCons : 1);
	uint32_t nbHeaders = 0;
	if(batch)
		nbHeaders = PxBatchConstraints(descs.data(), nbCons, bodies.data(), nbDyn, headers.data(), ordered.data(), nullptr, 0);
	else
	{
		for(uint32_t i = 0; i < nbCons; i++)
		{
			headers[i].startIndex = i;
			headers[i].stride = 1;
			headers[i].constraintType = 0;
			ordered[i] = descs[i];
		}
		nbHeaders = nbCons;
	}
	std::vector<uint32_t> order(nbCons);
	for(uint32_t k = 0; k < nbCons; k++) order[k] = *reinterpret_cast<const uint32_t*>(ordered[k].constraint);

	const float invDt = 1.0f / dt;
	Arena arena;
	arena.null = nullAlloc;
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		PxConstraintBatchHeader& header = headers[h];
		PxSolverContactDesc cd[4];
		for(uint32_t a = 0; a < header.stride; a++)
		{
			PxSolverConstraintDesc& desc = ordered[header.startIndex + a];
			const uint32_t i = order[header.startIndex + a];
			PxSolverContactDesc& c = cd[a];
			memset(&c, 0, sizeof(c));
			c.body0 = desc.bodyA;
			c.body1 = desc.bodyB;
			c.data0 = &data[desc.bodyADataIndex];
			c.data1 = &data[desc.bodyBDataIndex];
			c.bodyFrame0 = c.data0->body2World;
			c.bodyFrame1 = c.data1->body2World;
			c.contactForces = &forces[cs[i]];
			c.contacts = &points[cs[i]];
			c.numContacts = cc[i];
			c.frictionPtr = nullptr;
			c.frictionCount = 0;
			c.shapeInteraction = nullptr;
			c.maxCCDSeparation = 3.402823466e+38f;
			c.bodyState0 = eDYNAMIC_BODY;
			c.bodyState1 = desc.bodyBDataIndex < nbDyn ? eDYNAMIC_BODY : eSTATIC_BODY;
			c.desc = &desc;
			c.invMassScales = PxConstraintInvMassScale{1.0f, 1.0f, 1.0f, 1.0f};
		}
		if(!PxCreateContactConstraints(&header, 1, cd, arena, invDt, -2.0f, 0.04f, 0.025f, nullptr)) { fprintf(stderr, "contact prep failed\n"); return 3; }
	}

	std::vector<PxVec3> motionLin(nbDyn ? nbDyn : 1), motionAng(nbDyn ? nbDyn : 1);
	memset(bodies.data(), 0, bodies.size() * sizeof(PxSolverBody));
	PxSolveConstraints(headers.data(), nbHeaders, ordered.data(), bodies.data(), motionLin.data(), motionAng.data(), nbDyn, iters[0], iters[1], 0.0f, 0.0f,
	                   0, nullptr, nullptr, nullptr);
	PxIntegrateSolverBodies(data.data(), bodies.data(), motionLin.data(), motionAng.data(), nbDyn, dt);
	for(uint32_t a = 0; a < nbDyn; a++)
	{
		const PxSolverBodyData& d = data[a];
		const float v[13] = {d.linearVelocity.x, d.linearVelocity.y, d.linearVelocity.z, d.angularVelocity.x, d.angularVelocity.y, d.angularVelocity.z,
		                     d.body2World.q.x, d.body2World.q.y, d.body2World.q.z, d.body2World.q.w, d.body2World.p.x, d.body2World.p.y,
		                     d.body2World.p.z};
		writeAll(v, 13);
	}
	writeAll(&nbHeaders, 1);
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		const uint32_t hv[3] = {headers[h].startIndex, headers[h].stride, headers[h].constraintType};
		writeAll(hv, 3);
	}
	writeAll(order.data(), nbCons);
	writeAll(forces.data(), nbContacts);
	return 0;
}
