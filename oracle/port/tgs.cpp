// ORACLE (test infrastructure, never shipped): CPU restatement of the TGS
// immediate-mode contact path:
//   PxConstructSolverBodiesTGS / PxConstructStaticSolverBodyTGS
//     (physx/source/immediatemode/src/NpImmediateMode.cpp:1365,1380) ->
//     bodyCoreComputeUnconstrainedVelocity (lowleveldynamics/src/DyBodyCoreIntegrator.h:38),
//     copyToSolverBodyDataStep (lowleveldynamics/src/DyTGSDynamics.cpp:154)
//   PxBatchConstraintsTGS (NpImmediateMode.cpp:278, createHeaders :159) ->
//     classifyConstraintDesc / writeConstraintDesc (lowleveldynamics/src/DyConstraintPartition.cpp:476,571)
//   PxCreateContactConstraintsTGS (NpImmediateMode.cpp:1386) ->
//     createFinalizeSolverContactsStep (lowleveldynamics/src/DyTGSContactPrep.cpp:1297),
//     createContactPatches / correlatePatches / growPatches (DyFrictionCorrelation.cpp:56,133,187),
//     setupFinalizeSolverConstraints (DyTGSContactPrep.cpp:426), constructContactConstraintStep (:322)
//   PxSolveConstraintsTGS (NpImmediateMode.cpp:1630) -> solveContact (DyTGSContactPrep.cpp:1581),
//     solveDynamicContactsStep (:1492), integrateCoreStep (DyTGSDynamics.cpp:1403)
//   PxIntegrateSolverBodiesTGS (NpImmediateMode.cpp:1719)
// with fresh friction data (frictionPtr = NULL), unit mass scales, zero rest
// distance / offset slop, no torsional friction: the settings of the reference's
// immediate-mode snippet.  Headers of stride 4 follow the reference's 4-wide block
// path (createFinalizeSolverContacts4Step / setupFinalizeSolverConstraints4Step,
// lowleveldynamics/src/DyTGSContactPrepBlock.cpp:1398,219; solveContact4_Block
// :2280), restated one lane at a time; every other constraint follows the
// per-pair path.  The results equal the reference's bit for bit (tests).
#include "pxmath.h"
#include "tgs_frame.h"
#include "tgs_bodies.h"
#include <string.h>
#include <vector>
#include <algorithm>

#define OX extern "C" __attribute__((visibility("default")))

using namespace orc;

namespace
{
struct PointRow { V3 raXnI, rbXnI; float velMultiplier, separation, biasCoefficient, targetVelocity, recipResponse, maxImpulse, force; };
struct FrictionRow { V3 normal; float error; V3 raXnI; float targetVel; V3 rbXnI; float velMultiplier; float appliedForce, frictionScale, biasScale; };
struct PatchRows
{
	V3 normal;
	float invMass0, invMass1, angDom0, angDom1, maxPenBias, staticFriction, dynamicFriction;
	int pointStart, nbPoints, frictionStart, nbFriction;
	int anchorCount;     // anchors of the friction patch the rows were built from
	int brokenSlot;      // written friction patch that receives this patch's broken flag
	int broken;          // friction clamped during the latest solve of the patch
};
// block: the constraint is one lane of a 4-wide header and uses the block
// path's rows and solve (createFinalizeSolverContacts4Step, solveContact4_Block)
// written: the friction patches the constraint leaves for the next frame
struct ConstraintRows { int bodyA, bodyB; int patchStart, nbPatches; bool block; std::vector<FrictionPatch> written; };

struct ContactIn { V3 n; float sep; V3 p; float staticFriction, dynamicFriction, restitution; };

// ------------------------------------------------------------ bodies
void unconstrainedVelocity(V3 g, float dt, float linDamp, float angDamp, float maxLinSq, float maxAngSq, V3& lv, V3& av)
{
	const float ld = linDamp * dt, ad = angDamp * dt;
	const float oml = 1.0f - ld, oma = 1.0f - ad;
	lv = add(lv, scale(scale(g, dt), 1.0f));   // gravity*dt*accelScale
	const float lm = oml >= 0.0f ? oml : 0.0f;  // fsel(x, x, 0)
	const float am = oma >= 0.0f ? oma : 0.0f;
	lv = scale(lv, lm);
	av = scale(av, am);
	const float l2 = lenSqS(lv);
	if(l2 > maxLinSq) lv = scale(lv, sqrtf(maxLinSq / l2));
	const float a2 = lenSqS(av);
	if(a2 > maxAngSq) av = scale(av, sqrtf(maxAngSq / a2));
}

M33 transformInertia(V3 d, const M33& M)
{
	// Cm::transformInertiaTensor (common/src/CmUtils.h:57); M(r, c) = column c, row r
	auto m = [&](int r, int c) { const V3& col = c == 0 ? M.c0 : (c == 1 ? M.c1 : M.c2); return getc(col, r); };
	const float axx = d.x * m(0, 0), axy = d.x * m(1, 0), axz = d.x * m(2, 0);
	const float byx = d.y * m(0, 1), byy = d.y * m(1, 1), byz = d.y * m(2, 1);
	const float czx = d.z * m(0, 2), czy = d.z * m(1, 2), czz = d.z * m(2, 2);
	const float i00 = axx * m(0, 0) + byx * m(0, 1) + czx * m(0, 2);
	const float i11 = axy * m(1, 0) + byy * m(1, 1) + czy * m(1, 2);
	const float i22 = axz * m(2, 0) + byz * m(2, 1) + czz * m(2, 2);
	const float i01 = axx * m(1, 0) + byx * m(1, 1) + czx * m(1, 2);
	const float i02 = axx * m(2, 0) + byx * m(2, 1) + czx * m(2, 2);
	const float i12 = axy * m(2, 0) + byy * m(2, 1) + czy * m(2, 2);
	M33 r;
	r.c0 = v3(i00, i01, i02);
	r.c1 = v3(i01, i11, i12);
	r.c2 = v3(i02, i12, i22);
	return r;
}

void copyToSolverBody(V3 lv, V3 av, float invMass, V3 invInertia, const Tr& pose, float maxDepen, float maxImpulse, float maxAngVelSq,
                      bool kinematic, BodyVel& vel, BodyTx& tx, BodyData& data)
{
	const M33 rot = m33FromQuatCol(pose.q);   // PxMat33Padded
	const V3 sqrtInv = v3(invInertia.x == 0.0f ? 0.0f : sqrtf(invInertia.x), invInertia.y == 0.0f ? 0.0f : sqrtf(invInertia.y),
	                      invInertia.z == 0.0f ? 0.0f : sqrtf(invInertia.z));
	const V3 sqrtBody = v3(sqrtInv.x == 0.0f ? 0.0f : 1.0f / sqrtInv.x, sqrtInv.y == 0.0f ? 0.0f : 1.0f / sqrtInv.y,
	                       sqrtInv.z == 0.0f ? 0.0f : 1.0f / sqrtInv.z);
	tx.sqrtInvInertia = transformInertia(sqrtInv, rot);
	tx.p = pose.p;
	tx.dq.x = tx.dq.y = tx.dq.z = 0.0f; tx.dq.w = 1.0f;
	const M33 sqrtInertia = transformInertia(sqrtBody, rot);
	vel.lin = lv;
	vel.ang = m33MulVS(sqrtInertia, av);
	vel.dLin = zero3();
	vel.dAng = zero3();
	vel.kinematic = kinematic;
	vel.maxAngVel = sqrtf(maxAngVelSq);
	data.invMass = invMass;
	data.penBiasClamp = maxDepen;
	data.maxContactImpulse = maxImpulse;
	data.origLin = lv;
	data.origAng = av;
}

// ------------------------------------------------------------ batching
void batchConstraints(const uint32_t* bodyA, const uint32_t* bodyB, int n, int nbDyn, BatchOut& out)
{
	const uint32_t MAXP = 32;
	std::vector<uint32_t> progress(nbDyn, 0), maxNormal(nbDyn, 0), maxFriction(nbDyn, 0);
	std::vector<uint32_t> perPartition(MAXP, 0);
	std::vector<int> overflow;
	// pass 1: classification in input order
	for(int i = 0; i < n; i++)
	{
		const bool aA = bodyA[i] < uint32_t(nbDyn), aB = bodyB[i] < uint32_t(nbDyn);
		if(aA && aB)
		{
			uint32_t& pA = progress[bodyA[i]];
			uint32_t& pB = progress[bodyB[i]];
			const uint32_t mask = ~pA & ~pB;
			if(!mask) { overflow.push_back(i); continue; }
			const uint32_t part = __builtin_ctz(mask);
			pA |= 1u << part; pB |= 1u << part;
			perPartition[part]++;
			maxNormal[bodyA[i]] = std::max(maxNormal[bodyA[i]], part + 1);
			maxNormal[bodyB[i]] = std::max(maxNormal[bodyB[i]], part + 1);
		}
		else
		{
			if(aA) maxFriction[bodyA[i]]++;
			if(aB) maxFriction[bodyB[i]]++;
		}
	}
	uint32_t start = 0;
	std::vector<int> pending = overflow;
	while(!pending.empty())
	{
		std::fill(progress.begin(), progress.end(), 0u);
		start += MAXP;
		perPartition.resize(perPartition.size() + MAXP, 0);
		std::vector<int> next;
		for(int i : pending)
		{
			uint32_t& pA = progress[bodyA[i]];
			uint32_t& pB = progress[bodyB[i]];
			const uint32_t mask = ~pA & ~pB;
			if(!mask) { next.push_back(i); continue; }
			const uint32_t part = __builtin_ctz(mask);
			pA |= 1u << part; pB |= 1u << part;
			perPartition[start + part]++;
			maxNormal[bodyA[i]] = std::max(maxNormal[bodyA[i]], start + part + 1);
			maxNormal[bodyB[i]] = std::max(maxNormal[bodyB[i]], start + part + 1);
		}
		pending.swap(next);
	}
	// reserveSpaceForStaticConstraints
	for(int b = 0; b < nbDyn; b++)
	{
		const uint32_t need = maxNormal[b] + maxFriction[b];
		if(need > perPartition.size()) perPartition.resize(need, 0);
		for(uint32_t k = 0; k < maxFriction[b]; k++) perPartition[maxNormal[b] + k]++;
	}
	// exclusive prefix
	uint32_t acc = 0;
	for(uint32_t& c : perPartition) { const uint32_t t = c; c = acc; acc += t; }
	// pass 2: write
	std::fill(progress.begin(), progress.end(), 0u);
	std::vector<uint32_t> staticProgress(nbDyn, 0);
	out.order.assign(n, -1);
	std::vector<int> ov;
	for(int i = 0; i < n; i++)
	{
		const bool aA = bodyA[i] < uint32_t(nbDyn), aB = bodyB[i] < uint32_t(nbDyn);
		if(aA && aB)
		{
			uint32_t& pA = progress[bodyA[i]];
			uint32_t& pB = progress[bodyB[i]];
			const uint32_t mask = ~pA & ~pB;
			if(!mask) { ov.push_back(i); continue; }
			const uint32_t part = __builtin_ctz(mask);
			pA |= 1u << part; pB |= 1u << part;
			out.order[perPartition[part]++] = i;
		}
		else
		{
			const uint32_t b = aA ? bodyA[i] : (aB ? bodyB[i] : 0xffffffffu);
			if(b == 0xffffffffu) continue;  // static-static: dropped from the ordered list
			const uint32_t idx = maxNormal[b] + staticProgress[b]++;
			out.order[perPartition[idx]++] = i;
		}
	}
	start = 0;
	while(!ov.empty())
	{
		std::fill(progress.begin(), progress.end(), 0u);
		start += MAXP;
		std::vector<int> next;
		for(int i : ov)
		{
			uint32_t& pA = progress[bodyA[i]];
			uint32_t& pB = progress[bodyB[i]];
			const uint32_t mask = ~pA & ~pB;
			if(!mask) { next.push_back(i); continue; }
			const uint32_t part = __builtin_ctz(mask);
			pA |= 1u << part; pB |= 1u << part;
			out.order[perPartition[start + part]++] = i;
		}
		ov.swap(next);
	}
	// maxPartition: leading partitions whose end offsets keep increasing
	uint32_t maxPartition = 0, prev = 0;
	for(size_t a = 0; a < perPartition.size(); a++, maxPartition++)
	{
		if(perPartition[a] == prev) break;
		prev = perPartition[a];
	}
	// createHeaders (NpImmediateMode.cpp:159): up to 4 consecutive descs of one type
	out.headerStart.clear();
	out.headerStride.clear();
	uint32_t cur = 0;
	uint32_t maxJ = n == 0 ? 0 : perPartition[0];
	for(uint32_t a = 0; a < uint32_t(n);)
	{
		out.headerStart.push_back(a);
		const uint32_t loopMax = std::min(maxJ - a, 4u);
		uint32_t j = 0;
		if(loopMax > 0)
		{
			j = 1;
			if(cur < maxPartition)
				for(; j < loopMax; ++j) {}
		}
		out.headerStride.push_back(j);
		if(maxJ == a + j && maxJ != uint32_t(n))
		{
			cur++;
			maxJ = perPartition[cur];
		}
		a += j;
	}
}

// ------------------------------------------------------------ friction correlation (fresh patches)
struct Correlation
{
	struct ContactPatch { int start, count, next; float restitution, staticFriction, dynamicFriction; V3 bmin, bmax; };
	ContactPatch contactPatches[256];
	int contactPatchCount = 0;
	FrictionPatch frictionPatches[32];
	V3 frictionPatchWorldNormal[32];
	int frictionPatchContactCounts[32];
	V3 patchMin[32], patchMax[32];
	int correlationListHeads[32];
	int contactID[32][2];
	int frictionPatchCount = 0;
};

void createContactPatches(Correlation& c, const ContactIn* cb, int n, float tol)
{
	if(!n) return;
	int pc = 0;
	Correlation::ContactPatch* cur = &c.contactPatches[pc];
	auto init = [&](Correlation::ContactPatch& p, int i) {
		p.start = i; p.count = 1; p.next = 0;
		p.restitution = cb[i].restitution; p.staticFriction = cb[i].staticFriction; p.dynamicFriction = cb[i].dynamicFriction;
	};
	init(c.contactPatches[pc++], 0);
	V3 mn = cb[0].p, mx = cb[0].p;
	int patchIndex = 0, count = 1;
	for(int i = 1; i < n; i++)
	{
		const ContactIn& cc = cb[i];
		const ContactIn& pc0 = cb[patchIndex];
		if(cc.staticFriction == pc0.staticFriction && cc.dynamicFriction == pc0.dynamicFriction && cc.restitution == pc0.restitution &&
		   dotS(cc.n, pc0.n) >= tol)
		{
			mn = vmin(mn, cc.p);
			mx = vmax(mx, cc.p);
			count++;
		}
		else
		{
			patchIndex = i;
			cur->count = count;
			count = 1;
			cur->bmin = mn; cur->bmax = mx;
			cur = &c.contactPatches[pc];
			init(c.contactPatches[pc++], i);
			mn = cc.p; mx = cc.p;
		}
	}
	if(count != 1) cur->count = count;
	cur->bmin = mn; cur->bmax = mx;
	c.contactPatchCount = pc;
}

// getFrictionPatches (lowleveldynamics/src/DyContactPrepShared.h:73): last
// frame's patches that are not broken, have anchors, still face each other
// (body normals within PXC_SAME_NORMAL) and whose anchors have not separated
// along the normal by the correlation distance start the patch list, without
// contacts yet.
void getFrictionPatches(Correlation& c, const FrictionPatch* prev, int count, const Tr& f0, const Tr& f1, float correlationDistance)
{
	if(!prev || !count) return;
	const Q qinv = qConj(f0.q);
	Tr b1to0;
	b1to0.p = qRotateS(qinv, sub(f1.p, f0.p));
	b1to0.q = qMulS(qinv, f1.q);
	for(int k = 0; k < count; k++)
	{
		const FrictionPatch& patch = prev[k];
		if(patch.broken || patch.anchorCount == 0) continue;
		if(!(dotS(patch.body0Normal, qRotateS(b1to0.q, patch.body1Normal)) > 0.999f)) continue;
		bool separated = false;
		for(int a = 0; a < patch.anchorCount; a++)
		{
			const V3 p1in0 = add(qRotateS(b1to0.q, patch.body1Anchors[a]), b1to0.p);
			if(!(fabsf(dotS(sub(patch.body0Anchors[a], p1in0), patch.body0Normal)) < correlationDistance)) { separated = true; break; }
		}
		if(separated) continue;
		if(c.frictionPatchCount == 32) return;
		const int i = c.frictionPatchCount++;
		c.contactID[i][0] = 0xffff;
		c.contactID[i][1] = 0xffff;
		c.frictionPatchWorldNormal[i] = qRotateS(f0.q, patch.body0Normal);
		c.frictionPatchContactCounts[i] = 0;
		c.patchMin[i] = v3(FLT_MAX, FLT_MAX, FLT_MAX);     // PxBounds3::setEmpty
		c.patchMax[i] = v3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
		c.correlationListHeads[i] = -1;
		c.frictionPatches[i] = patch;
	}
}

void correlatePatches(Correlation& c, const ContactIn* cb, const Tr& f0, const Tr& f1, float tol)
{
	int fpc = c.frictionPatchCount;
	for(int i = 0; i < c.contactPatchCount; i++)
	{
		Correlation::ContactPatch& cp = c.contactPatches[i];
		const V3 n = cb[cp.start].n;
		int j = 0;
		for(; j < fpc && ((dotS(n, c.frictionPatchWorldNormal[j]) < tol) || c.frictionPatches[j].restitution != cp.restitution ||
		                  c.frictionPatches[j].staticFriction != cp.staticFriction || c.frictionPatches[j].dynamicFriction != cp.dynamicFriction);
		    j++)
			;
		if(j == fpc)
		{
			if(j == 32) continue;
			FrictionPatch& fp = c.frictionPatches[fpc];
			fp.body0Normal = qRotateInvS(f0.q, n);
			fp.body1Normal = qRotateInvS(f1.q, n);
			fp.relativeQuat = qMulS(qConj(f0.q), f1.q);
			fp.anchorCount = 0;
			fp.broken = 0;
			fp.staticFriction = cp.staticFriction; fp.dynamicFriction = cp.dynamicFriction; fp.restitution = cp.restitution;
			c.frictionPatchWorldNormal[j] = n;
			c.frictionPatchContactCounts[fpc] = cp.count;
			c.patchMin[fpc] = cp.bmin; c.patchMax[fpc] = cp.bmax;
			c.contactID[fpc][0] = 0xffff;
			c.contactID[fpc][1] = 0xffff;
			fpc++;
			cp.next = -1;
		}
		else
		{
			c.patchMin[j] = vmin(c.patchMin[j], cp.bmin);
			c.patchMax[j] = vmax(c.patchMax[j], cp.bmax);
			c.frictionPatchContactCounts[j] += cp.count;
			cp.next = c.correlationListHeads[j];
		}
		c.correlationListHeads[j] = i;
	}
	c.frictionPatchCount = fpc;
}

V3 trTransformS(const Tr& t, V3 v) { return add(qRotateS(t.q, v), t.p); }
V3 trTransformInvS(const Tr& t, V3 v) { return qRotateInvS(t.q, sub(v, t.p)); }

void growPatches(Correlation& c, const ContactIn* cb, const Tr& f0, const Tr& f1, float thr)
{
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		FrictionPatch& fp = c.frictionPatches[i];
		if(fp.anchorCount == 2 || c.correlationListHeads[i] == -1)
		{
			const V3 d = sub(c.patchMax[i], c.patchMin[i]);
			const float diag = lenSqS(d);
			const float an = lenSqS(sub(fp.body0Anchors[0], fp.body0Anchors[1]));
			if(c.frictionPatchContactCounts[i] == 0 || (an * 4.0f) >= diag) continue;
			fp.anchorCount = 0;
		}
		V3 wa[2];
		int ac = 0;
		float pointDistSq = 0.0f, d0, d1;
		if(fp.anchorCount == 1) wa[ac++] = trTransformS(f0, fp.body0Anchors[0]);
		const float eps = 1e-8f;
		for(int patch = c.correlationListHeads[i]; patch != -1; patch = c.contactPatches[patch].next)
		{
			const Correlation::ContactPatch& cp = c.contactPatches[patch];
			for(int j = 0; j < cp.count; j++)
			{
				const V3 wp = cb[cp.start + j].p;
				if(cb[cp.start + j].sep < thr)
				{
					switch(ac)
					{
					case 0:
						c.contactID[i][0] = cp.start + j;
						wa[0] = wp;
						ac++;
						break;
					case 1:
						pointDistSq = lenSqS(sub(wp, wa[0]));
						if(pointDistSq > eps) { c.contactID[i][1] = cp.start + j; wa[1] = wp; ac++; }
						break;
					default:
						d0 = lenSqS(sub(wp, wa[0]));
						d1 = lenSqS(sub(wp, wa[1]));
						if(d0 > d1)
						{
							if(d0 > pointDistSq) { c.contactID[i][1] = cp.start + j; wa[1] = wp; pointDistSq = d0; }
						}
						else if(d1 > pointDistSq) { c.contactID[i][0] = cp.start + j; wa[0] = wp; pointDistSq = d1; }
					}
				}
			}
		}
		for(int j = fp.anchorCount; j < ac; j++)
		{
			fp.body0Anchors[j] = trTransformInvS(f0, wa[j]);
			fp.body1Anchors[j] = trTransformInvS(f1, wa[j]);
		}
		if(ac == 0) fp.body0Anchors[0] = fp.body1Anchors[0] = zero3();
		fp.anchorCount = ac;
	}
}

// ------------------------------------------------------------ rows
struct Rows
{
	std::vector<ConstraintRows> cons;
	std::vector<PatchRows> patches;
	std::vector<PointRow> points;
	std::vector<FrictionRow> friction;
};

float constructPoint(const M33& s0, const M33& s1, float imn0, float imn1, V3 p0, V3 p1, V3 n, float nv0, float nv1, V3 av0, V3 av1,
                     float invDtp8, float invStepDt, float totalDt, float invTotalDt, float restitution, float bounce, const ContactIn& ct,
                     bool kin0, bool kin1, PointRow& row)
{
	const float zero = 0.0f;
	const float cTarget = dotA(n, zero3());  // targetVel is zero in immediate mode
	const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
	V3 raXn = cross(ra, n), rbXn = cross(rb, n);
	const float angV0 = dotA(raXn, av0), angV1 = dotA(rbXn, av1);
	const float vrel1 = nv0 + angV0, vrel2 = nv1 + angV1;
	const float vrel = vrel1 - vrel2;
	// offsetSlop == 0: raXn/rbXn are kept unless 0 > |.| (never)
	const V3 ri0 = m33MulV(s0, raXn), ri1 = m33MulV(s1, rbXn);
	const float i0 = dotA(ri0, ri0) * 1.0f, i1 = dotA(ri1, ri1) * 1.0f;
	const float resp0 = imn0 + i0, resp1 = i1 - imn1;
	const float unitResponse = resp0 + resp1;
	const float penetration = ct.sep - 0.0f;
	const bool isSeparated = penetration > zero;
	const float penInvDt = penetration * invTotalDt;
	const bool isGreater2 = (restitution > zero && bounce > vrel) && (-vrel > penInvDt);
	const float ratio = totalDt + (isGreater2 ? penetration / vrel : -totalDt);
	const float recipResponse = unitResponse > zero ? 1.0f / unitResponse : zero;
	const float biasCoeff = -(isSeparated ? invStepDt : invDtp8);
	const float velMultiplier = recipResponse;
	float totalError = penetration;
	float targetVelocity = cTarget + (isGreater2 ? (-vrel) * restitution : zero);
	totalError = targetVelocity * ratio + totalError;
	if(kin0) targetVelocity = targetVelocity - vrel1;
	if(kin1) targetVelocity = targetVelocity + vrel2;
	row.raXnI = ri0;
	row.rbXnI = ri1;
	row.velMultiplier = velMultiplier;
	row.separation = totalError;
	row.biasCoefficient = biasCoeff;
	row.targetVelocity = targetVelocity;
	row.recipResponse = recipResponse;
	row.maxImpulse = FLT_MAX;
	row.force = 0.0f;
	return penetration;
}

// prev / prevCount: the friction patches this constraint left last frame
// (frictionPtr / frictionCount; none for a fresh pair).
void prepConstraint(int ci, const ContactIn* contacts, int nbContacts, int a, int b, const BodyVel* vels, const BodyTx* txs, const BodyData* datas,
                    const Tr& f0, const Tr& f1, float invStepDt, float invTotalDt, float totalDt, float stepDt, float bounce, float fricOffset,
                    float correlationDistance, float biasCoefficient, const FrictionPatch* prev, int prevCount, Rows& rows)
{
	ConstraintRows cr;
	cr.bodyA = a; cr.bodyB = b;
	cr.patchStart = int(rows.patches.size());
	cr.nbPatches = 0;
	cr.block = false;
	if(nbContacts == 0) { rows.cons[ci] = cr; return; }
	Correlation c;
	getFrictionPatches(c, prev, prevCount, f0, f1, correlationDistance);
	createContactPatches(c, contacts, nbContacts, 0.999f);
	correlatePatches(c, contacts, f0, f1, 0.999f);
	growPatches(c, contacts, f0, f1, fricOffset + 0.0f);

	const BodyData& d0 = datas[a];
	const BodyData& d1 = datas[b];
	const bool kin0 = vels[a].kinematic, kin1 = vels[b].kinematic;
	const float invMass0 = 1.0f * d0.invMass;
	const float invMass1 = (-1.0f) * d1.invMass;   // nDom1 * invMass1
	const float maxPenBias = std::max(d0.penBiasClamp, d1.penBiasClamp);
	const V3 p0 = f0.p, p1 = f1.p;
	const V3 lv0 = d0.origLin, lv1 = d1.origLin, av0 = d0.origAng, av1 = d1.origAng;
	const M33& s0 = txs[a].sqrtInvInertia;
	const M33& s1 = txs[b].sqrtInvInertia;
	const float invDt = invStepDt, dt = stepDt;
	const float scale_ = std::min(0.8f, biasCoefficient);
	const float p8 = scale_;
	const float invDtp8 = invDt * p8;
	const float frictionBiasScale = invDt * scale_;
	(void)dt;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		const int count = c.frictionPatchContactCounts[i];
		if(count == 0) continue;
		const FrictionPatch& fp = c.frictionPatches[i];
		const int first = c.correlationListHeads[i];
		const ContactIn& base0 = contacts[c.contactPatches[first].start];
		PatchRows pr;
		pr.invMass0 = invMass0;
		pr.invMass1 = -invMass1;
		pr.angDom0 = 1.0f; pr.angDom1 = 1.0f;
		const V3 n = contacts[c.contactPatches[c.correlationListHeads[i]].start].n;
		const float nLenSq = dotA(n, n);
		const float nv0 = dotA(lv0, n), nv1 = dotA(lv1, n);
		const float imn0 = invMass0 * nLenSq, imn1 = invMass1 * nLenSq;
		pr.normal = n;
		pr.maxPenBias = base0.restitution < 0.0f ? -FLT_MAX : maxPenBias;
		pr.pointStart = int(rows.points.size());
		float maxPenetration = FLT_MAX;
		for(int patch = c.correlationListHeads[i]; patch != -1; patch = c.contactPatches[patch].next)
		{
			const Correlation::ContactPatch& cp = c.contactPatches[patch];
			for(int j = 0; j < cp.count; j++)
			{
				PointRow row;
				maxPenetration = fmin_(maxPenetration, constructPoint(s0, s1, imn0, imn1, p0, p1, n, nv0, nv1, av0, av1, invDtp8, invDt, totalDt,
				                                                      invTotalDt, base0.restitution, bounce, contacts[cp.start + j], kin0, kin1, row));
				rows.points.push_back(row);
			}
		}
		pr.nbPoints = int(rows.points.size()) - pr.pointStart;
		pr.staticFriction = base0.staticFriction;
		pr.dynamicFriction = base0.dynamicFriction;
		const bool haveFriction = fp.anchorCount != 0;
		pr.frictionStart = int(rows.friction.size());
		pr.nbFriction = haveFriction ? fp.anchorCount * 2 : 0;
		if(haveFriction)
		{
			const V3 linVrel = sub(lv0, lv1);
			const V3 t0f1 = v3(0.0f, -n.z, n.y), t0f2 = v3(-n.y, n.x, 0.0f);
			const V3 t0Fallback = 0.70710678f > fabsf(n.x) ? t0f1 : t0f2;
			V3 t0 = sub(linVrel, scale(n, dotA(n, linVrel)));
			t0 = dotA(t0, t0) > 0.0001f ? t0 : t0Fallback;
			t0 = normalizeA(t0);
			const V3 t1 = normalizeA(cross(n, t0));
			const float nv00 = dotA(lv0, t0), nv01 = dotA(lv1, t0), nv10 = dotA(lv0, t1), nv11 = dotA(lv1, t1);
			const V3 relTr = sub(p0, p1);
			const float frictionScale = fp.anchorCount == 2 ? 0.5f : 1.0f;
			for(int j = 0; j < fp.anchorCount; j++)
			{
				const V3 ra = qRotate(f0.q, fp.body0Anchors[j]);
				const V3 rb = qRotate(f1.q, fp.body1Anchors[j]);
				const V3 error = add(sub(ra, rb), relTr);
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					FrictionRow fr;
					const V3 raXn = cross(ra, t), rbXn = cross(rb, t);
					const V3 ri0 = m33MulV(s0, raXn), ri1 = m33MulV(s1, rbXn);
					const float resp0 = imn0 + dotA(ri0, ri0) * 1.0f;
					const float resp1 = dotA(ri1, ri1) * 1.0f - imn1;
					const float unitResponse = resp0 + resp1;
					const float velMultiplier = unitResponse > 0.0f ? p8 / unitResponse : 0.0f;
					float targetVel = dotA(zero3(), t);
					if(kin0) targetVel = targetVel - ((dir == 0 ? nv00 : nv10) + dotA(raXn, av0));
					if(kin1) targetVel = targetVel + ((dir == 0 ? nv01 : nv11) + dotA(rbXn, av1));
					fr.normal = t;
					fr.error = dotA(error, t);
					fr.raXnI = ri0;
					fr.targetVel = targetVel;
					fr.rbXnI = ri1;
					fr.velMultiplier = velMultiplier;
					fr.appliedForce = 0.0f;
					fr.frictionScale = frictionScale;
					fr.biasScale = frictionBiasScale;
					rows.friction.push_back(fr);
				}
			}
		}
		// the patch is written to the friction memory in this order
		// (createFinalizeSolverContactsStep, DyTGSContactPrep.cpp:1391-1398)
		pr.anchorCount = fp.anchorCount;
		pr.brokenSlot = int(cr.written.size());
		pr.broken = 0;
		cr.written.push_back(fp);
		rows.patches.push_back(pr);
		cr.nbPatches++;
	}
	rows.cons[ci] = std::move(cr);
}

// ------------------------------------------------------------ 4-wide block path, one lane
// PxCreateContactConstraintsTGS sends every header of stride 4 whose four
// descriptors hold at most 64 contacts through createFinalizeSolverContacts4Step
// (lowleveldynamics/src/DyTGSContactPrepBlock.cpp:1398), which builds the rows of
// the four constraints side by side in SIMD lanes
// (setupFinalizeSolverConstraints4Step, :219), and PxSolveConstraintsTGS solves
// them with solveContact4_Block (:2280).  The lanes never mix: a lane whose
// constraint has fewer patches, contacts or anchors than another is padded with
// rows of zero response that leave every value unchanged.  So each lane is the
// per-constraint computation below, with the block path's own arithmetic:
// sums in the order of its multiply-add chains, the transposed inertia product,
// the unit normal assumed in the solve, friction coefficients pre-scaled by the
// anchor count and the friction clamp carried across a patch's anchors.

// x*x' + y*y' then + z*z' (V4MulAdd(z, .., V4MulAdd(y, .., V4Mul(x, ..))))
inline float dotXYZ(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// z*z' + y*y' then + x*x' (V4MulAdd(x, .., V4MulAdd(y, .., V4Mul(z, ..))))
inline float dotZYX(V3 a, V3 b) { return (a.z * b.z + a.y * b.y) + a.x * b.x; }
// the block path's sqrtInvInertia product: lane-transposed columns dotted with v
inline V3 m33TMulXYZ(const M33& m, V3 v) { return v3(dotXYZ(m.c0, v), dotXYZ(m.c1, v), dotXYZ(m.c2, v)); }
// QuatRotate4V (physx/include/foundation/PxVecQuat.h:208): V4Dot3 = (x + y) + z
inline V3 qRotate4V(Q q, V3 v)
{
	const float w2 = q.w * q.w + (-0.5f);
	const V3 a = scale(v, w2);
	const V3 u = qv(q);
	const V3 temp = scaleAdd(cross(u, v), q.w, a);
	return scale(scaleAdd(u, dotXYZ(u, v), temp), 2.0f);
}

// One lane of setupFinalizeSolverConstraints4Step.  blockDynamic: some
// constraint of the header has a dynamic body B (the header-wide isDynamic);
// kinematic bodies B add their velocity terms as the reference's hasKinematic
// branch does.
void prepConstraintBlock(int ci, const ContactIn* contacts, int nbContacts, int a, int b, const BodyVel* vels, const BodyTx* txs,
                         const BodyData* datas, const Tr& f0, const Tr& f1, float invStepDt, float invTotalDt, float totalDt, float bounce,
                         float fricOffset, float correlationDistance, float biasCoefficient, bool blockDynamic, const FrictionPatch* prev,
                         int prevCount, Rows& rows)
{
	ConstraintRows cr;
	cr.bodyA = a; cr.bodyB = b;
	cr.patchStart = int(rows.patches.size());
	cr.nbPatches = 0;
	cr.block = true;
	if(nbContacts == 0) { rows.cons[ci] = cr; return; }
	Correlation c;
	getFrictionPatches(c, prev, prevCount, f0, f1, correlationDistance);
	createContactPatches(c, contacts, nbContacts, 0.999f);
	correlatePatches(c, contacts, f0, f1, 0.999f);
	growPatches(c, contacts, f0, f1, fricOffset + 0.0f);
	// The block path then drops the patches that received no contact
	// (createFinalizeSolverContacts4Step, DyTGSContactPrepBlock.cpp:1452-1466)
	// by moving the later list heads and contact counts down -- but not the
	// patches themselves, so a later patch's contacts pair with an earlier
	// patch's anchors, and the earlier patches are the ones written out.
	for(int p = c.frictionPatchCount; p > 0; --p)
		if(c.correlationListHeads[p - 1] == -1)
		{
			for(int p2 = p; p2 < c.frictionPatchCount; ++p2)
			{
				c.correlationListHeads[p2 - 1] = c.correlationListHeads[p2];
				c.frictionPatchContactCounts[p2 - 1] = c.frictionPatchContactCounts[p2];
			}
			c.frictionPatchCount--;
		}

	const BodyData& d0 = datas[a];
	const BodyData& d1 = datas[b];
	// kinematicScale: 1 for a solver body flagged kinematic (static bodies are,
	// PxConstructStaticSolverBodyTGS); the descriptors of this path carry no
	// eKINEMATIC_BODY state, so the hasKinematic branch is never taken
	const float kin0 = vels[a].kinematic ? 1.0f : 0.0f;
	const float kin1 = vels[b].kinematic ? 1.0f : 0.0f;
	const bool bKinematic = false;
	const float invMass0D0 = 1.0f * d0.invMass, invMass1D1 = 1.0f * d1.invMass;
	const float angDom0 = 1.0f, angDom1 = 1.0f;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 p0 = f0.p, p1 = f1.p;
	const V3 lv0 = d0.origLin, lv1 = d1.origLin, av0 = d0.origAng, av1 = d1.origAng;
	const M33& s0 = txs[a].sqrtInvInertia;
	const M33& s1 = txs[b].sqrtInvInertia;
	const float invDt = invStepDt;
	const float p8 = std::min(0.8f, biasCoefficient);
	const float frictionBiasScale = invDt * p8;
	const float invDtp8 = invDt * p8;
	const V3 vrel = sub(lv0, lv1);
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		const int count = c.frictionPatchContactCounts[i];
		if(count == 0) continue;
		const FrictionPatch& fp = c.frictionPatches[i];
		const ContactIn& base0 = contacts[c.contactPatches[c.correlationListHeads[i]].start];
		const float restitution = -base0.restitution;   // the block setup negates restitution
		PatchRows pr;
		pr.invMass0 = invMass0D0;
		pr.invMass1 = invMass1D1;
		pr.angDom0 = angDom0; pr.angDom1 = angDom1;
		const V3 n = base0.n;
		pr.normal = n;
		pr.maxPenBias = maxPenBias;
		const float norVel0 = dotXYZ(n, lv0), norVel1 = dotXYZ(n, lv1);
		const float relNorVel = norVel0 - norVel1;
		pr.pointStart = int(rows.points.size());
		for(int patch = c.correlationListHeads[i]; patch != -1; patch = c.contactPatches[patch].next)
		{
			const Correlation::ContactPatch& cp = c.contactPatches[patch];
			for(int j = 0; j < cp.count; j++)
			{
				const ContactIn& ct = contacts[cp.start + j];
				PointRow row;
				const float cTargetNorVel = dotZYX(zero3(), n);   // contact target velocity is zero
				const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
				const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
				const float relAngVel0 = dotXYZ(raXn, av0), relAngVel1 = dotXYZ(rbXn, av1);
				// offsetSlop == 0: no raXn/rbXn component is cleared
				const V3 dav0 = m33TMulXYZ(s0, raXn);
				const float dot0 = dotZYX(dav0, dav0);
				float unitResponse = dot0 * angDom0 + invMass0D0;
				const float vrel0 = norVel0 + relAngVel0, vrel1 = norVel1 + relAngVel1;
				V3 dav1 = zero3();
				if(blockDynamic)
				{
					dav1 = m33TMulXYZ(s1, rbXn);
					const float dot1 = dotZYX(dav1, dav1);
					unitResponse = unitResponse + (dot1 * angDom1 + invMass1D1);
				}
				const float vrelD = vrel0 - vrel1;
				float penetration = ct.sep - 0.0f;
				const float penInvDt = penetration * invTotalDt;
				const bool isSeparated = penetration > 0.0f;
				const bool isGreater2 = (0.0f > restitution && bounce > vrelD) && (-vrelD > penInvDt);
				const float ratio = isGreater2 ? totalDt + penetration / vrelD : 0.0f;
				const float recipResponse = unitResponse > 0.0f ? 1.0f / unitResponse : 0.0f;
				// restitution >= 0: not a compliant contact
				const float velMultiplier = recipResponse;
				const float scaledBias = -(isSeparated ? invDt : invDtp8);
				const float targetVelocity = (vrel1 * kin1 + (isGreater2 ? vrelD * restitution : 0.0f)) - vrel0 * kin0;
				penetration = targetVelocity * ratio + penetration;
				row.raXnI = dav0;
				row.rbXnI = dav1;
				row.velMultiplier = velMultiplier;
				row.targetVelocity = cTargetNorVel + targetVelocity;
				row.separation = penetration;
				row.biasCoefficient = scaledBias;
				row.recipResponse = recipResponse;
				row.maxImpulse = FLT_MAX;
				row.force = 0.0f;
				rows.points.push_back(row);
			}
		}
		pr.nbPoints = int(rows.points.size()) - pr.pointStart;
		const float coeff = fp.anchorCount == 2 ? 0.5f : 1.0f;
		pr.staticFriction = base0.staticFriction * coeff;
		pr.dynamicFriction = base0.dynamicFriction * coeff;
		pr.frictionStart = int(rows.friction.size());
		pr.nbFriction = fp.anchorCount * 2;
		if(fp.anchorCount)
		{
			const bool cond = 0.70710678f > fabsf(n.x);
			const V3 fallback = cond ? v3(0.0f, -n.z, n.y) : v3(-n.y, n.x, 0.0f);
			const V3 vs = v3(vrel.x - n.x * relNorVel, vrel.y - n.y * relNorVel, vrel.z - n.z * relNorVel);
			V3 t0 = dotZYX(vs, vs) > 0.0001f ? vs : fallback;
			const float recipLen = 1.0f / sqrtf(dotXYZ(t0, t0));
			t0 = scale(t0, recipLen);
			const V3 t1 = cross(n, t0);
			for(int j = 0; j < fp.anchorCount; j++)
			{
				const V3 ra = qRotate4V(f0.q, fp.body0Anchors[j]);
				const V3 rb = qRotate4V(f1.q, fp.body1Anchors[j]);
				const V3 error = sub(add(ra, p0), add(rb, p1));
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					const V3 raXn = cross(ra, t);
					const V3 dav0 = m33TMulXYZ(s0, raXn);
					float resp = dotXYZ(dav0, dav0) * angDom0 + invMass0D0;
					const float tVel0 = dotXYZ(t, lv0);
					const float vrel0 = ((tVel0 + raXn.x * av0.x) + raXn.y * av0.y) + raXn.z * av0.z;
					V3 dav1 = zero3();
					float vrel1 = 0.0f;
					if(blockDynamic || bKinematic)
					{
						const V3 rbXn = cross(rb, t);
						if(blockDynamic)
						{
							dav1 = m33TMulXYZ(s1, rbXn);
							resp = resp + (dotXYZ(dav1, dav1) * angDom1 + invMass1D1);
						}
						const float tVel1 = dotXYZ(t, lv1);
						vrel1 = ((tVel1 + rbXn.x * av1.x) + rbXn.y * av1.y) + rbXn.z * av1.z;
					}
					FrictionRow fr;
					fr.normal = t;
					fr.raXnI = dav0;
					fr.rbXnI = dav1;
					fr.velMultiplier = resp > 0.0f ? p8 / resp : 0.0f;
					fr.error = dotXYZ(t, error);
					fr.targetVel = (vrel1 * kin1 + dotXYZ(t, zero3())) - vrel0 * kin0;
					fr.biasScale = frictionBiasScale;
					fr.frictionScale = 1.0f;
					fr.appliedForce = 0.0f;
					rows.friction.push_back(fr);
				}
			}
		}
		// written in patch order; the broken-flag slot is completed per header
		pr.anchorCount = fp.anchorCount;
		pr.brokenSlot = int(cr.written.size());
		pr.broken = 0;
		cr.written.push_back(fp);
		rows.patches.push_back(pr);
		cr.nbPatches++;
	}
	rows.cons[ci] = std::move(cr);
}

// ------------------------------------------------------------ solve
void solveConstraint(const ConstraintRows& cr, Rows& rows, BodyVel* vels, float minPen, float elapsed)
{
	BodyVel& b0 = vels[cr.bodyA];
	BodyVel& b1 = vels[cr.bodyB];
	V3 lin0 = b0.lin, lin1 = b1.lin, ang0 = b0.ang, ang1 = b1.ang;
	const V3 angM0 = b0.dAng, angM1 = b1.dAng;
	const V3 relMotion = sub(b0.dLin, b1.dLin);
	for(int p = 0; p < cr.nbPatches; p++)
	{
		PatchRows& pr = rows.patches[cr.patchStart + p];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1;
		const float angD0 = pr.angDom0, angD1 = pr.angDom1;
		const V3 nIM0 = scale(n, invMassA), nIM1 = scale(n, invMassB);
		const float deltaV = dotA(relMotion, n);
		float accumulated = 0.0f;
		for(int i = 0; i < pr.nbPoints; i++)
		{
			PointRow& c = rows.points[pr.pointStart + i];
			const float angDelta0 = dotA(angM0, c.raXnI), angDelta1 = dotA(angM1, c.rbXnI);
			const float deltaAng = angDelta0 - angDelta1;
			const float targetVel = c.targetVelocity;
			const float deltaBias = (deltaV + deltaAng) - targetVel * elapsed;
			const float sep = fmax_(minPen, c.separation + deltaBias);
			const float bias = fmin_(-pr.maxPenBias, c.biasCoefficient * sep);
			const V3 v0 = add(mul(lin0, n), mul(ang0, c.raXnI));
			const V3 v1 = add(mul(lin1, n), mul(ang1, c.rbXnI));
			const float normalVel = sumElems(sub(v0, v1));
			const float biasNV = bias * c.recipResponse;
			const float lambda = biasNV - (normalVel - targetVel) * c.velMultiplier;
			const float applied = c.force;
			const float _deltaF = fmax_(lambda, -applied);
			const float _newForce = applied + _deltaF;
			const float newForce = fmin_(_newForce, c.maxImpulse);
			const float deltaF = newForce - applied;
			lin0 = scaleAdd(nIM0, deltaF, lin0);
			lin1 = negScaleSub(nIM1, deltaF, lin1);
			ang0 = scaleAdd(c.raXnI, deltaF * angD0, ang0);
			ang1 = negScaleSub(c.rbXnI, deltaF * angD1, ang1);
			c.force = newForce;
			accumulated = accumulated + newForce;
		}
		if(pr.nbFriction)
		{
			const float maxF = pr.staticFriction * accumulated;
			const float maxDynF = pr.dynamicFriction * accumulated;
			const int pairs = pr.nbFriction & 6;
			bool broken = false;
			for(int i = 0; i < pairs; i += 2)
			{
				FrictionRow& f0 = rows.friction[pr.frictionStart + i];
				FrictionRow& f1 = rows.friction[pr.frictionStart + i + 1];
				const float fs = f0.frictionScale;
				const float biasScale = f0.biasScale;
				float dv0 = (dotA(f0.raXnI, angM0) - dotA(f0.rbXnI, angM1)) + dotA(f0.normal, relMotion);
				float dv1 = (dotA(f1.raXnI, angM0) - dotA(f1.rbXnI, angM1)) + dotA(f1.normal, relMotion);
				dv0 = dv0 - f0.targetVel * elapsed;
				dv1 = dv1 - f1.targetVel * elapsed;
				const float e0 = f0.error + dv0, e1 = f1.error + dv1;
				const float bias0 = e0 * biasScale, bias1 = e1 * biasScale;
				const V3 dl00 = scale(f0.normal, invMassA), dl10 = scale(f0.normal, invMassB);
				const V3 dl01 = scale(f1.normal, invMassA), dl11 = scale(f1.normal, invMassB);
				const float nvel0 = sumElems(sub(add(mul(lin0, f0.normal), mul(ang0, f0.raXnI)), add(mul(lin1, f0.normal), mul(ang1, f0.rbXnI))));
				const float nvel1 = sumElems(sub(add(mul(lin0, f1.normal), mul(ang0, f1.raXnI)), add(mul(lin1, f1.normal), mul(ang1, f1.rbXnI))));
				const float tmp10 = f0.appliedForce - (bias0 - f0.targetVel) * f0.velMultiplier;
				const float tmp11 = f1.appliedForce - (bias1 - f1.targetVel) * f1.velMultiplier;
				const float ti0 = tmp10 - nvel0 * f0.velMultiplier;
				const float ti1 = tmp11 - nvel1 * f1.velMultiplier;
				const float total = sqrtf(ti0 * ti0 + ti1 * ti1);
				const bool clamp = total > fs * maxF;
				broken = broken || clamp;
				const float totalClamped = clamp ? fmin_(fs * maxDynF, total) : total;
				const float ratio = total > 0.0f ? totalClamped / total : 0.0f;
				const float nf0 = ti0 * ratio, nf1 = ti1 * ratio;
				const float df0 = nf0 - f0.appliedForce, df1 = nf1 - f1.appliedForce;
				lin0 = scaleAdd(dl00, df0, scaleAdd(dl01, df1, lin0));
				lin1 = negScaleSub(dl10, df0, negScaleSub(dl11, df1, lin1));
				ang0 = scaleAdd(f0.raXnI, df0 * angD0, scaleAdd(f1.raXnI, df1 * angD0, ang0));
				ang1 = negScaleSub(f0.rbXnI, df0 * angD1, negScaleSub(f1.rbXnI, df1 * angD1, ang1));
				f0.appliedForce = nf0;
				f1.appliedForce = nf1;
			}
			pr.broken = broken;
		}
	}
	b0.lin = lin0; b1.lin = lin1; b0.ang = ang0; b1.ang = ang1;
}

// One lane of solveContact4_Block (DyTGSContactPrepBlock.cpp:2280).  The linear
// part of the normal velocity is carried as relVel1 += (invMassA + invMassB) *
// deltaF and the linear velocities move once per patch; friction uses the
// pre-scaled coefficients, a 1e-5 allowance on the static bound, and once one
// anchor pair of a patch exceeds it the rest of the patch is clamped to the
// dynamic bound too.
void solveConstraintBlock(const ConstraintRows& cr, Rows& rows, BodyVel* vels, float minPen, float elapsed)
{
	BodyVel& b0 = vels[cr.bodyA];
	BodyVel& b1 = vels[cr.bodyB];
	V3 lin0 = b0.lin, lin1 = b1.lin, ang0 = b0.ang, ang1 = b1.ang;
	const V3 angD0v = b0.dAng, angD1v = b1.dAng;
	const V3 linDelta = sub(b0.dLin, b1.dLin);
	for(int p = 0; p < cr.nbPatches; p++)
	{
		PatchRows& pr = rows.patches[cr.patchStart + p];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1;
		const float sumInvMass = invMassA + invMassB;
		const float angD0 = pr.angDom0, angD1 = pr.angDom1;
		float relVel1 = dotXYZ(lin0, n) - dotXYZ(lin1, n);
		const float deltaNormalV = dotXYZ(linDelta, n);
		float accumDeltaF = 0.0f, accumulated = 0.0f;
		for(int i = 0; i < pr.nbPoints; i++)
		{
			PointRow& c = rows.points[pr.pointStart + i];
			const float applied = c.force;
			const float normalVel = relVel1 + (dotXYZ(c.raXnI, ang0) - dotXYZ(c.rbXnI, ang1));
			const float deltaAng = dotXYZ(angD0v, c.raXnI) - dotXYZ(angD1v, c.rbXnI);
			const float targetVel = c.targetVelocity;
			const float deltaBias = (deltaNormalV + deltaAng) - targetVel * elapsed;
			const float sep = fmax_(minPen, c.separation + deltaBias);
			const float bias = fmin_(-pr.maxPenBias, c.biasCoefficient * sep);
			const float tVelBias = bias * c.recipResponse;
			const float _deltaF = fmax_(tVelBias - (normalVel - targetVel) * c.velMultiplier, -applied);
			const float newForce = fmin_(applied + _deltaF, c.maxImpulse);
			const float deltaF = newForce - applied;
			accumDeltaF = accumDeltaF + deltaF;
			const float angDeltaF0 = deltaF * angD0, angDeltaF1 = deltaF * angD1;
			relVel1 = sumInvMass * deltaF + relVel1;
			ang0 = add(scale(c.raXnI, angDeltaF0), ang0);
			ang1 = sub(ang1, scale(c.rbXnI, angDeltaF1));
			c.force = newForce;
			accumulated = accumulated + newForce;
		}
		const float accIM0 = accumDeltaF * invMassA, accIM1 = accumDeltaF * invMassB;
		lin0 = add(scale(n, accIM0), lin0);
		lin1 = sub(lin1, scale(n, accIM1));
		if(pr.nbFriction)
		{
			const float maxF = pr.staticFriction * accumulated + 1e-5f;
			const float maxDynF = pr.dynamicFriction * accumulated;
			bool broken = false;
			for(int i = 0; i < pr.nbFriction; i += 2)
			{
				FrictionRow& f0 = rows.friction[pr.frictionStart + i];
				FrictionRow& f1 = rows.friction[pr.frictionStart + i + 1];
				const float nv0 = (dotXYZ(lin0, f0.normal) + dotXYZ(f0.raXnI, ang0)) - (dotXYZ(lin1, f0.normal) + dotXYZ(f0.rbXnI, ang1));
				const float nv1 = (dotXYZ(lin0, f1.normal) + dotXYZ(f1.raXnI, ang0)) - (dotXYZ(lin1, f1.normal) + dotXYZ(f1.rbXnI, ang1));
				const float dv0 = dotXYZ(linDelta, f0.normal), dv1 = dotXYZ(linDelta, f1.normal);
				const float da0 = dotXYZ(angD0v, f0.raXnI) - dotXYZ(angD1v, f0.rbXnI);
				const float da1 = dotXYZ(angD0v, f1.raXnI) - dotXYZ(angD1v, f1.rbXnI);
				const float e0 = f0.error + ((dv0 + da0) - f0.targetVel * elapsed);
				const float e1 = f1.error + ((dv1 + da1) - f1.targetVel * elapsed);
				const float bias0 = e0 * f0.biasScale, bias1 = e1 * f1.biasScale;
				const float tmp10 = f0.appliedForce - (bias0 - f0.targetVel) * f0.velMultiplier;
				const float tmp11 = f1.appliedForce - (bias1 - f1.targetVel) * f1.velMultiplier;
				const float ti0 = tmp10 - nv0 * f0.velMultiplier;
				const float ti1 = tmp11 - nv1 * f1.velMultiplier;
				const float total = sqrtf(ti0 * ti0 + ti1 * ti1);
				broken = broken || total > maxF;
				const float totalClamped = broken ? fmin_(total, maxDynF) : total;
				const float ratio = total > 0.0f ? totalClamped / total : 0.0f;
				const float nf0 = ti0 * ratio, nf1 = ti1 * ratio;
				const float df0 = nf0 - f0.appliedForce, df1 = nf1 - f1.appliedForce;
				f0.appliedForce = nf0;
				f1.appliedForce = nf1;
				const float im00 = df0 * invMassA, im10 = df0 * invMassB, ad00 = df0 * angD0, ad10 = df0 * angD1;
				const float im01 = df1 * invMassA, im11 = df1 * invMassB, ad01 = df1 * angD0, ad11 = df1 * angD1;
				lin0 = add(scale(f0.normal, im00), add(scale(f1.normal, im01), lin0));
				lin1 = sub(sub(lin1, scale(f1.normal, im11)), scale(f0.normal, im10));
				ang0 = add(scale(f0.raXnI, ad00), add(scale(f1.raXnI, ad01), ang0));
				ang1 = sub(sub(ang1, scale(f1.rbXnI, ad11)), scale(f0.rbXnI, ad10));
			}
			pr.broken = broken;
		}
	}
	b0.lin = lin0; b0.ang = ang0;
	// body B is stored only when its data index is not 0 (:2731-2750)
	if(cr.bodyB != 0) { b1.lin = lin1; b1.ang = ang1; }
}

void integrateStep(BodyVel& v, BodyTx& t, float dt)
{
	const V3 delta = scale(v.lin, dt);
	const V3 unmolested = v.ang;
	const V3 angMotion = m33MulVS(t.sqrtInvInertia, v.ang);
	const float w2 = lenSqS(angMotion);
	t.p = add(t.p, delta);
	if(w2 != 0.0f)
	{
		const float w = sqrtf(w2);
		const float vv = dt * w * 0.5f;
		float s = sinf(vv), q = cosf(vv);
		s /= w;
		const V3 pqr = scale(angMotion, s);
		const Q qv_ = {pqr.x, pqr.y, pqr.z, 0.0f};
		Q r = qMulS(qv_, t.dq);
		r.x += t.dq.x * q; r.y += t.dq.y * q; r.z += t.dq.z * q; r.w += t.dq.w * q;
		// PxQuat::getNormalized: s = 1/|q| then multiply
		const float m = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w);
		const float inv = 1.0f / m;
		t.dq.x = r.x * inv; t.dq.y = r.y * inv; t.dq.z = r.z * inv; t.dq.w = r.w * inv;
	}
	v.dAng = add(v.dAng, scale(unmolested, dt));
	v.dLin = add(v.dLin, delta);
}

Tr loadTr(const float* p)
{
	Tr t;
	t.q.x = p[0]; t.q.y = p[1]; t.q.z = p[2]; t.q.w = p[3];
	t.p = v3(p[4], p[5], p[6]);
	return t;
}
} // namespace

OX uint32_t orc_batch_constraints_tgs(const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, uint32_t nbDyn, uint32_t nbStatic,
                                      uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder)
{
	(void)nbStatic;
	BatchOut out;
	batchConstraints(bodyA, bodyB, int(n), int(nbDyn), out);
	for(size_t h = 0; h < out.headerStart.size(); h++)
	{
		outHeaderStart[h] = out.headerStart[h];
		outHeaderStride[h] = out.headerStride[h];
	}
	for(uint32_t i = 0; i < n; i++) outOrder[i] = uint32_t(out.order[i]);
	return uint32_t(out.headerStart.size());
}

// The snippet's sequence PxConstructSolverBodiesTGS ... PxIntegrateSolverBodiesTGS;
// friction is indexed by the caller's constraint index (frictionPtr / frictionCount).
uint32_t orc::tgsFrame(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA, const uint32_t* pairB,
                  uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount, const float* contacts, const float* material,
                  const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel, float bounceThreshold, float frictionOffsetThreshold,
                  float correlationDistance, float* outVel, float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder,
                  std::vector<std::vector<FrictionPatch>>* friction)
{
	std::vector<BodyVel> vels;
	std::vector<BodyTx> txs;
	std::vector<BodyData> datas;
	std::vector<Tr> poses;
	buildSolverBodies(rigid, nbDyn, staticPose, nbStatic, gravity, dt, vels, txs, datas, poses);
	BatchOut batch;
	batchConstraints(pairA, pairB, int(nbConstraints), int(nbDyn), batch);
	for(size_t h = 0; h < batch.headerStart.size(); h++)
	{
		outHeaderStart[h] = batch.headerStart[h];
		outHeaderStride[h] = batch.headerStride[h];
	}
	for(uint32_t i = 0; i < nbConstraints; i++) outOrder[i] = uint32_t(batch.order[i]);

	const float invDt = 1.0f / dt;
	const float stepDt = dt / float(nbPos);
	const float invStepDt = invDt * float(nbPos);
	// PxCreateContactConstraintsTGS(invDt = invStepDt, invTotalDt = invDt)
	const float biasCoefficient = 2.0f * sqrtf(invDt / invStepDt);
	const float totalDt = 1.0f / invDt;
	const float prepDt = 1.0f / invStepDt;
	Rows rows;
	rows.cons.resize(nbConstraints);
	// headers of stride 4 holding at most 64 contacts take the block path
	// (NpImmediateMode.cpp:1422-1444); isDynamic is per header
	std::vector<char> inBlock(nbConstraints, 0), blockDynamic(nbConstraints, 0);
	for(size_t h = 0; h < batch.headerStart.size(); h++)
	{
		if(batch.headerStride[h] != 4) continue;
		const uint32_t s = batch.headerStart[h];
		uint32_t total = 0;
		bool dyn = false;
		for(uint32_t l = 0; l < 4; l++)
		{
			const int ci = batch.order[s + l];
			if(ci < 0) continue;
			total += contactCount[ci];
			dyn = dyn || pairB[ci] < nbDyn;
		}
		if(total > 64) continue;
		for(uint32_t l = 0; l < 4; l++) { inBlock[s + l] = 1; blockDynamic[s + l] = dyn; }
	}
	std::vector<ContactIn> cin;
	for(uint32_t k = 0; k < nbConstraints; k++)
	{
		const int ci = batch.order[k];
		if(ci < 0) continue;
		cin.resize(contactCount[ci]);
		for(uint32_t c = 0; c < contactCount[ci]; c++)
		{
			const float* s = contacts + 8 * (contactStart[ci] + c);
			cin[c].n = v3(s[0], s[1], s[2]);
			cin[c].sep = s[3];
			cin[c].p = v3(s[4], s[5], s[6]);
			cin[c].staticFriction = material[3 * ci + 0];
			cin[c].dynamicFriction = material[3 * ci + 1];
			cin[c].restitution = material[3 * ci + 2];
		}
		const FrictionPatch* prev = friction && !(*friction)[ci].empty() ? (*friction)[ci].data() : nullptr;
		const int prevCount = friction ? int((*friction)[ci].size()) : 0;
		if(inBlock[k])
			prepConstraintBlock(ci, cin.data(), int(contactCount[ci]), int(pairA[ci]), int(pairB[ci]), vels.data(), txs.data(), datas.data(),
			                    poses[pairA[ci]], poses[pairB[ci]], invStepDt, invDt, totalDt, bounceThreshold, frictionOffsetThreshold,
			                    correlationDistance, biasCoefficient, blockDynamic[k] != 0, prev, prevCount, rows);
		else
			prepConstraint(ci, cin.data(), int(contactCount[ci]), int(pairA[ci]), int(pairB[ci]), vels.data(), txs.data(), datas.data(),
			               poses[pairA[ci]], poses[pairB[ci]], invStepDt, invDt, totalDt, prepDt, bounceThreshold, frictionOffsetThreshold,
			               correlationDistance, biasCoefficient, prev, prevCount, rows);
	}
	// Block headers: the broken flag of a lane's patch i goes to the written
	// patch counted by the header's earlier patch rows that had friction in any
	// lane (the block setup advances its write-back address only for those,
	// DyTGSContactPrepBlock.cpp:1218-1222).
	for(size_t h = 0; h < batch.headerStart.size(); h++)
	{
		const uint32_t s0 = batch.headerStart[h];
		if(batch.headerStride[h] != 4 || !inBlock[s0]) continue;
		int maxPatches = 0;
		for(uint32_t l = 0; l < 4; l++)
			if(batch.order[s0 + l] >= 0) maxPatches = std::max(maxPatches, rows.cons[batch.order[s0 + l]].nbPatches);
		int slot = 0;
		for(int i = 0; i < maxPatches; i++)
		{
			int maxAnchors = 0;
			for(uint32_t l = 0; l < 4; l++)
			{
				if(batch.order[s0 + l] < 0) continue;
				const ConstraintRows& cr = rows.cons[batch.order[s0 + l]];
				if(i < cr.nbPatches)
				{
					PatchRows& pr = rows.patches[cr.patchStart + i];
					pr.brokenSlot = slot;
					maxAnchors = std::max(maxAnchors, pr.anchorCount);
				}
			}
			if(maxAnchors) slot++;
		}
	}
	auto solve = [&](const ConstraintRows& cr, float minPen, float el) {
		if(cr.block) solveConstraintBlock(cr, rows, vels.data(), minPen, el);
		else solveConstraint(cr, rows, vels.data(), minPen, el);
	};
	float elapsed = 0.0f;
	for(uint32_t it = 0; it < nbPos; it++)
	{
		for(uint32_t k = 0; k < nbConstraints; k++)
			if(batch.order[k] >= 0) solve(rows.cons[batch.order[k]], -FLT_MAX, elapsed);
		for(uint32_t j = 0; j < nbDyn; j++) integrateStep(vels[j], txs[j], stepDt);
		elapsed += stepDt;
	}
	for(uint32_t it = 0; it < nbVel; it++)
		for(uint32_t k = 0; k < nbConstraints; k++)
			if(batch.order[k] >= 0) solve(rows.cons[batch.order[k]], 0.0f, elapsed);
	// write-back of the last iteration: a patch whose friction was clamped
	// marks its written friction patch broken (writeBackContact,
	// DyTGSContactPrep.cpp:1907; writeBackContact4_Block, DyTGSContactPrepBlock.cpp:2891)
	if(friction)
		for(uint32_t ci = 0; ci < nbConstraints; ci++)
		{
			ConstraintRows& cr = rows.cons[ci];
			for(int p = 0; p < cr.nbPatches; p++)
			{
				const PatchRows& pr = rows.patches[cr.patchStart + p];
				if(pr.nbFriction && pr.broken && pr.brokenSlot < int(cr.written.size())) cr.written[pr.brokenSlot].broken = 1;
			}
			(*friction)[ci] = cr.written;
		}
	finishSolverBodies(vels, txs, poses, nbDyn, outVel, outPose);
	return uint32_t(batch.headerStart.size());
}

// Same argument layout as the reference harness's pxref_tgs_solve.
OX uint32_t orc_tgs_solve(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA,
                          const uint32_t* pairB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                          const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel,
                          float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, float* outVel, float* outPose,
                          uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder, void* outBodyVelRaw, void* outTxIRaw)
{
	(void)outBodyVelRaw;
	(void)outTxIRaw;
	return tgsFrame(rigid, nbDyn, staticPose, nbStatic, pairA, pairB, nbConstraints, contactStart, contactCount, contacts, material, gravity, dt,
	                nbPos, nbVel, bounceThreshold, frictionOffsetThreshold, correlationDistance, outVel, outPose, outHeaderStart, outHeaderStride,
	                outOrder, nullptr);
}

void orc::buildSolverBodies(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const float* gravity, float dt,
                            std::vector<BodyVel>& vels, std::vector<BodyTx>& txs, std::vector<BodyData>& datas, std::vector<Tr>& poses)
{
	const uint32_t nbTotal = nbDyn + nbStatic;
	vels.assign(nbTotal, BodyVel());
	txs.assign(nbTotal, BodyTx());
	datas.assign(nbTotal, BodyData());
	poses.assign(nbTotal, Tr());
	const RigidBodyData* rb = static_cast<const RigidBodyData*>(rigid);
	const V3 g = v3(gravity[0], gravity[1], gravity[2]);
	for(uint32_t a = 0; a < nbDyn; a++)
	{
		const RigidBodyData& r = rb[a];
		V3 lv = v3(r.linVel[0], r.linVel[1], r.linVel[2]);
		V3 av = v3(r.angVel[0], r.angVel[1], r.angVel[2]);
		unconstrainedVelocity(g, dt, r.linearDamping, r.angularDamping, r.maxLinearVelocitySq, r.maxAngularVelocitySq, lv, av);
		Tr pose;
		pose.q.x = r.q[0]; pose.q.y = r.q[1]; pose.q.z = r.q[2]; pose.q.w = r.q[3];
		pose.p = v3(r.p[0], r.p[1], r.p[2]);
		poses[a] = pose;
		copyToSolverBody(lv, av, r.invMass, v3(r.invInertia[0], r.invInertia[1], r.invInertia[2]), pose, -r.maxDepenetrationVelocity,
		                 r.maxContactImpulse, r.maxAngularVelocitySq, false, vels[a], txs[a], datas[a]);
	}
	for(uint32_t s = 0; s < nbStatic; s++)
	{
		poses[nbDyn + s] = loadTr(staticPose + 7 * s);
		copyToSolverBody(zero3(), zero3(), 0.0f, zero3(), poses[nbDyn + s], -FLT_MAX, FLT_MAX, FLT_MAX, true, vels[nbDyn + s], txs[nbDyn + s],
		                 datas[nbDyn + s]);
	}
}

void orc::batchSolverConstraints(const uint32_t* bodyA, const uint32_t* bodyB, int n, int nbDyn, BatchOut& out)
{
	batchConstraints(bodyA, bodyB, n, nbDyn, out);
}

void orc::integrateSolverBody(BodyVel& v, BodyTx& t, float dt) { integrateStep(v, t, dt); }

void orc::finishSolverBodies(const std::vector<BodyVel>& vels, const std::vector<BodyTx>& txs, const std::vector<Tr>& poses, uint32_t nbDyn,
                             float* outVel, float* outPose)
{
	for(uint32_t a = 0; a < nbDyn; a++)
	{
		const V3 w = m33MulVS(txs[a].sqrtInvInertia, vels[a].ang);
		Q q = qMulS(txs[a].dq, poses[a].q);
		const float m = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
		const float inv = 1.0f / m;
		q.x *= inv; q.y *= inv; q.z *= inv; q.w *= inv;
		outVel[6 * a + 0] = vels[a].lin.x; outVel[6 * a + 1] = vels[a].lin.y; outVel[6 * a + 2] = vels[a].lin.z;
		outVel[6 * a + 3] = w.x; outVel[6 * a + 4] = w.y; outVel[6 * a + 5] = w.z;
		float* o = outPose + 7 * a;
		o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.w;
		o[4] = txs[a].p.x; o[5] = txs[a].p.y; o[6] = txs[a].p.z;
	}
}

#include "pgs.inl"
