// ORACLE (test infrastructure, never shipped): CPU restatement of the PGS
// immediate-mode contact path, part of the tgs.cpp translation unit (it shares
// its batching and friction-correlation restatements):
//   PxConstructSolverBodies / PxConstructStaticSolverBody
//     (physx/source/immediatemode/src/NpImmediateMode.cpp:55,70) ->
//     bodyCoreComputeUnconstrainedVelocity (lowleveldynamics/src/DyBodyCoreIntegrator.h:38),
//     copyToSolverBodyData (lowleveldynamics/src/DyRigidBodyToSolverBody.cpp:38)
//   PxBatchConstraints (NpImmediateMode.cpp:269): the partition rule of PxBatchConstraintsTGS
//   PxCreateContactConstraints (NpImmediateMode.cpp:292) ->
//     createFinalizeSolverContacts (lowleveldynamics/src/DyContactPrep.cpp:472),
//     setupFinalizeSolverConstraints (:49), constructContactConstraint
//     (DyContactPrepShared.h:298); headers of stride 4 with at most 64 contacts:
//     createFinalizeSolverContacts4 / setupFinalizeSolverConstraints4
//     (DyContactPrep4.cpp:1225,51)
//   PxSolveConstraints (NpImmediateMode.cpp:552): solveContact / solveContact_BStatic
//     (DySolverConstraints.cpp:221,373) with solveDynamicContacts / solveStaticContacts
//     (DySolverConstraintsShared.h:49,111), concludeContact (:508), writeBackContact
//     (:553); the block path solveContact4_Block / solveContact4_StaticBlock,
//     concludeContact4_Block, writeBackContact4_Block (DySolverConstraintsBlock.cpp:45,407,676,757)
//   PxIntegrateSolverBodies (NpImmediateMode.cpp:78) -> integrateCore
//     (DyBodyCoreIntegrator.h:83)
// with the immediate-mode snippet's settings: fresh friction data, unit mass
// scales, zero rest distance and offset slop, no target velocities, maximum
// impulses unbounded, non-negative restitution.

namespace
{
struct PgsBody       // PxSolverBodyData fields the path uses
{
	V3 lin, ang;
	float invMass, penBiasClamp, maxContactImpulse;
	M33 sqrtInvInertia;
	Tr pose;
};
struct PgsVel { V3 lin, ang; };   // PxSolverBody: delta linear velocity, angular state

// unbiasedErr: the per-pair path's error after the position iterations;
// scaledBias: the block path's bias removed at the conclude
struct PgsPoint { V3 raXn, rbXn; float velMultiplier, maxImpulse, biasedErr, unbiasedErr, impulseMultiplier, scaledBias; };
// per-pair rows: bias, targetVel; block rows: scaledBias (the solve's bias) and
// targetVelocity (what the conclude leaves in it)
struct PgsFriction { V3 normal, raXn, rbXn; float appliedForce, velMultiplier, bias, targetVel, scaledBias, targetVelocity; };
struct PgsPatch
{
	V3 normal;
	float invMass0, invMass1, angDom0, angDom1, staticFriction, dynamicFriction;
	int pointStart, nbPoints, frictionStart, nbFriction;
	int broken;
};
// a constraint's rows; block: one lane of a 4-wide header (the block path's
// arithmetic); blockDynamic: that header has a dynamic body B somewhere
struct PgsCons
{
	int bodyA, bodyB;
	bool block, blockDynamic;
	int patchStart, nbPatches;
	std::vector<float> force;   // applied normal impulse per point row
};
struct PgsRows
{
	std::vector<PgsCons> cons;
	std::vector<PgsPatch> patches;
	std::vector<PgsPoint> points;
	std::vector<PgsFriction> friction;
};

void pgsCopyToSolverBody(V3 lv, V3 av, float invMass, V3 invInertia, const Tr& pose, float maxDepen, float maxImpulse, PgsBody& b)
{
	const M33 rot = m33FromQuatCol(pose.q);   // PxMat33Padded
	const V3 sqrtInv = v3(invInertia.x == 0.0f ? 0.0f : sqrtf(invInertia.x), invInertia.y == 0.0f ? 0.0f : sqrtf(invInertia.y),
	                      invInertia.z == 0.0f ? 0.0f : sqrtf(invInertia.z));
	b.sqrtInvInertia = transformInertia(sqrtInv, rot);
	b.lin = lv;
	b.ang = av;
	b.invMass = invMass;
	b.penBiasClamp = maxDepen;
	b.maxContactImpulse = maxImpulse;
	b.pose = pose;
}

// ------------------------------------------------------------ per-pair rows
void pgsPrepConstraint(int ci, const ContactIn* contacts, int nbContacts, int a, int b, const std::vector<PgsBody>& bodies, float invDt, float dt,
                       float bounce, float fricOffset, PgsRows& rows)
{
	PgsCons cr;
	cr.bodyA = a; cr.bodyB = b;
	cr.block = false; cr.blockDynamic = false;
	cr.patchStart = int(rows.patches.size());
	cr.nbPatches = 0;
	if(nbContacts == 0) { rows.cons[ci] = cr; return; }
	const PgsBody& d0 = bodies[a];
	const PgsBody& d1 = bodies[b];
	const Tr& f0 = d0.pose;
	const Tr& f1 = d1.pose;
	Correlation c;
	createContactPatches(c, contacts, nbContacts, 0.999f);
	correlatePatches(c, contacts, f0, f1, 0.999f);
	growPatches(c, contacts, f0, f1, fricOffset + 0.0f);

	const float invMass0D0 = 1.0f * d0.invMass;
	const float invMass1D1 = (-1.0f) * d1.invMass;   // nDom1 * invMass1
	const float angD0 = 1.0f, angD1 = 1.0f;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 p0 = f0.p, p1 = f1.p;
	const V3 lv0 = d0.lin, lv1 = d1.lin, av0 = d0.ang, av1 = d1.ang;
	const M33& s0 = d0.sqrtInvInertia;
	const M33& s1 = d1.sqrtInvInertia;
	const float p8 = 0.8f;
	const float invDtp8 = invDt * p8;
	(void)dt;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		const int count = c.frictionPatchContactCounts[i];
		if(count == 0) continue;
		const FrictionPatch& fp = c.frictionPatches[i];
		const int first = c.correlationListHeads[i];
		const ContactIn& base0 = contacts[c.contactPatches[first].start];
		const float restitution = base0.restitution;
		PgsPatch pr;
		pr.invMass0 = invMass0D0;
		pr.invMass1 = -invMass1D1;
		pr.angDom0 = angD0; pr.angDom1 = angD1;
		const V3 n = contacts[c.contactPatches[c.correlationListHeads[i]].start].n;
		const float nLenSq = dotA(n, n);
		// V3SumElems(V3NegMulSub(normal, linVel1, V3Mul(normal, linVel0)))
		const float norVel = sumElems(sub(mul(n, lv0), mul(n, lv1)));
		const float imn0 = invMass0D0 * nLenSq, imn1 = invMass1D1 * nLenSq;
		pr.normal = n;
		pr.pointStart = int(rows.points.size());
		for(int patch = c.correlationListHeads[i]; patch != -1; patch = c.contactPatches[patch].next)
		{
			const Correlation::ContactPatch& cp = c.contactPatches[patch];
			for(int j = 0; j < cp.count; j++)
			{
				// constructContactConstraint (DyContactPrepShared.h:298)
				const ContactIn& ct = contacts[cp.start + j];
				const float cTargetVel = dotA(n, zero3());
				const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
				const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
				// offsetSlop is 0: the slop test keeps raXn / rbXn and vRelAng as they are
				const float vRelAng = dotA(raXn, av0) - dotA(rbXn, av1);
				const float vrel = norVel + vRelAng;
				const V3 ri0 = m33MulV(s0, raXn), ri1 = m33MulV(s1, rbXn);
				const float resp0 = imn0 + dotA(ri0, ri0) * angD0;
				const float resp1 = dotA(ri1, ri1) * angD1 - imn1;
				const float unitResponse = resp0 + resp1;
				const float penetration = ct.sep - 0.0f;
				const float penetrationInvDt = penetration * invDt;
				const bool isSeparated = penetration >= 0.0f;
				const bool collidingWithVrel = -vrel > penetrationInvDt;
				const bool isGreater2 = (restitution > 0.0f && bounce > vrel) && collidingWithVrel;
				float targetVelocity = cTargetVel + (isGreater2 ? (-vrel) * restitution : 0.0f);
				targetVelocity = targetVelocity - vrel;
				const float recipResponse = unitResponse > 0.0f ? 1.0f / unitResponse : 0.0f;
				const float velMultiplier = recipResponse;
				const float penetrationInvDtScaled = isSeparated ? penetrationInvDt : penetration * invDtp8;
				float scaledBias = velMultiplier * fmax_(maxPenBias, penetrationInvDtScaled);
				const bool ccdSeparationCondition = FLT_MAX >= penetration;
				scaledBias = (ccdSeparationCondition && isGreater2) ? 0.0f : scaledBias;
				PgsPoint row;
				row.raXn = ri0;
				row.rbXn = ri1;
				row.velMultiplier = velMultiplier;
				row.maxImpulse = FLT_MAX;
				row.impulseMultiplier = 1.0f;
				row.biasedErr = targetVelocity * velMultiplier + (-scaledBias);
				row.unbiasedErr = targetVelocity * velMultiplier + (isGreater2 ? 0.0f : -fmax_(scaledBias, 0.0f));
				rows.points.push_back(row);
			}
		}
		pr.nbPoints = int(rows.points.size()) - pr.pointStart;
		const float frictionCoefficient = fp.anchorCount == 2 ? 0.5f : 1.0f;
		pr.staticFriction = base0.staticFriction * frictionCoefficient;
		pr.dynamicFriction = base0.dynamicFriction * frictionCoefficient;
		const bool haveFriction = fp.anchorCount != 0;
		pr.frictionStart = int(rows.friction.size());
		pr.nbFriction = haveFriction ? fp.anchorCount * 2 : 0;
		pr.broken = 0;
		if(haveFriction)
		{
			const V3 linVrel = sub(lv0, lv1);
			const V3 t0f1 = v3(0.0f, -n.z, n.y), t0f2 = v3(-n.y, n.x, 0.0f);
			const V3 t0Fallback = 0.70710678f > fabsf(n.x) ? t0f1 : t0f2;
			V3 t0 = sub(linVrel, scale(n, dotA(n, linVrel)));
			t0 = dotA(t0, t0) > 0.0001f ? t0 : t0Fallback;
			t0 = normalizeA(t0);
			const V3 t1 = cross(n, t0);
			for(int j = 0; j < fp.anchorCount; j++)
			{
				const V3 ra = qRotate(f0.q, fp.body0Anchors[j]);
				const V3 rb = qRotate(f1.q, fp.body1Anchors[j]);
				// offsetSlop is 0: the error keeps every component
				const V3 error = sub(add(ra, p0), add(rb, p1));
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					const V3 raXn = cross(ra, t), rbXn = cross(rb, t);
					const V3 ri0 = m33MulV(s0, raXn), ri1 = m33MulV(s1, rbXn);
					const float resp0 = invMass0D0 + angD0 * dotA(ri0, ri0);
					const float resp1 = angD1 * dotA(ri1, ri1) - invMass1D1;
					const float resp = resp0 + resp1;
					const float velMultiplier = resp > 0.0f ? p8 / resp : 0.0f;
					float targetVel = dotA(zero3(), t);
					const float vrel1 = dotA(t, lv0) + dotA(raXn, av0);
					const float vrel2 = dotA(t, lv1) + dotA(rbXn, av1);
					const float vrel = vrel1 - vrel2;
					targetVel = targetVel - vrel;
					PgsFriction fr;
					fr.normal = t;
					fr.appliedForce = 0.0f;
					fr.raXn = ri0;
					fr.velMultiplier = velMultiplier;
					fr.rbXn = ri1;
					fr.bias = dotA(t, error) * invDt;
					fr.targetVel = targetVel;
					rows.friction.push_back(fr);
				}
			}
		}
		rows.patches.push_back(pr);
		cr.nbPatches++;
	}
	cr.force.assign(size_t(nbContacts), 0.0f);
	rows.cons[ci] = std::move(cr);
}

// ------------------------------------------------------------ 4-wide block rows, one lane
// PxCreateContactConstraints sends a header of stride 4 whose four descriptors
// hold at most 64 contacts through createFinalizeSolverContacts4
// (DyContactPrep4.cpp:1225), which builds the four constraints' rows side by
// side (setupFinalizeSolverConstraints4, :51); PxSolveConstraints solves them
// with solveContact4_Block / solveContact4_StaticBlock.  The lanes never mix
// (a lane with fewer patches, points or anchors gets padding rows of zero
// velocity multiplier), so each lane is computed alone here with the block
// path's arithmetic: the multiply-add chains of its dot products, the
// transposed inertia product, restitution negated, the tangent normalised by a
// reciprocal square root, and the friction rows' bias and target velocity
// folded into one scaled bias.  blockDynamic: some constraint of the header has
// a dynamic body B (the header-wide isDynamic).
void pgsPrepConstraintBlock(int ci, const ContactIn* contacts, int nbContacts, int a, int b, const std::vector<PgsBody>& bodies, float invDt,
                            float dt, float bounce, float fricOffset, bool blockDynamic, PgsRows& rows)
{
	PgsCons cr;
	cr.bodyA = a; cr.bodyB = b;
	cr.block = true; cr.blockDynamic = blockDynamic;
	cr.patchStart = int(rows.patches.size());
	cr.nbPatches = 0;
	if(nbContacts == 0) { rows.cons[ci] = cr; return; }
	const PgsBody& d0 = bodies[a];
	const PgsBody& d1 = bodies[b];
	const Tr& f0 = d0.pose;
	const Tr& f1 = d1.pose;
	Correlation c;
	createContactPatches(c, contacts, nbContacts, 0.999f);
	correlatePatches(c, contacts, f0, f1, 0.999f);
	growPatches(c, contacts, f0, f1, fricOffset + 0.0f);

	const float dom0 = 1.0f, dom1 = 1.0f, angDom0 = 1.0f, angDom1 = 1.0f;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 lv0 = d0.lin, lv1 = d1.lin, av0 = d0.ang, av1 = d1.ang;
	const float invMass0D0 = dom0 * d0.invMass, invMass1D1 = dom1 * d1.invMass;
	const M33& I0 = d0.sqrtInvInertia;
	const M33& I1 = d1.sqrtInvInertia;
	const V3 p0 = f0.p, p1 = f1.p;
	const float p8 = 0.8f;
	const float invDtp8 = invDt * p8;
	const V3 vrelv = sub(lv0, lv1);
	(void)dt;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.frictionPatchContactCounts[i] == 0) continue;
		const FrictionPatch& fp = c.frictionPatches[i];
		const int head = c.correlationListHeads[i];
		const ContactIn& base0 = contacts[c.contactPatches[head].start];
		const float restitution = -base0.restitution;
		PgsPatch pr;
		pr.invMass0 = invMass0D0;
		pr.invMass1 = invMass1D1;
		pr.angDom0 = angDom0; pr.angDom1 = angDom1;
		const V3 n = base0.n;
		pr.normal = n;
		const float relNorVel = dotXYZ(n, lv0) - dotXYZ(n, lv1);
		pr.pointStart = int(rows.points.size());
		for(int patch = head; patch != -1; patch = c.contactPatches[patch].next)
		{
			const Correlation::ContactPatch& cp = c.contactPatches[patch];
			for(int j = 0; j < cp.count; j++)
			{
				const ContactIn& ct = contacts[cp.start + j];
				const float cTargetNorVel = dotZYX(zero3(), n);
				const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
				const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
				// offsetSlop is 0: the slop test keeps raXn / rbXn and relAng as they are
				const float relAng = dotXYZ(raXn, av0) - dotXYZ(rbXn, av1);
				const V3 delAng0 = m33TMulXYZ(I0, raXn);
				float unitResponse = dotZYX(delAng0, delAng0) * angDom0 + invMass0D0;
				const float vrel = relNorVel + relAng;
				V3 delAng1 = zero3();
				if(blockDynamic)
				{
					delAng1 = m33TMulXYZ(I1, rbXn);
					const float resp1 = dotZYX(delAng1, delAng1) * angDom1 + invMass1D1;
					unitResponse = unitResponse + resp1;
				}
				const float penetration = ct.sep - 0.0f;
				const float penInvDtPt8 = fmax_(maxPenBias, penetration * invDtp8);
				const float penetrationInvDt = penetration * invDt;
				const bool isSeparated = penetration >= 0.0f;
				const bool collidingWithVrel = -vrel > penetrationInvDt;
				const float recipResponse = unitResponse > 0.0f ? 1.0f / unitResponse : 0.0f;
				// restitution >= 0 here, so the compliant branch (restitution > 0 after the negation) is not taken
				const float velMultiplier = recipResponse;
				const float impulseMultiplier = 1.0f - 0.0f;
				float scaledBias = (isSeparated ? penetrationInvDt : penInvDtPt8) * velMultiplier;
				const bool isGreater2 = (0.0f > restitution && bounce > vrel) && collidingWithVrel;
				const bool ccdSeparationCondition = FLT_MAX >= penetration;
				scaledBias = -((ccdSeparationCondition && isGreater2) ? 0.0f : scaledBias);
				const float targetVelocity = ((cTargetNorVel - vrel) + (isGreater2 ? vrel * restitution : 0.0f)) * velMultiplier;
				PgsPoint row;
				row.raXn = delAng0;
				row.rbXn = delAng1;
				row.velMultiplier = velMultiplier;
				row.biasedErr = targetVelocity + scaledBias;
				row.unbiasedErr = 0.0f;
				row.impulseMultiplier = impulseMultiplier;
				row.scaledBias = isGreater2 ? scaledBias : fmax_(0.0f, scaledBias);
				row.maxImpulse = FLT_MAX;
				rows.points.push_back(row);
			}
		}
		pr.nbPoints = int(rows.points.size()) - pr.pointStart;
		const float coefficient = fp.anchorCount == 2 ? 0.5f : 1.0f;
		pr.staticFriction = base0.staticFriction * coefficient;
		pr.dynamicFriction = base0.dynamicFriction * coefficient;
		const int anchors = fp.anchorCount;
		pr.frictionStart = int(rows.friction.size());
		pr.nbFriction = anchors * 2;
		pr.broken = 0;
		if(anchors)
		{
			const V3 fb1 = v3(0.0f, -n.z, n.y), fb2 = v3(-n.y, n.x, 0.0f);
			const V3 fallback = 0.70710678f > fabsf(n.x) ? fb1 : fb2;
			const V3 vs = v3(vrelv.x - n.x * relNorVel, vrelv.y - n.y * relNorVel, vrelv.z - n.z * relNorVel);
			V3 t0 = dotZYX(vs, vs) > 0.0001f ? vs : fallback;
			const float recipLen = 1.0f / sqrtf(dotXYZ(t0, t0));
			t0 = scale(t0, recipLen);
			const V3 t1 = cross(n, t0);
			for(int j = 0; j < anchors; j++)
			{
				const V3 ra = qRotate4V(f0.q, fp.body0Anchors[j]);
				const V3 rb = qRotate4V(f1.q, fp.body1Anchors[j]);
				const V3 error = sub(add(ra, p0), add(rb, p1));
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					const V3 raXn = cross(ra, t);
					const V3 delAng0 = m33TMulXYZ(I0, raXn);
					// the friction rows sum their squares z + (y + x), the normal rows x + (y + z)
					float resp = dotXYZ(delAng0, delAng0) * angDom0 + invMass0D0;
					const float tVel0 = dotXYZ(t, lv0);
					float vrel = ((tVel0 + raXn.x * av0.x) + raXn.y * av0.y) + raXn.z * av0.z;
					V3 delAng1 = zero3();
					if(blockDynamic)
					{
						const V3 rbXn = cross(rb, t);
						delAng1 = m33TMulXYZ(I1, rbXn);
						const float resp1 = dotXYZ(delAng1, delAng1) * angDom1 + invMass1D1;
						resp = resp + resp1;
						const float tVel1 = dotXYZ(t, lv1);
						const float vel1 = ((tVel1 + rbXn.x * av1.x) + rbXn.y * av1.y) + rbXn.z * av1.z;
						vrel = vrel - vel1;
					}
					const float velMultiplier = 1.0f * (resp > 0.0f ? p8 / resp : 0.0f);
					float bias = dotXYZ(t, error) * invDt;
					const float targetVel = dotXYZ(t, zero3()) - vrel;
					PgsFriction fr;
					fr.normal = t;
					fr.raXn = delAng0;
					fr.rbXn = delAng1;
					fr.appliedForce = 0.0f;
					fr.velMultiplier = velMultiplier;
					fr.targetVelocity = -(targetVel * velMultiplier);
					bias = bias - targetVel;
					fr.scaledBias = bias * velMultiplier;
					fr.bias = 0.0f;
					fr.targetVel = 0.0f;
					rows.friction.push_back(fr);
				}
			}
		}
		rows.patches.push_back(pr);
		cr.nbPatches++;
	}
	cr.force.assign(size_t(nbContacts), 0.0f);
	rows.cons[ci] = std::move(cr);
}

// One lane of solveContact4_Block (dynamic) / solveContact4_StaticBlock; the
// padding rows of the other lanes change nothing.  conclude: concludeContact4_Block
// after the solve.  storeB: the block path stores body B only when its data
// index is not 0.
void pgsSolveConstraintBlock(PgsCons& cr, PgsRows& rows, std::vector<PgsVel>& vels, bool dynamicBlock, bool doFriction, bool conclude, bool storeB)
{
	PgsVel& b0 = vels[cr.bodyA];
	PgsVel& b1 = vels[cr.bodyB];
	V3 lin0 = b0.lin, ang0 = b0.ang, lin1 = b1.lin, ang1 = b1.ang;
	int pointBase = 0;
	for(int k = 0; k < cr.nbPatches; k++)
	{
		PgsPatch& pr = rows.patches[cr.patchStart + k];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1, angD0 = pr.angDom0, angD1 = pr.angDom1;
		float accumulated = 0.0f, accumDeltaF = 0.0f;
		if(dynamicBlock)
		{
			const float sumInvMass = invMassA + invMassB;
			float relVel1 = dotXYZ(lin0, n) - dotXYZ(lin1, n);
			for(int i = 0; i < pr.nbPoints; i++)
			{
				const PgsPoint& c = rows.points[pr.pointStart + i];
				float& applied = cr.force[pointBase + i];
				const float appliedForce = applied;
				const float cnv2 = dotXYZ(c.raXn, ang0), cnv4 = dotXYZ(c.rbXn, ang1);
				const float normalVel = relVel1 + (cnv2 - cnv4);
				float deltaF = c.biasedErr - normalVel * c.velMultiplier;
				deltaF = fmax_(deltaF, -appliedForce);
				const float newApplied = fmin_(c.impulseMultiplier * appliedForce + deltaF, c.maxImpulse);
				deltaF = newApplied - appliedForce;
				accumDeltaF = accumDeltaF + deltaF;
				const float angDeltaF0 = deltaF * angD0, angDeltaF1 = deltaF * angD1;
				relVel1 = sumInvMass * deltaF + relVel1;
				ang0 = add(scale(c.raXn, angDeltaF0), ang0);
				ang1 = sub(ang1, scale(c.rbXn, angDeltaF1));
				applied = newApplied;
				accumulated = accumulated + newApplied;
			}
			const float im0 = accumDeltaF * invMassA, im1 = accumDeltaF * invMassB;
			lin0 = add(scale(n, im0), lin0);
			lin1 = sub(lin1, scale(n, im1));
		}
		else
		{
			float cnv1 = dotXYZ(lin0, n);
			for(int i = 0; i < pr.nbPoints; i++)
			{
				const PgsPoint& c = rows.points[pr.pointStart + i];
				float& applied = cr.force[pointBase + i];
				const float appliedForce = applied;
				const float normalVel = ((cnv1 + c.raXn.x * ang0.x) + c.raXn.y * ang0.y) + c.raXn.z * ang0.z;
				const float _deltaF = fmax_(c.biasedErr - normalVel * c.velMultiplier, -appliedForce);
				const float newApplied = fmin_(c.impulseMultiplier * appliedForce + _deltaF, c.maxImpulse);
				const float deltaF = newApplied - appliedForce;
				const float angDeltaF = angD0 * deltaF;
				accumDeltaF = accumDeltaF + deltaF;
				cnv1 = invMassA * deltaF + cnv1;
				ang0 = add(scale(c.raXn, angDeltaF), ang0);
				applied = newApplied;
				accumulated = accumulated + newApplied;
			}
			lin0 = add(scale(n, accumDeltaF * invMassA), lin0);
		}
		if(doFriction && pr.nbFriction)
		{
			const float maxFrictionImpulse = pr.staticFriction * accumulated;
			const float maxDynFrictionImpulse = pr.dynamicFriction * accumulated;
			const float negMaxDynFrictionImpulse = -maxDynFrictionImpulse;
			bool broken = false;
			for(int i = 0; i < pr.nbFriction; i++)
			{
				PgsFriction& f = rows.friction[pr.frictionStart + i];
				const V3 t = f.normal;
				const float appliedForce = f.appliedForce;
				float normalVel;
				if(dynamicBlock)
					normalVel = (dotXYZ(lin0, t) + dotXYZ(f.raXn, ang0)) - (dotXYZ(lin1, t) + dotXYZ(f.rbXn, ang1));
				else
					normalVel = dotXYZ(lin0, t) + dotXYZ(f.raXn, ang0);
				const float tmp1 = appliedForce - f.scaledBias;
				const float totalImpulse = tmp1 - normalVel * f.velMultiplier;
				broken = broken || fabsf(totalImpulse) > maxFrictionImpulse;
				const float newApplied = broken ? fmin_(maxDynFrictionImpulse, fmax_(negMaxDynFrictionImpulse, totalImpulse)) : totalImpulse;
				const float deltaF = newApplied - appliedForce;
				f.appliedForce = newApplied;
				if(dynamicBlock)
				{
					const float dIm0 = deltaF * invMassA, dIm1 = deltaF * invMassB, aD0 = deltaF * angD0, aD1 = deltaF * angD1;
					lin0 = add(scale(t, dIm0), lin0);
					lin1 = sub(lin1, scale(t, dIm1));
					ang0 = add(scale(f.raXn, aD0), ang0);
					ang1 = sub(ang1, scale(f.rbXn, aD1));
				}
				else
				{
					const float dIm = invMassA * deltaF, aD = angD0 * deltaF;
					lin0 = add(scale(t, dIm), lin0);
					ang0 = add(scale(f.raXn, aD), ang0);
				}
			}
			pr.broken = broken ? 1 : 0;
		}
		if(conclude)
		{
			for(int i = 0; i < pr.nbPoints; i++)
			{
				PgsPoint& c = rows.points[pr.pointStart + i];
				c.biasedErr = c.biasedErr - c.scaledBias;
			}
			for(int i = 0; i < pr.nbFriction; i++)
			{
				PgsFriction& f = rows.friction[pr.frictionStart + i];
				f.scaledBias = f.targetVelocity;
			}
		}
		pointBase += pr.nbPoints;
	}
	b0.lin = lin0;
	b0.ang = ang0;
	if(dynamicBlock && storeB)
	{
		b1.lin = lin1;
		b1.ang = ang1;
	}
}

// ------------------------------------------------------------ per-pair solve
// solveContact (dynamic B) / solveContact_BStatic; conclude: concludeContact
// after the solve; the impulses are kept per point row.
void pgsSolveConstraint(PgsCons& cr, PgsRows& rows, std::vector<PgsVel>& vels, bool dynamicB, bool doFriction, bool conclude)
{
	PgsVel& b0 = vels[cr.bodyA];
	PgsVel& b1 = vels[cr.bodyB];
	V3 linVel0 = b0.lin, angState0 = b0.ang, linVel1 = b1.lin, angState1 = b1.ang;
	int pointBase = 0;
	for(int k = 0; k < cr.nbPatches; k++)
	{
		PgsPatch& pr = rows.patches[cr.patchStart + k];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1, angDom0 = pr.angDom0, angDom1 = pr.angDom1;
		float accumulated = 0.0f;
		const V3 delLinVel0 = scale(n, invMassA);
		const V3 delLinVel1 = scale(n, invMassB);
		for(int i = 0; i < pr.nbPoints; i++)
		{
			const PgsPoint& c = rows.points[pr.pointStart + i];
			float& applied = cr.force[pointBase + i];
			const float appliedForce = applied;
			float normalVel;
			if(dynamicB)
			{
				const V3 v0 = add(mul(linVel0, n), mul(angState0, c.raXn));
				const V3 v1 = add(mul(linVel1, n), mul(angState1, c.rbXn));
				normalVel = sumElems(sub(v0, v1));
			}
			else
				normalVel = sumElems(add(mul(linVel0, n), mul(angState0, c.raXn)));
			const float _deltaF = fmax_(c.biasedErr - normalVel * c.velMultiplier, -appliedForce);
			const float _newForce = dynamicB ? c.impulseMultiplier * appliedForce + _deltaF : appliedForce * c.impulseMultiplier + _deltaF;
			const float newForce = fmin_(_newForce, c.maxImpulse);
			const float deltaF = newForce - appliedForce;
			linVel0 = add(scale(delLinVel0, deltaF), linVel0);
			angState0 = add(scale(c.raXn, deltaF * angDom0), angState0);
			if(dynamicB)
			{
				linVel1 = sub(linVel1, scale(delLinVel1, deltaF));
				angState1 = sub(angState1, scale(c.rbXn, deltaF * angDom1));
			}
			applied = newForce;
			accumulated = accumulated + newForce;
		}
		if(doFriction && pr.nbFriction)
		{
			const float maxFrictionImpulse = pr.staticFriction * accumulated;
			const float maxDynFrictionImpulse = pr.dynamicFriction * accumulated;
			const float negMaxDynFrictionImpulse = -maxDynFrictionImpulse;
			bool broken = false;
			for(int i = 0; i < pr.nbFriction; i++)
			{
				PgsFriction& f = rows.friction[pr.frictionStart + i];
				const V3 t = f.normal;
				const float appliedForce = f.appliedForce;
				const V3 dl0 = scale(t, invMassA);
				float normalVel;
				if(dynamicB)
				{
					const V3 v0 = add(mul(linVel0, t), mul(angState0, f.raXn));
					const V3 v1 = add(mul(linVel1, t), mul(angState1, f.rbXn));
					normalVel = sumElems(sub(v0, v1));
				}
				else
					normalVel = sumElems(add(mul(linVel0, t), mul(angState0, f.raXn)));
				const float tmp1 = appliedForce - (f.bias - f.targetVel) * f.velMultiplier;
				const float totalImpulse = tmp1 - normalVel * f.velMultiplier;
				const bool clamp = fabsf(totalImpulse) > maxFrictionImpulse;
				const float totalClamped = fmin_(maxDynFrictionImpulse, fmax_(negMaxDynFrictionImpulse, totalImpulse));
				const float newAppliedForce = clamp ? totalClamped : totalImpulse;
				broken = broken || clamp;
				const float deltaF = newAppliedForce - appliedForce;
				linVel0 = add(scale(dl0, deltaF), linVel0);
				angState0 = add(scale(f.raXn, deltaF * angDom0), angState0);
				if(dynamicB)
				{
					const V3 dl1 = scale(t, invMassB);
					linVel1 = sub(linVel1, scale(dl1, deltaF));
					angState1 = sub(angState1, scale(f.rbXn, deltaF * angDom1));
				}
				f.appliedForce = newAppliedForce;
			}
			pr.broken = broken ? 1 : 0;
		}
		if(conclude)
		{
			for(int i = 0; i < pr.nbPoints; i++)
			{
				PgsPoint& c = rows.points[pr.pointStart + i];
				c.biasedErr = c.unbiasedErr;
			}
			for(int i = 0; i < pr.nbFriction; i++) rows.friction[pr.frictionStart + i].bias = 0.0f;
		}
		pointBase += pr.nbPoints;
	}
	b0.lin = linVel0;
	b0.ang = angState0;
	if(dynamicB)
	{
		b1.lin = linVel1;
		b1.ang = angState1;
	}
}

// integrateCore (DyBodyCoreIntegrator.h:83) with PxSinCos as the C library's sinf / cosf
void pgsIntegrate(V3& motionLin, V3& motionAng, const PgsVel& sb, PgsBody& d, float dt)
{
	const V3 linearMotionVel = add(d.lin, motionLin);
	motionLin = linearMotionVel;
	d.pose.p = add(d.pose.p, scale(linearMotionVel, dt));
	V3 angularMotionVel = add(d.ang, m33MulVS(d.sqrtInvInertia, motionAng));
	float w = lenSqS(angularMotionVel);
	if(w != 0.0f)
	{
		w = sqrtf(w);
		const float maxW = 1e+7f;
		if(w > maxW)
		{
			angularMotionVel = scale(normalizeS(angularMotionVel), maxW);
			w = maxW;
		}
		const float v = dt * w * 0.5f;
		float s = sinf(v);
		const float q = cosf(v);
		s = s / w;
		const V3 pqr = scale(angularMotionVel, s);
		const Q quatVel = {pqr.x, pqr.y, pqr.z, 0.0f};
		Q result = qMulS(quatVel, d.pose.q);
		const Q& q0 = d.pose.q;
		result.x += q0.x * q; result.y += q0.y * q; result.z += q0.z * q; result.w += q0.w * q;
		const float m = sqrtf(result.x * result.x + result.y * result.y + result.z * result.z + result.w * result.w);
		const float r = 1.0f / m;
		d.pose.q.x = result.x * r; d.pose.q.y = result.y * r; d.pose.q.z = result.z * r; d.pose.q.w = result.w * r;
	}
	motionAng = angularMotionVel;
	d.lin = add(d.lin, sb.lin);
	d.ang = add(d.ang, m33MulVS(d.sqrtInvInertia, sb.ang));
}
} // namespace

// One PGS frame (the reference's immediate-mode PGS path, see the top of this
// file).  batch: PxBatchConstraints headers (else one header per constraint).
// Outputs as pxref_pgs_solve: velocities and poses of the dynamic bodies,
// headers (start, stride, type), the constraint order and, per contact of the
// caller's contact array, the written-back normal impulse in the order of the
// constraint's rows.
OX uint32_t orc_pgs_solve(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA,
                          const uint32_t* pairB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                          const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel,
                          float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, int batch, float* outVel,
                          float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outHeaderType, uint32_t* outOrder,
                          float* outForces)
{
	(void)correlationDistance;   // fresh friction data: nothing to correlate with
	const uint32_t nbTotal = nbDyn + nbStatic;
	std::vector<PgsBody> bodies(nbTotal);
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
		pgsCopyToSolverBody(lv, av, r.invMass, v3(r.invInertia[0], r.invInertia[1], r.invInertia[2]), pose, -r.maxDepenetrationVelocity,
		                    r.maxContactImpulse, bodies[a]);
	}
	for(uint32_t s = 0; s < nbStatic; s++)
		pgsCopyToSolverBody(zero3(), zero3(), 0.0f, zero3(), loadTr(staticPose + 7 * s), -FLT_MAX, FLT_MAX, bodies[nbDyn + s]);

	BatchOut bo;
	if(batch)
		batchConstraints(pairA, pairB, int(nbConstraints), int(nbDyn), bo);
	else
	{
		for(uint32_t i = 0; i < nbConstraints; i++)
		{
			bo.order.push_back(int(i));
			bo.headerStart.push_back(i);
			bo.headerStride.push_back(1);
		}
	}
	const size_t nbHeaders = bo.headerStart.size();
	for(uint32_t i = 0; i < nbConstraints; i++) outOrder[i] = uint32_t(bo.order[i]);

	const float invDt = 1.0f / dt;
	PgsRows rows;
	rows.cons.resize(nbConstraints);
	std::vector<ContactIn> cin;
	auto load = [&](uint32_t ci) {
		cin.resize(contactCount[ci]);
		for(uint32_t k = 0; k < contactCount[ci]; k++)
		{
			const float* s = contacts + 8 * (contactStart[ci] + k);
			ContactIn& c = cin[k];
			c.n = v3(s[0], s[1], s[2]); c.sep = s[3]; c.p = v3(s[4], s[5], s[6]);
			c.staticFriction = material[3 * ci]; c.dynamicFriction = material[3 * ci + 1]; c.restitution = material[3 * ci + 2];
		}
	};
	// header types (DY_SC_TYPE_*): the first constraint's row type; a static
	// first row becomes dynamic when another constraint of the header is
	std::vector<uint32_t> htype(nbHeaders, 0);
	for(size_t h = 0; h < nbHeaders; h++)
	{
		const uint32_t start = bo.headerStart[h], stride = bo.headerStride[h];
		// headers of stride 4 holding at most 64 contacts take the block path
		// (NpImmediateMode.cpp:312-330); isDynamic is per header
		uint32_t total = 0;
		bool dynamicB = false;
		for(uint32_t l = 0; l < stride; l++)
		{
			total += contactCount[bo.order[start + l]];
			dynamicB = dynamicB || pairB[bo.order[start + l]] < nbDyn;
		}
		const bool block = stride == 4 && total <= 64;
		for(uint32_t l = 0; l < stride; l++)
		{
			const uint32_t ci = uint32_t(bo.order[start + l]);
			load(ci);
			if(block)
				pgsPrepConstraintBlock(int(ci), cin.data(), int(contactCount[ci]), int(pairA[ci]), int(pairB[ci]), bodies, invDt, dt,
				                       bounceThreshold, frictionOffsetThreshold, dynamicB, rows);
			else
				pgsPrepConstraint(int(ci), cin.data(), int(contactCount[ci]), int(pairA[ci]), int(pairB[ci]), bodies, invDt, dt, bounceThreshold,
				                  frictionOffsetThreshold, rows);
		}
		uint32_t type;
		if(block)
			type = dynamicB ? 6u : 7u;   // DY_SC_TYPE_BLOCK_RB_CONTACT / _BLOCK_STATIC_RB_CONTACT
		else
		{
			type = pairB[bo.order[start]] >= nbDyn ? 5u : 1u;   // DY_SC_TYPE_STATIC_CONTACT / _RB_CONTACT
			if(type == 5u)
				for(uint32_t l = 1; l < stride; l++)
					if(pairB[bo.order[start + l]] < nbDyn) { type = 1u; break; }
		}
		htype[h] = type;
		outHeaderStart[h] = start;
		outHeaderStride[h] = stride;
		outHeaderType[h] = type;
	}

	std::vector<PgsVel> vels(nbTotal, PgsVel{zero3(), zero3()});
	auto iterate = [&](bool doFriction, bool conclude) {
		for(size_t h = 0; h < nbHeaders; h++)
			for(uint32_t l = 0; l < bo.headerStride[h]; l++)
			{
				PgsCons& cr = rows.cons[bo.order[bo.headerStart[h] + l]];
				if(cr.block)
					pgsSolveConstraintBlock(cr, rows, vels, htype[h] == 6u, doFriction, conclude, cr.bodyB != 0);
				else
					pgsSolveConstraint(cr, rows, vels, htype[h] == 1u, doFriction, conclude);
			}
	};
	for(uint32_t i = nbPos; i > 1; --i) iterate(i <= 3, false);
	iterate(true, true);
	std::vector<V3> motionLin(nbDyn), motionAng(nbDyn);
	for(uint32_t a = 0; a < nbDyn; a++) { motionLin[a] = vels[a].lin; motionAng[a] = vels[a].ang; }
	for(uint32_t i = nbVel; i > 1; --i) iterate(true, false);
	iterate(true, false);   // the write-back iteration solves as the others
	for(uint32_t a = 0; a < nbDyn; a++)
	{
		pgsIntegrate(motionLin[a], motionAng[a], vels[a], bodies[a], dt);
		const PgsBody& d = bodies[a];
		outVel[6 * a + 0] = d.lin.x; outVel[6 * a + 1] = d.lin.y; outVel[6 * a + 2] = d.lin.z;
		outVel[6 * a + 3] = d.ang.x; outVel[6 * a + 4] = d.ang.y; outVel[6 * a + 5] = d.ang.z;
		float* o = outPose + 7 * a;
		o[0] = d.pose.q.x; o[1] = d.pose.q.y; o[2] = d.pose.q.z; o[3] = d.pose.q.w;
		o[4] = d.pose.p.x; o[5] = d.pose.p.y; o[6] = d.pose.p.z;
	}
	if(outForces)
		for(uint32_t ci = 0; ci < nbConstraints; ci++)
			for(uint32_t k = 0; k < contactCount[ci] && k < rows.cons[ci].force.size(); k++) outForces[contactStart[ci] + k] = rows.cons[ci].force[k];
	return uint32_t(nbHeaders);
}
