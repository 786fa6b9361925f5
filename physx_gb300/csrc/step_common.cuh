// Device helpers shared by the batched world (world.cu) and the large-scene
// step (scene.cu): step parameters, pair kinds, shape bounds, the ABP overlap
// test and the per-kind contact generators.
#pragma once
#include "common.cuh"
#include "contacts.cuh"
#include "solver.cuh"

namespace gbpx
{
namespace world
{
struct StepParams
{
	float dt, gx, gy, gz;
	float contactDistance, toleranceLength, boundsMargin;
	float bounceThreshold, frictionOffsetThreshold, correlationDistance, staticFriction;
	uint32_t nbPos, nbVel;
	uint32_t persistent;   // carry contact manifolds and friction patches between steps
	uint32_t largeBodies;  // scenes of more solver bodies run one block per scene (world)
	uint32_t solveVariant; // solve kernel of the world: the resident solve, or a staging variant of the warp-per-scene solve
	uint32_t resBytes;     // shared-memory workspace of one resident-solve block (world)
	uint32_t resStream;    // resident solve: levels a scene may go deeper with its rows streamed through a two-slot ring
};

// no slot in last step's pair list (a new pair)
constexpr uint32_t NO_PREV = 0xffffffffu;

// Pair kinds: shape types ordered (t0 <= t1), code t0 * 4 + t1.  Dynamic
// bodies are spheres, capsules or boxes; statics may also be planes, so nine
// kinds occur (plane-plane never does: statics are not paired together).
constexpr uint32_t NB_KINDS = 9;
__device__ __forceinline__ uint32_t kindOf(int t0, int t1)
{
	const int a = t0 < t1 ? t0 : t1, b = t0 < t1 ? t1 : t0;
	switch(a * 4 + b)
	{
	case 0: return 0;    // sphere-sphere
	case 1: return 1;    // sphere-plane
	case 2: return 2;    // sphere-capsule
	case 3: return 3;    // sphere-box
	case 6: return 4;    // plane-capsule
	case 7: return 5;    // plane-box
	case 10: return 6;   // capsule-capsule
	case 11: return 7;   // capsule-box
	case 15: return 8;   // box-box
	default: return NB_KINDS;
	}
}

__device__ __forceinline__ Tr loadStaticPose(const float* s)
{
	Tr t;
	t.q.x = s[0]; t.q.y = s[1]; t.q.z = s[2]; t.q.w = s[3];
	t.p = v3(s[4], s[5], s[6]);
	return t;
}

// World-space AABB of a shape, before the margin (sphere, capsule along local
// X, box); planes are unbounded.
__device__ __forceinline__ void shapeBounds(int type, const float4 g, const Tr& pose, V3& mn, V3& mx)
{
	V3 e;
	if(type == 0) e = v3(g.x, g.x, g.x);
	else if(type == 2)
	{
		const V3 ax = qBasis0(pose.q);
		e = v3(fabsf(ax.x) * g.y + g.x, fabsf(ax.y) * g.y + g.x, fabsf(ax.z) * g.y + g.x);
	}
	else if(type == 3)
	{
		const M33 R = m33FromQuatCol(pose.q);
		e = v3((fabsf(R.c0.x) * g.x + fabsf(R.c1.x) * g.y) + fabsf(R.c2.x) * g.z,
		       (fabsf(R.c0.y) * g.x + fabsf(R.c1.y) * g.y) + fabsf(R.c2.y) * g.z,
		       (fabsf(R.c0.z) * g.x + fabsf(R.c1.z) * g.y) + fabsf(R.c2.z) * g.z);
	}
	else
	{
		mn = v3(-1e30f, -1e30f, -1e30f);
		mx = v3(1e30f, 1e30f, 1e30f);
		return;
	}
	mn = sub(pose.p, e);
	mx = add(pose.p, e);
}

__device__ __forceinline__ bool overlapBoxes(const float* a, const float* b)
{
	// ABP semantics: X on encoded keys, Y/Z closed float intervals
	const uint32_t aminx = encodeFloatBits(__float_as_uint(a[0])), amaxx = encodeFloatBits(__float_as_uint(a[3]));
	const uint32_t bminx = encodeFloatBits(__float_as_uint(b[0])), bmaxx = encodeFloatBits(__float_as_uint(b[3]));
	if(bminx > amaxx || aminx > bmaxx) return false;
	return !(b[4] < a[1] || a[4] < b[1] || b[5] < a[2] || a[5] < b[2]);
}

// Contacts of one pair kind (shape types TA <= TB), PxGenerateContacts semantics.
template <int TA, int TB>
__device__ __forceinline__ void generateKind(const float* ga, const float* gb, const Tr& pa, const Tr& pb, const StepParams& sp, np::Manifold& m,
                                             np::Buffer& out)
{
	const float cd = sp.contactDistance, tl = sp.toleranceLength;
	if constexpr(TA == 0 && TB == 0) np::sphereSphere(ga[0], gb[0], pa, pb, cd, out);
	else if constexpr(TA == 0 && TB == 1) np::spherePlane(ga[0], pa, pb, cd, out);
	else if constexpr(TA == 0 && TB == 2) np::sphereCapsule(ga[0], gb[0], gb[1], pa, pb, cd, out);
	else if constexpr(TA == 0 && TB == 3) np::sphereBox(ga[0], v3(gb[0], gb[1], gb[2]), pa, pb, cd, out);
	else if constexpr(TA == 1 && TB == 2) np::planeCapsule(gb[0], gb[1], pa, pb, cd, m, out);
	else if constexpr(TA == 1 && TB == 3) np::planeBox(v3(gb[0], gb[1], gb[2]), pa, pb, cd, tl, m, out);
	else if constexpr(TA == 2 && TB == 2) np::capsuleCapsule(ga[0], ga[1], gb[0], gb[1], pa, pb, cd, out);
	else if constexpr(TA == 2 && TB == 3) np::capsuleBox(ga[0], ga[1], v3(gb[0], gb[1], gb[2]), pa, pb, cd, tl, m, out);
	else if constexpr(TA == 3 && TB == 3) np::boxBox(v3(ga[0], ga[1], ga[2]), v3(gb[0], gb[1], gb[2]), pa, pb, cd, tl, m, out);
}

// Pair kinds whose PCM manifold persists between frames (the reference's
// gEnablePCMCaching table): plane-capsule, plane-box, capsule-box, box-box.
__host__ __device__ constexpr bool cachedPairKind(uint32_t kind) { return kind == 4 || kind == 5 || kind == 7 || kind == 8; }

// Row-preparation parameters of a step (PxCreateContactConstraintsTGS arguments).
__device__ __forceinline__ tgs::PrepParams prepParams(const StepParams& sp)
{
	const float invDt = 1.0f / sp.dt;
	tgs::PrepParams pp;
	pp.invStepDt = invDt * float(sp.nbPos);
	pp.invTotalDt = invDt;
	pp.totalDt = 1.0f / invDt;
	pp.stepDt = 1.0f / pp.invStepDt;
	pp.bounceThreshold = sp.bounceThreshold;
	pp.frictionOffsetThreshold = sp.frictionOffsetThreshold;
	pp.biasCoefficient = 2.0f * sqrtf(invDt / pp.invStepDt);
	pp.correlationDistance = sp.correlationDistance;
	return pp;
}
} // namespace world
} // namespace gbpx
