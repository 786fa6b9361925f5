// ORACLE (test infrastructure): the TGS frame of tgs.cpp as used by the
// persistent scene step of scene.cpp.
#pragma once
#include "pxmath.h"
#include <vector>

namespace orc
{
// FrictionPatch (lowleveldynamics/src/DyFrictionPatch.h:43): what
// PxCreateContactConstraintsTGS leaves in the caller's friction memory and
// reads back the next frame through frictionPtr / frictionCount.
struct FrictionPatch
{
	int broken;
	V3 body0Normal, body1Normal;
	V3 body0Anchors[2], body1Anchors[2];
	int anchorCount;
	float staticFriction, dynamicFriction, restitution;
	Q relativeQuat;
};


// One immediate-mode TGS frame over given contacts (tgs.cpp).  friction: per
// constraint, the friction patches it left last frame on input and the ones it
// leaves, with their broken flags, on output; null for fresh friction data.
uint32_t tgsFrame(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA, const uint32_t* pairB,
                  uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount, const float* contacts, const float* material,
                  const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel, float bounceThreshold, float frictionOffsetThreshold,
                  float correlationDistance, float* outVel, float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder,
                  std::vector<std::vector<FrictionPatch>>* friction);
} // namespace orc
