// ORACLE (test infrastructure): helpers of the narrowphase restatement that
// need iterative geometry (GJK/EPA) or polygon tests.
#pragma once
#include "pxmath.h"

namespace orc
{
// Gu::contains (physx/source/geomutils/src/pcm/GuPCMContactGenUtil.cpp:35):
// point-in-polygon on XY by ray crossing, with the endpoint shortcut and the
// epsilon-shifted crossing test of the reference (bounds reject done by caller).
static inline bool polyContainsXY(const V3* verts, int numVerts, V3 p)
{
	const float tx = p.x, ty = p.y;
	const float eps = FLT_EPSILON;
	int intersections = 0;
	for(int i = 0, j = numVerts - 1; i < numVerts; j = i++)
	{
		const float jy = verts[j].y, iy = verts[i].y, jx = verts[j].x, ix = verts[i].x;
		if((tx == jx && ty == jy) || (tx == ix && ty == iy)) return true;
		const bool yflag0 = jy > ty, yflag1 = iy > ty;
		if(yflag0 != yflag1)
		{
			const float jix = ix - jx, jiy = iy - jy, jty = ty - jy;
			const float part1 = jty * jix;
			const float part2 = (jx + eps) * jiy;
			const float part3 = tx * jiy;
			const bool comp = jiy > 0.0f;
			const float tmp = part1 + part2;
			const float comp1 = comp ? tmp : part3;
			const float comp2 = comp ? part3 : tmp;
			if(comp1 >= comp2)
			{
				if(intersections == 1) return false;
				intersections++;
			}
		}
	}
	return intersections > 0;
}

struct GjkResult
{
	V3 closestA, closestB, normal;
	float penDep;
};

} // namespace orc
