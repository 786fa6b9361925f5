// Convex-core contacts on the device: PhysX's contact generation for
// PxConvexCoreGeometry (a point / segment / box / ellipsoid / cylinder / cone
// core grown by a margin) against spheres, capsules, boxes, planes and other
// convex cores.  Restates, in this build's own code and data layout:
//   - makeConvexShape (geomutils/src/GuConvexGeometry.cpp:593): sphere = point
//     core + radius, capsule = segment core + radius, box = box core;
//   - the per-core support and contact-face functions, FaceClipper,
//     reducePolygon, rotatePoints and the convex-convex generateContacts
//     (geomutils/include/GuConvexSupport.h);
//   - the reference GJK distance and EPA depth (geomutils/include/GuRefGjkEpa.h);
//   - the plane-convex generateContacts (geomutils/src/GuConvexSupport.cpp:41);
//   - contactConvexCoreConvex / contactPlaneConvexCore
//     (geomutils/src/contact/GuContactConvexCoreConvex.cpp:49,
//      GuContactPlaneConvexCore.cpp:37), which these pairs dispatch to
//     (lowlevel/common/src/pipeline/PxcContactMethodImpl.cpp:274-345).
// The reference evaluates this path with its scalar PxVec3 / PxQuat types, so
// every expression below keeps their operation order (PxVec3::dot left to
// right, operator/ as a multiply by the reciprocal, getNormalized as a multiply
// by 1/sqrt); the translation unit is compiled without fused multiply-add.
// No state persists between calls (these pairs keep no contact cache).
//
// GB300 layout: one thread per pair, its GJK / EPA working set (two 32-vertex
// support caches, the EPA polytope of <= 60 faces) in thread-local memory; the
// pairs arrive bucketed, so a warp runs only this generator.
#pragma once
#include "vmath.cuh"

namespace gbpx
{
namespace cc
{
// PxConvexCore::Type
enum : int { CORE_POINT = 0, CORE_SEGMENT = 1, CORE_BOX = 2, CORE_ELLIPSOID = 3, CORE_CYLINDER = 4, CORE_CONE = 5, CORE_COUNT = 6 };
constexpr uint32_t MAX_FACE_POINTS = 4;   // ConvexCore::MAX_FACE_POINTS
constexpr uint32_t MAX_CONTACTS = 4;      // MAX_CONVEX_CONTACTS

// ---- scalar PxVec3 / PxQuat semantics
__device__ __forceinline__ float sgn(float a) { return a >= 0.0f ? 1.0f : -1.0f; }   // PxSign
__device__ __forceinline__ V3 divS(V3 a, float f) { return scale(a, 1.0f / f); }     // PxVec3::operator/
__device__ __forceinline__ float magS(V3 a) { return sqrtf(lenSqS(a)); }
// PxVec3::normalize: returns the magnitude, divides when it is positive
__device__ __forceinline__ float normalizeIn(V3& a)
{
	const float m = magS(a);
	if(m > 0.0f) a = scale(a, 1.0f / m);
	return m;
}
// PxVec3::normalizeFast
__device__ __forceinline__ float normalizeFastIn(V3& a)
{
	const float m = magS(a);
	a = scale(a, 1.0f / m);
	return m;
}
__device__ __forceinline__ float& at(V3& a, uint32_t i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ float at(const V3& a, uint32_t i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
// PxQuat::rotate / rotateInv (scalar form)
__device__ __forceinline__ V3 qrotS(const Q& q, V3 v)
{
	const float vx = 2.0f * v.x, vy = 2.0f * v.y, vz = 2.0f * v.z;
	const float w2 = q.w * q.w - 0.5f;
	const float dot2 = q.x * vx + q.y * vy + q.z * vz;
	return v3(vx * w2 + (q.y * vz - q.z * vy) * q.w + q.x * dot2, vy * w2 + (q.z * vx - q.x * vz) * q.w + q.y * dot2,
	          vz * w2 + (q.x * vy - q.y * vx) * q.w + q.z * dot2);
}
__device__ __forceinline__ V3 qrotInvS(const Q& q, V3 v)
{
	const float vx = 2.0f * v.x, vy = 2.0f * v.y, vz = 2.0f * v.z;
	const float w2 = q.w * q.w - 0.5f;
	const float dot2 = q.x * vx + q.y * vy + q.z * vz;
	return v3(vx * w2 - (q.y * vz - q.z * vy) * q.w + q.x * dot2, vy * w2 - (q.z * vx - q.x * vz) * q.w + q.y * dot2,
	          vz * w2 - (q.x * vy - q.y * vx) * q.w + q.z * dot2);
}
__device__ __forceinline__ V3 xformS(const Tr& t, V3 v) { return add(qrotS(t.q, v), t.p); }
__device__ __forceinline__ V3 xformInvS(const Tr& t, V3 v) { return qrotInvS(t.q, sub(v, t.p)); }
// PxQuat::getBasisVector0 and getInvBasisVector0..2
__device__ __forceinline__ V3 basis0(const Q& q)
{
	const float x2 = q.x * 2.0f, w2 = q.w * 2.0f;
	return v3((q.w * w2) - 1.0f + q.x * x2, (q.z * w2) + q.y * x2, (-q.y * w2) + q.z * x2);
}
__device__ __forceinline__ V3 invBasis0(const Q& q)
{
	const float x2 = q.x * 2.0f, w2 = q.w * 2.0f;
	return v3((q.w * w2) - 1.0f + q.x * x2, (-q.z * w2) + q.y * x2, (q.y * w2) + q.z * x2);
}
__device__ __forceinline__ V3 invBasis1(const Q& q)
{
	const float y2 = q.y * 2.0f, w2 = q.w * 2.0f;
	return v3((q.z * w2) + q.x * y2, (q.w * w2) - 1.0f + q.y * y2, (-q.x * w2) + q.z * y2);
}
__device__ __forceinline__ V3 invBasis2(const Q& q)
{
	const float z2 = q.z * 2.0f, w2 = q.w * 2.0f;
	return v3((-q.y * w2) + q.x * z2, (q.x * w2) + q.y * z2, (q.w * w2) - 1.0f + q.z * z2);
}
// PxComputeBasisVectors(dir, right, up) (foundation/PxMathUtils.h:297)
__device__ __forceinline__ void basisVectors(V3 dir, V3& right, V3& up)
{
	if(fabsf(dir.y) <= 0.9999f)
	{
		right = v3(dir.z, 0.0f, -dir.x);
		normalizeIn(right);
		up = v3(dir.y * right.z, dir.z * right.x - dir.x * right.z, -dir.y * right.x);
	}
	else
	{
		right = v3(1.0f, 0.0f, 0.0f);
		up = v3(0.0f, dir.z, -dir.y);
		normalizeIn(up);
	}
}
// PxVec4::dot with (p, 1)
__device__ __forceinline__ float planeDot(const float4& pl, V3 p) { return pl.x * p.x + pl.y * p.y + pl.z * p.z + pl.w * 1.0f; }

// A convex shape: core type, core data (<= 3 floats here), margin, pose (Gu::ConvexShape)
struct Shape
{
	int core;
	float d[3];
	float margin;
	Tr pose;
};

// ---- per-core support (no margin) and contact face, local frame
__device__ __noinline__ V3 localSupport(const Shape& s, V3 dir)
{
	switch(s.core)
	{
	case CORE_SEGMENT: return v3(sgn(dir.x) * s.d[0] * 0.5f, 0.0f, 0.0f);
	case CORE_BOX: return v3(sgn(dir.x) * s.d[0] * 0.5f, sgn(dir.y) * s.d[1] * 0.5f, sgn(dir.z) * s.d[2] * 0.5f);
	case CORE_ELLIPSOID:
	{
		// xform = diag(radii): transformTranspose, getNormalized, transform
		const V3 c0 = v3(s.d[0], 0.0f, 0.0f), c1 = v3(0.0f, s.d[1], 0.0f), c2 = v3(0.0f, 0.0f, s.d[2]);
		const V3 dir1 = normalizeS(v3(dotS(c0, dir), dotS(c1, dir), dotS(c2, dir)));
		return add(add(scale(c0, dir1.x), scale(c1, dir1.y)), scale(c2, dir1.z));
	}
	case CORE_CYLINDER:
	{
		const float h = s.d[0] * 0.5f, r = s.d[1];
		const V3 d = normalizeS(dir);
		const float eps = 1e-5f;
		if(fabsf(d.y) < eps && fabsf(d.z) < eps) return v3(sgn(d.x) * h, r, 0.0f);
		return add(v3(sgn(d.x) * h, 0.0f, 0.0f), scale(normalizeS(v3(0.0f, d.y, d.z)), r));
	}
	case CORE_CONE:
	{
		const float h = s.d[0], r = s.d[1];
		const float sinA = r / sqrtf(h * h + r * r);
		const float halfH = h * 0.5f;
		const V3 d = normalizeS(dir);
		const float eps = 1e-5f;
		if(d.x > sinA) return v3(halfH, 0.0f, 0.0f);
		if(fabsf(d.y) < eps && fabsf(d.z) < eps) return v3(-halfH, r, 0.0f);
		return add(v3(-halfH, 0.0f, 0.0f), scale(normalizeS(v3(0.0f, d.y, d.z)), r));
	}
	default: return v3(0.0f, 0.0f, 0.0f);   // point
	}
}

// rotatePoints (GuConvexSupport.h): turn the face points about center/normal until
// the first one lies toward ref.  The angle's acos and the quaternion's sin/cos are
// evaluated in double and rounded: the host C library's acosf/sinf/cosf that the
// reference calls are nearer to the correctly rounded values than the device's
// single-precision functions.
__device__ __noinline__ void rotatePoints(V3 center, V3 ref, V3 normal, V3* points, uint32_t count)
{
	const float eps = FLT_EPSILON;
	V3 dir0 = sub(points[0], center);
	if(normalizeIn(dir0) < eps) return;
	V3 dir1 = add(sub(ref, center), scale(normal, dotS(normal, sub(ref, center))));
	if(normalizeIn(dir1) < eps) return;
	V3 axis = cross(dir0, dir1);
	if(normalizeIn(axis) < eps) return;
	axis = dotS(normal, axis) > 0.0f ? normal : neg(normal);
	const float c = dotS(dir0, dir1);
	const float lo = -1.0f > c ? -1.0f : c;       // PxClamp(c, -1, 1) = PxMin(1, PxMax(-1, c))
	const float cc = 1.0f < lo ? 1.0f : lo;
	const float angle = float(acos(double(cc)));
	const float a = angle * 0.5f;
	double ds, dc;
	sincos(double(a), &ds, &dc);
	const float sn = float(ds);
	Q rot;
	rot.w = float(dc);
	rot.x = axis.x * sn; rot.y = axis.y * sn; rot.z = axis.z * sn;
	for(uint32_t i = 0; i < count; i++) points[i] = add(qrotS(rot, sub(points[i], center)), center);
}

// contactFace of each core (local frame): up to 4 points of the face toward dir.
__device__ __noinline__ uint32_t localContactFace(const Shape& s, V3 dir, V3 ref, V3& faceNormal, V3* fp)
{
	uint32_t numPoints = 0;
	const float dEps1 = 0.99f, dEps2 = 0.14f;
	switch(s.core)
	{
	case CORE_SEGMENT:
	{
		const float length = s.d[0];
		const V3 d = normalizeS(dir);
		fp[0] = fp[1] = fp[2] = fp[3] = faceNormal = v3(0.0f, 0.0f, 0.0f);
		if(fabsf(d.x) < dEps2)
		{
			faceNormal = normalizeS(v3(0.0f, d.y, d.z));
			fp[0] = v3(length * 0.5f, 0.0f, 0.0f);
			fp[1] = v3(-length * 0.5f, 0.0f, 0.0f);
			numPoints = 2;
		}
		return numPoints;
	}
	case CORE_BOX:
	{
		const V3 ext = v3(s.d[0], s.d[1], s.d[2]);
		const V3 d = normalizeS(dir);
		const float eps = FLT_EPSILON;
		fp[0] = fp[1] = fp[2] = fp[3] = faceNormal = v3(0.0f, 0.0f, 0.0f);
		for(uint32_t axis0 = 0; axis0 < 3 && numPoints == 0; ++axis0)
		{
			const uint32_t axis1 = (axis0 + 1) % 3, axis2 = (axis0 + 2) % 3;
			const float e0 = at(ext, axis0), e1 = at(ext, axis1), e2 = at(ext, axis2);
			const float da0 = at(d, axis0), da1 = at(d, axis1), da2 = at(d, axis2);
			if(fabsf(da0) > dEps1 && (e1 > eps || e2 > eps))
			{
				at(faceNormal, axis0) = sgn(da0);
				const float f0 = sgn(da0) * e0 * 0.5f;
				at(fp[0], axis0) = f0; at(fp[0], axis1) = e1 * 0.5f;  at(fp[0], axis2) = e2 * 0.5f;
				at(fp[1], axis0) = f0; at(fp[1], axis1) = -e1 * 0.5f; at(fp[1], axis2) = e2 * 0.5f;
				at(fp[2], axis0) = f0; at(fp[2], axis1) = -e1 * 0.5f; at(fp[2], axis2) = -e2 * 0.5f;
				at(fp[3], axis0) = f0; at(fp[3], axis1) = e1 * 0.5f;  at(fp[3], axis2) = -e2 * 0.5f;
				numPoints = 4;
			}
			else if(fabsf(da0) < dEps2 && e0 > eps && (fabsf(da1) < dEps1 || e2 < eps) && (fabsf(da2) < dEps1 || e1 < eps))
			{
				at(faceNormal, axis1) = da1;
				at(faceNormal, axis2) = da2;
				normalizeIn(faceNormal);
				const float f1 = sgn(da1) * e1 * 0.5f, f2 = sgn(da2) * e2 * 0.5f;
				at(fp[0], axis0) = e0 * 0.5f;  at(fp[0], axis1) = f1; at(fp[0], axis2) = f2;
				at(fp[1], axis0) = -e0 * 0.5f; at(fp[1], axis1) = f1; at(fp[1], axis2) = f2;
				numPoints = 2;
			}
		}
		return numPoints;
	}
	case CORE_ELLIPSOID:
	{
		const V3 rad = v3(s.d[0], s.d[1], s.d[2]);
		const V3 d = normalizeS(dir);
		const float eps = FLT_EPSILON;
		fp[0] = fp[1] = fp[2] = fp[3] = faceNormal = v3(0.0f, 0.0f, 0.0f);
		for(uint32_t axis0 = 0; axis0 < 3 && numPoints == 0; ++axis0)
		{
			const uint32_t axis1 = (axis0 + 1) % 3, axis2 = (axis0 + 2) % 3;
			const float r0 = at(rad, axis0), r1 = at(rad, axis1), r2 = at(rad, axis2);
			const float da0 = at(d, axis0);
			if(fabsf(da0) > dEps1 && r0 < eps && r1 > eps && r2 > eps)
			{
				at(faceNormal, axis0) = sgn(da0);
				at(fp[0], axis1) = r1;
				at(fp[1], axis1) = -r1;
				at(fp[2], axis2) = r2;
				at(fp[3], axis2) = -r2;
				numPoints = 4;
			}
			else if(fabsf(da0) < dEps2 && r0 > eps && r1 < eps && r2 < eps)
			{
				at(faceNormal, axis1) = at(d, axis1);
				at(faceNormal, axis2) = at(d, axis2);
				normalizeIn(faceNormal);
				at(fp[0], axis0) = r0;
				at(fp[1], axis0) = -r0;
				numPoints = 2;
			}
		}
		return numPoints;
	}
	case CORE_CYLINDER:
	{
		const float height = s.d[0], radius = s.d[1];
		const V3 d = normalizeS(dir);
		faceNormal = v3(0.0f, 0.0f, 0.0f);
		if(fabsf(d.x) > dEps1 && radius > 0.0f)
		{
			const float cx = sgn(d.x) * height * 0.5f;
			faceNormal = v3(sgn(d.x), 0.0f, 0.0f);
			fp[0] = v3(cx, radius, 0.0f);
			fp[1] = v3(cx, 0.0f, radius);
			fp[2] = v3(cx, -radius, 0.0f);
			fp[3] = v3(cx, 0.0f, -radius);
			numPoints = 4;
			rotatePoints(v3(cx, 0.0f, 0.0f), ref, faceNormal, fp, numPoints);
		}
		else if(fabsf(d.x) < dEps2 && height > 0.0f)
		{
			const V3 dr = faceNormal = normalizeS(v3(0.0f, d.y, d.z));
			fp[0] = add(v3(height * 0.5f, 0.0f, 0.0f), scale(dr, radius));
			fp[1] = add(v3(-height * 0.5f, 0.0f, 0.0f), scale(dr, radius));
			numPoints = 2;
		}
		return numPoints;
	}
	case CORE_CONE:
	{
		const float height = s.d[0], radius = s.d[1];
		faceNormal = v3(0.0f, 0.0f, 0.0f);
		if(height + radius > 0.0f)
		{
			const V3 d = normalizeS(dir);
			const float eps = 1e-5f;
			if((d.x < -dEps1 || (d.x > dEps1 && height < eps)) && radius > 0.0f)
			{
				const float cx = sgn(d.x) * height * 0.5f;
				faceNormal = v3(sgn(d.x), 0.0f, 0.0f);
				fp[0] = v3(cx, radius, 0.0f);
				fp[1] = v3(cx, 0.0f, radius);
				fp[2] = v3(cx, -radius, 0.0f);
				fp[3] = v3(cx, 0.0f, -radius);
				numPoints = 4;
				rotatePoints(v3(cx, 0.0f, 0.0f), ref, faceNormal, fp, numPoints);
			}
			else if(height > 0.0f)
			{
				const float sinA = radius / sqrtf(height * height + radius * radius);
				const float dX = d.x * sqrtf(1.0f - sinA * sinA) - sqrtf(1.0f - d.x * d.x) * sinA;
				if(fabsf(dX) < dEps2)
				{
					const V3 dr = normalizeS(v3(0.0f, d.y, d.z));
					faceNormal = normalizeS(v3(radius / height, dr.y, dr.z));
					fp[0] = v3(height * 0.5f, 0.0f, 0.0f);
					fp[1] = add(v3(-height * 0.5f, 0.0f, 0.0f), scale(dr, radius));
					numPoints = 2;
				}
			}
		}
		return numPoints;
	}
	default:
		faceNormal = v3(0.0f, 0.0f, 0.0f);
		return 0;   // point
	}
}

// ConvexShape::support (world, with margin) and ::contactFace (world)
__device__ __forceinline__ V3 support(const Shape& s, V3 dir)
{
	return add(xformS(s.pose, localSupport(s, qrotInvS(s.pose.q, dir))), scale(dir, s.margin));
}
__device__ __noinline__ uint32_t contactFace(const Shape& s, V3 dir, V3 point, V3& faceNormal, V3* fp)
{
	const uint32_t n = localContactFace(s, qrotInvS(s.pose.q, dir), xformInvS(s.pose, point), faceNormal, fp);
	faceNormal = qrotS(s.pose.q, faceNormal);
	for(uint32_t i = 0; i < n; i++) fp[i] = add(xformS(s.pose, fp[i]), scale(faceNormal, s.margin));
	return n;
}

// ---- RefGjkEpa::Convex: a shape's support points, welded within its accuracy
constexpr uint32_t CVX_MAX_VERTS = 32;
struct Cvx
{
	const Shape* s;
	V3 verts[CVX_MAX_VERTS];
	uint32_t n;
	float acc;
};
__device__ __noinline__ void cvxInit(Cvx& c, const Shape& s)
{
	c.s = &s;
	c.n = 0;
	const V3 X = v3(1, 0, 0), Y = v3(0, 1, 0), Z = v3(0, 0, 1);
	const V3 mn = v3(localSupport(s, neg(X)).x, localSupport(s, neg(Y)).y, localSupport(s, neg(Z)).z);
	const V3 mx = v3(localSupport(s, X).x, localSupport(s, Y).y, localSupport(s, Z).z);
	const V3 dim = sub(mx, mn);
	const float maxExtent = fmax_(dim.x, fmax_(dim.y, dim.z));
	c.acc = fmax_(maxExtent * 0.01f, FLT_EPSILON);
}
// getBounds().getCenter() in world space
__device__ __noinline__ V3 cvxCenter(const Cvx& c)
{
	const Shape& s = *c.s;
	const V3 X = invBasis0(s.pose.q), Y = invBasis1(s.pose.q), Z = invBasis2(s.pose.q);
	const V3 mn = v3(xformS(s.pose, localSupport(s, neg(X))).x, xformS(s.pose, localSupport(s, neg(Y))).y,
	                 xformS(s.pose, localSupport(s, neg(Z))).z);
	const V3 mx = v3(xformS(s.pose, localSupport(s, X)).x, xformS(s.pose, localSupport(s, Y)).y, xformS(s.pose, localSupport(s, Z)).z);
	return scale(add(mn, mx), 0.5f);
}
__device__ __noinline__ uint32_t cvxSupportIndex(Cvx& c, V3 dir)
{
	const Shape& s = *c.s;
	const V3 v = xformS(s.pose, localSupport(s, qrotInvS(s.pose.q, dir)));
	uint32_t closest = CVX_MAX_VERTS;
	const float weld = c.acc * c.acc;
	float distSq = FLT_MAX;
	for(int i = int(c.n) - 1; i >= 0; --i)
	{
		const float dSq = lenSqS(sub(c.verts[i], v));
		if(dSq < weld) return uint32_t(i);
		if(distSq > dSq) { distSq = dSq; closest = uint32_t(i); }
	}
	if(c.n == CVX_MAX_VERTS) return closest;
	c.verts[c.n++] = v;
	return c.n - 1;
}

// ---- RefGjkEpa::GjkDistance
struct GjkVert { V3 p; float s; uint32_t aI, bI; };
struct Gjk
{
	Cvx* A;
	Cvx* B;
	uint32_t n, iter;
	GjkVert v[4];
	V3 closest;
};
__device__ __forceinline__ GjkVert gjkVert(V3 p, float s, uint32_t a, uint32_t b) { GjkVert r; r.p = p; r.s = s; r.aI = a; r.bI = b; return r; }
__device__ __noinline__ float gjkAddPoint(Gjk& g, V3 dir)
{
	if(++g.iter > 100u) return FLT_MAX;   // MAX_ITERATIONS
	const uint32_t aI = cvxSupportIndex(*g.A, dir), bI = cvxSupportIndex(*g.B, neg(dir));
	const V3 p = sub(g.A->verts[aI], g.B->verts[bI]);
	for(uint32_t i = 0; i < g.n; ++i)
		if(g.v[i].aI == aI && g.v[i].bI == bI) return FLT_MAX;
	g.v[g.n++] = gjkVert(p, 0.0f, aI, bI);
	return dotS(p, neg(dir));
}
__device__ __forceinline__ void swapV(GjkVert& a, GjkVert& b) { const GjkVert t = a; a = b; b = t; }
__device__ __noinline__ void gjkComputeClosest(Gjk& g)
{
	GjkVert vs[4];
	for(int i = 0; i < 4; i++) { vs[i] = g.v[i]; vs[i].s = 0.0f; }
	uint32_t num = g.n;
	switch(num)
	{
	case 1:
		vs[0].s = 1.0f;
		break;
	case 2:
	{
		const V3 a = vs[0].p, b = vs[1].p;
		const V3 ba = sub(a, b);
		const float sba = dotS(ba, neg(b));
		if(sba <= 0.0f) { vs[0] = vs[1]; vs[0].s = 1.0f; num = 1; break; }
		vs[0].s = sba / lenSqS(ba);
		vs[1].s = 1.0f - vs[0].s;
		break;
	}
	case 3:
	{
		const V3 a = vs[0].p, b = vs[1].p, c = vs[2].p;
		const V3 ca = sub(a, c), cb = sub(b, c);
		const float sca = dotS(ca, neg(c)), scb = dotS(cb, neg(c));
		if(sca <= 0.0f && scb <= 0.0f) { vs[0] = vs[2]; vs[0].s = 1.0f; num = 1; break; }
		const V3 abc = cross(sub(b, a), sub(c, a));
		const float iabc = 1.0f / lenSqS(abc);
		const V3 pabc = scale(scale(abc, dotS(abc, a)), iabc);
		const float tca = dotS(abc, cross(sub(c, pabc), sub(a, pabc)));
		if(sca > 0.0f && tca <= 0.0f)
		{
			vs[1] = vs[2];
			vs[0].s = sca / lenSqS(ca);
			vs[1].s = 1.0f - vs[0].s;
			num = 2;
			break;
		}
		const float tbc = dotS(abc, cross(sub(b, pabc), sub(c, pabc)));
		if(scb > 0.0f && tbc <= 0.0f)
		{
			vs[0] = vs[1];
			vs[1] = vs[2];
			vs[0].s = scb / lenSqS(cb);
			vs[1].s = 1.0f - vs[0].s;
			num = 2;
			break;
		}
		vs[0].s = tbc * iabc;
		vs[1].s = tca * iabc;
		vs[2].s = 1.0f - vs[0].s - vs[1].s;
		if(dotS(abc, a) > 0.0f) swapV(vs[0], vs[1]);
		break;
	}
	case 4:
	{
		const V3 a = vs[0].p, b = vs[1].p, c = vs[2].p, d = vs[3].p;
		const V3 da = sub(a, d), db = sub(b, d), dc = sub(c, d);
		const float sda = dotS(da, neg(d)), sdb = dotS(db, neg(d)), sdc = dotS(dc, neg(d));
		if(sda <= 0.0f && sdb <= 0.0f && sdc <= 0.0f) { vs[0] = vs[3]; vs[0].s = 1.0f; num = 1; break; }
		const V3 dab = cross(sub(a, d), sub(b, d));
		const float idab = 1.0f / lenSqS(dab);
		const V3 pdab = scale(scale(dab, dotS(dab, d)), idab);
		const V3 dbc = cross(sub(b, d), sub(c, d));
		const float idbc = 1.0f / lenSqS(dbc);
		const V3 pdbc = scale(scale(dbc, dotS(dbc, d)), idbc);
		const V3 dca = cross(sub(c, d), sub(a, d));
		const float idca = 1.0f / lenSqS(dca);
		const V3 pdca = scale(scale(dca, dotS(dca, d)), idca);
		const float tda = dotS(dab, cross(sub(d, pdab), sub(a, pdab)));
		const float tad = dotS(dca, cross(sub(a, pdca), sub(d, pdca)));
		if(sda > 0.0f && tda <= 0.0f && tad <= 0.0f)
		{
			vs[1] = vs[3];
			vs[0].s = sda / lenSqS(da);
			vs[1].s = 1.0f - vs[0].s;
			num = 2;
			break;
		}
		const float tdb = dotS(dbc, cross(sub(d, pdbc), sub(b, pdbc)));
		const float tbd = dotS(dab, cross(sub(b, pdab), sub(d, pdab)));
		if(sdb > 0.0f && tdb <= 0.0f && tbd <= 0.0f)
		{
			vs[0] = vs[1];
			vs[1] = vs[3];
			vs[0].s = sdb / lenSqS(db);
			vs[1].s = 1.0f - vs[0].s;
			num = 2;
			break;
		}
		const float tcd = dotS(dbc, cross(sub(c, pdbc), sub(d, pdbc)));
		const float tdc = dotS(dca, cross(sub(d, pdca), sub(c, pdca)));
		if(sdc > 0.0f && tdc <= 0.0f && tcd <= 0.0f)
		{
			vs[0] = vs[2];
			vs[1] = vs[3];
			vs[0].s = sdc / lenSqS(dc);
			vs[1].s = 1.0f - vs[0].s;
			num = 2;
			break;
		}
		const V3 abc = cross(sub(b, a), sub(c, a));
		if(tda > 0.0f && tbd > 0.0f && dotS(dab, d) < 0.0f && dotS(abc, dab) > 0.0f)
		{
			vs[2] = vs[3];
			vs[0].s = tbd * idab;
			vs[1].s = tda * idab;
			vs[2].s = 1.0f - vs[0].s - vs[1].s;
			num = 3;
			break;
		}
		if(tdb > 0.0f && tcd > 0.0f && dotS(dbc, d) < 0.0f && dotS(abc, dbc) > 0.0f)
		{
			vs[0] = vs[1];
			vs[1] = vs[2];
			vs[2] = vs[3];
			vs[0].s = tcd * idbc;
			vs[1].s = tdb * idbc;
			vs[2].s = 1.0f - vs[0].s - vs[1].s;
			num = 3;
			break;
		}
		if(tdc > 0.0f && tad > 0.0f && dotS(dca, d) < 0.0f && dotS(abc, dca) > 0.0f)
		{
			vs[1] = vs[3];
			vs[0].s = tdc * idca;
			vs[2].s = tad * idca;
			vs[1].s = 1.0f - vs[0].s - vs[2].s;
			num = 3;
			break;
		}
		break;
	}
	default: break;
	}
	const V3 cl = add(add(add(scale(vs[0].p, vs[0].s), scale(vs[1].p, vs[1].s)), scale(vs[2].p, vs[2].s)), scale(vs[3].p, vs[3].s));
	if(magS(cl) < magS(g.closest) - FLT_EPSILON)
	{
		g.closest = cl;
		for(int i = 0; i < 4; i++) g.v[i] = vs[i];
		g.n = num;
	}
	else
		--g.n;
}

// computeGjkDistance: the gap between the cores (FLT_MAX beyond maxDist, 0 on overlap)
__device__ __noinline__ float gjkDistance(Cvx& A, Cvx& B, float maxDist, V3& pointA, V3& pointB, V3& axis)
{
	Gjk g;
	g.A = &A; g.B = &B;
	g.n = 0; g.iter = 0;
	g.closest = v3(FLT_MAX, FLT_MAX, FLT_MAX);
	for(int i = 0; i < 4; i++) g.v[i] = gjkVert(v3(0, 0, 0), 0.0f, 0, 0);
	V3 dir = sub(cvxCenter(B), cvxCenter(A));
	if(normalizeIn(dir) < FLT_EPSILON) dir = v3(1, 0, 0);
	gjkAddPoint(g, dir);
	const float distEps = 0.01f * fmin_(A.acc, B.acc);
	for(int guard = 0; guard < 256; guard++)   // the loop ends within 100 added points
	{
		gjkComputeClosest(g);
		const float closestDist = magS(g.closest);
		if(closestDist < distEps) return 0.0f;
		const V3 d = neg(normalizeS(g.closest));
		const float proj = gjkAddPoint(g, d);
		if(proj >= closestDist - distEps)
		{
			V3 pA = v3(0, 0, 0), pB = v3(0, 0, 0);
			for(uint32_t i = 0; i < g.n; ++i)
			{
				pA = add(pA, scale(A.verts[g.v[i].aI], g.v[i].s));
				pB = add(pB, scale(B.verts[g.v[i].bI], g.v[i].s));
			}
			pointA = pA; pointB = pB;
			axis = neg(d);
			return closestDist;
		}
		if(proj > maxDist) return FLT_MAX;
	}
	return FLT_MAX;
}

// ---- RefGjkEpa::EpaDepth
constexpr uint32_t EPA_MAX_VERTS = 32;
constexpr uint32_t EPA_MAX_FACES = 2 * EPA_MAX_VERTS - 4;
constexpr uint32_t EPA_MAX_EDGES = EPA_MAX_VERTS + EPA_MAX_FACES - 2;
struct EpaFace { float4 plane; uint8_t v[4]; };
struct Epa
{
	Cvx* A;
	Cvx* B;
	uint8_t va[EPA_MAX_VERTS], vb[EPA_MAX_VERTS];
	EpaFace f[EPA_MAX_FACES];
	uint32_t nv, nf;
	EpaFace closest, best;
	float proj;
};
__device__ __forceinline__ EpaFace epaFace(float4 pl, uint32_t a, uint32_t b, uint32_t c)
{
	EpaFace r; r.plane = pl; r.v[0] = uint8_t(a); r.v[1] = uint8_t(b); r.v[2] = uint8_t(c); r.v[3] = 0; return r;
}
__device__ __forceinline__ V3 epaVert(const Epa& e, uint32_t i) { return sub(e.A->verts[e.va[i]], e.B->verts[e.vb[i]]); }
__device__ __noinline__ bool epaMakePlane(const Epa& e, uint32_t i0, uint32_t i1, uint32_t i2, float4& plane)
{
	const V3 a = epaVert(e, i0), b = epaVert(e, i1), c = epaVert(e, i2);
	const V3 abc = add(add(cross(sub(b, a), sub(c, a)), cross(sub(c, b), sub(a, b))), cross(sub(a, c), sub(b, c)));
	const float labc = magS(abc);
	if(labc < FLT_EPSILON) return false;
	const V3 n = divS(abc, labc);
	plane = make_float4(n.x, n.y, n.z, dotS(n, neg(a)));
	return true;
}
__device__ __noinline__ float epaAddPoint(Epa& e, V3 dir)
{
	if(e.nv > EPA_MAX_VERTS - 1) return FLT_MAX;
	const uint32_t aI = cvxSupportIndex(*e.A, dir), bI = cvxSupportIndex(*e.B, neg(dir));
	const V3 p = sub(e.A->verts[aI], e.B->verts[bI]);
	const float proj = dotS(p, neg(dir));
	if(proj > e.proj) { e.proj = proj; e.best = e.closest; }
	for(uint32_t i = 0; i < e.nv; ++i)
		if(aI == e.va[i] && bI == e.vb[i]) return FLT_MAX;
	e.va[e.nv] = uint8_t(aI); e.vb[e.nv] = uint8_t(bI);
	e.nv++;
	if(e.nv < 3) return 0.0f;
	if(e.nv == 3)
	{
		float4 plane0, plane1;
		if(!epaMakePlane(e, 0, 1, 2, plane0) || !epaMakePlane(e, 1, 0, 2, plane1)) return FLT_MAX;
		e.f[e.nf++] = epaFace(plane0, 0, 1, 2);
		e.f[e.nf++] = epaFace(plane1, 1, 0, 2);
		return 0.0f;
	}
	const float testEps = 0.01f * fmin_(e.A->acc, e.B->acc);
	uint8_t edges[EPA_MAX_EDGES][2];
	uint32_t numEdges = 0;
	for(int i = int(e.nf) - 1; i >= 0; --i)
	{
		const EpaFace fc = e.f[i];
		if(planeDot(fc.plane, p) > testEps)
		{
			for(uint32_t j = 0; j < 3; ++j)
			{
				bool addE = true;
				const uint8_t v0 = fc.v[j], v1 = fc.v[(j + 1) % 3];
				for(int k = int(numEdges) - 1; k >= 0; --k)
				{
					if(v0 == edges[k][1] && v1 == edges[k][0])
					{
						addE = false;
						--numEdges;
						edges[k][0] = edges[numEdges][0];
						edges[k][1] = edges[numEdges][1];
						break;
					}
				}
				if(addE)
				{
					if(numEdges == EPA_MAX_EDGES) return FLT_MAX;   // beyond the reference's arrays
					edges[numEdges][0] = v0;
					edges[numEdges][1] = v1;
					numEdges++;
				}
			}
			e.f[i] = e.f[--e.nf];
		}
	}
	if(numEdges == 0) return FLT_MAX;
	if(e.nf > EPA_MAX_FACES - numEdges) return FLT_MAX;   // unsigned, as the reference's
	for(uint32_t i = 0; i < numEdges; ++i)
	{
		float4 plane;
		if(!epaMakePlane(e, edges[i][0], edges[i][1], e.nv - 1, plane)) return FLT_MAX;
		if(e.nf >= EPA_MAX_FACES) return FLT_MAX;
		e.f[e.nf++] = epaFace(plane, edges[i][0], edges[i][1], e.nv - 1);
	}
	return proj;
}
__device__ __noinline__ void epaComputeClosest(Epa& e)
{
	uint32_t c = 0xffffffffu;
	float cw = -FLT_MAX;
	for(uint32_t i = 0; i < e.nf; ++i)
	{
		const float w = e.f[i].plane.w;
		if(w > cw) { c = i; cw = w; }
	}
	if(c == 0xffffffffu) c = 0;
	e.closest = e.f[c];
	if(e.nf == 2) e.best = e.closest;
}
// computeEpaDepth: the overlap depth as a negative distance, FLT_MAX if the polytope fails
__device__ __noinline__ float epaDepth(Cvx& A, Cvx& B, V3& pointA, V3& pointB, V3& axis)
{
	Epa e;
	e.A = &A; e.B = &B;
	e.nv = 0; e.nf = 0;
	e.closest = epaFace(make_float4(0.0f, 0.0f, 0.0f, 0.0f), 0, 0, 0);
	e.best = e.closest;
	e.proj = -FLT_MAX;
	V3 dir0 = sub(cvxCenter(B), cvxCenter(A));
	if(normalizeIn(dir0) < FLT_EPSILON) dir0 = v3(1, 0, 0);
	V3 dir1, dir2;
	basisVectors(dir0, dir1, dir2);
	epaAddPoint(e, dir0);
	epaAddPoint(e, neg(dir0));
	epaAddPoint(e, dir1);
	if(e.nv < 3) epaAddPoint(e, neg(dir1));
	if(e.nv < 3) epaAddPoint(e, dir2);
	if(e.nv < 3) epaAddPoint(e, neg(dir2));
	e.proj = -FLT_MAX;
	if(e.nf == 0) return FLT_MAX;
	const float distEps = 0.01f * fmin_(A.acc, B.acc);
	for(int guard = 0; guard < 64; guard++)   // each pass adds a vertex (at most 32) or ends
	{
		epaComputeClosest(e);
		const float closestDist = e.closest.plane.w;
		const V3 d = v3(e.closest.plane.x, e.closest.plane.y, e.closest.plane.z);
		const float proj = epaAddPoint(e, d);
		if(proj >= closestDist - distEps)
		{
			const uint32_t i0 = e.best.v[0], i1 = e.best.v[1], i2 = e.best.v[2];
			const V3 va0 = A.verts[e.va[i0]], va1 = A.verts[e.va[i1]], va2 = A.verts[e.va[i2]];
			const V3 vb0 = B.verts[e.vb[i0]], vb1 = B.verts[e.vb[i1]], vb2 = B.verts[e.vb[i2]];
			const V3 a = sub(va0, vb0), b = sub(va1, vb1), c = sub(va2, vb2);
			const V3 abc = cross(sub(b, a), sub(c, a));
			const float iabc = 1.0f / lenSqS(abc);
			const V3 pabc = scale(scale(abc, dotS(abc, a)), iabc);
			const float tbc = dotS(abc, cross(sub(b, pabc), sub(c, pabc)));
			const float tca = dotS(abc, cross(sub(c, pabc), sub(a, pabc)));
			const float tab = dotS(abc, cross(sub(a, pabc), sub(b, pabc)));
			const float sa = tbc * iabc, sb = tca * iabc, sc = tab * iabc;
			pointA = add(add(scale(va0, sa), scale(va1, sb)), scale(va2, sc));
			pointB = add(add(scale(vb0, sa), scale(vb1, sb)), scale(vb2, sc));
			axis = neg(v3(e.best.plane.x, e.best.plane.y, e.best.plane.z));
			return e.best.plane.w;
		}
	}
	return FLT_MAX;
}

// ---- reducePolygon: up to 4 indices of pts forming the largest quad (keep1st keeps pts[0])
__device__ __noinline__ uint32_t reducePolygon(const V3* pts, uint32_t count, V3 normal, uint32_t inds[4], bool keep1st)
{
	const float eps = FLT_EPSILON;
	uint32_t pi0 = 0xffffffffu, pi1 = 0xffffffffu;
	if(keep1st)
	{
		pi0 = 0;
		float maxDist = -FLT_MAX;
		const V3 p0 = pts[pi0];
		for(uint32_t j = 0; j < count; ++j)
		{
			const float dist = lenSqS(sub(pts[j], p0));
			if(dist > maxDist + eps) { maxDist = dist; pi1 = j; }
		}
	}
	else
	{
		float maxDist = -FLT_MAX;
		for(uint32_t i = 0; i < count; ++i)
			for(uint32_t j = 0; j < count; ++j)
			{
				const float dist = lenSqS(sub(pts[j], pts[i]));
				if(dist > maxDist + eps) { maxDist = dist; pi0 = i; pi1 = j; }
			}
	}
	if(pi0 == 0xffffffffu || pi1 == 0xffffffffu) return 0;
	if(pi0 == pi1) { inds[0] = pi0; return 1; }
	uint32_t pi2 = 0xffffffffu, pi3 = 0xffffffffu;
	{
		const V3 p0 = pts[pi0], p1 = pts[pi1];
		const V3 n01 = cross(normal, sub(p1, p0));
		float minDist = 0.0f, maxDist = 0.0f;
		for(uint32_t i = 0; i < count; ++i)
		{
			const float d = dotS(n01, sub(pts[i], p0));
			if(d < minDist - eps) { pi2 = i; minDist = d; }
			if(d > maxDist + eps) { pi3 = i; maxDist = d; }
		}
	}
	uint32_t n = 0;
	inds[n++] = pi0;
	inds[n++] = pi1;
	if(pi2 != 0xffffffffu && pi2 != pi0 && pi2 != pi1) inds[n++] = pi2;
	if(pi3 != 0xffffffffu && pi3 != pi0 && pi3 != pi1 && pi3 != pi2) inds[n++] = pi3;
	return n;
}

// ---- FaceClipper: the contact patch from both contact faces and the GJK/EPA points
constexpr uint32_t MAX_CLIP_PLANES = MAX_FACE_POINTS * 2;
constexpr uint32_t MAX_POLYGON_POINTS = MAX_CLIP_PLANES + 4 + 1;
struct Clip
{
	V3 point0, point1, axis;
	V3 faceNormal0, faceNormal1;
	V3 fp0[MAX_FACE_POINTS], fp1[MAX_FACE_POINTS];
	uint32_t n0, n1;
	float4 out[MAX_CONTACTS];
	uint32_t nOut;
};
__device__ __noinline__ void clipNone(Clip& c)
{
	const V3 m = scale(add(c.point0, c.point1), 0.5f);
	c.out[0] = make_float4(m.x, m.y, m.z, dotS(c.axis, sub(c.point0, c.point1)));
	c.nOut = 1;
}
__device__ __noinline__ void clip2x2(Clip& c)
{
	const float eps = 1e-5f;
	const V3 a = c.fp0[0], b = c.fp0[1], cc = c.fp1[0], d = c.fp1[1];
	const V3 axis = c.axis;
	if(fabsf(dotS(cross(sub(b, a), sub(d, cc)), axis)) > eps) return clipNone(c);
	uint32_t n = 0;
	float4 pts[4];
	if(dotS(sub(a, cc), sub(d, cc)) > -eps && dotS(sub(a, d), sub(cc, d)) > -eps)
	{
		const V3 a1 = add(cc, divS(scale(sub(d, cc), dotS(sub(d, cc), sub(a, cc))), lenSqS(sub(d, cc))));
		const V3 m = scale(add(a, a1), 0.5f);
		pts[n++] = make_float4(m.x, m.y, m.z, dotS(axis, sub(a, a1)));
	}
	if(dotS(sub(b, cc), sub(d, cc)) > -eps && dotS(sub(b, d), sub(cc, d)) > -eps)
	{
		const V3 b1 = add(cc, divS(scale(sub(d, cc), dotS(sub(d, cc), sub(b, cc))), lenSqS(sub(d, cc))));
		const V3 m = scale(add(b, b1), 0.5f);
		pts[n++] = make_float4(m.x, m.y, m.z, dotS(axis, sub(b, b1)));
	}
	if(dotS(sub(cc, a), sub(b, a)) > -eps && dotS(sub(cc, b), sub(a, b)) > -eps)
	{
		const V3 c1 = add(a, divS(scale(sub(b, a), dotS(sub(b, a), sub(cc, a))), lenSqS(sub(b, a))));
		const V3 m = scale(add(c1, cc), 0.5f);
		pts[n++] = make_float4(m.x, m.y, m.z, dotS(axis, sub(c1, cc)));
	}
	if(dotS(sub(d, a), sub(b, a)) > -eps && dotS(sub(d, b), sub(a, b)) > -eps)
	{
		const V3 d1 = add(a, divS(scale(sub(b, a), dotS(sub(b, a), sub(d, a))), lenSqS(sub(b, a))));
		const V3 m = scale(add(d1, d), 0.5f);
		pts[n++] = make_float4(m.x, m.y, m.z, dotS(axis, sub(d1, d)));
	}
	const float mergeEps = 1e-6f;
	for(int i = int(n) - 1; i >= 0; --i)
		for(int j = i - 1; j >= 0; --j)
		{
			const V3 dd = v3(pts[i].x - pts[j].x, pts[i].y - pts[j].y, pts[i].z - pts[j].z);
			if(lenSqS(dd) < mergeEps)
			{
				if(pts[i].w < pts[j].w) pts[j] = pts[i];
				pts[i] = pts[--n];
				break;
			}
		}
	for(uint32_t i = 0; i < n; ++i) c.out[i] = pts[i];
	c.nOut = n;
}
__device__ __noinline__ void makePlanes(const Clip& c, const V3* fp, uint32_t num, float4* planes, uint32_t& numPlanes)
{
	if(num < 3) return;
	const V3 axis = c.axis;
	const float eps = 1e-5f;
	for(uint32_t i = 0; i < num; ++i)
	{
		const V3 s = fp[i];
		for(uint32_t j = i + 1; j < num; ++j)
		{
			const V3 e = fp[j];
			V3 n = cross(sub(e, s), axis);
			if(lenSqS(n) < eps * eps) continue;
			normalizeFastIn(n);
			uint32_t pos = 0, negc = 0;
			for(uint32_t k = 0; k < num; ++k)
			{
				if(k == i || k == j) continue;
				const float d = dotS(sub(fp[k], s), n);
				if(d > eps) pos++;
				else negc++;
			}
			if(pos && negc) continue;
			if(pos) n = neg(n);
			if(numPlanes < MAX_CLIP_PLANES) planes[numPlanes++] = make_float4(-n.x, -n.y, -n.z, dotS(n, s));
		}
	}
}
__device__ __noinline__ void clipPoly(float4 plane, V3* pts, uint32_t& num)
{
	float dist[MAX_POLYGON_POINTS];
	for(uint32_t i = 0; i < num; ++i) dist[i] = planeDot(plane, pts[i]);
	const float eps = 1e-5f;
	uint32_t nn = 0;
	V3 np[MAX_POLYGON_POINTS];
	for(uint32_t i = 0; i < num; ++i)
	{
		const uint32_t i0 = i, i1 = (i + 1) % num;
		const float d0 = dist[i0], d1 = dist[i1];
		const V3 p0 = pts[i0], p1 = pts[i1];
		if(d0 > -eps)
		{
			if(nn < MAX_POLYGON_POINTS) np[nn++] = p0;
			if(d1 < -eps && d0 - d1 > eps && nn < MAX_POLYGON_POINTS) np[nn++] = add(p0, scale(sub(p1, p0), d0 / (d0 - d1)));
		}
		else if(d1 > -eps && d1 - d0 > eps && nn < MAX_POLYGON_POINTS)
			np[nn++] = add(p0, scale(sub(p1, p0), d0 / (d0 - d1)));
	}
	num = nn;
	for(uint32_t i = 0; i < num; ++i) pts[i] = np[i];
}
__device__ __noinline__ void clipNxN(Clip& c)
{
	uint32_t numPlanes = 0;
	float4 planes[MAX_CLIP_PLANES];
	makePlanes(c, c.fp0, c.n0, planes, numPlanes);
	makePlanes(c, c.fp1, c.n1, planes, numPlanes);
	uint32_t np = 0;
	V3 poly[MAX_POLYGON_POINTS];
	// makePolygon
	if(c.n0 == 2) { poly[np++] = c.fp0[0]; poly[np++] = c.fp0[1]; }
	else if(c.n1 == 2) { poly[np++] = c.fp1[0]; poly[np++] = c.fp1[1]; }
	else
	{
		V3 X, Y;
		basisVectors(c.axis, X, Y);
		float minX = FLT_MAX, maxX = -FLT_MAX, minY = FLT_MAX, maxY = -FLT_MAX;
		for(uint32_t i = 0; i < c.n0; ++i)
		{
			const float pX = dotS(c.fp0[i], X), pY = dotS(c.fp0[i], Y);
			minX = fmin_(minX, pX); maxX = fmax_(maxX, pX);
			minY = fmin_(minY, pY); maxY = fmax_(maxY, pY);
		}
		for(uint32_t i = 0; i < c.n1; ++i)
		{
			const float pX = dotS(c.fp1[i], X), pY = dotS(c.fp1[i], Y);
			minX = fmin_(minX, pX); maxX = fmax_(maxX, pX);
			minY = fmin_(minY, pY); maxY = fmax_(maxY, pY);
		}
		const V3 ref = scale(add(c.point0, c.point1), 0.5f);
		const float refX = dotS(ref, X), refY = dotS(ref, Y);
		poly[np++] = add(add(ref, scale(X, minX - refX)), scale(Y, minY - refY));
		poly[np++] = add(add(ref, scale(X, maxX - refX)), scale(Y, minY - refY));
		poly[np++] = add(add(ref, scale(X, maxX - refX)), scale(Y, maxY - refY));
		poly[np++] = add(add(ref, scale(X, minX - refX)), scale(Y, maxY - refY));
	}
	for(uint32_t i = 0; i < numPlanes; ++i) clipPoly(planes[i], poly, np);
	if(np < MAX_POLYGON_POINTS) poly[np++] = scale(add(c.point0, c.point1), 0.5f);
	const float4 plane0 = make_float4(c.faceNormal0.x, c.faceNormal0.y, c.faceNormal0.z, -dotS(c.faceNormal0, c.fp0[0]));
	const float4 plane1 = make_float4(c.faceNormal1.x, c.faceNormal1.y, c.faceNormal1.z, -dotS(c.faceNormal1, c.fp1[0]));
	const V3 axis = c.axis;
	float4 pd[MAX_POLYGON_POINTS];
	for(uint32_t i = 0; i < np; ++i)
	{
		const V3 p = poly[i];
		const V3 p0 = sub(p, divS(scale(axis, planeDot(plane0, p)), dotS(axis, v3(plane0.x, plane0.y, plane0.z))));
		const V3 p1 = sub(p, divS(scale(axis, planeDot(plane1, p)), dotS(axis, v3(plane1.x, plane1.y, plane1.z))));
		const V3 m = scale(add(p0, p1), 0.5f);
		pd[i] = make_float4(m.x, m.y, m.z, dotS(axis, sub(p0, p1)));
	}
	uint32_t minI = 0;
	float minD = pd[0].w;
	for(uint32_t i = 0; i < np; ++i)
		if(pd[i].w < minD) { minD = pd[i].w; minI = i; }
	{ const float4 t = pd[0]; pd[0] = pd[minI]; pd[minI] = t; }
	V3 xyz[MAX_POLYGON_POINTS];
	for(uint32_t i = 0; i < np; ++i) xyz[i] = v3(pd[i].x, pd[i].y, pd[i].z);
	uint32_t inds[4];
	const uint32_t n = reducePolygon(xyz, np, axis, inds, true);
	for(uint32_t i = 0; i < n; ++i) c.out[i] = pd[inds[i]];
	c.nOut = n;
}

// generateContacts(convex0, convex1): normal (from 1 toward 0), up to 4 points and separations
__device__ __noinline__ uint32_t convexConvex(const Shape& s0, const Shape& s1, float contactDist, V3& normal, V3* points, float* dists)
{
	const float maxDist = s0.margin + s1.margin + contactDist;
	V3 point0 = v3(0, 0, 0), point1 = v3(0, 0, 0), axis = v3(0, 0, 0);
	float dist;
	{
		Cvx A, B;
		cvxInit(A, s0);
		cvxInit(B, s1);
		dist = gjkDistance(A, B, maxDist, point0, point1, axis);
	}
	if(dist < FLT_EPSILON)
	{
		Cvx A, B;
		cvxInit(A, s0);
		cvxInit(B, s1);
		dist = epaDepth(A, B, point0, point1, axis);
	}
	if(dist > maxDist) return 0;
	// cullDir is zero here: cullDir.dot(axis) < -1e-5 never holds
	point0 = sub(point0, scale(axis, s0.margin));
	point1 = add(point1, scale(axis, s1.margin));
	Clip c;
	c.point0 = point0; c.point1 = point1; c.axis = axis;
	c.n0 = contactFace(s0, neg(axis), point0, c.faceNormal0, c.fp0);
	c.n1 = contactFace(s1, axis, point1, c.faceNormal1, c.fp1);
	if(c.n0 < 2 || c.n1 < 2) clipNone(c);
	else if(c.n0 == 2 && c.n1 == 2) clip2x2(c);
	else clipNxN(c);
	normal = axis;
	for(uint32_t i = 0; i < c.nOut; ++i)
	{
		points[i] = v3(c.out[i].x, c.out[i].y, c.out[i].z);
		dists[i] = c.out[i].w;
	}
	return c.nOut;
}

// generateContacts(plane, convex1): the plane is x = 0 of its pose
__device__ __noinline__ uint32_t planeConvex(const Tr& planePose, const Shape& s1, float contactDist, V3& normal, V3* points, float* dists)
{
	const V3 pn = basis0(planePose.q);
	const float pd = -dotS(planePose.p, pn);
	normal = neg(pn);
	const V3 point1 = support(s1, normal);
	const float dist = dotS(point1, pn) + pd;
	uint32_t num = 0;
	if(dist < contactDist)
	{
		V3 faceNormal, fp[MAX_FACE_POINTS];
		const uint32_t np = contactFace(s1, normal, point1, faceNormal, fp);
		if(np == 0)
		{
			points[num] = add(point1, scale(scale(normal, dist), 0.5f));
			dists[num] = dist;
			++num;
		}
		for(uint32_t i = 0; i < np; ++i)
		{
			const V3 p1 = fp[i];
			const float d = dotS(p1, pn) + pd;
			points[num] = add(p1, scale(scale(normal, d), 0.5f));
			dists[num] = d;
			++num;
		}
	}
	return num;
}

// makeConvexShape from this build's shape encoding: type (low byte PxGeometryType:
// 0 sphere, 2 capsule, 3 box, 4 convex core with its PxConvexCore::Type in bits
// 8..15) and 4 floats (sphere: radius; capsule: radius, halfHeight; box: half
// extents; convex core: up to 3 core floats, margin).
__device__ __forceinline__ void makeShape(int type, const float* g, const Tr& pose, Shape& s)
{
	s.pose = pose;
	s.d[0] = s.d[1] = s.d[2] = 0.0f;
	switch(type & 0xff)
	{
	case 0: s.core = CORE_POINT; s.margin = g[0]; break;
	case 2: s.core = CORE_SEGMENT; s.d[0] = g[1] * 2.0f; s.margin = g[0]; break;
	case 3: s.core = CORE_BOX; s.d[0] = g[0] * 2.0f; s.d[1] = g[1] * 2.0f; s.d[2] = g[2] * 2.0f; s.margin = 0.0f; break;
	default:
		s.core = (type >> 8) & 0xff;
		s.d[0] = g[0]; s.d[1] = g[1]; s.d[2] = g[2];
		s.margin = g[3];
		break;
	}
}

// One pair with type0 <= type1 (low bytes) and at least one convex core:
// contactPlaneConvexCore for a plane, else contactConvexCoreConvex (poses shifted
// to their midpoint while the contacts are generated).  Returns the count.
__device__ __noinline__ uint32_t generatePair(int t0, const float* g0, int t1, const float* g1, const Tr& p0, const Tr& p1, float contactDist,
                                              V3& normal, V3* points, float* dists)
{
	if((t0 & 0xff) == 1)
	{
		Shape s1;
		makeShape(t1, g1, p1, s1);
		return planeConvex(p0, s1, contactDist, normal, points, dists);
	}
	const V3 shift = scale(add(p0.p, p1.p), 0.5f);
	Tr q0 = p0, q1 = p1;
	q0.p = sub(p0.p, shift);
	q1.p = sub(p1.p, shift);
	Shape s0, s1;
	makeShape(t0, g0, q0, s0);
	makeShape(t1, g1, q1, s1);
	const uint32_t n = convexConvex(s0, s1, contactDist, normal, points, dists);
	for(uint32_t i = 0; i < n; i++) points[i] = add(points[i], shift);
	return n;
}
} // namespace cc
} // namespace gbpx
