// Primitive contact generation (sphere / plane / capsule / box) for the GB300
// rigid-body step: PxGenerateContacts semantics
// (physx/source/immediatemode/src/NpImmediateMode.cpp:732-849), with a fresh
// PxCache or with the pair's persistent contact manifold (a 288-byte record,
// refreshed, invalidated or rebuilt as the reference does).  Per-pair generators
// follow physx/source/geomutils/src/pcm/: GuPCMContactSphereSphere.cpp:36,
// SpherePlane.cpp:36, SphereCapsule.cpp:56, SphereBox.cpp:37,
// PlaneCapsule.cpp:36, PlaneBox.cpp:36, CapsuleCapsule.cpp:79, BoxBox.cpp:332
// and :848; manifold reduction and output follow
// GuPersistentContactManifold.cpp:552-1313.  One thread runs one pair; the
// kernels in np.cu group pairs by type so a warp runs one generator.
//
// Box-box edge clipping divides by the reference's approximate reciprocal
// (V3RecipFast, GuPCMContactBoxBox.cpp:140): recipFast restates the x86 RCPPS
// result bit for bit, so the clipped points round as the reference's do.
#pragma once
#include "vmath.cuh"

namespace gbpx
{
namespace np
{
// Gu::contains (physx/source/geomutils/src/pcm/GuPCMContactGenUtil.cpp:35):
// point-in-polygon on XY by ray crossing, with the reference's endpoint
// shortcut and epsilon-shifted crossing test (bounds reject done by the caller).
__device__ __forceinline__ bool polyContainsXY(const V3* verts, int numVerts, V3 p)
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

enum { SPHERE = 0, PLANE = 1, CAPSULE = 2, BOX = 3 };
const int MAXC = 16;    // largest pre-reduction count: box-box clipping (4 + 4 + 8)
const int MAXOUT = 4;   // largest per-pair output after manifold reduction

struct Contact { V3 n; float sep; V3 p; };
struct Buffer
{
	Contact c[MAXOUT];
	int count = 0;
	__device__ void add(V3 p, V3 n, float s) { if(count < MAXOUT) { c[count].n = n; c[count].sep = s; c[count].p = p; count++; } }
};

// PersistentContact: local point on A, local point on B, local normal + penetration
struct PC { V3 a, b, n; float pen; };

// PersistentContactManifold state (GuPersistentContactManifold.h:144): the
// points, and what the next frame's refresh / invalidate tests read -- the
// relative transform when contacts were last generated (p = FLT_MAX when
// cleared) and, for box-box, both bodies' orientations then.
struct Manifold
{
	PC pts[4];
	int num = 0;
	Tr rel;
	Q quatA, quatB;
	int warmA[4], warmB[4], warmSize = 0;   // GJK warm start: last simplex's vertex indices
	__device__ Manifold()
	{
		rel.q = Q{0.0f, 0.0f, 0.0f, 1.0f};
		rel.p = v3(FLT_MAX, FLT_MAX, FLT_MAX);
		quatA = quatB = Q{0.0f, 0.0f, 0.0f, 1.0f};
	}
};

static __device__ float distPointSegSq(V3 a, V3 b, V3 p)
{
	const V3 ap = sub(p, a), ab = sub(b, a);
	const float nom = dotA(ap, ab), denom = dotA(ab, ab);
	const float tv = fclamp(nom / denom, 0.0f, 1.0f);
	const float t = denom == 0.0f ? 0.0f : tv;
	const V3 v = negScaleSub(ab, t, ap);
	return dotA(v, v);
}

// ----------------------------------------------------------------- sphere
static __device__ bool sphereSphere(float r0, float r1, const Tr& t0, const Tr& t1, float cDist, Buffer& out)
{
	const V3 d = sub(t0.p, t1.p);
	const float distSq = dotA(d, d);
	const float rs = r0 + r1, infl = rs + cDist;
	if(infl * infl > distSq)
	{
		const float dist = sqrtf(distSq);
		const V3 n = (1e-5f >= dist) ? unitX() : scaleInv(d, dist);
		const V3 p = scaleAdd(n, r1, t1.p);
		out.add(p, n, dist - rs);
		return true;
	}
	return false;
}

static __device__ bool spherePlane(float r, const Tr& t0, const Tr& t1, float cDist, Buffer& out)
{
	const V3 c = trTransformInv(t1, t0.p);
	const float sep = c.x - r;
	if(cDist >= sep)
	{
		const V3 n = qBasis0(t1.q);
		const V3 p = negScaleSub(n, r, t0.p);
		out.add(p, n, sep);
		return true;
	}
	return false;
}

static __device__ bool sphereCapsule(float sr, float cr, float hh, const Tr& t0, const Tr& t1, float cDist, Buffer& out)
{
	const V3 b0 = qBasis0(t1.q);
	const V3 tmp = scale(b0, hh);
	const V3 s = add(t1.p, tmp), e = sub(t1.p, tmp);
	const float rs = sr + cr, infl = rs + cDist;
	// distancePointSegmentSquared with the segment parameter
	const V3 ap = sub(t0.p, s), ab = sub(e, s);
	const float nom = dotA(ap, ab), denom = dotA(ab, ab);
	const float tv = fclamp(nom / denom, 0.0f, 1.0f);
	const float t = denom == 0.0f ? 0.0f : tv;
	const V3 v = negScaleSub(ab, t, ap);
	const float sqDist = dotA(v, v);
	if(infl * infl > sqDist)
	{
		const V3 p = scaleAdd(sub(e, s), t, s);
		const V3 dir = sub(t0.p, p);
		const float len = sqrtf(dotA(dir, dir));
		const V3 n = len > FLT_EPSILON ? scaleInv(dir, len) : unitX();
		const V3 point = negScaleSub(n, sr, t0.p);
		out.add(point, n, sqrtf(sqDist) - rs);
		return true;
	}
	return false;
}

static __device__ bool sphereBox(float r, V3 ext, const Tr& t0, const Tr& t1, float cDist, Buffer& out)
{
	const V3 c = trTransformInv(t1, t0.p);
	const float infl = r + cDist;
	const V3 p = vmax(vmin(c, ext), neg(ext));  // V3Clamp
	const V3 v = sub(c, p);
	const float lenSq = dotA(v, v);
	if(infl * infl > lenSq)
	{
		const V3 ac = vabs(c);
		if(ext.x >= ac.x && ext.y >= ac.y && ext.z >= ac.z)
		{
			const V3 ap = vabs(p);
			const V3 d = sub(ext, ap);
			const bool con0 = d.x >= d.z && d.y >= d.z && d.z >= d.z;
			const bool con1 = d.x >= d.x && d.y >= d.x && d.z >= d.x;
			const V3 sign = v3(p.x >= 0.0f ? 1.0f : -1.0f, p.y >= 0.0f ? 1.0f : -1.0f, p.z >= 0.0f ? 1.0f : -1.0f);
			const V3 tx = mul(v3(1, 0, 0), sign), ty = mul(v3(0, 1, 0), sign), tz = mul(v3(0, 0, 1), sign);
			const V3 ln = con0 ? tz : (con1 ? tx : ty);
			const float dist = -(con0 ? d.z : (con1 ? d.x : d.y));
			const V3 n = qRotate(t1.q, ln);
			const V3 point = sub(t0.p, scale(n, dist));
			out.add(point, n, dist - r);
		}
		else
		{
			const float recipLen = 1.0f / sqrtf(lenSq);
			const float len = 1.0f / recipLen;
			const V3 ln = scale(v, recipLen);
			const V3 n = qRotate(t1.q, ln);
			out.add(trTransform(t1, p), n, len - r);
		}
		return true;
	}
	return false;
}

// ----------------------------------------------------------------- manifold helpers
// PxMatTransformV
struct MatTr { M33 R; V3 p; };
static __device__ MatTr matFromTr(const Tr& t) { MatTr m; m.R = m33FromQuatCol(t.q); m.p = t.p; return m; }
static __device__ V3 mtTransform(const MatTr& m, V3 v) { return add(m33MulV(m.R, v), m.p); }
static __device__ V3 mtRotate(const MatTr& m, V3 v) { return m33MulV(m.R, v); }
static __device__ V3 mtRotateInv(const MatTr& m, V3 v) { return m33TMulV(m.R, v); }
static __device__ V3 mtTransformInv(const MatTr& m, V3 v) { return m33TMulV(m.R, sub(v, m.p)); }
static __device__ bool replacePoint(Manifold& m, const PC& c, float thr)
{
	const float sd = thr * thr;
	for(int i = 0; i < m.num; i++)
	{
		const V3 db = sub(m.pts[i].b, c.b), da = sub(m.pts[i].a, c.a);
		const float sb = dotA(db, db), sa = dotA(da, da);
		if(sd > fmin_(sb, sa)) { m.pts[i] = c; return true; }
	}
	return false;
}

static __device__ void addPoint2(Manifold& m, const PC& c, float thr)
{
	if(replacePoint(m, c, thr)) return;
	if(m.num < 2) { m.pts[m.num++] = c; return; }
	// reduceContactSegment
	const V3 v0 = sub(m.pts[0].b, c.b), v1 = sub(m.pts[1].b, c.b);
	if(dotA(v0, v0) > dotA(v1, v1)) m.pts[1] = c; else m.pts[0] = c;
}

// addManifoldContactsToContactBuffer for sphere/capsule vs primitive (GuPersistentContactManifold.cpp:783)
static __device__ void outputCapsuleLike(const Manifold& m, V3 normal, V3 projN, const Tr& tA, float radius, float cDist, Buffer& out)
{
	for(int i = 0; i < m.num; i++)
	{
		const float dist = m.pts[i].pen - radius;
		if(cDist >= dist) out.add(negScaleSub(projN, radius, trTransform(tA, m.pts[i].a)), normal, dist);
	}
}

// addManifoldContactsToContactBuffer(normal, transf1, contactOffset) (GuPersistentContactManifold.cpp:739)
static __device__ void outputWithOffset(const Manifold& m, V3 normal, const Tr& tB, float cDist, Buffer& out)
{
	for(int i = 0; i < m.num; i++)
	{
		const float dist = m.pts[i].pen;
		if(cDist >= dist) out.add(trTransform(tB, m.pts[i].b), normal, dist);
	}
}

// reduceBatchContactsCluster (GuPersistentContactManifold.cpp:859)
static __device__ void reduceCluster(Manifold& m, const PC* pts, int n)
{
	bool chosen[MAXC] = {};
	const float FMAX = FLT_MAX;
	float maxDist = FMAX;
	int index = 0;
	int indices[4];
	for(int i = 0; i < n; i++)
		if(maxDist > pts[i].pen) { maxDist = pts[i].pen; index = i; }
	m.pts[0] = pts[index]; chosen[index] = true; indices[0] = index;
	V3 v = sub(pts[0].b, m.pts[0].b);
	maxDist = dotA(v, v); index = 0;
	for(int i = 1; i < n; i++)
	{
		v = sub(pts[i].b, m.pts[0].b);
		const float d = dotA(v, v);
		if(d > maxDist) { maxDist = d; index = i; }
	}
	m.pts[1] = pts[index]; chosen[index] = true; indices[1] = index;
	maxDist = -FMAX; index = -1;
	v = sub(m.pts[1].b, m.pts[0].b);
	const V3 cn0 = m.pts[0].n;
	V3 nrm = cross(v, cn0);
	const float sqLen = dotA(nrm, nrm);
	nrm = sqLen > 0.0f ? scaleInv(nrm, sqrtf(sqLen)) : cn0;
	float minDist = FMAX;
	int index1 = -1;
	for(int i = 0; i < n; i++)
	{
		if(chosen[i]) continue;
		v = sub(pts[i].b, m.pts[0].b);
		const float d = dotA(v, nrm);
		if(d > maxDist) { maxDist = d; index = i; }
		if(minDist > d) { minDist = d; index1 = i; }
	}
	m.pts[2] = pts[index]; chosen[index] = true; indices[2] = index;
	if(minDist * maxDist > 0.0f)
	{
		maxDist = -FMAX;
		for(int i = 0; i < n; i++)
		{
			if(chosen[i]) continue;
			v = sub(pts[i].b, m.pts[0].b);
			const float d = dotA(v, nrm);
			if(d > maxDist) { maxDist = d; index1 = i; }
		}
	}
	m.pts[3] = pts[index1]; chosen[index1] = true; indices[3] = index1;
	for(int i = 0; i < n; i++)
	{
		if(chosen[i]) continue;
		maxDist = FMAX;
		const float pen = pts[i].pen;
		index = 0;
		for(int j = 0; j < 4; j++)
		{
			const V3 v1 = sub(pts[i].b, m.pts[j].b);
			const float dist = dotA(v1, v1);
			if(maxDist > dist) { maxDist = dist; index = j; }
		}
		if(pts[indices[index]].pen > pen) indices[index] = i;
	}
	for(int k = 0; k < 4; k++) m.pts[k] = pts[indices[k]];
}

// reduceBatchContacts (GuPersistentContactManifold.cpp:1008)
static __device__ void reduceBatch(Manifold& m, const PC* pts, int n, float tolLen)
{
	int chosenIdx[4];
	int cand[MAXC];
	float maxPen = pts[0].pen, minPen = maxPen;
	int index = 0, candIndex = 0;
	cand[0] = 0;
	int nbC = n;
	for(int i = 1; i < n; i++)
	{
		cand[i] = i;
		const float pen = pts[i].pen;
		minPen = fmax_(minPen, pen);
		if(maxPen > pen) { maxPen = pen; index = i; candIndex = i; }
	}
	chosenIdx[0] = index;
	nbC--; cand[candIndex] = cand[nbC];
	V3 v = sub(pts[cand[0]].b, pts[chosenIdx[0]].b);
	float maxDist = dotA(v, v);
	index = cand[0]; candIndex = 0;
	for(int i = 1; i < nbC; i++)
	{
		v = sub(pts[cand[i]].b, pts[chosenIdx[0]].b);
		const float d = dotA(v, v);
		if(d > maxDist) { maxDist = d; index = cand[i]; candIndex = i; }
	}
	chosenIdx[1] = index;
	nbC--; cand[candIndex] = cand[nbC];
	v = sub(pts[chosenIdx[1]].b, pts[chosenIdx[0]].b);
	const V3 cn0 = pts[chosenIdx[0]].n;
	V3 nrm = cross(v, cn0);
	const float sqLen = dotA(nrm, nrm);
	nrm = sqLen > 0.0f ? scaleInv(nrm, sqrtf(sqLen)) : cn0;
	maxDist = -FLT_MAX; index = 0xff; candIndex = 0xff;
	float minDist = FLT_MAX;
	int index1 = 0xff, candIndex1 = 0xff;
	for(int i = 0; i < nbC; i++)
	{
		v = sub(pts[cand[i]].b, pts[chosenIdx[0]].b);
		const float d = dotA(v, nrm);
		if(d > maxDist) { maxDist = d; index = cand[i]; candIndex = i; }
		if(minDist > d) { minDist = d; index1 = cand[i]; candIndex1 = i; }
	}
	chosenIdx[2] = index;
	nbC--; cand[candIndex] = cand[nbC];
	if(nbC == candIndex1) candIndex1 = candIndex;
	if(minDist * maxDist > 0.0f)
	{
		maxDist = -FLT_MAX;
		for(int i = 0; i < nbC; i++)
		{
			v = sub(pts[cand[i]].b, pts[chosenIdx[0]].b);
			const float d = dotA(v, nrm);
			if(d > maxDist) { maxDist = d; index1 = cand[i]; candIndex1 = i; }
		}
	}
	chosenIdx[3] = index1;
	nbC--; cand[candIndex1] = cand[nbC];
	const float eps = tolLen * 0.02f;
	if(eps > maxPen && minPen > eps)
	{
		for(int i = 0; i < 4; i++)
		{
			float pen = pts[chosenIdx[i]].pen;
			if(pen > eps)
			{
				candIndex = 0xff;
				for(int j = 0; j < nbC; j++)
				{
					const float pen1 = pts[cand[j]].pen;
					if(pen > pen1 && eps > pen1) { pen = pen1; candIndex = j; }
				}
				if(candIndex < nbC)
				{
					const int orig = chosenIdx[i];
					chosenIdx[i] = cand[candIndex];
					cand[candIndex] = orig;
				}
			}
			m.pts[i] = pts[chosenIdx[i]];
		}
	}
	else
		for(int i = 0; i < 4; i++) m.pts[i] = pts[chosenIdx[i]];
}

// reduceBatchContacts2 (GuPersistentContactManifold.cpp:1177)
static __device__ void reduceBatch2(Manifold& m, const PC* pts, int n)
{
	bool chosen[MAXC] = {};
	float maxDis = pts[0].pen;
	int index = 0;
	for(int i = 1; i < n; i++)
		if(maxDis > pts[i].pen) { maxDis = pts[i].pen; index = i; }
	m.pts[0] = pts[index]; chosen[index] = true;
	V3 v = sub(pts[0].b, m.pts[0].b);
	maxDis = dotA(v, v); index = 0;
	for(int i = 1; i < n; i++)
	{
		v = sub(pts[i].b, m.pts[0].b);
		const float d = dotA(v, v);
		if(d > maxDis) { maxDis = d; index = i; }
	}
	m.pts[1] = pts[index]; chosen[index] = true;
	int second = index;
	const float maxDepth = pts[index].pen;
	for(int i = 0; i < n; i++)
	{
		if(chosen[i]) continue;
		const V3 d0 = sub(m.pts[0].b, pts[i].b), d1 = sub(m.pts[1].b, pts[i].b);
		if(dotA(d0, d0) > dotA(d1, d1))
			if(maxDepth > pts[i].pen) second = i;
	}
	if(second != index) m.pts[1] = pts[second];
}

static __device__ void addBatch(Manifold& m, const PC* pts, int n, float tolLen)
{
	if(n <= 4) { for(int i = 0; i < n; i++) m.pts[i] = pts[i]; m.num = n; }
	else { reduceBatch(m, pts, n, tolLen); m.num = 4; }
}

static __device__ void addBatchCluster(Manifold& m, const PC* pts, int n)
{
	if(n <= 4) { for(int i = 0; i < n; i++) m.pts[i] = pts[i]; m.num = n; }
	else { reduceCluster(m, pts, n); m.num = 4; }
}

static __device__ void addBatch2(Manifold& m, const PC* pts, int n)
{
	if(n <= 2) { for(int i = 0; i < n; i++) m.pts[i] = pts[i]; m.num = n; }
	else { reduceBatch2(m, pts, n); m.num = 2; }
}

// ----------------------------------------------------------------- manifold persistence
// GuPersistentContactManifold.cpp:175-187
static __device__ __forceinline__ float kInvalidateThresholds(int n) { return n == 0 ? 0.5f : (n == 1 ? 0.125f : (n == 2 ? 0.25f : 0.375f)); }
static __device__ __forceinline__ float kInvalidateThresholds2(int n) { return n == 0 ? 0.5f : (n == 1 ? 0.1f : 0.75f); }
static __device__ __forceinline__ float kInvalidateQuatThresholds(int n) { return n == 0 ? 0.9998f : 0.9999f; }
static __device__ __forceinline__ float kInvalidateQuatThresholds2(int n) { return n == 0 ? 0.9995f : (n == 1 ? 0.9999f : 0.9997f); }

// V4Dot / QuatDot of the SSE2 layer: (y*y' + w*w') + (z*z' + x*x')
static __device__ float quatDot(Q a, Q b) { return (a.y * b.y + a.w * b.w) + (a.z * b.z + a.x * b.x); }

// refreshContactPoints (GuPersistentContactManifold.h:723): re-project every
// point with the current relative transform, drop those that slid further than
// the threshold, update the penetration of the rest.
static __device__ void refreshManifold(Manifold& m, const MatTr& aToB, float projectBreakingThreshold)
{
	const float sq = projectBreakingThreshold * projectBreakingThreshold;
	for(int i = m.num; i > 0; --i)
	{
		PC& p = m.pts[i - 1];
		const V3 aInB = add(m33MulV(aToB.R, p.a), aToB.p);
		const V3 v = sub(aInB, p.b);
		const float dist = dotA(v, p.n);
		const V3 projected = negScaleSub(p.n, dist, aInB);
		const V3 diff = sub(p.b, projected);
		if(dotA(diff, diff) > sq)
		{
			m.num--;
			m.pts[i - 1] = m.pts[m.num];
		}
		else
			p.pen = dist;
	}
}

// maxTransformPositionDelta: V4ExtractMax(|curP - rel.p|, w = 0)
static __device__ float maxPositionDelta(const Manifold& m, V3 curP)
{
	const V3 d = vabs(sub(curP, m.rel.p));
	return fmax_(fmax_(d.x, 0.0f), fmax_(d.z, d.y));
}

// invalidate_BoxConvex (GuPersistentContactManifold.h:190)
static __device__ bool invalidateBoxConvex(const Manifold& m, const Tr& cur, Q quatA, Q quatB, float minMargin, float radiusA, float radiusB)
{
	const float thresholdP = minMargin * kInvalidateThresholds(m.num);
	const float deltaP = maxPositionDelta(m, cur.p);
	const float thresholdQ = kInvalidateQuatThresholds(m.num);
	const float dqA = quatDot(quatA, m.quatA), dqB = quatDot(quatB, m.quatB);
	if(deltaP > thresholdP || thresholdQ > dqA || thresholdQ > dqB) return true;
	// the angles only meet a threshold: the device acosf (within 2 ulp of the host
	// C library's) decides the same except within a few ulp of the threshold
	const float aRadian = dqA < 1.0f ? acosf(dqA) : 0.0f;
	const float bRadian = dqB < 1.0f ? acosf(dqB) : 0.0f;
	return aRadian * radiusA > thresholdP || bRadian * radiusB > thresholdP;
}

// invalidate_SphereCapsule (GuPersistentContactManifold.h:227)
static __device__ bool invalidateSphereCapsule(const Manifold& m, const Tr& cur, float minMargin)
{
	const float thresholdP = minMargin * kInvalidateThresholds2(m.num);
	const float deltaP = maxPositionDelta(m, cur.p);
	const float dq = quatDot(cur.q, m.rel.q);
	return deltaP > thresholdP || kInvalidateQuatThresholds2(m.num) > dq;
}

// invalidate_PrimitivesPlane (GuPersistentContactManifold.h:245)
static __device__ bool invalidatePrimitivesPlane(const Manifold& m, const Tr& cur, float minMargin, float ratio)
{
	const float thresholdP = minMargin * ratio;
	const float deltaP = maxPositionDelta(m, cur.p);
	const float dq = quatDot(cur.q, m.rel.q);
	return deltaP > thresholdP || 0.99996f > dq;
}

// getWorldNormal (GuPersistentContactManifold.h:691): the manifold's summed
// normal (first point's if the sum vanishes), rotated into world space and
// normalized (QuatRotateAndNormalize)
static __device__ V3 manifoldWorldNormal(const Manifold& m, const Tr& trB)
{
	V3 n = m.pts[0].n;
	for(int i = 1; i < m.num; i++) n = add(n, m.pts[i].n);
	const V3 nn = dotA(n, n) > FLT_EPSILON ? n : m.pts[0].n;
	const Q q = trB.q;
	const float w2 = q.w * q.w + (-0.5f);
	const V3 u = qv(q);
	const V3 temp = scaleAdd(cross(u, nn), q.w, scale(nn, w2));
	return normalizeA(scaleAdd(u, dotA(u, nn), temp));
}

// distancePointTriangleSquaredLocal (GuPersistentContactManifold.cpp:61)
static __device__ float distPointTriangleSq(V3 p, V3 a, V3 b, V3 c)
{
	const V3 ab = sub(b, a), ac = sub(c, a), bc = sub(c, b);
	const V3 ap = sub(p, a), bp = sub(p, b), cp = sub(p, c);
	const float d1 = dotA(ab, ap), d2 = dotA(ac, ap), d3 = dotA(ab, bp);
	const float d4 = dotA(ac, bp), d5 = dotA(ab, cp), d6 = dotA(ac, cp);
	const float unom = d4 - d3, udenom = d5 - d6;
	if(0.0f > d1 && 0.0f > d2) { const V3 vv = sub(p, a); return dotA(vv, vv); }
	if(d3 >= 0.0f && d3 >= d4) { const V3 vv = sub(p, b); return dotA(vv, vv); }
	if(d6 >= 0.0f && d6 >= d5) { const V3 vv = sub(p, c); return dotA(vv, vv); }
	const float vc = d1 * d4 - d3 * d2;
	if(0.0f > vc && d1 >= 0.0f && 0.0f > d3)
	{
		const float s = d1 / (d1 - d3);
		const V3 vv = sub(p, scaleAdd(ab, s, a));
		return dotA(vv, vv);
	}
	const float va = d3 * d6 - d5 * d4;
	if(0.0f > va && d4 >= d3 && d5 >= d6)
	{
		const float u = unom / (unom + udenom);
		const V3 vv = sub(p, scaleAdd(bc, u, b));
		return dotA(vv, vv);
	}
	const float vb = d5 * d2 - d1 * d6;
	if(0.0f > vb && d2 >= 0.0f && 0.0f > d6)
	{
		const float t = d2 / (d2 - d6);
		const V3 vv = sub(p, scaleAdd(ac, t, a));
		return dotA(vv, vv);
	}
	const V3 n = cross(ab, ac);
	const float nn = dotA(n, n);
	const float t = nn > 0.0f ? dotA(n, sub(a, p)) / nn : 0.0f;
	const V3 vv = sub(p, add(p, scale(n, t)));
	return dotA(vv, vv);
}

// reduceContactsForPCM (GuPersistentContactManifold.cpp:603): four manifold
// points plus a new one down to four
static __device__ void reduceForPCM(Manifold& m, const PC& c)
{
	bool chosen[5] = {false, false, false, false, false};
	PC tmp[5];
	for(int i = 0; i < 4; i++) tmp[i] = m.pts[i];
	tmp[4] = c;
	float maxDist = c.pen;
	int index = 4;
	for(int i = 0; i < 4; i++)
		if(maxDist > tmp[i].pen) { maxDist = tmp[i].pen; index = i; }
	chosen[index] = true;
	m.pts[0] = tmp[index];
	V3 dir = sub(tmp[0].b, m.pts[0].b);
	maxDist = dotA(dir, dir);
	index = 0;
	for(int i = 1; i < 5; i++)
		if(!chosen[i])
		{
			dir = sub(tmp[i].b, m.pts[0].b);
			const float d = dotA(dir, dir);
			if(d > maxDist) { maxDist = d; index = i; }
		}
	chosen[index] = true;
	m.pts[1] = tmp[index];
	maxDist = -FLT_MAX;
	for(int i = 0; i < 5; i++)
		if(!chosen[i])
		{
			const float d = distPointSegSq(m.pts[0].b, m.pts[1].b, tmp[i].b);
			if(d > maxDist) { maxDist = d; index = i; }
		}
	chosen[index] = true;
	m.pts[2] = tmp[index];
	maxDist = -FLT_MAX;
	for(int i = 0; i < 5; i++)
		if(!chosen[i])
		{
			const float d = distPointTriangleSq(tmp[i].b, m.pts[0].b, m.pts[1].b, m.pts[2].b);
			if(d > maxDist) { maxDist = d; index = i; }
		}
	if(chosen[index]) { m.num = 3; return; }
	chosen[index] = true;
	m.pts[3] = tmp[index];
	int notChosen = 0;
	for(int a = 0; a < 5; a++)
		if(!chosen[a]) { notChosen = a; break; }
	float closest = FLT_MAX;
	index = 0;
	for(int a = 0; a < 4; a++)
	{
		const V3 dif = sub(m.pts[a].a, tmp[notChosen].a);
		const float d2 = dotA(dif, dif);
		if(closest > d2) { closest = d2; index = a; }
	}
	if(m.pts[index].pen > tmp[notChosen].pen) m.pts[index] = tmp[notChosen];
}

// addManifoldPoint (GuPersistentContactManifold.cpp:1246)
static __device__ void addPoint4(Manifold& m, const PC& c, float thr)
{
	if(replacePoint(m, c, thr)) return;
	if(m.num < 4) { m.pts[m.num++] = c; return; }
	reduceForPCM(m, c);
}

static __device__ float boxMargin(V3 ext, float tolLen)
{
	const float mn = fmin_(ext.x, fmin_(ext.y, ext.z));
	return fmin_(mn * 0.15f, tolLen * 0.15f);
}

// ----------------------------------------------------------------- plane
// pcmContactPlaneCapsule (GuPCMContactPlaneCapsule.cpp:36); m is the pair's
// persistent manifold (a fresh one for a fresh cache)
static __device__ bool planeCapsule(float r, float hh, const Tr& tPlane, const Tr& tCap, float cDist, Manifold& m, Buffer& out)
{
	const Tr& transf0 = tCap;
	const Tr& transf1 = tPlane;
	const Tr aToB = trInvMul(transf1, transf0);
	const V3 planeN = normalizeA(qBasis0(transf1.q));
	const V3 cn = neg(planeN);
	const V3 localN = unitX();
	const V3 bv = qBasis0(aToB.q);
	const V3 tmp = scale(bv, hh);
	const V3 s = add(aToB.p, tmp), e = sub(aToB.p, tmp);
	const float infl = r + cDist;
	const float replaceThr = r * 0.001f;
	const float projectThr = r * 0.05f;
	const int initial = m.num;
	refreshManifold(m, matFromTr(aToB), projectThr);
	const bool lost = m.num != initial;
	if(lost || invalidatePrimitivesPlane(m, aToB, r, 0.02f))
	{
		m.num = 0;
		m.rel = aToB;
		const float sd0 = s.x;
		if(infl > sd0)
		{
			PC c; c.a = trTransformInv(aToB, s); c.b = negScaleSub(localN, sd0, s); c.n = localN; c.pen = sd0;
			addPoint2(m, c, replaceThr);
		}
		const float sd1 = e.x;
		if(infl > sd1)
		{
			PC c; c.a = trTransformInv(aToB, e); c.b = negScaleSub(localN, sd1, e); c.n = localN; c.pen = sd1;
			addPoint2(m, c, replaceThr);
		}
	}
	outputCapsuleLike(m, cn, planeN, transf0, r, cDist, out);
	return m.num > 0;
}

// pcmContactPlaneBox (GuPCMContactPlaneBox.cpp:36)
static __device__ bool planeBox(V3 ext, const Tr& tPlane, const Tr& tBox, float cDist, float tolLen, Manifold& m, Buffer& out)
{
	const Tr& transf0 = tBox;
	const Tr& transf1 = tPlane;
	const Tr cur = trInvMul(transf1, transf0);
	const V3 negN = normalizeA(neg(qBasis0(transf1.q)));
	const V3 localN = unitX();
	const float margin = boxMargin(ext, tolLen);
	const float projectThr = margin * 0.2f;
	// PxMatTransformV(cur): rotation matrix columns from the quaternion
	const MatTr aToB = matFromTr(cur);
	const int initial = m.num;
	refreshManifold(m, aToB, projectThr);
	const bool lost = m.num != initial;
	if(lost || invalidatePrimitivesPlane(m, cur, margin, 0.2f))
	{
		m.num = 0;
		m.rel = cur;
		const M33& R = aToB.R;
		const float bx = ext.x, by = ext.y, bz = ext.z;
		const V3 t0 = scale(R.c0, bx), t1 = scale(R.c1, by), t2 = scale(R.c2, bz);
		const V3 nt2 = neg(t2);
		const float px = cur.p.x;
		const V3 t01 = add(t0, t1), t02 = sub(t0, t1);
		const float sv[8] = {add(t2, t01).x, add(nt2, t01).x, add(t2, t02).x, add(nt2, t02).x,
		                     sub(t2, t02).x, sub(nt2, t02).x, sub(t2, t01).x, sub(nt2, t01).x};
		const V3 corners[8] = {v3(bx, by, bz), v3(bx, by, -bz), v3(bx, -by, bz), v3(bx, -by, -bz),
		                       v3(-bx, by, bz), v3(-bx, by, -bz), v3(-bx, -by, bz), v3(-bx, -by, -bz)};
		const float acc = cDist - px;
		PC pts[8];
		int n = 0;
		for(int k = 0; k < 8; k++)
		{
			if(acc > sv[k])
			{
				const float pen = sv[k] + px;
				// aToB.transform(p) with the matrix form of the relative transform
				const V3 wp = add(m33MulV(R, corners[k]), cur.p);
				pts[n].a = corners[k];
				pts[n].b = negScaleSub(localN, pen, wp);
				pts[n].n = localN;
				pts[n].pen = pen;
				n++;
			}
		}
		addBatchCluster(m, pts, n);
	}
	outputWithOffset(m, negN, transf1, cDist, out);
	return m.num > 0;
}

// ----------------------------------------------------------------- capsule-capsule
static __device__ float segSegSq(V3 p1, V3 d1, V3 p2, V3 d2, float& s, float& t)
{
	const float eps = FLT_EPSILON;
	const V3 r = sub(p1, p2);
	// V3Dot4 sums (x + y) + z (PxVecMath.h:1320)
	const float a = dotS(d1, d1), e = dotS(d2, d2), b = dotS(d1, d2), c = dotS(d1, r);
	const float aR = a > eps ? 1.0f / a : 0.0f;
	const float eR = e > eps ? 1.0f / e : 0.0f;
	const float f = dotA(d2, r);
	const float denom = a * e - b * b;
	const float temp = b * f - c * e;
	const float s0 = fclamp(temp / denom, 0.0f, 1.0f);
	const float sTmp = eps > denom ? 0.5f : s0;
	const float tTmp = (b * sTmp + f) * eR;
	const float t2 = fclamp(tTmp, 0.0f, 1.0f);
	const float comp = (b * t2 - c) * aR;
	const float s2 = fclamp(comp, 0.0f, 1.0f);
	s = s2; t = t2;
	const V3 c1 = scaleAdd(d1, s2, p1), c2 = scaleAdd(d2, t2, p2);
	const V3 vv = sub(c1, c2);
	return dotA(vv, vv);
}

static __device__ bool capsuleCapsule(float r0, float hh0, float r1, float hh1, const Tr& t0, const Tr& t1, float cDist, Buffer& out)
{
	const V3 off = scale(add(t0.p, t1.p), 0.5f);
	const V3 p0 = sub(t0.p, off), p1 = sub(t1.p, off);
	const V3 b0 = qBasis0(t0.q), tmp0 = scale(b0, hh0);
	const V3 s0 = add(p0, tmp0), e0 = sub(p0, tmp0), d0 = sub(e0, s0);
	const V3 b1 = qBasis0(t1.q), tmp1 = scale(b1, hh1);
	const V3 s1 = add(p1, tmp1), e1 = sub(p1, tmp1), d1 = sub(e1, s1);
	const float sumR = r0 + r1, infl = sumR + cDist, inflSq = infl * infl;
	const float a = dotA(d0, d0), e = dotA(d1, d1);
	const float eps = 1e-6f;
	float tt0, tt1;
	const float sqDist0 = segSegSq(s0, d0, s1, d1, tt0, tt1);
	if(!(inflSq >= sqDist0)) return false;
	const V3 dir0 = eps > a ? zero3() : scaleInv(d0, sqrtf(a));
	const V3 dir1 = eps > e ? zero3() : scaleInv(d1, sqrtf(e));
	const float cosv = fabsf(dotA(dir0, dir1));
	if(cosv > 0.9998f)
	{
		// pcmDistancePointSegmentTValue22: project s1,e1 onto segment 0 and s0,e0 onto segment 1
		const V3 ab0 = sub(e0, s0), ab1 = sub(e1, s1);
		const float n00 = dotS(sub(s1, s0), ab0), n10 = dotS(sub(e1, s0), ab0);   // V3Dot4 order
		const float n01 = dotS(sub(s0, s1), ab1), n11 = dotS(sub(e0, s1), ab1);
		const float den0 = dotA(ab0, ab0), den1 = dotA(ab1, ab1);
		float tv[4] = {n00 / den0, n10 / den0, n01 / den1, n11 / den1};
		if(den0 == 0.0f) tv[0] = tv[1] = 0.0f;
		if(den1 == 0.0f) tv[2] = tv[3] = 0.0f;
		int nc = 0;
		for(int k = 0; k < 4; k++)
		{
			if(!(tv[k] >= 0.0f && 1.0f >= tv[k])) continue;
			V3 from, proj, v;
			if(k < 2)
			{
				proj = scaleAdd(d0, tv[k], s0);
				v = sub(proj, k == 0 ? s1 : e1);
				from = proj;
			}
			else
			{
				proj = scaleAdd(d1, tv[k], s1);
				from = k == 2 ? s0 : e0;
				v = sub(from, proj);
			}
			const float sq = dotA(v, v);
			if(sq > eps && inflSq > sq)
			{
				const float dist = sqrtf(sq);
				const V3 n = scaleInv(v, dist);
				const V3 p = add(negScaleSub(n, r0, from), off);
				out.add(p, n, dist - sumR);
				nc++;
			}
		}
		if(nc) return true;
	}
	const V3 cA = scaleAdd(d0, tt0, s0), cB = scaleAdd(d1, tt1, s1);
	const bool con = eps > sqDist0;
	const V3 n_ = con ? (a > eps ? d0 : unitX()) : sub(cA, cB);
	const V3 n = normalizeA(n_);
	const V3 p = add(negScaleSub(n, r0, cA), off);
	const float dist = con ? 0.0f : sqrtf(sqDist0);
	out.add(p, n, dist - sumR);
	return true;
}

// ----------------------------------------------------------------- box-box
static __device__ M33 transpose(const M33& m)
{
	M33 t;
	t.c0 = v3(m.c0.x, m.c1.x, m.c2.x);
	t.c1 = v3(m.c0.y, m.c1.y, m.c2.y);
	t.c2 = v3(m.c0.z, m.c1.z, m.c2.z);
	return t;
}
// a.transformInv(b) for matrix transforms (PxVecTransform.h:277)
static __device__ MatTr mtInvMul(const MatTr& a, const MatTr& b)
{
	MatTr r;
	const M33 at = transpose(a.R);
	r.R.c0 = m33MulV(at, b.R.c0);
	r.R.c1 = m33MulV(at, b.R.c1);
	r.R.c2 = m33MulV(at, b.R.c2);
	r.p = m33TMulV(a.R, sub(b.p, a.p));
	return r;
}


static __device__ void incidentPolygon(V3* pts, V3& faceN, V3 axis, const MatTr& t10, V3 ext)
{
	float ex = ext.x, ey = ext.y, ez = ext.z;
	const V3 u0 = t10.R.c0, u1 = t10.R.c1, u2 = t10.R.c2;
	const float d0 = dotA(u0, axis), d1 = dotA(u1, axis), d2 = dotA(u2, axis);
	const float a0 = fabsf(d0), a1 = fabsf(d1), a2 = fabsf(d2);
	if(a0 >= a1 && a0 >= a2)
	{
		const bool con = d0 > 0.0f;
		faceN = con ? neg(u0) : u0;
		ex = con ? -ex : ex;
		const V3 r0 = scale(u0, ex), r1 = scale(u1, ey), r2 = scale(u2, ez);
		const V3 tp0 = add(t10.p, r0), tp1 = add(r1, r2), tp2 = sub(r1, r2);
		pts[0] = add(tp0, tp1); pts[1] = add(tp0, tp2); pts[2] = sub(tp0, tp1); pts[3] = sub(tp0, tp2);
	}
	else if(a1 >= a2)
	{
		const bool con = d1 > 0.0f;
		faceN = con ? neg(u1) : u1;
		ey = con ? -ey : ey;
		const V3 r0 = scale(u0, ex), r1 = scale(u1, ey), r2 = scale(u2, ez);
		const V3 tp0 = add(t10.p, r1), tp1 = add(r0, r2), tp2 = sub(r0, r2);
		pts[0] = add(tp0, tp1); pts[1] = add(tp0, tp2); pts[2] = sub(tp0, tp1); pts[3] = sub(tp0, tp2);
	}
	else
	{
		const bool con = d2 > 0.0f;
		faceN = con ? neg(u2) : u2;
		ez = con ? -ez : ez;
		const V3 r0 = scale(u0, ex), r1 = scale(u1, ey), r2 = scale(u2, ez);
		const V3 tp0 = add(t10.p, r2), tp1 = add(r0, r1), tp2 = sub(r0, r1);
		pts[0] = add(tp0, tp1); pts[1] = add(tp0, tp2); pts[2] = sub(tp0, tp1); pts[3] = sub(tp0, tp2);
	}
}

// GuPCMContactGenUtil contains(): point-in-polygon on the XY plane with a bounds reject
static __device__ bool containsXY(const V3* verts, int n, V3 p, V3 bmin, V3 bmax)
{
	if(p.x < bmin.x || p.x > bmax.x || p.y < bmin.y || p.y > bmax.y) return false;
	return polyContainsXY(verts, n, p);
}

static __device__ bool segAABB(V3 p0, V3 d, V3 mx, V3 mn, float& tmin, float& tmax)
{
	const float eps = 1e-6f;
	const V3 ad = vabs(d);
	bool par[3] = {eps > ad.x, eps > ad.y, eps > ad.z};
	const float p[3] = {p0.x, p0.y, p0.z}, lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z}, dd[3] = {d.x, d.y, d.z};
	for(int k = 0; k < 3; k++)
		if(par[k] && (p[k] > hi[k] || lo[k] > p[k])) return false;
	float t1[3], t2[3];
	for(int k = 0; k < 3; k++)
	{
		const float odd = recipFast(dd[k]);   // V3RecipFast (GuPCMContactBoxBox.cpp:140)
		t1[k] = par[k] ? 0.0f : (lo[k] - p[k]) * odd;
		t2[k] = par[k] ? FLT_MAX : (hi[k] - p[k]) * odd;
	}
	float ft1 = -FLT_MAX, ft2 = FLT_MAX;
	for(int k = 0; k < 3; k++)
	{
		const float a = fmin_(t1[k], t2[k]), b = fmax_(t1[k], t2[k]);
		ft1 = fmax_(ft1, a);
		ft2 = fmin_(ft2, b);
	}
	const float tminf = fmax_(ft1, 0.0f), tmaxf = fmin_(1.0f, ft2);
	tmin = tminf; tmax = tmaxf;
	return !(tminf > tmaxf || tminf > 1.0f);
}

static __device__ void calculateContacts(float exX, float exY, V3* pts, V3 incN, V3 localN, PC* mc, int& num, float cDist)
{
	const float FMAX = FLT_MAX;
	const float extX = exX * 1.0001f, extY = exY * 1.0001f;
	const float nextX = -extX, nextY = -extY;
	bool pPen[4], pArea[4];
	V3 bmin = v3(FMAX, FMAX, FMAX), bmax = neg(bmin);
	const V3 bound = v3(extX, extY, FMAX);
	for(int i = 0; i < 4; i++)
	{
		bmin = vmin(bmin, pts[i]);
		bmax = vmax(bmax, pts[i]);
		const float z = -pts[i].z;
		if(cDist > z)
		{
			pPen[i] = true;
			const V3 ap = vabs(pts[i]);
			if(bound.x >= ap.x && bound.y >= ap.y && bound.z >= ap.z)
			{
				pArea[i] = true;
				mc[num].a = v3(pts[i].x, pts[i].y, 0.0f);
				mc[num].b = pts[i];
				mc[num].n = localN;
				mc[num].pen = z;
				num++;
			}
			else pArea[i] = false;
		}
		else { pPen[i] = false; pArea[i] = false; }
	}
	if(num == 4) return;
	const float denom = incN.z;
	const V3 qs[4] = {v3(extX, extY, 0.0f), v3(extX, nextY, 0.0f), v3(nextX, extY, 0.0f), v3(nextX, nextY, 0.0f)};
	for(int k = 0; k < 4; k++)
	{
		const V3 q0 = qs[k];
		if(containsXY(pts, 4, q0, bmin, bmax))
		{
			const float nom = dotA(incN, sub(pts[0], q0));
			const float t = nom / denom;
			const float pen = -t;
			if(cDist > pen)
			{
				mc[num].a = q0;
				mc[num].b = v3(q0.x, q0.y, t);
				mc[num].n = localN;
				mc[num].pen = pen;
				num++;
			}
		}
	}
	const V3 ext = v3(extX, extY, FMAX);
	const V3 negExt = v3(nextX, nextY, -(cDist + FLT_EPSILON));
	for(int rStart = 0, rEnd = 3; rStart < 4; rEnd = rStart++)
	{
		const V3 p0 = pts[rStart], p1 = pts[rEnd];
		if(!pPen[rStart] && !pPen[rEnd]) continue;
		const bool con0 = pPen[rStart] && pArea[rStart];
		const bool con1 = pPen[rEnd] && pArea[rEnd];
		if(con0 && con1) continue;
		const V3 d = sub(p1, p0);
		float tmin, tmax;
		if(segAABB(p0, d, ext, negExt, tmin, tmax))
		{
			if(!con0)
			{
				const V3 ip = scaleAdd(d, tmin, p0);
				mc[num].a = v3(ip.x, ip.y, 0.0f); mc[num].b = ip; mc[num].n = localN; mc[num].pen = -ip.z; num++;
			}
			if(!con1)
			{
				const V3 ip = scaleAdd(d, tmax, p0);
				mc[num].a = v3(ip.x, ip.y, 0.0f); mc[num].b = ip; mc[num].n = localN; mc[num].pen = -ip.z; num++;
			}
		}
	}
}

// doBoxBoxGenerateContacts (GuPCMContactBoxBox.cpp:332); returns false on separation
static __device__ bool boxBoxGenerate(V3 e0, V3 e1, const MatTr& T0, const MatTr& T1, float cDist, PC* mc, int& num)
{
	const float ea[3] = {e0.x, e0.y, e0.z}, eb[3] = {e1.x, e1.y, e1.z};
	const MatTr t10 = mtInvMul(T0, T1);
	const M33 r01 = transpose(t10.R);
	const V3 uEps = v3(1e-6f, 1e-6f, 1e-6f);
	const float tx = t10.p.x, ty = t10.p.y, tz = t10.p.z;
	const V3 col[3] = {t10.R.c0, t10.R.c1, t10.R.c2};
	const V3 a10[3] = {add(vabs(col[0]), uEps), add(vabs(col[1]), uEps), add(vabs(col[2]), uEps)};
	const V3 a01[3] = {add(vabs(r01.c0), uEps), add(vabs(r01.c1), uEps), add(vabs(r01.c2), uEps)};
	float sign[6], overlap[6];
	const float tt[3] = {tx, ty, tz};
	for(int k = 0; k < 3; k++)
	{
		sign[k] = tt[k];
		const V3 v = mul(a01[k], e1);
		const float rb = v.x + (v.y + v.z);
		overlap[k] = ((ea[k] + rb) - fabsf(sign[k])) + cDist;
		if(0.0f > overlap[k]) return false;
	}
	for(int k = 0; k < 3; k++)
	{
		sign[3 + k] = dotA(t10.p, col[k]);
		const V3 v = mul(a10[k], e0);
		const float ra = v.x + (v.y + v.z);
		overlap[3 + k] = ((ra + eb[k]) - fabsf(sign[3 + k])) + cDist;
		if(0.0f > overlap[3 + k]) return false;
	}
	// 9 edge-edge axes (separation tests only)
	for(int i = 0; i < 3; i++)
	{
		for(int j = 0; j < 3; j++)
		{
			const V3 c = col[j];
			const V3 aC = a10[j];
			const V3 aR = a01[i];
			float absSign, ra, rb;
			if(i == 0)
			{
				absSign = fabsf(c.y * tz - c.z * ty);
				ra = aC.z * ea[1] + aC.y * ea[2];
			}
			else if(i == 1)
			{
				absSign = fabsf(c.z * tx - c.x * tz);
				ra = aC.z * ea[0] + aC.x * ea[2];
			}
			else
			{
				absSign = fabsf(c.x * ty - c.y * tx);
				ra = aC.y * ea[0] + aC.x * ea[1];
			}
			if(j == 0) rb = aR.z * eb[1] + aR.y * eb[2];
			else if(j == 1) rb = aR.z * eb[0] + aR.x * eb[2];
			else rb = aR.y * eb[0] + aR.x * eb[1];
			const float rs = (ra + rb) + cDist;
			if(absSign > rs) return false;
		}
	}
	int feature = 0;
	float minOv = overlap[0];
	for(int i = 1; i < 6; i++) if(minOv > overlap[i]) { minOv = overlap[i]; feature = i; }

	const V3 ax0 = T0.R.c0, ax1 = T0.R.c1, ax2 = T0.R.c2;
	const V3 bx0 = T1.R.c0, bx1 = T1.R.c1, bx2 = T1.R.c2;
	MatTr nt;
	V3 mtd, incN, pts[4];
	bool flip = false;
	switch(feature)
	{
	case 0:
		if(0.0f >= sign[0]) { mtd = ax0; nt.R.c0 = neg(ax2); nt.R.c1 = ax1; nt.R.c2 = ax0; nt.p = negScaleSub(ax0, ea[0], T0.p); }
		else { mtd = neg(ax0); nt.R.c0 = ax2; nt.R.c1 = ax1; nt.R.c2 = neg(ax0); nt.p = scaleAdd(ax0, ea[0], T0.p); }
		{
			const MatTr t1n = mtInvMul(nt, T1);
			const V3 ln = mtRotateInv(nt, mtd);
			incidentPolygon(pts, incN, neg(ln), t1n, e1);
			calculateContacts(ea[2], ea[1], pts, incN, ln, mc, num, cDist);
		}
		break;
	case 1:
		if(0.0f >= sign[1]) { mtd = ax1; nt.R.c0 = ax0; nt.R.c1 = neg(ax2); nt.R.c2 = ax1; nt.p = negScaleSub(ax1, ea[1], T0.p); }
		else { mtd = neg(ax1); nt.R.c0 = ax0; nt.R.c1 = ax2; nt.R.c2 = neg(ax1); nt.p = scaleAdd(ax1, ea[1], T0.p); }
		{
			const MatTr t1n = mtInvMul(nt, T1);
			const V3 ln = mtRotateInv(nt, mtd);
			incidentPolygon(pts, incN, neg(ln), t1n, e1);
			calculateContacts(ea[0], ea[2], pts, incN, ln, mc, num, cDist);
		}
		break;
	case 2:
		if(0.0f >= sign[2]) { mtd = ax2; nt.R.c0 = ax0; nt.R.c1 = ax1; nt.R.c2 = ax2; nt.p = negScaleSub(ax2, ea[2], T0.p); }
		else { mtd = neg(ax2); nt.R.c0 = ax0; nt.R.c1 = neg(ax1); nt.R.c2 = neg(ax2); nt.p = scaleAdd(ax2, ea[2], T0.p); }
		{
			const MatTr t1n = mtInvMul(nt, T1);
			const V3 ln = mtRotateInv(nt, mtd);
			incidentPolygon(pts, incN, neg(ln), t1n, e1);
			calculateContacts(ea[0], ea[1], pts, incN, ln, mc, num, cDist);
		}
		break;
	case 3:
		flip = true;
		if(0.0f >= sign[3]) { mtd = bx0; nt.R.c0 = bx2; nt.R.c1 = bx1; nt.R.c2 = neg(bx0); nt.p = scaleAdd(bx0, eb[0], T1.p); }
		else { mtd = neg(bx0); nt.R.c0 = neg(bx2); nt.R.c1 = bx1; nt.R.c2 = bx0; nt.p = negScaleSub(bx0, eb[0], T1.p); }
		{
			const MatTr t1n = mtInvMul(nt, T0);
			const V3 ln = mtRotateInv(nt, mtd);
			incidentPolygon(pts, incN, ln, t1n, e0);
			calculateContacts(eb[2], eb[1], pts, incN, ln, mc, num, cDist);
		}
		break;
	case 4:
		flip = true;
		if(0.0f >= sign[4]) { mtd = bx1; nt.R.c0 = bx0; nt.R.c1 = bx2; nt.R.c2 = neg(bx1); nt.p = scaleAdd(bx1, eb[1], T1.p); }
		else { mtd = neg(bx1); nt.R.c0 = bx0; nt.R.c1 = neg(bx2); nt.R.c2 = bx1; nt.p = negScaleSub(bx1, eb[1], T1.p); }
		{
			const MatTr t1n = mtInvMul(nt, T0);
			const V3 ln = mtRotateInv(nt, mtd);
			incidentPolygon(pts, incN, ln, t1n, e0);
			calculateContacts(eb[0], eb[2], pts, incN, ln, mc, num, cDist);
		}
		break;
	default:
		flip = true;
		if(0.0f >= sign[5]) { mtd = bx2; nt.R.c0 = bx0; nt.R.c1 = neg(bx1); nt.R.c2 = neg(bx2); nt.p = scaleAdd(bx2, eb[2], T1.p); }
		else { mtd = neg(bx2); nt.R.c0 = bx0; nt.R.c1 = bx1; nt.R.c2 = bx2; nt.p = negScaleSub(bx2, eb[2], T1.p); }
		{
			const MatTr t1n = mtInvMul(nt, T0);
			const V3 ln = mtRotateInv(nt, mtd);
			incidentPolygon(pts, incN, ln, t1n, e0);
			calculateContacts(eb[0], eb[1], pts, incN, ln, mc, num, cDist);
		}
		break;
	}
	if(num)
	{
		if(flip) for(int i = 0; i < num; i++) { const V3 t_ = mc[i].a; mc[i].a = mc[i].b; mc[i].b = t_; };
		const MatTr n1 = mtInvMul(T1, nt), n0 = mtInvMul(T0, nt);
		const V3 lnB = mtRotate(n1, mc[0].n);
		for(int i = 0; i < num; i++)
		{
			mc[i].a = mtTransform(n0, mc[i].a);
			mc[i].b = mtTransform(n1, mc[i].b);
			mc[i].n = lnB;
		}
	}
	return true;
}

#include "gjk_epa.cuh"

// the simplex indices gjkPenetration leaves in the manifold for the next call
static __device__ void keepWarmStart(Manifold& m, const GjkOut& g)
{
	m.warmSize = g.warmSize;
	for(int i = 0; i < g.warmSize; i++) { m.warmA[i] = g.aInd[i]; m.warmB[i] = g.bInd[i]; }
}


// pcmContactBoxBox (GuPCMContactBoxBox.cpp:848)
static __device__ bool boxBox(V3 e0, V3 e1, const Tr& tA, const Tr& tB, float cDist, float tolLen, Manifold& m, Buffer& out)
{
	const Tr cur = trInvMul(tB, tA);
	const MatTr aToB = matFromTr(cur);
	const float m0 = boxMargin(e0, tolLen), m1 = boxMargin(e1, tolLen);
	const float minMargin = fmin_(m0, m1);
	const int initial = m.num;
	refreshManifold(m, aToB, minMargin * 0.8f);
	const bool lost = m.num != initial;
	const float radiusA = sqrtf(dotA(e0, e0)), radiusB = sqrtf(dotA(e1, e1));
	if(lost || invalidateBoxConvex(m, cur, tA.q, tB.q, minMargin, radiusA, radiusB))
	{
		m.rel = cur;
		m.quatA = tA.q;
		m.quatB = tB.q;
		MatTr T0 = matFromTr(tA), T1 = matFromTr(tB);
		T0.R.c0 = normalizeA(T0.R.c0); T0.R.c1 = normalizeA(T0.R.c1); T0.R.c2 = normalizeA(T0.R.c2);
		T1.R.c0 = normalizeA(T1.R.c0); T1.R.c1 = normalizeA(T1.R.c1); T1.R.c2 = normalizeA(T1.R.c2);
		PC mc[MAXC];
		int num = 0;
		if(!boxBoxGenerate(e0, e1, T0, T1, cDist, mc, num)) return false;
		if(num > 0)
		{
			addBatch(m, mc, num, tolLen);
			const V3 wn = normalizeA(mtRotate(T1, m.pts[0].n));
			for(int i = 0; i < m.num; i++) out.add(mtTransform(T1, m.pts[i].b), wn, m.pts[i].pen);
			return true;
		}
		// Edge-edge configuration: GJK / EPA between the core boxes
		// (GuPCMContactBoxBox.cpp:917-957), one point added to the manifold.
		const GjkConvex ca = makeRelativeBox(e0, aToB);
		const GjkConvex cb = makeBox(e1);
		GjkOut g;
		int status = gjkPenetration(ca, cb, aToB.p, cDist, g);   // the warm start is cleared first
		keepWarmStart(m, g);
		if(status == EPA_CONTACT) status = epaPenetration(ca, cb, g, tolLen, g);
		if(status != GJK_CONTACT && status != EPA_CONTACT) return false;
		PC c;
		c.a = mtTransformInv(aToB, g.closestA);
		c.b = g.closestB;
		c.n = g.normal;
		c.pen = g.penDep;
		addPoint4(m, c, minMargin * 0.05f);
		const V3 wn = normalizeA(qRotate(tB.q, g.normal));
		outputWithOffset(m, wn, tB, cDist, out);
		return true;
	}
	if(m.num > 0)
	{
		outputWithOffset(m, manifoldWorldNormal(m, tB), tB, cDist, out);
		return true;
	}
	return false;
}

// ----------------------------------------------------------------- capsule-box
// pcmContactCapsuleBox (GuPCMContactCapsuleBox.cpp:73)
static __device__ bool capsuleBox(float r, float hh, V3 ext, const Tr& tCap, const Tr& tBox, float cDist, float tolLen, Manifold& m, Buffer& out)
{
	const Tr cur = trInvMul(tBox, tCap);
	const MatTr aToB = matFromTr(cur);
	const int initial = m.num;
	const float margin = boxMargin(ext, tolLen);
	const float minMargin = fmin_(margin, r);
	refreshManifold(m, aToB, minMargin * 0.8f);
	const bool lost = m.num != initial;
	if(lost || invalidateSphereCapsule(m, cur, minMargin))
	{
		m.rel = cur;
		const V3 axis = mtRotate(aToB, scale(unitX(), hh));
		const V3 p0 = add(aToB.p, axis), p1 = sub(aToB.p, axis);
		const GjkConvex cap = makeCapsule(p0, p1, r);
		const GjkConvex box = makeBox(ext);
		// the reference seeds the search with the capsule centre minus the box's world position
		const V3 initialDir = sub(aToB.p, tBox.p);
		GjkOut g;
		int status = gjkPenetration(cap, box, initialDir, cDist, g, m.warmA, m.warmB, m.warmSize);
		keepWarmStart(m, g);
		if(status == GJK_NON_INTERSECT) return false;
		PC mc[MAXC];
		int num = 0;
		bool overlapTest = false;
		bool full = true;
		if(status == GJK_DEGENERATE)
			overlapTest = true;
		else
		{
			if(status == GJK_CONTACT)
			{
				mc[num].a = mtTransformInv(aToB, g.closestA); mc[num].b = g.closestB; mc[num].n = g.normal; mc[num].pen = g.penDep; num++;
			}
			else
			{
				status = epaPenetration(cap, box, g, tolLen, g);
				if(status == EPA_CONTACT)
				{
					mc[num].a = mtTransformInv(aToB, g.closestA); mc[num].b = g.closestB; mc[num].n = g.normal; mc[num].pen = g.penDep; num++;
				}
				else
					overlapTest = true;
			}
			full = initial == 0 || lost || overlapTest;
		}
		if(!full)
		{
			// a GJK / EPA point added to the existing manifold
			PC c;
			c.a = trTransformInv(cur, g.closestA);
			c.b = g.closestB;
			c.n = g.normal;
			c.pen = g.penDep;
			addPoint2(m, c, minMargin * 0.1f);
			const V3 wn = qRotate(tBox.q, g.normal);
			outputCapsuleLike(m, wn, wn, tCap, r, cDist, out);
			return true;
		}
		// fullContactsGenerationCapsuleBox (GuPCMContactCapsuleBox.cpp:43)
		V3 normal = g.normal;
		const int orig = num;
		if(!capsuleBoxFull(p0, p1, r, ext, aToB, mc, num, cDist, normal, g.closestB, box.margin, overlapTest, tolLen)) return false;
		int first = 0;
		if(orig != 0 && num != orig) { num--; first = 1; }
		addBatch2(m, mc + first, num);
		const V3 wn = qRotate(tBox.q, normal);
		outputCapsuleLike(m, wn, wn, tCap, r, cDist, out);
		return true;
	}
	if(m.num > 0)
	{
		const V3 wn = manifoldWorldNormal(m, tBox);
		outputCapsuleLike(m, wn, wn, tCap, r, cDist, out);
		return true;
	}
	return false;
}

// Whether box-box / capsule-box contact generation takes its full path this
// frame: the pair's manifold, refreshed to the current transforms, lost a point
// or is invalidated (the decision boxBox / capsuleBox above make).  Used only to
// order the pairs of a kind so that the lanes of a warp take the same path; the
// generators decide again on their own.
static __device__ bool boxBoxFullPath(V3 e0, V3 e1, const Tr& tA, const Tr& tB, float tolLen, Manifold m)
{
	const Tr cur = trInvMul(tB, tA);
	const MatTr aToB = matFromTr(cur);
	const float minMargin = fmin_(boxMargin(e0, tolLen), boxMargin(e1, tolLen));
	const int initial = m.num;
	refreshManifold(m, aToB, minMargin * 0.8f);
	if(m.num != initial) return true;
	return invalidateBoxConvex(m, cur, tA.q, tB.q, minMargin, sqrtf(dotA(e0, e0)), sqrtf(dotA(e1, e1)));
}

static __device__ bool capsuleBoxFullPath(float r, V3 ext, const Tr& tCap, const Tr& tBox, float tolLen, Manifold m)
{
	const Tr cur = trInvMul(tBox, tCap);
	const MatTr aToB = matFromTr(cur);
	const float minMargin = fmin_(boxMargin(ext, tolLen), r);
	const int initial = m.num;
	refreshManifold(m, aToB, minMargin * 0.8f);
	if(m.num != initial) return true;
	return invalidateSphereCapsule(m, cur, minMargin);
}

// One pair (types in the reference's table order, t0 <= t1).  m: the pair's
// persistent manifold, read and updated by the cached kinds (plane-capsule,
// plane-box, capsule-box, box-box: gEnablePCMCaching, PxsContext.cpp:89).
static __device__ int generate(int t0, const float* g0, int t1, const float* g1, const Tr& p0, const Tr& p1, float cDist, float tolLen, Manifold& m, Buffer& out)
{
	switch(t0 * 4 + t1)
	{
	case SPHERE * 4 + SPHERE: sphereSphere(g0[0], g1[0], p0, p1, cDist, out); break;
	case SPHERE * 4 + PLANE: spherePlane(g0[0], p0, p1, cDist, out); break;
	case SPHERE * 4 + CAPSULE: sphereCapsule(g0[0], g1[0], g1[1], p0, p1, cDist, out); break;
	case SPHERE * 4 + BOX: sphereBox(g0[0], v3(g1[0], g1[1], g1[2]), p0, p1, cDist, out); break;
	case PLANE * 4 + CAPSULE: planeCapsule(g1[0], g1[1], p0, p1, cDist, m, out); break;
	case PLANE * 4 + BOX: planeBox(v3(g1[0], g1[1], g1[2]), p0, p1, cDist, tolLen, m, out); break;
	case CAPSULE * 4 + CAPSULE: capsuleCapsule(g0[0], g0[1], g1[0], g1[1], p0, p1, cDist, out); break;
	case CAPSULE * 4 + BOX: capsuleBox(g0[0], g0[1], v3(g1[0], g1[1], g1[2]), p0, p1, cDist, tolLen, m, out); break;
	case BOX * 4 + BOX: boxBox(v3(g0[0], g0[1], g0[2]), v3(g1[0], g1[1], g1[2]), p0, p1, cDist, tolLen, m, out); break;
	default: break;  // plane-plane: no contact generation in the reference table
	}
	return out.count;
}

// One pair's persistent contact manifold between calls (the state a PxCache
// carries for the cached pair kinds), 288 bytes: relative transform (q, p),
// both bodies' orientations, point count, a flag (0 = fresh cache), the GJK
// warm start and up to four points (local point on A, local point on B, local
// normal, penetration).
struct __align__(16) ManifoldRecord
{
	float relQ[4], relP[4], quatA[4], quatB[4];
	uint32_t num, used, warmSize, pad;
	float pts[4][12];
	uint8_t warmA[4], warmB[4];
	uint32_t pad2[2];
};
static_assert(sizeof(ManifoldRecord) == 288, "manifold record layout");

// does the pair kind (types ordered t0 <= t1) keep a manifold between frames
// (gEnablePCMCaching, physx/source/lowlevel/software/src/PxsContext.cpp:89)
static __device__ __forceinline__ bool cachedKind(int t0, int t1)
{
	return (t0 == PLANE && (t1 == CAPSULE || t1 == BOX)) || (t0 == CAPSULE && t1 == BOX) || (t0 == BOX && t1 == BOX);
}

static __device__ void loadManifold(const ManifoldRecord& r, Manifold& m)
{
	if(!r.used) { m = Manifold(); return; }
	m.rel.q.x = r.relQ[0]; m.rel.q.y = r.relQ[1]; m.rel.q.z = r.relQ[2]; m.rel.q.w = r.relQ[3];
	m.rel.p = v3(r.relP[0], r.relP[1], r.relP[2]);
	m.quatA.x = r.quatA[0]; m.quatA.y = r.quatA[1]; m.quatA.z = r.quatA[2]; m.quatA.w = r.quatA[3];
	m.quatB.x = r.quatB[0]; m.quatB.y = r.quatB[1]; m.quatB.z = r.quatB[2]; m.quatB.w = r.quatB[3];
	m.num = int(r.num);
	m.warmSize = int(r.warmSize);
	for(int i = 0; i < 4; i++) { m.warmA[i] = r.warmA[i]; m.warmB[i] = r.warmB[i]; }
	for(int i = 0; i < m.num; i++)
	{
		const float* f = r.pts[i];
		m.pts[i].a = v3(f[0], f[1], f[2]);
		m.pts[i].b = v3(f[4], f[5], f[6]);
		m.pts[i].n = v3(f[8], f[9], f[10]);
		m.pts[i].pen = f[11];
	}
}

static __device__ void storeManifold(const Manifold& m, ManifoldRecord& r)
{
	r.relQ[0] = m.rel.q.x; r.relQ[1] = m.rel.q.y; r.relQ[2] = m.rel.q.z; r.relQ[3] = m.rel.q.w;
	r.relP[0] = m.rel.p.x; r.relP[1] = m.rel.p.y; r.relP[2] = m.rel.p.z; r.relP[3] = 0.0f;
	r.quatA[0] = m.quatA.x; r.quatA[1] = m.quatA.y; r.quatA[2] = m.quatA.z; r.quatA[3] = m.quatA.w;
	r.quatB[0] = m.quatB.x; r.quatB[1] = m.quatB.y; r.quatB[2] = m.quatB.z; r.quatB[3] = m.quatB.w;
	r.num = uint32_t(m.num);
	r.used = 1;
	r.warmSize = uint32_t(m.warmSize);
	r.pad = 0;
	for(int i = 0; i < 4; i++)
	{
		r.warmA[i] = i < m.warmSize ? uint8_t(m.warmA[i]) : 0;
		r.warmB[i] = i < m.warmSize ? uint8_t(m.warmB[i]) : 0;
	}
	for(int i = 0; i < m.num; i++)
	{
		float* f = r.pts[i];
		f[0] = m.pts[i].a.x; f[1] = m.pts[i].a.y; f[2] = m.pts[i].a.z; f[3] = 0.0f;
		f[4] = m.pts[i].b.x; f[5] = m.pts[i].b.y; f[6] = m.pts[i].b.z; f[7] = 0.0f;
		f[8] = m.pts[i].n.x; f[9] = m.pts[i].n.y; f[10] = m.pts[i].n.z; f[11] = m.pts[i].pen;
	}
}

static __device__ Tr loadTr(const float* p)
{
	Tr t;
	t.q.x = p[0]; t.q.y = p[1]; t.q.z = p[2]; t.q.w = p[3];
	t.p = v3(p[4], p[5], p[6]);
	return t;
}
} // namespace np
} // namespace gbpx
