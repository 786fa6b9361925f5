// Device GJK / EPA and capsule-box manifold generation, included by
// contacts.cuh inside gbpx::np.  Same algorithm and evaluation order as the
// reference's penetration GJK (physx/source/geomutils/src/gjk/
// GuGJKPenetration.h:88, GuGJKSimplex.h/.cpp, common/GuBarycentricCoordinates.cpp),
// EPA (gjk/GuEPA.cpp, GuEPAFacet.h, common/src/CmPriorityQueue.h, CmIDPool.h)
// and capsule-box full-manifold generation (pcm/GuPCMContactGenSphereCapsule.cpp:154-420,
// pcm/GuPCMContactGenUtil.cpp:83/:201, pcm/GuPersistentContactManifold.cpp:289,
// pcm/GuPCMShapeConvex.cpp:50).  EPA keeps its polytope (64 facets, 64 support
// points) in thread-local memory; it only runs for the rare deep/edge-edge pairs.
#pragma once

enum GjkStatus { GJK_NON_INTERSECT = 0, GJK_CONTACT, GJK_UNDEFINED, GJK_DEGENERATE, EPA_CONTACT, EPA_DEGENERATE, EPA_FAIL };
enum { GJK_MAX_ITERATIONS = 128 };

struct GjkConvex
{
	int kind;            // 0 box, 1 box through relative transform, 2 capsule segment
	V3 ext;              // box half extents
	V3 p0, p1;           // capsule segment
	float margin, minMargin;
	bool marginIsRadius;
	MatTr aToB, aToBT;   // relative transform and its transposed rotation

	__device__ V3 boxPoint(int idx) const
	{
		return v3((idx & 1) ? ext.x : -ext.x, (idx & 2) ? ext.y : -ext.y, (idx & 4) ? ext.z : -ext.z);
	}
	__device__ V3 supportPoint(int idx) const
	{
		if(kind == 2) return idx ? p0 : p1;
		const V3 p = boxPoint(idx);
		return kind == 1 ? add(m33MulV(aToB.R, p), aToB.p) : p;
	}
	__device__ V3 support(V3 dir, int& idx) const
	{
		if(kind == 2)
		{
			const bool c = dotA(p0, dir) > dotA(p1, dir);
			idx = c ? 1 : 0;
			return c ? p0 : p1;
		}
		const V3 d = kind == 1 ? m33MulV(aToBT.R, dir) : dir;
		idx = (d.x > 0.0f ? 1 : 0) | (d.y > 0.0f ? 2 : 0) | (d.z > 0.0f ? 4 : 0);
		const V3 p = v3(d.x > 0.0f ? ext.x : -ext.x, d.y > 0.0f ? ext.y : -ext.y, d.z > 0.0f ? ext.z : -ext.z);
		return kind == 1 ? add(m33MulV(aToB.R, p), aToB.p) : p;
	}
	__device__ V3 support(V3 dir) const { int i; return support(dir, i); }
};

static __device__ __forceinline__ float minExtent(V3 e) { return fmin_(fmin_(e.x, e.y), e.z); }

// BoxV(center, extents): margin = 0.15 min extent, minMargin = 0.05 min extent (GuVecBox.h:60)
static __device__ __forceinline__ GjkConvex makeBox(V3 ext)
{
	GjkConvex c;
	c.kind = 0;
	c.ext = ext;
	const float m = minExtent(ext);
	c.margin = m * 0.15f;
	c.minMargin = m * 0.05f;
	c.marginIsRadius = false;
	return c;
}
static __device__ __forceinline__ M33 transpose33(const M33& m)
{
	M33 t;
	t.c0 = v3(m.c0.x, m.c1.x, m.c2.x);
	t.c1 = v3(m.c0.y, m.c1.y, m.c2.y);
	t.c2 = v3(m.c0.z, m.c1.z, m.c2.z);
	return t;
}
static __device__ __forceinline__ GjkConvex makeRelativeBox(V3 ext, const MatTr& aToB)
{
	GjkConvex c = makeBox(ext);
	c.kind = 1;
	c.aToB = aToB;
	c.aToBT.R = transpose33(aToB.R);
	c.aToBT.p = aToB.p;
	return c;
}
static __device__ __forceinline__ GjkConvex makeCapsule(V3 p0, V3 p1, float r)
{
	GjkConvex c;
	c.kind = 2;
	c.p0 = p0;
	c.p1 = p1;
	c.margin = r;
	c.minMargin = r;
	c.marginIsRadius = true;
	return c;
}

// closestPtPointSegment (GuGJKSimplex.h:88)
static __device__ __forceinline__ V3 gjkSegment(V3* Q, int& size)
{
	const V3 a = Q[0], b = Q[1];
	const V3 ab = sub(b, a);
	const float denom = dotA(ab, ab);
	const V3 ap = neg(a);
	const float nom = dotA(ap, ab);
	if(FLT_EPSILON >= denom)
	{
		size = 1;
		return Q[0];
	}
	const float t = fclamp(nom / denom, 0.0f, 1.0f);
	return scaleAdd(ab, t, a);
}

// closestPtPointTriangleBaryCentric (GuGJKSimplex.h:190)
static __device__ __forceinline__ float gjkTriBary(V3 a, V3 b, V3 c, int* idx, int& size, V3& closestPt)
{
	size = 3;
	const V3 ab = sub(b, a), ac = sub(c, a);
	const V3 n = cross(ab, ac);
	const float nn = dotA(n, n);
	if(nn == 0.0f) return FLT_MAX;
	const V3 bCrossC = cross(b, c), cCrossA = cross(c, a), aCrossB = cross(a, b);
	const float va = dotA(n, bCrossC), vb = dotA(n, cCrossA), vc = dotA(n, aCrossB);
	if(va >= 0.0f && vb >= 0.0f && vc >= 0.0f)
	{
		const float t = dotA(n, a) / nn;
		const V3 q = scale(n, t);
		closestPt = q;
		return dotA(q, q);
	}
	const V3 ap = neg(a), bp = neg(b), cp = neg(c);
	const float d1 = dotA(ab, ap), d2 = dotA(ac, ap), d3 = dotA(ab, bp), d4 = dotA(ac, bp), d5 = dotA(ab, cp), d6 = dotA(ac, cp);
	const float unom = d4 - d3, udenom = d5 - d6;
	size = 2;
	if(0.0f >= vc && d1 >= 0.0f && 0.0f >= d3)
	{
		const float toRecip = d1 - d3;
		const float recip = fabsf(toRecip) > FLT_EPSILON ? 1.0f / toRecip : 0.0f;
		const V3 q = scaleAdd(ab, d1 * recip, a);
		closestPt = q;
		return dotA(q, q);
	}
	if(0.0f >= va && d4 >= d3 && d5 >= d6)
	{
		const V3 bc = sub(c, b);
		const float toRecip = unom + udenom;
		const float recip = fabsf(toRecip) > FLT_EPSILON ? 1.0f / toRecip : 0.0f;
		idx[0] = idx[1];
		idx[1] = idx[2];
		const V3 q = scaleAdd(bc, unom * recip, b);
		closestPt = q;
		return dotA(q, q);
	}
	if(0.0f >= vb && d2 >= 0.0f && 0.0f >= d6)
	{
		const float toRecip = d2 - d6;
		const float recip = fabsf(toRecip) > FLT_EPSILON ? 1.0f / toRecip : 0.0f;
		idx[1] = idx[2];
		const V3 q = scaleAdd(ac, d2 * recip, a);
		closestPt = q;
		return dotA(q, q);
	}
	size = 1;
	if(0.0f >= d1 && 0.0f >= d2)
	{
		closestPt = a;
		return dotA(a, a);
	}
	if(d3 >= 0.0f && d3 >= d4)
	{
		idx[0] = idx[1];
		closestPt = b;
		return dotA(b, b);
	}
	idx[0] = idx[2];
	closestPt = c;
	return dotA(c, c);
}

struct Simplex
{
	V3 Q[4], A[4], B[4];
	int aInd[4], bInd[4];
	int size;
	__device__ void keep(const int* idx, int n)
	{
		V3 q[3], a[3], b[3];
		int ai[3], bi[3];
		for(int i = 0; i < n; i++) { q[i] = Q[idx[i]]; a[i] = A[idx[i]]; b[i] = B[idx[i]]; ai[i] = aInd[idx[i]]; bi[i] = bInd[idx[i]]; }
		for(int i = 0; i < n; i++) { Q[i] = q[i]; A[i] = a[i]; B[i] = b[i]; aInd[i] = ai[i]; bInd[i] = bi[i]; }
	}
};

// closestPtPointTriangle with index bookkeeping (GuGJKSimplex.h:330)
static __device__ __forceinline__ V3 gjkTriangle(Simplex& s)
{
	s.size = 3;
	const float eps2 = FLT_EPSILON * FLT_EPSILON;
	const V3 a = s.Q[0], b = s.Q[1], c = s.Q[2];
	const V3 signArea = cross(sub(b, a), sub(c, a));
	const float area = dotA(signArea, signArea);
	if(eps2 >= area)
	{
		s.size = 2;
		return gjkSegment(s.Q, s.size);
	}
	int sz;
	int idx[3] = {0, 1, 2};
	V3 closestPt = zero3();
	gjkTriBary(a, b, c, idx, sz, closestPt);
	if(sz != 3)
	{
		s.keep(idx, 2);
		s.size = sz;
	}
	return closestPt;
}

// PointOutsideOfPlane4 (GuGJKSimplex.h:52)
static __device__ __forceinline__ void outsideOfPlane4(V3 a, V3 b, V3 c, V3 d, bool* out)
{
	const V3 ab = sub(b, a), ac = sub(c, a), ad = sub(d, a), bd = sub(d, b), bc = sub(c, b);
	const V3 v0 = cross(ab, ac), v1 = cross(ac, ad), v2 = cross(ad, ab), v3_ = cross(bd, bc);
	const float sa[4] = {dotA(v0, a), dotA(v1, a), dotA(v2, a), dotA(v3_, a)};
	const float sd[4] = {dotA(v0, d), dotA(v1, b), dotA(v2, c), dotA(v3_, b)};
	for(int i = 0; i < 4; i++) out[i] = sa[i] * sd[i] >= 0.0f;
}

// closestPtPointTetrahedron with index bookkeeping (GuGJKSimplex.cpp:150)
static __device__ __forceinline__ V3 gjkTetrahedron(Simplex& s)
{
	const V3 a = s.Q[0], b = s.Q[1], c = s.Q[2], d = s.Q[3];
	const V3 n = normalizeA(cross(sub(b, a), sub(c, a)));
	const float signDist = dotA(n, sub(d, a));
	if(1e-4f > fabsf(signDist))
	{
		s.size = 3;
		return gjkTriangle(s);
	}
	bool outside[4];
	outsideOfPlane4(a, b, c, d, outside);
	if(!outside[0] && !outside[1] && !outside[2] && !outside[3]) return zero3();

	// getClosestPtPointTriangle (GuGJKSimplex.cpp:40): best of the faces the origin is outside of
	const int faces[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
	float best = FLT_MAX;
	int idx[3] = {0, 1, 2};
	V3 closest = zero3();
	if(outside[0]) best = gjkTriBary(s.Q[0], s.Q[1], s.Q[2], idx, s.size, closest);
	for(int f = 1; f < 4; f++)
	{
		if(!outside[f]) continue;
		int sz = 3;
		int t[3] = {faces[f][0], faces[f][1], faces[f][2]};
		V3 tc;
		const float sq = gjkTriBary(s.Q[t[0]], s.Q[t[1]], s.Q[t[2]], t, sz, tc);
		if(best > sq)
		{
			closest = tc;
			best = sq;
			idx[0] = t[0]; idx[1] = t[1]; idx[2] = t[2];
			s.size = sz;
		}
	}
	s.keep(idx, 3);
	return closest;
}

static __device__ __forceinline__ V3 gjkDoSimplex(Simplex& s, V3 support)
{
	switch(s.size)
	{
	case 1: return support;
	case 2: return gjkSegment(s.Q, s.size);
	case 3: return gjkTriangle(s);
	default: return gjkTetrahedron(s);
	}
}

// getClosestPoint (GuGJKSimplex.h:116) with barycentricCoordinates
static __device__ __forceinline__ void gjkClosestPoints(const Simplex& s, V3 closest, V3& ca, V3& cb, int size)
{
	if(size == 1)
	{
		ca = s.A[0];
		cb = s.B[0];
	}
	else if(size == 2)
	{
		const V3 v0 = sub(s.Q[0], closest), v1 = sub(s.Q[1], closest);
		const V3 d = sub(v1, v0);
		const float den = dotA(d, d);
		const float num = dotA(neg(v0), d);
		const float r = den > 0.0f ? 1.0f / den : 0.0f;
		const float v = num * r;
		ca = scaleAdd(sub(s.A[1], s.A[0]), v, s.A[0]);
		cb = scaleAdd(sub(s.B[1], s.B[0]), v, s.B[0]);
	}
	else if(size == 3)
	{
		const V3 ab = sub(s.Q[1], s.Q[0]), ac = sub(s.Q[2], s.Q[0]);
		const V3 n = cross(ab, ac);
		const V3 pa = sub(s.Q[0], closest), pb = sub(s.Q[1], closest), pc = sub(s.Q[2], closest);
		const float va = dotA(n, cross(pb, pc)), vb = dotA(n, cross(pc, pa)), vc = dotA(n, cross(pa, pb));
		const float total = va + (vb + vc);
		const float r = total == 0.0f ? 0.0f : 1.0f / total;
		const float v = vb * r, w = vc * r;
		ca = add(s.A[0], add(scale(sub(s.A[1], s.A[0]), v), scale(sub(s.A[2], s.A[0]), w)));
		cb = add(s.B[0], add(scale(sub(s.B[1], s.B[0]), v), scale(sub(s.B[2], s.B[0]), w)));
	}
}

struct GjkOut
{
	V3 closestA, closestB, normal;
	float penDep;
	int aInd[4], bInd[4];
	int warmSize;
};

// gjkPenetration, takeCoreShape = true (GuGJKPenetration.h:88).  warmA/warmB/
// warmSize: the simplex vertex indices kept from the pair's previous call
// (the manifold's warm start), 0 for none.  Every exit records the final
// simplex's indices in out (assignWarmStartValue), the degenerate exit one
// vertex fewer.
static __device__ __noinline__ int gjkPenetration(const GjkConvex& a, const GjkConvex& b, V3 initialDir, float contactDist, GjkOut& out,
                                 const int* warmA = nullptr, const int* warmB = nullptr, int warmSize = 0)
{
	const float minMargin = fmin_(a.minMargin, b.minMargin);
	const float eps = minMargin * 0.1f;
	const float relDif = 1.0f - 0.000225f;
	const float tMarginA = a.marginIsRadius ? a.margin : 0.0f;
	const float tMarginB = b.marginIsRadius ? b.margin : 0.0f;
	const float sumExpandedMargin = (tMarginA + tMarginB) + contactDist;
	float dist = FLT_MAX, prevDist = dist;
	V3 prevClos = zero3();
	bool notTerminated = true, notDegenerated = true;
	Simplex s;
	s.size = 0;
	V3 closest, v;
	auto record = [&](int n) {
		out.warmSize = n;
		for(int i = 0; i < n; i++) { out.aInd[i] = s.aInd[i]; out.bInd[i] = s.bInd[i]; }
	};
	if(warmSize != 0)
	{
		V3 support = zero3();
		for(int i = 0; i < warmSize; i++)
		{
			s.aInd[i] = warmA[i];
			s.bInd[i] = warmB[i];
			const V3 sa = a.supportPoint(warmA[i]), sb = b.supportPoint(warmB[i]);
			support = sub(sa, sb);
			s.A[s.size] = sa;
			s.B[s.size] = sb;
			s.Q[s.size++] = support;
		}
		closest = gjkDoSimplex(s, support);
		dist = sqrtf(dotA(closest, closest));
		v = scaleInv(closest, dist);
		prevDist = dist;
		prevClos = closest;
		notTerminated = dist > eps;
	}
	else
	{
		closest = dotA(initialDir, initialDir) > 0.0f ? initialDir : unitX();
		v = normalizeA(closest);
	}
	// The distance strictly decreases every iteration over a finite set of
	// support points, so the loop ends; the cap only bounds pathological input.
	for(int iter = 0; notTerminated; iter++)
	{
		if(iter == GJK_MAX_ITERATIONS)
		{
			notDegenerated = false;
			break;
		}
		if(s.size == 4) break;   // a full simplex only remains when it encloses the origin
		prevDist = dist;
		prevClos = closest;
		int ia, ib;
		const V3 sa = a.support(neg(closest), ia);
		const V3 sb = b.support(closest, ib);
		s.aInd[s.size] = ia;
		s.bInd[s.size] = ib;
		const V3 support = sub(sa, sb);
		const float vw = dotA(v, support);
		if(vw > sumExpandedMargin)
		{
			record(s.size);
			return GJK_NON_INTERSECT;
		}
		if(vw > dist * relDif)
		{
			record(s.size);
			out.normal = v;
			gjkClosestPoints(s, closest, out.closestA, out.closestB, s.size);
			out.penDep = dist;
			return GJK_CONTACT;
		}
		s.A[s.size] = sa;
		s.B[s.size] = sb;
		s.Q[s.size++] = support;
		closest = gjkDoSimplex(s, support);
		dist = sqrtf(dotA(closest, closest));
		v = scaleInv(closest, dist);
		notDegenerated = prevDist > dist;
		notTerminated = dist > eps && notDegenerated;
	}
	if(!notDegenerated)
	{
		record(s.size - 1);
		V3 ca = zero3(), cb = zero3();
		gjkClosestPoints(s, prevClos, ca, cb, s.size);
		out.normal = scaleInv(prevClos, prevDist);
		out.closestA = ca;
		out.closestB = cb;
		out.penDep = prevDist;
		return GJK_DEGENERATE;
	}
	record(s.size);
	return EPA_CONTACT;
}

// ---- EPA
enum { EPA_MAX_FACETS = 64, EPA_MAX_EDGES = 32, EPA_MAX_POINTS = 64 };

struct EpaFacet
{
	V3 n;
	float dist;
	int8_t adj[3];       // adjacent facet per edge, -1 = none
	int8_t adjEdge[3];
	int8_t idx[3];
	bool obsolete, inHeap;
};

struct Epa
{
	V3 aBuf[EPA_MAX_POINTS], bBuf[EPA_MAX_POINTS];
	EpaFacet f[EPA_MAX_FACETS];
	uint8_t heap[EPA_MAX_FACETS];
	int heapSize;
	// deferred ID pool (physx/source/common/src/CmIDPool.h)
	uint8_t freeIds[EPA_MAX_FACETS], deferred[EPA_MAX_FACETS];
	int curId, nbFree, nbDeferred;
	// edge buffer (GuEPAFacet.h:176)
	uint8_t edgeFacet[EPA_MAX_EDGES], edgeIndex[EPA_MAX_EDGES];
	int nbEdges;
	bool edgeOverflow;

	__device__ int newId() { return nbFree ? freeIds[--nbFree] : curId++; }
	__device__ void freeId(int id) { if(id == curId - 1) --curId; else freeIds[nbFree++] = uint8_t(id); }
	__device__ void processDeferred() { for(int i = 0; i < nbDeferred; i++) freeId(deferred[i]); nbDeferred = 0; }
	__device__ int remainingIds() const { return EPA_MAX_FACETS - (curId - nbFree); }

	// Cm::PriorityQueueBase push/pop (physx/source/common/src/CmPriorityQueue.h), ordered by plane distance
	__device__ void push(int id)
	{
		int i = heapSize, parent = (i - 1) >> 1;
		while(i > 0 && f[id].dist < f[heap[parent]].dist)
		{
			heap[i] = heap[parent];
			i = parent;
			parent = (i - 1) >> 1;
		}
		heap[i] = uint8_t(id);
		heapSize++;
	}
	__device__ int pop()
	{
		const int hs = --heapSize;
		const int top = heap[0];
		const int last = heap[hs];
		int i = 0, child;
		for(; (child = 2 * i + 1) < hs; i = child)
		{
			const int right = child + 1;
			if(right < hs && f[heap[right]].dist < f[heap[child]].dist) child = right;
			if(f[last].dist < f[heap[child]].dist) break;
			heap[i] = heap[child];
		}
		heap[i] = uint8_t(last);
		return top;
	}

	// Facet::isValid2 (GuEPA.cpp:129)
	__device__ bool setPlane(int id, float upper)
	{
		EpaFacet& F = f[id];
		const V3 p0 = sub(aBuf[F.idx[0]], bBuf[F.idx[0]]);
		const V3 p1 = sub(aBuf[F.idx[1]], bBuf[F.idx[1]]);
		const V3 p2 = sub(aBuf[F.idx[2]], bBuf[F.idx[2]]);
		const V3 dn = cross(sub(p1, p0), sub(p2, p0));
		float nv = dotA(dn, dn);
		const bool con = nv > FLT_EPSILON;
		nv = con ? nv : 1.0f;
		F.n = scale(dn, 1.0f / sqrtf(nv));
		F.dist = dotA(F.n, p0);
		return con && upper >= F.dist;
	}
	// EPA::addFacet (GuEPA.cpp:161)
	__device__ int addFacet(int i0, int i1, int i2, float upper)
	{
		const int id = newId();
		EpaFacet& F = f[id];
		F.idx[0] = int8_t(i0); F.idx[1] = int8_t(i1); F.idx[2] = int8_t(i2);
		F.adj[0] = F.adj[1] = F.adj[2] = -1;
		F.adjEdge[0] = F.adjEdge[1] = F.adjEdge[2] = -1;
		F.obsolete = false;
		if(setPlane(id, upper))
		{
			push(id);
			F.inHeap = true;
		}
		else
			F.inHeap = false;
		return id;
	}
	__device__ void link(int a, int e0, int b, int e1)
	{
		f[a].adj[e0] = int8_t(b);
		f[a].adjEdge[e0] = int8_t(e1);
		f[b].adj[e1] = int8_t(a);
		f[b].adjEdge[e1] = int8_t(e0);
	}
	__device__ static int inc3(int i) { return i == 2 ? 0 : i + 1; }
	__device__ float planeDistTo(int id, V3 p) const
	{
		const EpaFacet& F = f[id];
		return dotA(F.n, sub(p, sub(aBuf[F.idx[0]], bBuf[F.idx[0]])));
	}
	// Facet::silhouette (GuEPA.cpp:189-239)
	__device__ void silhouetteFrom(int start, int startEdge, V3 w)
	{
		int stF[EPA_MAX_FACETS], stE[EPA_MAX_FACETS];
		stF[0] = start;
		stE[0] = startEdge;
		int size = 1;
		while(size--)
		{
			const int fi = stF[size], index = stE[size];
			EpaFacet& F = f[fi];
			if(F.obsolete) continue;
			if(0.0f > planeDistTo(fi, w))
			{
				if(nbEdges < EPA_MAX_EDGES)
				{
					edgeFacet[nbEdges] = uint8_t(fi);
					edgeIndex[nbEdges] = uint8_t(index);
					nbEdges++;
				}
				else
				{
					edgeOverflow = true;
					return;
				}
			}
			else
			{
				F.obsolete = true;
				const int next = inc3(index), next2 = inc3(next);
				// a broken adjacency or a full stack ends the expansion as degenerate
				if(size + 2 > EPA_MAX_FACETS || F.adj[next] < 0 || F.adj[next2] < 0) { edgeOverflow = true; return; }
				stF[size] = F.adj[next2]; stE[size] = F.adjEdge[next2]; size++;
				stF[size] = F.adj[next]; stE[size] = F.adjEdge[next]; size++;
				if(!F.inHeap) deferred[nbDeferred++] = uint8_t(fi);
			}
		}
	}
	__device__ void silhouette(int fi, V3 w)
	{
		f[fi].obsolete = true;
		for(int e = 0; e < 3; e++)
		{
			if(f[fi].adj[e] < 0) { edgeOverflow = true; return; }
			silhouetteFrom(f[fi].adj[e], f[fi].adjEdge[e], w);
		}
	}
	// Facet::getClosestPoint (GuEPAFacet.h:226) + calculateContactInformation (GuEPA.cpp:288)
	__device__ void contactInfo(int fi, GjkOut& out) const
	{
		const EpaFacet& F = f[fi];
		const V3 pa0 = aBuf[F.idx[0]], pa1 = aBuf[F.idx[1]], pa2 = aBuf[F.idx[2]];
		const V3 pb0 = bBuf[F.idx[0]], pb1 = bBuf[F.idx[1]], pb2 = bBuf[F.idx[2]];
		const V3 p0 = sub(pa0, pb0), p1 = sub(pa1, pb1), p2 = sub(pa2, pb2);
		const V3 v0 = sub(p1, p0), v1 = sub(p2, p0);
		const V3 cp = scale(F.n, F.dist);
		const V3 v2 = sub(cp, p0);
		const float d00 = dotA(v0, v0), d01 = dotA(v0, v1), d11 = dotA(v1, v1), d20 = dotA(v2, v0), d21 = dotA(v2, v1);
		const float det = d00 * d11 - d01 * d01;
		const float recip = det > FLT_EPSILON ? 1.0f / det : 0.0f;
		const float l1 = (d11 * d20 - d01 * d21) * recip;
		const float l2 = (d00 * d21 - d01 * d20) * recip;
		const float u = 1.0f - (l1 + l2);
		out.closestA = scaleAdd(pa0, u, scaleAdd(pa1, l1, scale(pa2, l2)));
		out.closestB = scaleAdd(pb0, u, scaleAdd(pb1, l1, scale(pb2, l2)));
		out.normal = neg(F.n);
		out.penDep = -fabsf(F.dist);
	}
	__device__ bool expandTriangle(int& nv, float upper)
	{
		nv = 3;
		const int f0 = addFacet(0, 1, 2, upper);
		const int f1 = addFacet(1, 0, 2, upper);
		if(heapSize == 0) return false;
		link(f0, 0, f1, 0);
		link(f0, 1, f1, 2);
		link(f0, 2, f1, 1);
		return true;
	}
	__device__ bool expandSegment(const GjkConvex& a, const GjkConvex& b, int& nv, float upper)
	{
		const V3 q0 = sub(aBuf[0], bBuf[0]), q1 = sub(aBuf[1], bBuf[1]);
		const V3 v = sub(q1, q0);
		const V3 av = vabs(v);
		V3 axis = unitX();
		if(av.x > av.y && av.z > av.y) axis = v3(0, 1, 0);
		else if(av.x > av.z) axis = v3(0, 0, 1);
		const V3 n = normalizeA(cross(axis, v));
		aBuf[2] = a.support(neg(n));
		bBuf[2] = b.support(n);
		return expandTriangle(nv, upper);
	}
	__device__ bool expandPoint(const GjkConvex& a, const GjkConvex& b, int& nv, float upper)
	{
		const V3 q0 = sub(aBuf[0], bBuf[0]);
		aBuf[1] = a.support(neg(unitX()));
		bBuf[1] = b.support(unitX());
		const V3 q1 = sub(aBuf[1], bBuf[1]);
		if(q0.x == q1.x && q0.y == q1.y && q0.z == q1.z) return false;
		return expandSegment(a, b, nv, upper);
	}
};

// epaPenetration, takeCoreShape = true (GuEPA.cpp:93, EPA::PenetrationDepth :317)
static __device__ __noinline__ int epaPenetration(const GjkConvex& a, const GjkConvex& b, const GjkOut& simplex, float toleranceLength, GjkOut& out)
{
	Epa e;
	e.heapSize = 0;
	e.curId = e.nbFree = e.nbDeferred = 0;
	e.nbEdges = 0;
	e.edgeOverflow = false;
	const int size = simplex.warmSize;
	for(int i = 0; i < size; i++)
	{
		e.aBuf[i] = a.supportPoint(simplex.aInd[i]);
		e.bBuf[i] = b.supportPoint(simplex.bInd[i]);
	}
	float upper = FLT_MAX;
	int nv = 0;
	switch(size)
	{
	case 1: if(!e.expandPoint(a, b, nv, upper)) return EPA_FAIL; break;
	case 2: if(!e.expandSegment(a, b, nv, upper)) return EPA_FAIL; break;
	case 3: if(!e.expandTriangle(nv, upper)) return EPA_FAIL; break;
	default:
	{
		const V3 p0 = sub(e.aBuf[0], e.bBuf[0]), p1 = sub(e.aBuf[1], e.bBuf[1]);
		const V3 p2 = sub(e.aBuf[2], e.bBuf[2]), p3 = sub(e.aBuf[3], e.bBuf[3]);
		const V3 n = normalizeA(cross(sub(p1, p0), sub(p2, p0)));
		if(dotA(n, sub(p3, p0)) > 0.0f)
		{
			const V3 ta = e.aBuf[1], tb = e.bBuf[1];
			e.aBuf[1] = e.aBuf[2]; e.bBuf[1] = e.bBuf[2];
			e.aBuf[2] = ta; e.bBuf[2] = tb;
		}
		const int f0 = e.addFacet(0, 1, 2, upper);
		const int f1 = e.addFacet(0, 3, 1, upper);
		const int f2 = e.addFacet(0, 2, 3, upper);
		const int f3 = e.addFacet(1, 3, 2, upper);
		if(e.heapSize == 0) return EPA_FAIL;
		e.link(f0, 0, f1, 2);
		e.link(f0, 1, f3, 2);
		e.link(f0, 2, f2, 0);
		e.link(f1, 0, f2, 2);
		e.link(f1, 1, f3, 0);
		e.link(f2, 1, f3, 1);
		nv = 4;
		break;
	}
	}
	const float eps = fmin_(a.minMargin, b.minMargin) * 0.1f;
	int facet = -1;
	do
	{
		e.processDeferred();
		facet = e.pop();
		e.f[facet].inHeap = false;
		if(!e.f[facet].obsolete)
		{
			const V3 n = e.f[facet].n;
			const float pd = e.f[facet].dist;
			const V3 ta = a.support(n);
			const V3 tb = b.support(neg(n));
			const V3 q = sub(ta, tb);
			const float dist = dotA(q, n);
			if(eps >= fabsf(dist - pd))
			{
				e.contactInfo(facet, out);
				const float tolEps = 1e-3f * toleranceLength;
				const V3 dif = sub(out.closestA, out.closestB);
				const float pen = fabsf(out.penDep) + tolEps;
				const float sq = dotA(dif, dif);
				const float len = sq > 0.0f ? sqrtf(sq) : 0.0f;
				return len > pen ? EPA_DEGENERATE : EPA_CONTACT;
			}
			upper = fmin_(upper, dist);
			e.aBuf[nv] = ta;
			e.bBuf[nv] = tb;
			const int index = nv++;
			e.nbEdges = 0;
			e.edgeOverflow = false;
			e.silhouette(facet, q);
			if(e.nbEdges == 0 || e.edgeOverflow)
			{
				e.contactInfo(facet, out);
				return EPA_DEGENERATE;
			}
			if(e.nbEdges > e.remainingIds())
			{
				e.contactInfo(facet, out);
				return EPA_DEGENERATE;
			}
			auto src = [&](int k) { return int(e.f[e.edgeFacet[k]].idx[e.edgeIndex[k]]); };
			auto tgt = [&](int k) { return int(e.f[e.edgeFacet[k]].idx[Epa::inc3(e.edgeIndex[k])]); };
			const int first = e.addFacet(tgt(0), src(0), index, upper);
			e.link(first, 0, e.edgeFacet[0], e.edgeIndex[0]);
			int last = first;
			for(int k = 1; k < e.nbEdges; k++)
			{
				const int nf = e.addFacet(tgt(k), src(k), index, upper);
				e.link(nf, 0, e.edgeFacet[k], e.edgeIndex[k]);
				e.link(nf, 2, last, 1);
				last = nf;
			}
			e.link(first, 2, last, 1);
		}
		e.freeId(facet);
	} while(e.heapSize > 0 && upper > e.f[e.heap[0]].dist && nv != EPA_MAX_POINTS);
	e.contactInfo(facet, out);
	return EPA_DEGENERATE;
}


static __constant__ uint8_t kBoxQuads[24] = {0, 3, 2, 1, 1, 2, 6, 5, 5, 6, 7, 4, 4, 7, 3, 0, 3, 7, 6, 2, 4, 0, 1, 5};
static __constant__ int kBoxFaceAxis[6] = {2, 0, 2, 0, 1, 1};
static __constant__ float kBoxFaceSign[6] = {-1.0f, 1.0f, 1.0f, -1.0f, 1.0f, -1.0f};
static __constant__ int kBoxFaceMinVert[6] = {4, 0, 0, 1, 0, 2};

struct PolyBox
{
	V3 verts[8];
	V3 n[6];
	float d[6];
	__device__ explicit PolyBox(V3 h)
	{
		const V3 lo = neg(h);
		verts[0] = v3(lo.x, lo.y, lo.z); verts[1] = v3(h.x, lo.y, lo.z);
		verts[2] = v3(h.x, h.y, lo.z);   verts[3] = v3(lo.x, h.y, lo.z);
		verts[4] = v3(lo.x, lo.y, h.z);  verts[5] = v3(h.x, lo.y, h.z);
		verts[6] = v3(h.x, h.y, h.z);    verts[7] = v3(lo.x, h.y, h.z);
		for(int i = 0; i < 6; i++)
		{
			float c[3] = {0.0f, 0.0f, 0.0f};
			c[kBoxFaceAxis[i]] = kBoxFaceSign[i];
			n[i] = v3(c[0], c[1], c[2]);
			d[i] = -getc(h, kBoxFaceAxis[i]);
		}
	}
	__device__ V3 vert(int face, int k) const { return verts[kBoxQuads[face * 4 + k]]; }
};

// PxPlane::distance with PxVec3::dot
static __device__ float planeDistance(V3 n, float d, V3 p) { return dotS(n, p) + d; }

// testPolyDataAxis + testSATCapsulePoly (GuPCMContactGenSphereCapsule.cpp:41/:154)
static __device__ bool satCapsuleBox(V3 p0, V3 p1, float r, const PolyBox& pb, V3 ext, float cDist, V3& axisOut)
{
	float minOverlap = FLT_MAX;
	V3 axis = v3(0, 1, 0);
	for(int i = 0; i < 6; i++)
	{
		const V3 n = pb.n[i];
		const float magnitude = 1.0f / sqrtf(dotA(n, n));
		const V3 planeN = scale(n, magnitude);
		const float min0 = dotA(n, pb.verts[kBoxFaceMinVert[i]]) * magnitude;
		const float max0 = (-pb.d[i]) * magnitude;
		const float t0 = dotA(p0, planeN), t1 = dotA(p1, planeN);
		const float min1 = fmin_(t0, t1) - r, max1 = fmax_(t0, t1) + r;
		if(min1 > max0 + cDist || min0 > max1 + cDist) return false;
		const float ov = max0 - min1;
		if(minOverlap > ov) { minOverlap = ov; axis = planeN; }
	}
	const V3 capAxis = sub(p1, p0);
	for(int i = 0; i < 6; i++)
	{
		for(int s = 0, e = 3; s < 4; e = s++)
		{
			const V3 edge = sub(pb.vert(i, e), pb.vert(i, s));
			const V3 dir = cross(capAxis, edge);
			const float lenSq = dotA(dir, dir);
			if(FLT_EPSILON > lenSq) continue;
			const V3 n = scaleInv(dir, sqrtf(lenSq));
			const V3 sp = v3(n.x > 0.0f ? ext.x : -ext.x, n.y > 0.0f ? ext.y : -ext.y, n.z > 0.0f ? ext.z : -ext.z);
			const float max0 = dotA(n, sp), min0 = -max0;
			const float t0 = dotA(p0, n), t1 = dotA(p1, n);
			const float min1 = fmin_(t0, t1) - r, max1 = fmax_(t0, t1) + r;
			if(min1 > max0 + cDist || min0 > max1 + cDist) return false;
			const float ov = max0 - min1;
			if(minOverlap > ov) { minOverlap = ov; axis = n; }
		}
	}
	axisOut = axis;
	return true;
}

// getPolygonIndex for a box (no edge data; GuPCMContactGenUtil.cpp:83)
static __device__ int boxPolygonIndex(const PolyBox& pb, V3 normal)
{
	float minProj = dotA(normal, pb.n[0]);
	int best = 0;
	for(int i = 1; i < 6; i++)
	{
		const float proj = dotA(normal, pb.n[i]);
		if(minProj > proj) { minProj = proj; best = i; }
	}
	return best;
}

// getWitnessPolygonIndex (GuPCMContactGenUtil.cpp:201)
static __device__ int boxWitnessPolygonIndex(const PolyBox& pb, V3 normal, V3 closest, float tolerance)
{
	float pd[6];
	const float eps = -tolerance;
	float dist = planeDistance(pb.n[0], pb.d[0], closest);
	float minDist = dist >= eps ? fabsf(dist) : FLT_MAX;
	pd[0] = minDist;
	float maxDist = dist;
	int closestFace = 0, maxFace = 0;
	for(int i = 1; i < 6; i++)
	{
		dist = planeDistance(pb.n[i], pb.d[i], closest);
		pd[i] = dist >= eps ? fabsf(dist) : FLT_MAX;
		if(minDist > pd[i]) { minDist = pd[i]; closestFace = i; }
		if(dist > maxDist) { maxDist = dist; maxFace = i; }
	}
	if(minDist == FLT_MAX) return maxFace;
	float bestProj = dotA(normalizeA(pb.n[closestFace]), normal);
	const int first = closestFace;
	for(int i = 0; i < 6; i++)
	{
		if(tolerance > pd[i] - minDist && first != i)
		{
			const float proj = dotA(normalizeA(pb.n[i]), normal);
			if(bestProj > proj) { closestFace = i; bestProj = proj; }
		}
	}
	return closestFace;
}

// findRotationMatrixFromZAxis (GuPersistentContactManifold.cpp:289)
static __device__ M33 rotationFromZAxis(V3 to)
{
	const float e = to.z, f = fabsf(e);
	M33 m;
	if(0.9999f > f)
	{
		const float vx = -to.y, vy = to.x;
		const float h = 1.0f / (1.0f + e);
		const float hvx = h * vx, hvxy = hvx * vy;
		m.c0 = v3(hvx * vx + e, hvxy, vy);
		m.c1 = v3(hvxy, h * (vy * vy) + e, -vx);
		m.c2 = v3(-vy, vx, e);
		return m;
	}
	const V3 u = v3(0.0f, 1.0f, -1.0f);   // (0,1,0) - (0,0,1)
	const V3 v = sub(v3(0, 1, 0), to);
	const float dotU = dotA(u, u), dotV = dotA(v, v), dotUV = dotA(u, v);
	const float c1 = -(2.0f / dotU), c2 = -(2.0f / dotV);
	const float c3 = c1 * (c2 * dotUV);
	const V3 c1u = scale(u, c1), c2v = scale(v, c2), c3v = scale(v, c3);
	m.c0 = scaleAdd(u, c1u.x, scaleAdd(v, c2v.x, scale(u, c3v.x)));
	m.c0.x = m.c0.x + 1.0f;
	m.c1 = scaleAdd(u, c1u.y, scaleAdd(v, c2v.y, scale(u, c3v.y)));
	m.c1.y = m.c1.y + 1.0f;
	m.c2 = scaleAdd(u, c1u.z, scaleAdd(v, c2v.z, scale(u, c3v.z)));
	m.c2.z = m.c2.z + 1.0f;
	return m;
}

// generatedCapsuleBoxFaceContacts (GuPCMContactGenSphereCapsule.cpp:221)
static __device__ void capsuleBoxFaceContacts(V3 p0, V3 p1, float r, const PolyBox& pb, int face, const MatTr& aToB, PC* mc, int& num, float cDist, V3 normal)
{
	const float radius = r + cDist;
	const V3 planeN = normalizeA(pb.n[face]);
	const V3 a = pb.vert(face, 0);
	const float denom0 = dotA(planeN, sub(p0, a)), denom1 = dotA(planeN, sub(p1, a));
	const float proj = dotA(planeN, normal);
	const float numer = proj > 0.0f ? 1.0f / proj : 0.0f;
	const float t0 = denom0 * numer, t1 = denom1 * numer;
	const bool con0 = radius >= t0, con1 = radius >= t1;
	if(!(con0 || con1)) return;
	const M33 rot = rotationFromZAxis(planeN);
	V3 pts[4];
	V3 bmin = v3(FLT_MAX, FLT_MAX, FLT_MAX), bmax = neg(bmin);
	for(int i = 0; i < 4; i++)
	{
		pts[i] = m33MulV(rot, pb.vert(face, i));
		bmin = vmin(bmin, pts[i]);
		bmax = vmax(bmax, pts[i]);
	}
	if(con0)
	{
		const V3 q = negScaleSub(normal, t0, p0);
		if(containsXY(pts, 4, m33MulV(rot, q), bmin, bmax))
		{
			mc[num].a = mtTransformInv(aToB, p0); mc[num].b = q; mc[num].n = normal; mc[num].pen = t0; num++;
		}
	}
	if(con1)
	{
		const V3 q = negScaleSub(normal, t1, p1);
		if(containsXY(pts, 4, m33MulV(rot, q), bmin, bmax))
		{
			mc[num].a = mtTransformInv(aToB, p1); mc[num].b = q; mc[num].n = normal; mc[num].pen = t1; num++;
		}
	}
}

// generateEE (GuPCMContactGenSphereCapsule.cpp:312)
static __device__ void capsuleBoxEE(V3 p, V3 q, V3 normal, V3 a, V3 b, const MatTr& aToB, PC* mc, int& num, float inflatedRadius)
{
	const float expandedRatio = 0.005f;
	const V3 ab = sub(b, a);
	const V3 n = cross(ab, normal);
	const float d = dotA(n, a), np = dotA(n, p), nq = dotA(n, q);
	const float signP = np - d, signQ = nq - d;
	if(signP * signQ > 0.0f) return;
	const V3 pq = sub(q, p);
	const float npq = dotA(n, pq);
	if(npq == 0.0f) return;
	const float segT = (d - np) / npq;
	const V3 lpA = scaleAdd(pq, segT, p);
	const V3 perN = cross(normal, pq);
	const V3 ap = sub(lpA, a);
	const float nom = dotA(perN, ap), den = dotA(perN, ab);
	const float t = nom / den;
	const float mx = 1.0f + expandedRatio, mn = 0.0f - expandedRatio;
	if(t > mx || mn > t) return;
	const V3 v = negScaleSub(ab, t, ap);
	const float sd = dotA(v, normal);
	if(inflatedRadius >= sd)
	{
		mc[num].a = mtTransformInv(aToB, lpA);
		mc[num].b = sub(lpA, v);
		mc[num].n = normal;
		mc[num].pen = sd;
		num++;
	}
}

// generateCapsuleBoxFullContactManifold (GuPCMContactGenSphereCapsule.cpp:379)
static __device__ bool capsuleBoxFull(V3 p0, V3 p1, float r, V3 ext, const MatTr& aToB, PC* mc, int& num, float cDist, V3& normal, V3 closest,
                    float margin, bool overlapTest, float tolLen)
{
	const PolyBox pb(ext);
	const int orig = num;
	int face;
	if(overlapTest)
	{
		if(!satCapsuleBox(p0, p1, r, pb, ext, cDist, normal)) return false;
		face = boxPolygonIndex(pb, neg(normal));
	}
	else
	{
		const float lo = tolLen * 1e-2f, hi = tolLen * 5e-2f;
		const float tolerance = fmin_(hi, fmax_(lo, margin));
		face = boxWitnessPolygonIndex(pb, neg(normal), closest, tolerance);
	}
	capsuleBoxFaceContacts(p0, p1, r, pb, face, aToB, mc, num, cDist, normal);
	if(num - orig < 2)
	{
		const float inflated = r + cDist;
		for(int s = 0, e = 3; s < 4; e = s++) capsuleBoxEE(p0, p1, normal, pb.vert(face, s), pb.vert(face, e), aToB, mc, num, inflated);
	}
	return true;
}

