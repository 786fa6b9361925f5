// ORACLE (test infrastructure, never shipped): one frame of the reference's
// immediate-mode loop (physx/snippets/snippetimmediatemode/SnippetImmediateMode.cpp:473
// stepPhysics) for many independent scenes, with a fresh broadphase, fresh
// PxCache and fresh friction data per frame:
//   bounds (shape AABB + margin) -> ABP pair set (every body is created, so the
//   set is every overlapping pair under BpBroadPhaseABP.cpp's closed-interval
//   test) ordered by (id0, id1) -> PxGenerateContacts per pair ->
//   constraints = pairs with contacts -> TGS solve + integrate -> write-back.
// Built from the restated broadphase/narrowphase/TGS entry points of this
// directory; the reference harness (oracle/ref/harness.cpp, pxref_scene_step)
// does the same with the reference's own functions.
#include "pxmath.h"
#include "tgs_frame.h"
#include <string.h>
#include <map>
#include <vector>
#include <algorithm>

#define OX extern "C" __attribute__((visibility("default")))

using namespace orc;

extern "C" int orc_np_run(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0, const float* pose1,
                          uint32_t nbPairs, float contactDistance, float meshContactMargin, float toleranceLength, float* outContacts,
                          uint32_t maxPerPair, uint32_t* outCounts);
extern "C" uint32_t orc_tgs_solve(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA,
                                  const uint32_t* pairB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                                  const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel,
                                  float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, float* outVel, float* outPose,
                                  uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder, void* outBodyVelRaw, void* outTxIRaw);
extern "C" int orc_np_run_cached(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0,
                                 const float* pose1, uint32_t nbPairs, float contactDistance, float meshContactMargin, float toleranceLength,
                                 float* outContacts, uint32_t maxPerPair, uint32_t* outCounts, void* manifolds);

namespace
{
inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
inline uint32_t encodeFloat(uint32_t ir) { return (ir & 0x80000000u) ? ~ir : (ir | 0x80000000u); }

struct Rigid   // PxRigidBodyData
{
	float linVel[3]; float invMass; float angVel[3]; float maxDepen; float invInertia[3]; float maxImpulse;
	float q[4]; float p[3]; float linDamp, angDamp, maxLinSq, maxAngSq; uint32_t pad;
};

// Shape AABB: sphere r; capsule |axis|*halfHeight + r; box sum of |columns|*extents; planes unbounded.
void shapeBounds(int type, const float* g, const Tr& pose, float margin, float* out)
{
	V3 e;
	if(type == 0) e = v3(g[0], g[0], g[0]);
	else if(type == 2)
	{
		const V3 ax = qBasis0(pose.q);
		e = v3(fabsf(ax.x) * g[1] + g[0], fabsf(ax.y) * g[1] + g[0], fabsf(ax.z) * g[1] + g[0]);
	}
	else if(type == 3)
	{
		const M33 R = m33FromQuatCol(pose.q);
		e = v3((fabsf(R.c0.x) * g[0] + fabsf(R.c1.x) * g[1]) + fabsf(R.c2.x) * g[2],
		       (fabsf(R.c0.y) * g[0] + fabsf(R.c1.y) * g[1]) + fabsf(R.c2.y) * g[2],
		       (fabsf(R.c0.z) * g[0] + fabsf(R.c1.z) * g[1]) + fabsf(R.c2.z) * g[2]);
	}
	else
	{
		for(int k = 0; k < 3; k++) { out[k] = -1e30f - margin; out[3 + k] = 1e30f + margin; }
		return;
	}
	const V3 mn = sub(pose.p, e), mx = add(pose.p, e);
	out[0] = mn.x - margin; out[1] = mn.y - margin; out[2] = mn.z - margin;
	out[3] = mx.x + margin; out[4] = mx.y + margin; out[5] = mx.z + margin;
}

bool overlap(const float* a, const float* b)
{
	const uint32_t aminx = encodeFloat(fbits(a[0])), amaxx = encodeFloat(fbits(a[3]));
	const uint32_t bminx = encodeFloat(fbits(b[0])), bmaxx = encodeFloat(fbits(b[3]));
	if(bminx > amaxx || aminx > bmaxx) return false;
	return !(b[4] < a[1] || a[4] < b[1] || b[5] < a[2] || a[5] < b[2]);
}

// Every overlapping pair of the n dynamic and m static boxes except static-static,
// as (id0 < id1) sorted by (id0, id1).  A sweep over the boxes sorted by encoded
// min X tests each pair whose X intervals overlap exactly once; the set is the
// one the all-pairs closed-interval test gives.
void overlappingPairs(const std::vector<float>& box, uint32_t n, uint32_t m, std::vector<uint32_t>& A, std::vector<uint32_t>& B)
{
	const uint32_t total = n + m;
	std::vector<uint32_t> idx(total);
	for(uint32_t i = 0; i < total; i++) idx[i] = i;
	auto minKey = [&](uint32_t i) { return encodeFloat(fbits(box[6 * size_t(i)])); };
	std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return minKey(a) < minKey(b); });
	std::vector<uint64_t> keys;
	for(uint32_t s = 0; s < total; s++)
	{
		const uint32_t i = idx[s];
		const uint32_t maxKey = encodeFloat(fbits(box[6 * size_t(i) + 3]));
		for(uint32_t t = s + 1; t < total && minKey(idx[t]) <= maxKey; t++)
		{
			const uint32_t j = idx[t];
			if(i >= n && j >= n) continue;   // statics are not paired together
			if(!overlap(&box[6 * size_t(i)], &box[6 * size_t(j)])) continue;
			const uint32_t a = i < j ? i : j, b = i < j ? j : i;
			keys.push_back((uint64_t(a) << 32) | b);
		}
	}
	std::sort(keys.begin(), keys.end());
	A.resize(keys.size());
	B.resize(keys.size());
	for(size_t k = 0; k < keys.size(); k++) { A[k] = uint32_t(keys[k] >> 32); B[k] = uint32_t(keys[k]); }
}
} // namespace

// Persistent pair state between frames (the snippet's WITH_PERSISTENCY mode,
// SnippetImmediateMode.cpp:47): per overlapping pair its contact manifold
// (288-byte record of np.cpp, zero = fresh cache) and the friction patches its
// contact constraint left.  A pair starts fresh when it starts overlapping and
// loses its state when it stops; a pair without contacts loses its friction.
namespace
{
struct PairState
{
	uint8_t manifold[288];
	std::vector<FrictionPatch> friction;
	PairState() { memset(manifold, 0, sizeof(manifold)); }
};
struct Persistent
{
	std::vector<std::map<std::pair<uint32_t, uint32_t>, PairState>> scenes;
};

int sceneStep(Persistent* ps, uint32_t nbScenes, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, void* rigidIO, const int* types,
              const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
              const float* params, const uint32_t* iterations);
} // namespace

OX void* orc_persistent_create() { return new Persistent; }
OX void orc_persistent_release(void* h) { delete static_cast<Persistent*>(h); }

// orc_scene_step with persistent contact manifolds and friction patches (state in h).
OX int orc_scene_step_persistent(void* h, uint32_t nbScenes, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, void* rigidIO,
                                 const int* types, const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes,
                                 const float* staticGeoms, const float* params, const uint32_t* iterations)
{
	return sceneStep(static_cast<Persistent*>(h), nbScenes, sceneBodyCount, sceneStaticCount, rigidIO, types, geoms, friction, staticPoses,
	                 staticTypes, staticGeoms, params, iterations);
}

// Steps every scene once.  rigid: all dynamic bodies (PxRigidBodyData) scene by
// scene; params as gbpx_world_create (dt, g xyz, contactDistance,
// toleranceLength, boundsMargin, bounceThreshold, frictionOffsetThreshold,
// correlationDistance, staticFriction); iterations (pos, vel).
OX int orc_scene_step(uint32_t nbScenes, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, void* rigidIO, const int* types,
                      const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
                      const float* params, const uint32_t* iterations)
{
	return sceneStep(nullptr, nbScenes, sceneBodyCount, sceneStaticCount, rigidIO, types, geoms, friction, staticPoses, staticTypes, staticGeoms,
	                 params, iterations);
}

namespace
{
int sceneStep(Persistent* ps, uint32_t nbScenes, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, void* rigidIO, const int* types,
              const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
              const float* params, const uint32_t* iterations)
{
	if(ps && ps->scenes.size() < nbScenes) ps->scenes.resize(nbScenes);
	Rigid* rigid = static_cast<Rigid*>(rigidIO);
	const float dt = params[0];
	const float g[3] = {params[1], params[2], params[3]};
	const float cDist = params[4], tolLen = params[5], margin = params[6];
	uint32_t b0 = 0, s0 = 0;
	for(uint32_t s = 0; s < nbScenes; s++)
	{
		const uint32_t n = sceneBodyCount[s], m = sceneStaticCount[s];
		std::vector<float> box(6 * size_t(n + m));
		std::vector<Tr> pose(n + m);
		std::vector<int> type(n + m);
		std::vector<float> geom(4 * size_t(n + m));
		for(uint32_t i = 0; i < n + m; i++)
		{
			if(i < n)
			{
				const Rigid& r = rigid[b0 + i];
				pose[i].q = Q{r.q[0], r.q[1], r.q[2], r.q[3]};
				pose[i].p = v3(r.p[0], r.p[1], r.p[2]);
				type[i] = types[b0 + i];
				memcpy(&geom[4 * i], geoms + 4 * size_t(b0 + i), 16);
			}
			else
			{
				const float* sp = staticPoses + 7 * size_t(s0 + i - n);
				pose[i].q = Q{sp[0], sp[1], sp[2], sp[3]};
				pose[i].p = v3(sp[4], sp[5], sp[6]);
				type[i] = staticTypes[s0 + i - n];
				memcpy(&geom[4 * i], staticGeoms + 4 * size_t(s0 + i - n), 16);
			}
			shapeBounds(type[i], &geom[4 * i], pose[i], margin, &box[6 * i]);
		}
		// every overlapping pair, (id0, id1) order, statics after dynamics
		std::vector<uint32_t> A, B;
		overlappingPairs(box, n, m, A, B);
		// order (i, j): dynamic partners come first for each i, then statics (n + k > every j)
		const size_t np = A.size();
		std::vector<int> t0(np), t1(np);
		std::vector<float> g0(4 * np), g1(4 * np), p0(7 * np), p1(7 * np);
		for(size_t k = 0; k < np; k++)
		{
			t0[k] = type[A[k]]; t1[k] = type[B[k]];
			memcpy(&g0[4 * k], &geom[4 * A[k]], 16);
			memcpy(&g1[4 * k], &geom[4 * B[k]], 16);
			const Tr& pa = pose[A[k]];
			const Tr& pb = pose[B[k]];
			const float qa[7] = {pa.q.x, pa.q.y, pa.q.z, pa.q.w, pa.p.x, pa.p.y, pa.p.z};
			const float qb[7] = {pb.q.x, pb.q.y, pb.q.z, pb.q.w, pb.p.x, pb.p.y, pb.p.z};
			memcpy(&p0[7 * k], qa, 28);
			memcpy(&p1[7 * k], qb, 28);
		}
		std::vector<float> cts(np * 4 * 8);
		std::vector<uint32_t> cnt(np);
		std::vector<PairState*> state(np, nullptr);
		if(ps)
		{
			std::map<std::pair<uint32_t, uint32_t>, PairState> next;
			std::map<std::pair<uint32_t, uint32_t>, PairState>& cur = ps->scenes[s];
			for(size_t k = 0; k < np; k++)
			{
				const std::pair<uint32_t, uint32_t> key(A[k], B[k]);
				auto it = cur.find(key);
				next[key] = it != cur.end() ? it->second : PairState();
			}
			cur.swap(next);
			std::vector<uint8_t> rec(np * 288 + 288);
			for(size_t k = 0; k < np; k++)
			{
				state[k] = &cur[std::make_pair(A[k], B[k])];
				memcpy(&rec[k * 288], state[k]->manifold, 288);
			}
			if(np) orc_np_run_cached(t0.data(), g0.data(), t1.data(), g1.data(), p0.data(), p1.data(), uint32_t(np), cDist, 0.01f, tolLen, cts.data(),
			                         4, cnt.data(), rec.data());
			for(size_t k = 0; k < np; k++)
			{
				memcpy(state[k]->manifold, &rec[k * 288], 288);
				if(!cnt[k]) state[k]->friction.clear();
			}
		}
		else if(np)
			orc_np_run(t0.data(), g0.data(), t1.data(), g1.data(), p0.data(), p1.data(), uint32_t(np), cDist, 0.01f, tolLen, cts.data(), 4,
			           cnt.data());
		std::vector<uint32_t> ca, cb, cs, cc;
		std::vector<float> packed, mat;
		std::vector<std::vector<FrictionPatch>> fric;
		std::vector<PairState*> cstate;
		for(size_t k = 0; k < np; k++)
		{
			if(!cnt[k]) continue;
			if(ps)
			{
				cstate.push_back(state[k]);
				fric.push_back(state[k]->friction);
			}
			ca.push_back(A[k]); cb.push_back(B[k]);
			cs.push_back(uint32_t(packed.size() / 8)); cc.push_back(cnt[k]);
			packed.insert(packed.end(), &cts[k * 32], &cts[k * 32] + 8 * cnt[k]);
			const float fa = friction[b0 + A[k]];
			const float fb = B[k] < n ? friction[b0 + B[k]] : params[10];
			const float mu = (fa + fb) * 0.5f;
			mat.push_back(mu); mat.push_back(mu); mat.push_back(0.0f);
		}
		std::vector<float> vel(6 * size_t(n)), outPose(7 * size_t(n));
		std::vector<uint32_t> hs(2 * ca.size() + 2), hst(2 * ca.size() + 2), ord(ca.size() + 1);
		std::vector<float> statics(7 * size_t(m));
		for(uint32_t k = 0; k < m; k++) memcpy(&statics[7 * k], staticPoses + 7 * size_t(s0 + k), 28);
		if(ps)
		{
			tgsFrame(&rigid[b0], n, statics.data(), m, ca.data(), cb.data(), uint32_t(ca.size()), cs.data(), cc.data(), packed.data(), mat.data(), g,
			         dt, iterations[0], iterations[1], params[7], params[8], params[9], vel.data(), outPose.data(), hs.data(), hst.data(), ord.data(),
			         &fric);
			for(size_t k = 0; k < cstate.size(); k++) cstate[k]->friction = fric[k];
		}
		else
			orc_tgs_solve(&rigid[b0], n, statics.data(), m, ca.data(), cb.data(), uint32_t(ca.size()), cs.data(), cc.data(), packed.data(),
			              mat.data(), g, dt, iterations[0], iterations[1], params[7], params[8], params[9], vel.data(), outPose.data(), hs.data(),
			              hst.data(), ord.data(), nullptr, nullptr);
		for(uint32_t i = 0; i < n; i++)
		{
			Rigid& r = rigid[b0 + i];
			memcpy(r.linVel, &vel[6 * i], 12);
			memcpy(r.angVel, &vel[6 * i + 3], 12);
			memcpy(r.q, &outPose[7 * i], 16);
			memcpy(r.p, &outPose[7 * i + 4], 12);
		}
		b0 += n;
		s0 += m;
	}
	return 0;
}
} // namespace
