// PxGenerateContacts of libgbpx_immediate.so over moving frames with one PxCache
// per pair kept between frames and cache memory from a PxCacheAllocator, the
// way the reference's immediate-mode snippet keeps its pair caches
// (SnippetImmediateMode.cpp:657-676).  Used by tests/test_immediate_dropin_gpu.py.
//
// stdin (binary): nbPairs, nbFrames (u32); per pair type0, type1 (i32; a
// convex core is 4 | its PxConvexCore::Type << 8) and geometry (4 + 4 floats); per frame the poses of both shapes (7 + 7 floats per
// pair, PxTransform).
// stdout (binary): per frame per pair the contact count (u32) and per contact
// normal xyz, separation, point xyz, 0 (8 floats).
#include "gbpx_immediate.h"

#include <cstdint>
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

struct Shape
{
	union { PxGeometry any; PxSphereGeometry sphere; PxCapsuleGeometry capsule; PxBoxGeometry box; PxPlaneGeometry plane; PxConvexCoreGeometry convex; };
	Shape() { memset(this, 0, sizeof(*this)); }
	void set(int type, const float* g)
	{
		any.mType = type & 0xff;
		if(type == 0) sphere.radius = g[0];
		if(type == 2) { capsule.radius = g[0]; capsule.halfHeight = g[1]; }
		if(type == 3) box.halfExtents = PxVec3{g[0], g[1], g[2]};
		if((type & 0xff) == 4)
		{
			// PxConvexCoreGeometry: core type in bits 8..15 of the input type, core floats, margin
			convex.mCoreType = type >> 8;
			memcpy(convex.mCore, g, 3 * sizeof(float));
			convex.mMargin = g[3];
		}
	}
};

struct Recorder : PxContactRecorder
{
	std::vector<std::vector<PxContactPoint>> perPair;
	bool recordContacts(const PxContactPoint* cp, uint32_t n, uint32_t index) override
	{
		perPair[index].assign(cp, cp + n);
		return true;
	}
};

// cache memory of the last two frames: a frame's caches are read by the next one
struct CacheAllocator : PxCacheAllocator
{
	std::vector<void*> blocks[2];
	int frame = 0;
	uint8_t* allocateCacheData(const uint32_t byteSize) override
	{
		void* p = nullptr;
		if(posix_memalign(&p, 16, byteSize ? byteSize : 16)) return nullptr;
		blocks[frame & 1].push_back(p);
		return static_cast<uint8_t*>(p);
	}
	void nextFrame()
	{
		frame++;
		for(void* p : blocks[frame & 1]) free(p);
		blocks[frame & 1].clear();
	}
	~CacheAllocator() override
	{
		for(auto& b : blocks)
			for(void* p : b) free(p);
	}
};
} // namespace

int main()
{
	uint32_t hdr[2];
	readAll(hdr, 2);
	const uint32_t nbPairs = hdr[0], nbFrames = hdr[1];
	std::vector<int> t0(nbPairs), t1(nbPairs);
	std::vector<float> geom(8 * size_t(nbPairs));
	readAll(t0.data(), nbPairs);
	readAll(t1.data(), nbPairs);
	readAll(geom.data(), geom.size());
	std::vector<Shape> s0(nbPairs), s1(nbPairs);
	std::vector<const PxGeometry*> g0(nbPairs), g1(nbPairs);
	for(uint32_t k = 0; k < nbPairs; k++)
	{
		s0[k].set(t0[k], &geom[8 * size_t(k)]);
		s1[k].set(t1[k], &geom[8 * size_t(k) + 4]);
		g0[k] = &s0[k].any;
		g1[k] = &s1[k].any;
	}
	std::vector<PxCache> caches(nbPairs);
	memset(caches.data(), 0, caches.size() * sizeof(PxCache));
	CacheAllocator alloc;
	std::vector<PxTransform> p0(nbPairs), p1(nbPairs);
	for(uint32_t f = 0; f < nbFrames; f++)
	{
		alloc.nextFrame();
		readAll(p0.data(), nbPairs);
		readAll(p1.data(), nbPairs);
		Recorder rec;
		rec.perPair.resize(nbPairs);
		if(nbPairs && !PxGenerateContacts(g0.data(), g1.data(), p0.data(), p1.data(), caches.data(), nbPairs, rec, 0.04f, 0.01f, 1.0f, alloc))
			return 3;
		for(uint32_t k = 0; k < nbPairs; k++)
		{
			const uint32_t n = uint32_t(rec.perPair[k].size());
			fwrite(&n, 4, 1, stdout);
			for(const PxContactPoint& c : rec.perPair[k])
			{
				const float o[8] = {c.normal.x, c.normal.y, c.normal.z, c.separation, c.point.x, c.point.y, c.point.z, 0.0f};
				fwrite(o, 4, 8, stdout);
			}
		}
	}
	return 0;
}
