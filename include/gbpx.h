/*
 * gbpx.h -- C ABI of the GB300-native rigid-body immediate-mode step.
 *
 * Plain C: pointers and sizes only.  Every entry point returns a status code
 * (GBPX_OK == 0, negative on error) unless documented otherwise.  Host arrays
 * use the reference's layouts; the reference interface each function replaces
 * is cited beside it (paths relative to the PhysX source tree).
 *
 * Layout conventions:
 *   bounds   PxBounds3: 6 floats per handle (min x y z, max x y z)
 *   pose     PxTransform: 7 floats (qx qy qz qw px py pz)
 *   pair     PxBroadPhasePair: 2 uint32 (id0 < id1)
 */
#ifndef GBPX_H
#define GBPX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBPX_OK 0
#define GBPX_ERR_INVALID (-1)
#define GBPX_ERR_CUDA (-2)
#define GBPX_ERR_CAPACITY (-3)
#define GBPX_ERR_NOMEM (-4)
#define GBPX_ERR_STATE (-5)
#define GBPX_ERR_BUDGET (-6)
#define GBPX_ERR_TIMEOUT (-7)

/* ------------------------------------------------------------------- runtime */
int gbpx_device_count(int* out);
int gbpx_device_info(int device, char* name, int nameBytes, int* smCount, int* computeCapability);
int gbpx_device_synchronize(void);

/* ---------------------------------------------------------------- broadphase
 * ABP-compatible broadphase.  Replaces:
 *   PxCreateBroadPhase(PxBroadPhaseDesc(eABP))   physx/include/PxBroadPhase.h:629
 *   PxBroadPhase::release                        physx/include/PxBroadPhase.h:505
 *   PxBroadPhase::update(data, continuation)     physx/include/PxBroadPhase.h:576
 *   PxBroadPhase::fetchResults(results)          physx/include/PxBroadPhase.h:588
 * Created/lost pair sets are bit-exact with the reference ABP; each list is
 * returned sorted by (id0, id1).  The returned arrays stay owned by the
 * broadphase until the next update (as in the reference). */
int gbpx_bp_create(int discardStaticVsKinematic, int discardKinematicVsKinematic, void** outBroadPhase);
void gbpx_bp_release(void* broadPhase);
/* PxBroadPhaseUpdateData (physx/include/PxBroadPhase.h:312): bounds, groups and
 * distances are persistent user arrays indexed by handle, `capacity` entries. */
int gbpx_bp_update(void* broadPhase, const uint32_t* created, uint32_t nbCreated, const uint32_t* updated, uint32_t nbUpdated,
                   const uint32_t* removed, uint32_t nbRemoved, const float* bounds, const uint32_t* groups,
                   const float* distances, uint32_t capacity);
int gbpx_bp_fetch_results(void* broadPhase, const uint32_t** createdPairs, uint32_t* nbCreated, const uint32_t** lostPairs,
                          uint32_t* nbLost);
/* live boxes, updated boxes, found pairs, active pairs of the last update */
int gbpx_bp_stats(void* broadPhase, uint64_t* out4);
/* PxGetBroadPhaseStaticFilterGroup / DynamicFilterGroup / KinematicFilterGroup
 * (physx/include/PxBroadPhase.h:264-291) */
uint32_t gbpx_bp_static_filter_group(void);
uint32_t gbpx_bp_dynamic_filter_group(uint32_t id);
uint32_t gbpx_bp_kinematic_filter_group(uint32_t id);

/* -------------------------------------------------------------- narrowphase
 * immediate::PxGenerateContacts (physx/include/PxImmediateMode.h:267) for
 * sphere / plane / capsule / box pairs with a fresh PxCache per pair.
 * type: PxGeometryType (0 sphere, 1 plane, 2 capsule, 3 box); geom: 4 floats
 * (sphere r | capsule r, halfHeight | box hx, hy, hz); pose: PxTransform.
 * outContacts: nbPairs x maxPerPair x 8 floats (normal xyz, separation,
 * point xyz, 0); outCounts: contacts per pair.  The normal points along the
 * direction shape0 must move, as PxContactPoint (geomutils/PxContactPoint.h:39). */
int gbpx_generate_contacts(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0,
                           const float* pose1, uint32_t nbPairs, float contactDistance, float meshContactMargin,
                           float toleranceLength, float* outContacts, uint32_t maxPerPair, uint32_t* outCounts);

#ifdef __cplusplus
}
#endif

#endif /* GBPX_H */
