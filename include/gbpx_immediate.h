/*
 * gbpx_immediate.h -- the reference's immediate-mode entry points on the path,
 * exported by libgbpx_immediate.so under their own (C-linkage) names:
 *
 *   PxGenerateContacts               physx/include/PxImmediateMode.h:267
 *   PxConstructSolverBodiesTGS       physx/include/PxImmediateMode.h:592
 *   PxConstructStaticSolverBodyTGS   physx/include/PxImmediateMode.h:601
 *   PxBatchConstraintsTGS            physx/include/PxImmediateMode.h:620
 *   PxCreateContactConstraintsTGS    physx/include/PxImmediateMode.h:642
 *   PxCreateJointConstraintsTGS      physx/include/PxImmediateMode.h:659
 *   PxCreateJointConstraintsWithImmediateShadersTGS
 *                                    physx/include/PxImmediateMode.h:696
 *   PxSolveConstraintsTGS            physx/include/PxImmediateMode.h:716
 *   PxIntegrateSolverBodiesTGS       physx/include/PxImmediateMode.h:729
 *   PxConstructSolverBodies          physx/include/PxImmediateMode.h:111
 *   PxConstructStaticSolverBody      physx/include/PxImmediateMode.h:118
 *   PxBatchConstraints               physx/include/PxImmediateMode.h:137
 *   PxCreateContactConstraints       physx/include/PxImmediateMode.h:159
 *   PxSolveConstraints               physx/include/PxImmediateMode.h:231
 *   PxIntegrateSolverBodies          physx/include/PxImmediateMode.h:245
 *   PxGetBroadPhaseStaticFilterGroup     physx/include/PxBroadPhase.h:264
 *   PxGetBroadPhaseDynamicFilterGroup    physx/include/PxBroadPhase.h:278
 *   PxGetBroadPhaseKinematicFilterGroup  physx/include/PxBroadPhase.h:291
 *   PxCreateBroadPhase                   physx/include/PxBroadPhase.h:629
 *   PxCreateAABBManager                  physx/include/PxBroadPhase.h:796
 *   PxSetProfilerCallback                physx/include/foundation/PxFoundation.h:195
 *   PxGetProfilerCallback                physx/include/foundation/PxFoundation.h:190
 *
 * The reference declares these PX_C_EXPORT (extern "C"), so a program built
 * against the reference's headers links them from this library instead.  This
 * header restates, in namespace gbpx_px, the byte layouts those signatures use
 * (checked against the reference by tests/test_immediate_layout.py) and the
 * callback interfaces with the same virtual-function order.  It is for building
 * the library and its tests; a PhysX program keeps including PhysX's headers.
 * Do not include it together with PxImmediateMode.h.
 *
 * Behaviour: as the reference's persistent mode, a PxCache handed back keeps
 * the pair's contact manifold (for plane-capsule, plane-box, capsule-box and
 * box-box pairs, in memory from the PxCacheAllocator), and a contact
 * descriptor's frictionPtr / frictionCount handed back keep its friction
 * patches (memory from reserveFrictionData, broken flags written by
 * PxSolveConstraintsTGS); fresh caches and null friction pointers start over.
 * The bytes behind both are this library's own layout, opaque to the caller as
 * the reference's are.  The supported pair set is sphere / plane / capsule /
 * box, and convex cores; contact descriptors must use unit inverse-mass
 * scales, restDistance 0 and no maximum impulse, and articulations are not
 * supported (the functions return false, or do nothing, for input outside this
 * set).  The PGS functions start every frame from fresh friction data:
 * PxCreateContactConstraints hands back no friction patches (frictionPtr NULL,
 * frictionCount 0).  All arithmetic runs on the GPU through libgbpx.
 *
 * PxCreateBroadPhase accepts eABP and ePABP descriptors (the same pair sets;
 * the GPU sweep stands in for both) and returns NULL for other types, as the
 * reference does for descriptors it cannot serve.  Its PxBroadPhase gives the
 * reference ABP's created and lost pairs bit for bit, each list sorted by
 * (mID0, mID1); the update's continuation task is not used (eABP is
 * single-threaded in the reference too); getAllocator() hands out page-locked
 * host memory, from which bounds reach the device fastest.  PxCreateAABBManager
 * wraps such a broadphase with the reference's object bookkeeping (one manager
 * per broadphase).  A PxProfilerCallback installed with PxSetProfilerCallback
 * receives a zone for every stage of the library's work (the reference reports
 * its PX_PROFILE_ZONEs the same way).
 */
#ifndef GBPX_IMMEDIATE_H
#define GBPX_IMMEDIATE_H

#include <stddef.h>
#include <stdint.h>

namespace gbpx_px
{
struct PxVec3 { float x, y, z; };
struct PxQuat { float x, y, z, w; };
struct PxTransform { PxQuat q; PxVec3 p; };
struct PxMat33 { PxVec3 column0, column1, column2; };

// PxGeometryType: eSPHERE 0, ePLANE 1, eCAPSULE 2, eBOX 3
struct PxGeometry { int mType; float mTypePadding; };
struct PxSphereGeometry : PxGeometry { float radius; };
struct PxCapsuleGeometry : PxGeometry { float radius, halfHeight; };
struct PxBoxGeometry : PxGeometry { PxVec3 halfExtents; };
struct PxPlaneGeometry : PxGeometry {};
// PxConvexCoreGeometry (geometry/PxConvexCoreGeometry.h:227): PxConvexCore::Type,
// the core's data (MAX_CORE_SIZE = 6 floats: segment length; box extents;
// ellipsoid radii; cylinder / cone height, radius) and the margin
struct PxConvexCoreGeometry : PxGeometry { int mCoreType; uint8_t mCore[24]; float mMargin; };

struct alignas(16) PxContactPoint
{
	alignas(16) PxVec3 normal;
	float separation;
	alignas(16) PxVec3 point;
	float maxImpulse;
	alignas(16) PxVec3 targetVel;
	float staticFriction;
	uint8_t materialFlags;
	uint32_t internalFaceIndex1;
	float dynamicFriction;
	float restitution;
	float damping;
};

struct PxCache { uint8_t* mCachedData; uint16_t mCachedSize; uint8_t mPairData; uint8_t mManifoldFlags; };

class PxCacheAllocator
{
public:
	virtual uint8_t* allocateCacheData(const uint32_t byteSize) = 0;
	virtual ~PxCacheAllocator() {}
};

class PxContactRecorder
{
public:
	virtual bool recordContacts(const PxContactPoint* contactPoints, uint32_t nbContacts, uint32_t index) = 0;
	virtual ~PxContactRecorder() {}
};

struct alignas(16) PxRigidBodyData
{
	alignas(16) PxVec3 linearVelocity;
	float invMass;
	PxVec3 angularVelocity;
	float maxDepenetrationVelocity;
	PxVec3 invInertia;
	float maxContactImpulse;
	PxTransform body2World;
	float linearDamping, angularDamping, maxLinearVelocitySq, maxAngularVelocitySq;
	uint32_t pad;
};

struct alignas(16) PxTGSSolverBodyVel
{
	alignas(16) PxVec3 linearVelocity;
	uint16_t maxDynamicPartition;
	uint16_t nbStaticInteractions;
	PxVec3 angularVelocity;
	uint32_t partitionMask;
	PxVec3 deltaAngDt;
	float maxAngVel;
	PxVec3 deltaLinDt;
	uint16_t lockFlags;
	bool isKinematic;
	uint8_t pad;
};

struct PxTGSSolverBodyTxInertia
{
	PxQuat deltaBody2WorldQ;
	PxVec3 body2WorldP;
	PxMat33 sqrtInvInertia;
};

struct alignas(16) PxTGSSolverBodyData
{
	alignas(16) PxVec3 originalLinearVelocity;
	float maxContactImpulse;
	PxVec3 originalAngularVelocity;
	float penBiasClamp;
	float invMass;
	uint32_t nodeIndex;
	float reportThreshold;
	uint32_t pad;
};

// PxSolverBody (physx/include/solver/PxSolverDefs.h:54): the PGS solver's
// delta linear velocity and angular state
struct alignas(16) PxSolverBody
{
	alignas(16) PxVec3 linearVelocity;
	uint16_t maxSolverNormalProgress;
	uint16_t maxSolverFrictionProgress;
	PxVec3 angularState;
	uint32_t solverProgress;
};

// PxSolverBodyData (PxSolverDefs.h:74)
struct alignas(16) PxSolverBodyData
{
	alignas(16) PxVec3 linearVelocity;
	float invMass;
	PxVec3 angularVelocity;
	float reportThreshold;
	PxMat33 sqrtInvInertia;
	float penBiasClamp;
	uint32_t nodeIndex;
	float maxContactImpulse;
	PxTransform body2World;
	uint16_t pad;
};

struct PxConstraintBatchHeader { uint32_t startIndex; uint16_t stride; uint16_t constraintType; };

struct alignas(16) PxSolverConstraintDesc
{
	union { PxSolverBody* bodyA; PxTGSSolverBodyVel* tgsBodyA; void* articulationA; };
	union { PxSolverBody* bodyB; PxTGSSolverBodyVel* tgsBodyB; void* articulationB; };
	uint32_t bodyADataIndex, bodyBDataIndex;
	uint32_t linkIndexA, linkIndexB;
	uint8_t* constraint;
	void* writeBack;
	void* writeBackFriction;
	uint16_t progressA, progressB;
	uint16_t constraintLengthOver16;   // constraintType before preparation
};

struct alignas(16) PxConstraintInvMassScale { float linear0, angular0, linear1, angular1; };

// PxSolverConstraintPrepDescBase::BodyState
enum { eDYNAMIC_BODY = 1, eSTATIC_BODY = 2, eKINEMATIC_BODY = 4, eARTICULATION = 8 };

struct PxTGSSolverContactDesc
{
	PxConstraintInvMassScale invMassScales;
	PxSolverConstraintDesc* desc;
	const PxTGSSolverBodyVel* body0;
	const PxTGSSolverBodyVel* body1;
	const PxTGSSolverBodyTxInertia* body0TxI;
	const PxTGSSolverBodyTxInertia* body1TxI;
	const PxTGSSolverBodyData* bodyData0;
	const PxTGSSolverBodyData* bodyData1;
	PxTransform bodyFrame0;
	PxTransform bodyFrame1;
	int bodyState0;
	int bodyState1;
	void* shapeInteraction;
	uint8_t* frictionPtr;
	const PxContactPoint* contacts;
	uint32_t numContacts;
	uint8_t frictionCount;
	bool hasMaxImpulse;
	bool disableStrongFriction;
	bool hasForceThresholds;
	float restDistance;
	float maxCCDSeparation;
	float* contactForces;
	uint32_t startFrictionPatchIndex;
	uint32_t numFrictionPatches;
	uint32_t startContactPatchIndex;
	uint16_t numContactPatches;
	uint16_t axisConstraintCount;
	float maxImpulse;
	float torsionalPatchRadius;
	float minTorsionalPatchRadius;
	float offsetSlop;
};

// PxSolverContactDesc (PxSolverDefs.h:157,221): the PGS contact descriptor
struct PxSolverContactDesc
{
	PxConstraintInvMassScale invMassScales;
	PxSolverConstraintDesc* desc;
	const PxSolverBody* body0;
	const PxSolverBody* body1;
	const PxSolverBodyData* data0;
	const PxSolverBodyData* data1;
	PxTransform bodyFrame0;
	PxTransform bodyFrame1;
	int bodyState0;
	int bodyState1;
	void* shapeInteraction;
	uint8_t* frictionPtr;
	const PxContactPoint* contacts;
	uint32_t numContacts;
	uint8_t frictionCount;
	bool hasMaxImpulse;
	bool disableStrongFriction;
	bool hasForceThresholds;
	float restDistance;
	float maxCCDSeparation;
	float* contactForces;
	uint32_t startFrictionPatchIndex;
	uint32_t numFrictionPatches;
	uint32_t startContactPatchIndex;
	uint16_t numContactPatches;
	uint16_t axisConstraintCount;
	float offsetSlop;
};

// Px1DConstraint (physx/include/PxConstraintDesc.h:194): one joint row
struct alignas(16) Px1DConstraint
{
	PxVec3 linear0; float geometricError;
	PxVec3 angular0; float velocityTarget;
	PxVec3 linear1; float minImpulse;
	PxVec3 angular1; float maxImpulse;
	float mods[2];     // spring stiffness / damping, or restitution / bounce velocity threshold
	uint16_t flags;    // Px1DConstraintFlag
	uint16_t solveHint;
	uint32_t pad;
};

struct PxVec3p { PxVec3 v; uint32_t padding; };   // PxVec3Padded

// PxTGSSolverConstraintPrepDesc (physx/include/solver/PxSolverDefs.h:615-668)
struct PxTGSSolverConstraintPrepDesc
{
	PxConstraintInvMassScale invMassScales;
	PxSolverConstraintDesc* desc;
	const PxTGSSolverBodyVel* body0;
	const PxTGSSolverBodyVel* body1;
	const PxTGSSolverBodyTxInertia* body0TxI;
	const PxTGSSolverBodyTxInertia* body1TxI;
	const PxTGSSolverBodyData* bodyData0;
	const PxTGSSolverBodyData* bodyData1;
	PxTransform bodyFrame0;
	PxTransform bodyFrame1;
	int bodyState0;
	int bodyState1;
	void* writeback;   // Dy::ConstraintWriteback (linearImpulse, broken bit 31, angularImpulse, residual) or null
	Px1DConstraint* rows;
	uint32_t numRows;
	float linBreakForce, angBreakForce;
	float minResponseThreshold;
	bool disablePreprocessing;
	bool improvedSlerp;
	bool driveLimitsAreForces;
	bool extendedLimits;
	bool disableConstraint;
	PxVec3p body0WorldOffset;
	PxVec3p cA2w;
	PxVec3p cB2w;
};

// PxConstraintSolverPrep (PxConstraintDesc.h:278): a joint shader filling up to
// maxConstraints rows; returns the rows it wrote.
typedef uint32_t (*PxConstraintSolverPrep)(Px1DConstraint* constraints, PxVec3p& bodyAWorldOffset, uint32_t maxConstraints,
                                           PxConstraintInvMassScale& invMassScale, const void* constantBlock, const PxTransform& bodyAToWorld,
                                           const PxTransform& bodyBToWorld, bool useExtendedLimits, PxVec3p& cAtW, PxVec3p& cBtW);
// PxImmediateConstraint (PxImmediateMode.h:192)
struct PxImmediateConstraint
{
	PxConstraintSolverPrep prep;
	const void* constantBlock;
};

class PxConstraintAllocator
{
public:
	virtual uint8_t* reserveConstraintData(const uint32_t byteSize) = 0;
	virtual uint8_t* reserveFrictionData(const uint32_t byteSize) = 0;
	virtual ~PxConstraintAllocator() {}
};

// The reference's profiler callback (physx/include/foundation/PxProfiler.h:40-110),
// same virtual functions in the same order.
class PxProfilerCallback
{
public:
	virtual ~PxProfilerCallback() {}
	virtual void* zoneStart(const char* eventName, bool detached, uint64_t contextId) = 0;
	virtual void zoneEnd(void* profilerData, const char* eventName, bool detached, uint64_t contextId) = 0;
	virtual void recordData(int32_t value, const char* valueName, uint64_t contextId) { (void)value; (void)valueName; (void)contextId; }
	virtual void recordData(float value, const char* valueName, uint64_t contextId) { (void)value; (void)valueName; (void)contextId; }
	virtual void recordFrame(const char* name, uint64_t contextId) { (void)name; (void)contextId; }
};

// ---- low- and high-level broadphase (physx/include/PxBroadPhase.h) ----
struct PxBounds3 { PxVec3 minimum, maximum; };
struct PxBroadPhaseType { enum Enum { eSAP, eMBP, eABP, ePABP, eGPU, eLAST }; };
class PxBaseTask;
class PxCudaContextManager;
class PxBroadPhaseRegions;   // only MBP has regions: never returned here

class PxAllocatorCallback   // physx/include/foundation/PxAllocatorCallback.h
{
public:
	virtual ~PxAllocatorCallback() {}
	virtual void* allocate(size_t size, const char* typeName, const char* filename, int line) = 0;
	virtual void deallocate(void* ptr) = 0;
};

struct PxBroadPhaseCaps { uint32_t mMaxNbRegions; };

class PxBroadPhaseDesc
{
public:
	PxBroadPhaseDesc(PxBroadPhaseType::Enum type = PxBroadPhaseType::eLAST)
	    : mType(type), mContextID(0), mContextManager(nullptr), mFoundLostPairsCapacity(256 * 1024), mDiscardStaticVsKinematic(false),
	      mDiscardKinematicVsKinematic(false)
	{
	}
	PxBroadPhaseType::Enum mType;
	uint64_t mContextID;
	PxCudaContextManager* mContextManager;
	uint32_t mFoundLostPairsCapacity;
	bool mDiscardStaticVsKinematic;
	bool mDiscardKinematicVsKinematic;
};

typedef uint32_t PxBpIndex;
typedef uint32_t PxBpFilterGroup;

class PxBroadPhaseUpdateData
{
public:
	PxBroadPhaseUpdateData(const PxBpIndex* created, uint32_t nbCreated, const PxBpIndex* updated, uint32_t nbUpdated, const PxBpIndex* removed,
	                       uint32_t nbRemoved, const PxBounds3* bounds, const PxBpFilterGroup* groups, const float* distances, uint32_t capacity)
	    : mCreated(created), mNbCreated(nbCreated), mUpdated(updated), mNbUpdated(nbUpdated), mRemoved(removed), mNbRemoved(nbRemoved),
	      mBounds(bounds), mGroups(groups), mDistances(distances), mCapacity(capacity)
	{
	}
	const PxBpIndex* mCreated;
	const uint32_t mNbCreated;
	const PxBpIndex* mUpdated;
	const uint32_t mNbUpdated;
	const PxBpIndex* mRemoved;
	const uint32_t mNbRemoved;
	const PxBounds3* mBounds;
	const PxBpFilterGroup* mGroups;
	const float* mDistances;
	const uint32_t mCapacity;
};

struct PxBroadPhasePair { PxBpIndex mID0, mID1; };

struct PxBroadPhaseResults
{
	PxBroadPhaseResults() : mNbCreatedPairs(0), mCreatedPairs(nullptr), mNbDeletedPairs(0), mDeletedPairs(nullptr) {}
	uint32_t mNbCreatedPairs;
	const PxBroadPhasePair* mCreatedPairs;
	uint32_t mNbDeletedPairs;
	const PxBroadPhasePair* mDeletedPairs;
};

// Same virtual functions, in the same order, as the reference's PxBroadPhase
// (physx/include/PxBroadPhase.h:492-618): a caller's virtual calls land in the
// same vtable slots.
class PxBroadPhase
{
protected:
	PxBroadPhase() {}
	virtual ~PxBroadPhase() {}
public:
	virtual void release() = 0;
	virtual PxBroadPhaseType::Enum getType() const = 0;
	virtual void getCaps(PxBroadPhaseCaps& caps) const = 0;
	virtual PxBroadPhaseRegions* getRegions() = 0;
	virtual PxAllocatorCallback* getAllocator() = 0;
	virtual uint64_t getContextID() const = 0;
	virtual void setScratchBlock(void* scratchBlock, uint32_t size) = 0;
	virtual void update(const PxBroadPhaseUpdateData& updateData, PxBaseTask* continuation = nullptr) = 0;
	virtual void fetchResults(PxBroadPhaseResults& results) = 0;
	void updateAndFetchResults(PxBroadPhaseResults& results, const PxBroadPhaseUpdateData& updateData)
	{
		update(updateData);
		fetchResults(results);
	}
};

// The reference's PxAABBManager (physx/include/PxBroadPhase.h:642-796), same order.
class PxAABBManager
{
protected:
	PxAABBManager() {}
	virtual ~PxAABBManager() {}
public:
	virtual void release() = 0;
	virtual PxBroadPhase& getBroadPhase() = 0;
	virtual const PxBounds3* getBounds() const = 0;
	virtual const float* getDistances() const = 0;
	virtual const PxBpFilterGroup* getGroups() const = 0;
	virtual uint32_t getCapacity() const = 0;
	virtual void addObject(PxBpIndex index, const PxBounds3& bounds, PxBpFilterGroup group, float distance = 0.0f) = 0;
	virtual void removeObject(PxBpIndex index) = 0;
	virtual void updateObject(PxBpIndex index, const PxBounds3* bounds = nullptr, const float* distance = nullptr) = 0;
	virtual void update(PxBaseTask* continuation = nullptr) = 0;
	virtual void fetchResults(PxBroadPhaseResults& results) = 0;
	void updateAndFetchResults(PxBroadPhaseResults& results)
	{
		update();
		fetchResults(results);
	}
};
} // namespace gbpx_px

extern "C" {
bool PxGenerateContacts(const gbpx_px::PxGeometry* const* geom0, const gbpx_px::PxGeometry* const* geom1, const gbpx_px::PxTransform* pose0,
                        const gbpx_px::PxTransform* pose1, gbpx_px::PxCache* contactCache, uint32_t nbPairs,
                        gbpx_px::PxContactRecorder& contactRecorder, float contactDistance, float meshContactMargin, float toleranceLength,
                        gbpx_px::PxCacheAllocator& allocator);
void PxConstructSolverBodiesTGS(const gbpx_px::PxRigidBodyData* inRigidData, gbpx_px::PxTGSSolverBodyVel* outSolverBodyVel,
                                gbpx_px::PxTGSSolverBodyTxInertia* outSolverBodyTxInertia, gbpx_px::PxTGSSolverBodyData* outSolverBodyData,
                                uint32_t nbBodies, const gbpx_px::PxVec3& gravity, float dt, bool gyroscopicForces);
void PxConstructStaticSolverBodyTGS(const gbpx_px::PxTransform& globalPose, gbpx_px::PxTGSSolverBodyVel& solverBodyVel,
                                    gbpx_px::PxTGSSolverBodyTxInertia& solverBodyTxInertia, gbpx_px::PxTGSSolverBodyData& solverBodyData);
uint32_t PxBatchConstraintsTGS(const gbpx_px::PxSolverConstraintDesc* solverConstraintDescs, uint32_t nbConstraints,
                               gbpx_px::PxTGSSolverBodyVel* solverBodies, uint32_t nbBodies, gbpx_px::PxConstraintBatchHeader* outBatchHeaders,
                               gbpx_px::PxSolverConstraintDesc* outOrderedConstraintDescs, void** articulations, uint32_t nbArticulations);
bool PxCreateContactConstraintsTGS(gbpx_px::PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, gbpx_px::PxTGSSolverContactDesc* contactDescs,
                                   gbpx_px::PxConstraintAllocator& allocator, float invDt, float invTotalDt, float bounceThreshold,
                                   float frictionOffsetThreshold, float correlationDistance);
bool PxCreateJointConstraintsTGS(gbpx_px::PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, gbpx_px::PxTGSSolverConstraintPrepDesc* jointDescs,
                                 gbpx_px::PxConstraintAllocator& allocator, float dt, float totalDt, float invDt, float invTotalDt, float lengthScale);
bool PxCreateJointConstraintsWithImmediateShadersTGS(gbpx_px::PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders,
                                                     gbpx_px::PxImmediateConstraint* constraints,
                                                     gbpx_px::PxTGSSolverConstraintPrepDesc* jointDescs, gbpx_px::PxConstraintAllocator& allocator,
                                                     float dt, float totalDt, float invDt, float invTotalDt, float lengthScale);
void PxSolveConstraintsTGS(const gbpx_px::PxConstraintBatchHeader* batchHeaders, uint32_t nbBatchHeaders,
                           const gbpx_px::PxSolverConstraintDesc* solverConstraintDescs, gbpx_px::PxTGSSolverBodyVel* solverBodies,
                           gbpx_px::PxTGSSolverBodyTxInertia* txInertias, uint32_t nbSolverBodies, uint32_t nbPositionIterations,
                           uint32_t nbVelocityIterations, float dt, float invDt, uint32_t nbSolverArticulations, void** solverArticulations,
                           void* Z, void* deltaV);
void PxIntegrateSolverBodiesTGS(gbpx_px::PxTGSSolverBodyVel* solverBody, const gbpx_px::PxTGSSolverBodyTxInertia* txInertia,
                                gbpx_px::PxTransform* poses, uint32_t nbBodiesToIntegrate, float dt);
void PxConstructSolverBodies(const gbpx_px::PxRigidBodyData* inRigidData, gbpx_px::PxSolverBodyData* outSolverBodyData, uint32_t nbBodies,
                             const gbpx_px::PxVec3& gravity, float dt, bool gyroscopicForces);
void PxConstructStaticSolverBody(const gbpx_px::PxTransform& globalPose, gbpx_px::PxSolverBodyData& solverBodyData);
uint32_t PxBatchConstraints(const gbpx_px::PxSolverConstraintDesc* solverConstraintDescs, uint32_t nbConstraints, gbpx_px::PxSolverBody* solverBodies,
                            uint32_t nbBodies, gbpx_px::PxConstraintBatchHeader* outBatchHeaders,
                            gbpx_px::PxSolverConstraintDesc* outOrderedConstraintDescs, void** articulations, uint32_t nbArticulations);
bool PxCreateContactConstraints(gbpx_px::PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, gbpx_px::PxSolverContactDesc* contactDescs,
                                gbpx_px::PxConstraintAllocator& allocator, float invDt, float bounceThreshold, float frictionOffsetThreshold,
                                float correlationDistance, void* ZV);
void PxSolveConstraints(const gbpx_px::PxConstraintBatchHeader* batchHeaders, uint32_t nbBatchHeaders,
                        const gbpx_px::PxSolverConstraintDesc* solverConstraintDescs, const gbpx_px::PxSolverBody* solverBodies,
                        gbpx_px::PxVec3* linearMotionVelocity, gbpx_px::PxVec3* angularMotionVelocity, uint32_t nbSolverBodies,
                        uint32_t nbPositionIterations, uint32_t nbVelocityIterations, float dt, float invDt, uint32_t nbSolverArticulations,
                        void** solverArticulations, void* Z, void* deltaV);
void PxIntegrateSolverBodies(gbpx_px::PxSolverBodyData* solverBodyData, gbpx_px::PxSolverBody* solverBody, gbpx_px::PxVec3* linearMotionVelocity,
                             gbpx_px::PxVec3* angularMotionState, uint32_t nbBodiesToIntegrate, float dt);
gbpx_px::PxBpFilterGroup PxGetBroadPhaseStaticFilterGroup();
gbpx_px::PxBpFilterGroup PxGetBroadPhaseDynamicFilterGroup(uint32_t id);
gbpx_px::PxBpFilterGroup PxGetBroadPhaseKinematicFilterGroup(uint32_t id);
gbpx_px::PxBroadPhase* PxCreateBroadPhase(const gbpx_px::PxBroadPhaseDesc& desc);
gbpx_px::PxAABBManager* PxCreateAABBManager(gbpx_px::PxBroadPhase& broadphase);
void PxSetProfilerCallback(gbpx_px::PxProfilerCallback* profiler);
gbpx_px::PxProfilerCallback* PxGetProfilerCallback();
}

#endif /* GBPX_IMMEDIATE_H */
