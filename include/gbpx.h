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

#include <stddef.h>
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
int gbpx_set_device(int device);
/* profiler range: a profiler started with capture off records only the
 * kernels launched between these calls */
int gbpx_profiler_start(void);
int gbpx_profiler_stop(void);
/* Profiler zones (the reference's PX_PROFILE_ZONE, physx/include/common/PxProfileZone.h,
 * reported to a PxProfilerCallback, physx/include/foundation/PxProfiler.h:58-69):
 * every stage of the library's calls is an NVTX range and, once installed here,
 * a zoneStart / zoneEnd pair on these callbacks (zoneEnd gets zoneStart's return
 * value).  Both null removes them; install while no library call runs. */
typedef void* (*gbpx_zone_start_fn)(const char* name, int detached, uint64_t contextId, void* user);
typedef void (*gbpx_zone_end_fn)(void* data, const char* name, int detached, uint64_t contextId, void* user);
int gbpx_set_profiler_callback(gbpx_zone_start_fn zoneStart, gbpx_zone_end_fn zoneEnd, void* user);

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
/* sweep kernels of the following updates: 1 = shared-memory tiled (default),
 * 0 = one warp per updated box / one thread per other box; both find the same pairs */
int gbpx_bp_set_sweep(void* broadPhase, int tiled);
/* timing of the last update + fetchResults: out2[0] host milliseconds staging the
 * user's arrays, out2[1] device milliseconds from the first upload to the results
 * in host memory (CUDA events) */
int gbpx_bp_timing(void* broadPhase, float* out2);
/* PxGetBroadPhaseStaticFilterGroup / DynamicFilterGroup / KinematicFilterGroup
 * (physx/include/PxBroadPhase.h:264-291) */
uint32_t gbpx_bp_static_filter_group(void);
uint32_t gbpx_bp_dynamic_filter_group(uint32_t id);
uint32_t gbpx_bp_kinematic_filter_group(uint32_t id);

/* -------------------------------------------------------------- narrowphase
 * immediate::PxGenerateContacts (physx/include/PxImmediateMode.h:267) for
 * sphere / plane / capsule / box / convex-core pairs with a fresh PxCache per
 * pair.  type: PxGeometryType (0 sphere, 1 plane, 2 capsule, 3 box, 4 convex
 * core) in the low byte; for a convex core (PxConvexCoreGeometry,
 * physx/include/geometry/PxConvexCoreGeometry.h) bits 8..15 hold its
 * PxConvexCore::Type (0 point, 1 segment, 2 box, 3 ellipsoid, 4 cylinder,
 * 5 cone), so type = 4 | coreType << 8.  geom: 4 floats (sphere r | capsule r,
 * halfHeight | box hx, hy, hz | convex core: the core's floats — segment
 * length; box extents xyz; ellipsoid radii xyz; cylinder or cone height,
 * radius — then the margin in geom[3]); pose: PxTransform.  Convex-core pairs
 * give at most 4 contacts (GuConvexSupport.h MAX_CONVEX_CONTACTS) and keep no
 * cache.
 * outContacts: nbPairs x maxPerPair x 8 floats (normal xyz, separation,
 * point xyz, 0); outCounts: contacts per pair.  The normal points along the
 * direction shape0 must move, as PxContactPoint (geomutils/PxContactPoint.h:39). */
int gbpx_generate_contacts(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0,
                           const float* pose1, uint32_t nbPairs, float contactDistance, float meshContactMargin,
                           float toleranceLength, float* outContacts, uint32_t maxPerPair, uint32_t* outCounts);
/* The same with persistent caches, as PxGenerateContacts with a PxCache per pair
 * kept between calls: manifolds (nbPairs x 288 bytes, host memory, zero for a
 * fresh cache) carries the contact manifold of the plane-capsule, plane-box,
 * capsule-box and box-box pairs (gEnablePCMCaching,
 * physx/source/lowlevel/software/src/PxsContext.cpp:89) from one call to the
 * next: refresh and invalidation (geomutils/src/pcm/GuPersistentContactManifold.h:190-271),
 * incremental points and the GJK warm start.  It is read and updated. */
int gbpx_generate_contacts_cached(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0,
                                  const float* pose1, uint32_t nbPairs, float contactDistance, float meshContactMargin,
                                  float toleranceLength, float* outContacts, uint32_t maxPerPair, uint32_t* outCounts, void* manifolds);

/* No counterpart in the reference: the same contact generation for callers
 * that may not allocate device memory during the call (a cudaMalloc or
 * cudaFree in a frame loop synchronises the device and fragments the pool;
 * some host applications own all device memory through their own pools).
 * Inputs and outputs are the caller's device arrays (layouts as above;
 * dOutContacts holds 4 contacts x 8 floats per pair and is 16-byte aligned),
 * the work is enqueued on `stream` (a cudaStream_t, NULL = default stream).
 * Caches are fresh (no PxCache is read or written).  Geometry types must be
 * the ones above: the device arrays are not checked on the host, and other
 * values give undefined contacts.
 * Scratch is a fixed 1 MiB device array, so nbPairs <= 262144
 * (GBPX_ERR_CAPACITY above).  The scratch is shared by every call on a
 * device: calls that may overlap must be serialised by the caller.  The first
 * call on a device looks the scratch address up. */
int gbpx_generate_contacts_device_noalloc(const int* dType0, const float* dGeom0, const int* dType1, const float* dGeom1,
                                          const float* dPose0, const float* dPose1, uint32_t nbPairs, float contactDistance,
                                          float toleranceLength, float* dOutContacts, uint32_t* dOutCounts, void* stream);

/* ---------------------------------------------------------------------- TGS
 * Rigid bodies use PxRigidBodyData (physx/include/PxImmediateMode.h:68, 96 B).
 *
 * PxConstructSolverBodiesTGS (physx/include/PxImmediateMode.h:592): writes
 * PxTGSSolverBodyVel (64 B), PxTGSSolverBodyTxInertia (64 B) and
 * PxTGSSolverBodyData (48 B) records per body. */
int gbpx_construct_solver_bodies_tgs(const void* rigidBodies, uint32_t nbBodies, const float* gravity, float dt, void* outBodyVel,
                                     void* outTxInertia, void* outBodyData);
/* PxBatchConstraintsTGS (physx/include/PxImmediateMode.h:620): constraint i
 * joins bodies bodyA[i], bodyB[i]; indices >= nbDynamic are static/kinematic.
 * Returns the header count; headers are (start, stride), outOrder lists the
 * caller's constraint indices in solve order. */
uint32_t gbpx_batch_constraints_tgs(const uint32_t* bodyA, const uint32_t* bodyB, uint32_t nbConstraints, uint32_t nbDynamic,
                                    uint32_t nbStatic, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder);
/* One TGS step from given contacts: PxConstructSolverBodiesTGS,
 * PxBatchConstraintsTGS, PxCreateContactConstraintsTGS (:642),
 * PxSolveConstraintsTGS (:716) and PxIntegrateSolverBodiesTGS (:729) with
 * the immediate-mode settings (fresh friction data, unit mass scales).
 * contacts: 8 floats each (normal, separation, point, 0), <= 4 per constraint;
 * material: (static friction, dynamic friction, restitution) per constraint.
 * outVelocity: linear + world angular (6 floats) per dynamic body; outPose:
 * PxTransform per dynamic body. */
int gbpx_tgs_solve(const void* rigidBodies, uint32_t nbDynamic, const float* staticPoses, uint32_t nbStatic, const uint32_t* bodyA,
                   const uint32_t* bodyB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                   const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPositionIterations,
                   uint32_t nbVelocityIterations, float bounceThreshold, float frictionOffsetThreshold, float correlationDistance,
                   float* outVelocity, float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outOrder,
                   uint32_t* outNbHeaders);

/* Split-phase TGS on solver bodies in the reference's layouts, the stages a
 * caller of physx::immediate drives itself (used by libgbpx_immediate.so):
 *   PxConstructStaticSolverBodyTGS   physx/include/PxImmediateMode.h:601
 *   PxCreateContactConstraintsTGS    physx/include/PxImmediateMode.h:642
 *   PxSolveConstraintsTGS            physx/include/PxImmediateMode.h:716
 *   PxIntegrateSolverBodiesTGS       physx/include/PxImmediateMode.h:729
 * Constraint rows are this build's own format, gbpx_constraint_row_stride()
 * bytes per constraint at most. */
uint32_t gbpx_constraint_row_stride(void);
/* The integrator's sine and cosine of the half angle (no reference
 * counterpart; numerics check): for each of n angles (host array) out gets 4
 * floats: the sine and cosine the solver uses, and double-precision sin / cos
 * rounded to float. */
int gbpx_eval_sincos_angle(const float* x, uint32_t n, float* out);
int gbpx_construct_static_solver_bodies_tgs(const float* poses, uint32_t n, void* outVel, void* outTxI, void* outData);
/* one descriptor per constraint: both bodies' records (64/64/48 B), frames
 * (PxTransform) and PxContactPoints (80 B); laneFlags[k] (null: all per-pair):
 * bit 0 = lane of a stride-4 header on the reference's 4-wide block path
 * (createFinalizeSolverContacts4Step, lowleveldynamics/src/DyTGSContactPrepBlock.cpp:1398),
 * bit 1 = that header has a dynamic body B, bit 2 = bodyBDataIndex is 0;
 * frictionIn / frictionOut (null: fresh friction data, none kept): per
 * constraint a 464-byte record (uint32 count, 12 bytes padding, 4 friction
 * patches of 112 bytes), the patches the constraint left last frame
 * (frictionPtr / frictionCount of PxTGSSolverContactDesc) and the ones it
 * leaves this frame; invDt = nbPositionIterations / dt, invTotalDt = 1 / dt.
 * Rows to outRows + k * stride, used bytes to outRowBytes[k]. */
int gbpx_create_contact_constraints_tgs(uint32_t n, const void* vel0, const void* vel1, const void* txI0, const void* txI1, const void* data0,
                                        const void* data1, const float* frame0, const float* frame1, const uint32_t* contactStart,
                                        const uint32_t* contactCount, const void* contactPoints, uint32_t nbPoints, const uint8_t* laneFlags,
                                        const void* frictionIn, void* frictionOut, float invDt, float invTotalDt, float bounceThreshold,
                                        float frictionOffsetThreshold, float correlationDistance, void* outRows, uint32_t* outRowBytes);
/* rows (n x stride, solve order, impulses updated in place); constraint k joins
 * bodyA[k], bodyB[k]; constraints in [waveEnds[w-1], waveEnds[w]) touch distinct
 * bodies; the first nbIntegrate bodies are integrated every position iteration;
 * dt = time step / nbPositionIterations; outBroken (null: not wanted): per
 * constraint, bit p set when patch p's friction was clamped in the last
 * iteration, which marks the friction patch it wrote broken. */
int gbpx_solve_constraints_tgs(void* rows, const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, const uint32_t* waveEnds, uint32_t nbWaves,
                               void* bodyVel, void* bodyTxI, uint32_t nbBodies, uint32_t nbIntegrate, uint32_t nbPos, uint32_t nbVel, float dt,
                               uint32_t* outBroken);
int gbpx_integrate_solver_bodies_tgs(void* bodyVel, const void* bodyTxI, float* poses, uint32_t n);
/* PxBatchConstraintsTGS over a list mixing contacts and joints: kind[i] = the
 * constraint's PxSolverConstraintDesc type (0 contact, 1 joint); a header only
 * joins consecutive constraints of one type (createHeaders,
 * physx/source/immediatemode/src/NpImmediateMode.cpp:159). */
uint32_t gbpx_batch_typed_constraints_tgs(const uint32_t* bodyA, const uint32_t* bodyB, const uint8_t* kind, uint32_t nbConstraints,
                                          uint32_t nbDynamic, uint32_t nbStatic, uint32_t* outHeaderStart, uint32_t* outHeaderStride,
                                          uint32_t* outOrder);

/* ---------------------------------------------------------------------- PGS
 * One immediate-mode PGS frame (PxConstructSolverBodies,
 * PxConstructStaticSolverBody, PxBatchConstraints, PxCreateContactConstraints,
 * PxSolveConstraints, PxIntegrateSolverBodies: physx/include/PxImmediateMode.h;
 * physx/source/immediatemode/src/NpImmediateMode.cpp:55-78,269,292,552) from
 * given contacts.  Inputs as gbpx_tgs_solve (body A of every constraint
 * dynamic, 1..4 contacts per constraint); batch != 0 batches with
 * PxBatchConstraints's rule, else one header per constraint in the caller's
 * order.  Headers of stride 4 with at most 64 contacts take the reference's
 * 4-wide block path.  Outputs: per dynamic body the linear and angular
 * velocity (6 floats) and pose (7 floats) after integration; headers (start,
 * stride, constraintType: DY_SC_TYPE_RB_CONTACT 1, _STATIC_CONTACT 5,
 * _BLOCK_RB_CONTACT 6, _BLOCK_STATIC_RB_CONTACT 7) and the constraint order
 * (arrays of at least nbConstraints); outForces (may be NULL): per contact the
 * normal impulse the last velocity iteration writes back, in the
 * constraint's row order (as PxSolverContactDesc::contactForces receives it). */
int gbpx_pgs_solve(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* pairA,
                   const uint32_t* pairB, uint32_t nbConstraints, const uint32_t* contactStart, const uint32_t* contactCount,
                   const float* contacts, const float* material, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel,
                   float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, int batch, float* outVel,
                   float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outHeaderType, uint32_t* outOrder,
                   float* outForces, uint32_t* outNbHeaders);

/* The PGS stages on solver bodies in the reference's layouts (PxSolverBodyData
 * 112 B, PxSolverBody 32 B), for the physx::immediate drop-in: records of
 * gbpx_pgs_record_bytes() each. */
uint32_t gbpx_pgs_record_bytes(void);
/* PxConstructSolverBodies (rigid: nb PxRigidBodyData) or, with rigid NULL,
 * PxConstructStaticSolverBody (poses: nb PxTransform) into nb PxSolverBodyData. */
int gbpx_construct_solver_bodies_pgs(const void* rigid, const float* poses, uint32_t nb, const float* gravity, float dt, void* outData);
/* PxCreateContactConstraints, one contact descriptor per constraint: both
 * bodies' PxSolverBodyData, the body frames, contactPoints[contactStart[k] ..
 * +contactCount[k]] (PxContactPoint, 80 B, 1..4 per constraint).  laneFlags[k]:
 * bit 0 a lane of a stride-4 header on the 4-wide block path, bit 1 that header
 * has a dynamic body B, bit 2 the block solve stores body B (bodyBDataIndex != 0),
 * bit 3 the per-pair solve treats body B as dynamic (DY_SC_TYPE_RB_CONTACT). */
int gbpx_create_contact_constraints_pgs(uint32_t n, const void* data0, const void* data1, const float* frame0, const float* frame1,
                                        const uint32_t* contactStart, const uint32_t* contactCount, const void* contactPoints,
                                        uint32_t nbPoints, const uint8_t* laneFlags, float invDt, float bounceThreshold,
                                        float frictionOffsetThreshold, void* outRecords);
/* PxSolveConstraints over n records in solve order (updated in place), record k
 * joining bodies bodyA[k], bodyB[k] (>= nbBodies: a zero body outside the
 * caller's array); wave w = records [waveEnds[w-1], waveEnds[w]) touching
 * distinct bodies.  bodies: nbBodies PxSolverBody (zeroed), updated in place;
 * outMotionLin / outMotionAng: the velocities after the position iterations. */
int gbpx_solve_constraints_pgs(void* records, const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, const uint32_t* waveEnds,
                               uint32_t nbWaves, void* bodies, uint32_t nbBodies, uint32_t nbPos, uint32_t nbVel, float* outMotionLin,
                               float* outMotionAng);
/* PxIntegrateSolverBodies (integrateCore): data (PxSolverBodyData) updated in
 * place, the motion velocities replaced by those integrated with. */
int gbpx_integrate_solver_bodies_pgs(void* data, const void* bodies, float* motionLin, float* motionAng, uint32_t n, float dt);

/* -------------------------------------------------------- joints (1D constraints)
 * Replace, on the rigid-body path:
 *   PxCreateJointConstraintsTGS      physx/include/PxImmediateMode.h:659
 *     (NpImmediateMode.cpp:1480: per-pair setupSolverConstraintStep, or the
 *     4-wide setupSolverConstraintStep4 for a header of stride 4 whose joints
 *     all have rows)
 *   the joint half of PxSolveConstraintsTGS (solve1DStep / solve1DStep4,
 *     conclude, write-back)
 * Rows are the caller's Px1DConstraint (80 bytes, <= 12 per joint).  Per joint
 * 20 parameter floats: PxConstraintInvMassScale (linear0, angular0, linear1,
 * angular1), cA2w, cB2w, body0WorldOffset, linBreakForce, angBreakForce,
 * minResponseThreshold, flags (a float holding 1 disablePreprocessing |
 * 4 driveLimitsAreForces; 2 improvedSlerp is refused with GBPX_ERR_INVALID),
 * 3 unused.  Joint records are this build's own format,
 * gbpx_joint_record_bytes() each. */
uint32_t gbpx_joint_record_bytes(void);
/* One joint per entry: the bodies' records in the reference's layouts, frames
 * (PxTransform), rows[rowStart[k] .. +rowCount[k]], params + 20 k, block[k] = 1
 * for a lane of a 4-wide header.  Times as the immediate-mode snippet passes
 * them to PxCreateJointConstraintsTGS: stepDt, simDt, 1/stepDt, 1/simDt, lengthScale. */
int gbpx_create_joint_constraints_tgs(uint32_t n, const void* vel0, const void* vel1, const void* txI0, const void* txI1, const void* data0,
                                      const void* data1, const float* frame0, const float* frame1, const uint32_t* rowStart, const uint32_t* rowCount,
                                      const void* rows, uint32_t nbRows, const float* params, const uint8_t* block, float stepDt, float simDt,
                                      float recipStepDt, float recipSimDt, float lengthScale, void* outRecords);
/* PxSolveConstraintsTGS over contacts and joints: wave w solves contacts
 * [waveEnds[w-1], waveEnds[w]) and joints [jointWaveEnds[w-1], jointWaveEnds[w])
 * (distinct dynamic bodies); otherwise as gbpx_solve_constraints_tgs.
 * outJointForce / outJointBroken (null: not wanted): per joint the write-back
 * impulse (linear, angular: 6 floats) and broken flag. */
int gbpx_solve_constraints_joints_tgs(void* rows, const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, const uint32_t* waveEnds,
                                      void* jointRecords, const uint32_t* jointA, const uint32_t* jointB, uint32_t nbJoints,
                                      const uint32_t* jointWaveEnds, uint32_t nbWaves, void* bodyVel, void* bodyTxI, uint32_t nbBodies,
                                      uint32_t nbIntegrate, uint32_t nbPos, uint32_t nbVel, float dt, uint32_t* outBroken, float* outJointForce,
                                      uint32_t* outJointBroken);
/* One immediate-mode TGS frame of joints, the snippet's joint sequence
 * (SnippetImmediateMode.cpp:838-1061) with the caller's rows: construct
 * bodies, PxBatchConstraintsTGS over the joints (batchJoints = 0: one header of
 * stride 1 per joint in input order), PxCreateJointConstraintsTGS per header,
 * nbPos + nbVel iterations, PxIntegrateSolverBodiesTGS.  Outputs: velocity
 * (linear, world angular) and pose per dynamic body, headers (start, stride,
 * DY_SC_TYPE_RB_1D = 2 or DY_SC_TYPE_BLOCK_1D = 8), joint order, per joint the
 * write-back impulse (6 floats) and broken flag. */
int gbpx_joint_frame(const void* rigidBodies, uint32_t nbDynamic, const float* staticPoses, uint32_t nbStatic, const uint32_t* jointA,
                     const uint32_t* jointB, uint32_t nbJoints, const uint32_t* rowStart, const uint32_t* rowCount, const void* rows,
                     const float* params, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel, uint32_t batchJoints, float* outVelocity,
                     float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outHeaderType, uint32_t* outOrder,
                     float* outForce, uint32_t* outBroken, uint32_t* outNbHeaders);

/* -------------------------------------------------------- batched world
 * Many independent scenes advanced together: one persistent launch per step
 * (optionally a CUDA graph), all state resident on the device.  Each scene's
 * frame is the reference immediate-mode loop (physx/snippets/
 * snippetimmediatemode/SnippetImmediateMode.cpp:473): all overlapping pairs,
 * contacts, TGS.  With persistence on (the snippet's WITH_PERSISTENCY default)
 * every overlapping pair keeps its PCM contact manifold and the friction
 * patches of its contact constraint from step to step; a pair starts fresh
 * when it starts overlapping.  With persistence off every step uses fresh
 * caches and friction data.  No single reference function is replaced: this
 * is the multi-scene driver of the functions above.
 * params (12 floats): dt, gravity xyz, contactDistance, toleranceLength,
 * boundsMargin, bounceThreshold, frictionOffsetThreshold, correlationDistance,
 * staticFriction, persistence (0 or 1); iterations: position, velocity. */
int gbpx_world_create(uint32_t nbScenes, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, const void* rigidBodies,
                      const int* types, const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes,
                      const float* staticGeoms, const float* params, const uint32_t* iterations, uint32_t pairsPerBody, void** outWorld);
void gbpx_world_release(void* world);
int gbpx_world_step(void* world, uint32_t nbSteps, int useGraph);
int gbpx_world_synchronize(void* world);
int gbpx_world_get_bodies(void* world, void* outRigidBodies);
int gbpx_world_set_bodies(void* world, const void* rigidBodies);
int gbpx_world_status(void* world, uint32_t* outStatus);
/* out8: scenes, dynamic bodies, statics, pair slots, broadphase grid blocks,
 * device bytes, kernels launched per step, large-scene threshold */
int gbpx_world_info(void* world, uint64_t* out8);
int gbpx_world_scene_pairs(void* world, uint32_t scene, uint32_t* outKeys, uint32_t* outContactCounts, uint32_t capacity,
                           uint32_t* outCount);
int gbpx_world_time_steps(void* world, uint32_t nbSteps, int useGraph, float* outMs);
int gbpx_world_time_plain(void* world, uint32_t firstScene, uint32_t nbScenes, float* outMs);
/* out4: pairs, pairs with contacts, contacts, bytes of packed constraint rows (last step) */
int gbpx_world_stats(void* world, uint64_t* out4);
/* Scenes of more than largeBodies solver bodies (bodies + statics) run the
 * broadphase, batching and solve one block (8 warps) per scene, smaller scenes
 * one warp per scene; default 512.  Results do not depend on it. */
int gbpx_world_set_large_bodies(void* world, uint32_t largeBodies);
/* Autotuner keyed on the scene-size histogram: times candidate thresholds of
 * gbpx_world_set_large_bodies, then the solve kernel, then the preparation
 * and heavy narrowphase blocks per SM (gbpx_world_set_occupancy), on a
 * size-stratified sample of sampleScenes
 * scenes (a temporary world in the current state, `steps` graph steps each),
 * sets the fastest and caches it per histogram.  The sample must load the GPU
 * like the whole world (pass the scene count to copy every scene).  outMs: the
 * chosen configuration's ms per step on the sample (0 when cached). */
int gbpx_world_autotune(void* world, uint32_t sampleScenes, uint32_t steps, uint32_t* outLargeBodies, uint32_t* outSolveVariant,
                        float* outMs);
/* The world's tuning: out5 = block-per-scene threshold, solve kernel,
 * preparation and heavy narrowphase blocks per SM (0 = as many as fit),
 * streamed-row levels of the resident solve. */
int gbpx_world_tuning(void* world, uint32_t* out5);
/* Streamed rows in the resident solve (0 .. 3, default 1): a scene whose
 * on-chip footprint needs a level above `levels` is solved one level deeper
 * (by a group of at least two warps), its rows streamed chunk by chunk
 * (consecutive constraints of one partition) through a two-slot ring of bulk
 * copies while the previous chunk is solved, so more scenes are in flight per
 * SM; scenes too large for any slice stream their rows too (levels > 0).  The
 * autotuner sets it after the solve kernel.  Results do not depend on it. */
int gbpx_world_set_resident_stream(void* world, uint32_t levels);
/* Workspace of the warp-per-scene solve: variants 0-2 keep the body
 * velocities in shared memory and stage rows in 0 / 256 / 512 bytes per lane
 * (2 is the default), variants 3-5 the same with the velocities left in HBM,
 * 6 / 7 stage 400 bytes with the velocities on chip / in HBM (a smaller
 * workspace leaves room for more warps per SM).  Results do not depend
 * on it.  The autotuner sets it after the threshold. */
int gbpx_world_set_solve_variant(void* world, uint32_t variant);
/* Persistent blocks per SM of the row preparation and of the capsule-box and
 * box-box narrowphase kernels (0 = as many as fit, the default): their threads
 * keep large working sets in local memory, and fewer threads in flight keep it
 * in L1 / L2.  Results do not depend on it. */
int gbpx_world_set_occupancy(void* world, uint32_t prepBlocksPerSm, uint32_t narrowphaseBlocksPerSm);
/* Pairs of each pair kind in the last step, in the kind order of the
 * narrowphase launches (sphere-sphere ... box-box): 9 counts. */
int gbpx_world_kind_counts(void* world, uint32_t* out9);
/* average device milliseconds per kernel of a step (un-captured steps, events
 * between launches), in launch order; outMs has "kernels per step" entries */
int gbpx_world_time_stages(void* world, uint32_t nbSteps, float* outMs);
int gbpx_world_step_host(void* world, const void* rigidIn, void* rigidOut, uint32_t nbSteps, int useGraph, float* outMs);
int gbpx_host_alloc(size_t bytes, void** out);

/* ------------------------------------------------------------- serving
 * Request loop over a live pool of scenes resident in HBM (no reference
 * counterpart: it drives the batched step above).  Scenes are admitted into
 * fixed-capacity slots grouped by body-count class (class c: slots[c] slots of
 * capacity[c] bodies, staticsPerSlot statics), each class split into
 * lanesPerClass lanes; each lane steps on its own stream.  A request advances
 * one scene by n steps; each pump issues, per lane, one step over every scene
 * that still owes steps (continuous batching), with at most two steps in
 * flight per lane, and completes requests whose steps have finished.  Latency
 * runs from the request's arrival time to the host observing its last step
 * done. */
int gbpx_server_create(uint32_t nbClasses, const uint32_t* capacity, const uint32_t* slots, uint32_t staticsPerSlot, const float* params,
                       const uint32_t* iterations, uint32_t pairsPerBody, uint32_t lanesPerClass, void** outServer);
void gbpx_server_release(void* server);
/* device bytes of one slot (for sizing a pool against a memory budget), with or
 * without the persistent pair state; not a status code */
uint64_t gbpx_server_slot_bytes(uint32_t capacity, uint32_t staticsPerSlot, uint32_t pairsPerBody, int persistent);
/* GBPX_ERR_BUDGET when no free slot of sufficient capacity exists */
int gbpx_server_admit(void* server, uint32_t nbBodies, const void* rigidBodies, const int* types, const float* geoms, const float* friction,
                      uint32_t nbStatics, const float* staticPoses, const int* staticTypes, const float* staticGeoms, uint32_t* outScene);
/* GBPX_ERR_STATE while the scene still owes requested steps */
int gbpx_server_retire(void* server, uint32_t scene);
/* arrival: seconds on the server clock, negative for now */
int gbpx_server_submit(void* server, uint32_t scene, uint32_t nbSteps, uint64_t tag, double arrival);
int gbpx_server_pump(void* server, uint32_t* outIssued);
int gbpx_server_clock(void* server, double* outSeconds);
int gbpx_server_poll(void* server, uint64_t* outTags, double* outLatencySeconds, uint32_t capacity, uint32_t* outCount);
int gbpx_server_read_scene(void* server, uint32_t scene, void* outRigidBodies);
/* Eviction and re-admission (checkpoint / resume of served state): the snapshot
 * of a scene that owes no steps -- bodies, shapes, statics and, with persistent
 * pair state, its sorted pair list with each pair's contact manifold and
 * friction patches -- in this library's layout; *outBytes gets its size and out
 * (capacity bytes, GBPX_ERR_CAPACITY if short) the snapshot unless null.
 * Restoring admits it as a new scene (the smallest class that holds its bodies,
 * statics and pairs) whose following steps give the results the scene would
 * have had. */
int gbpx_server_snapshot_scene(void* server, uint32_t scene, void* out, uint64_t capacity, uint64_t* outBytes);
int gbpx_server_restore_scene(void* server, const void* snapshot, uint64_t bytes, uint32_t* outScene);
/* out4: body-steps completed, class steps completed, live scenes, steps in flight */
int gbpx_server_stats(void* server, uint64_t* out4);
/* The open-loop serving load run in the library (no per-request host language
 * round trips): Poisson arrivals at `rate` of "advance a live scene by n ~
 * U{minSteps..maxSteps} steps" for `seconds`; the pool is filled from a library
 * of nbLib scenes with one static shape each (scene k's bodies at libOffsets[k]
 * .. libOffsets[k + 1], nbLib + 1 offsets), and a scene that owes nothing after
 * its lifetime (U{lifeMin..lifeMax} steps) is retired and replaced.  out16:
 * seconds, submitted, completed, body-steps, p50 and p99 request latency (ms),
 * the same for 257..512-body scenes, their p50 and p99 latency per requested
 * step, live scenes, retired, admitted after the start, lane steps, lanes, 0. */
int gbpx_server_run_load(void* server, double seconds, double rate, uint32_t minSteps, uint32_t maxSteps, uint32_t lifeMin, uint32_t lifeMax,
                         uint64_t seed, uint32_t nbLib, const uint32_t* libOffsets, const void* libRigid, const int* libTypes,
                         const float* libGeoms, const float* libFriction, const float* libStaticPoses, const int* libStaticTypes,
                         const float* libStaticGeoms, double* out16);
void gbpx_host_free(void* p);

/* ---- One large scene (no reference counterpart: the snippet's frame over one
 * scene of any size, every stage spread over the whole GPU) ----
 * Layout as one scene of gbpx_world_create (PxRigidBodyData, types, 4-float
 * geoms and friction per dynamic body; static PxTransforms, types, geoms;
 * 12 params, 2 iterations).  The broadphase is the ABP of gbpx_bp_* with every
 * dynamic body updated each frame; PxBatchConstraintsTGS runs on the host. */
int gbpx_scene_create(uint32_t nbDyn, const void* rigidBodies, const int* types, const float* geoms, const float* friction, uint32_t nbStatic,
                      const float* staticPoses, const int* staticTypes, const float* staticGeoms, const float* params, const uint32_t* iterations,
                      void** outScene);
void gbpx_scene_release(void* scene);
int gbpx_scene_step(void* scene, uint32_t nbSteps);
int gbpx_scene_get_bodies(void* scene, void* outRigidBodies);
int gbpx_scene_set_bodies(void* scene, const void* rigidBodies);
/* out4: pairs, constraints, contacts, partitions of the last step */
int gbpx_scene_stats(void* scene, uint64_t* out4);
/* PxBatchConstraintsTGS's rule on the device (enable = 1, the default: an exact
 * parallel reproduction of the sequential greedy assignment) or on the host
 * (0).  Same order and partitions either way; a frame in which a body has more
 * than 32 dynamic constraints is batched on the host. */
int gbpx_scene_set_device_batching(void* scene, int enable);
/* out2[0]: colouring passes of the last frame's device batching; out2[1]: 1
 * when that frame was batched on the device. */
int gbpx_scene_batch_info(void* scene, uint32_t* out2);
/* outMs[0] = ms per frame, outMs[1..6] per stage: bounds + broadphase,
 * narrowphase, constraint list + batching, bodies + rows, iterations, write-back */
int gbpx_scene_time_steps(void* scene, uint32_t nbSteps, float* outMs);
/* end to end: bodies uploaded from rigidIn, nbSteps frames, downloaded to rigidOut */
int gbpx_scene_step_host(void* scene, const void* rigidIn, void* rigidOut, uint32_t nbSteps, float* outMs);

#ifdef __cplusplus
}
#endif

#endif /* GBPX_H */
