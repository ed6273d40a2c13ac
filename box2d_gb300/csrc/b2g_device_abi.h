/*
 * Thin C ABI between the C17 host side of the GB300 step library and its CUDA kernels,
 * plus the plain-old-data records both sides agree on.
 *
 * Device memory layout (one world = one b2gDeviceWorld):
 *   bodies, indexed by body id (static and awake alike): transform, center, inverse mass
 *     data, extents, awake index, type/flags, shape list range
 *   awake solver state, indexed by awake index (the reference's awake-set order,
 *     body.c:200-260): b2BodyState as two float4 (v.x, v.y, w, flags) and
 *     (dp.x, dp.y, dq.c, dq.s), plus the integration parameters
 *   shapes, indexed by shape id: geometry, material, AABB, fat AABB, enlarge flag
 *   contacts, indexed by contact id (stable across color moves): the b2ContactSim fields
 *   graph colors: per color an array of contact ids and joint ids in the reference's array
 *     order; contact constraints are laid out color by color, one slot per contact
 *
 * Every function returns 0 on success or a CUDA error code.
 */
#ifndef B2G_DEVICE_ABI_H
#define B2G_DEVICE_ABI_H

#include "box2d_gb300.h"

#ifdef __cplusplus
extern "C"
{
#endif

#define B2G_OVERFLOW_INDEX ( B2_GRAPH_COLOR_COUNT - 1 )

/* body flag bits (body.h b2BodyFlags) */
enum
{
	B2G_LOCK_X = 0x1,
	B2G_LOCK_Y = 0x2,
	B2G_LOCK_Z = 0x4,
	B2G_IS_FAST = 0x8,
	B2G_IS_BULLET = 0x10,
	B2G_SPEED_CAPPED = 0x20,
	B2G_HAD_TOI = 0x40,
	B2G_ALLOW_FAST_ROTATION = 0x80,
	B2G_ENLARGE_BOUNDS = 0x100,
	B2G_DYNAMIC_FLAG = 0x200,
	B2G_DIRTY_MASS = 0x400,
	B2G_ENABLE_SLEEP = 0x800,
	B2G_ENABLE_RECYCLING = 0x1000,
	B2G_TRANSIENT = B2G_IS_FAST | B2G_SPEED_CAPPED | B2G_HAD_TOI,
};

/* contact sim flag bits (contact.h b2ContactFlags) */
enum
{
	B2G_C_TOUCHING = 0x1,
	B2G_C_HIT_EVENT = 0x2,
	B2G_C_ENABLE_EVENTS = 0x4,
	B2G_C_RECYCLE = 0x8,
	B2G_S_TOUCHING = 0x10000,
	B2G_S_DISJOINT = 0x20000,
	B2G_S_STARTED = 0x40000,
	B2G_S_STOPPED = 0x80000,
	B2G_S_HIT_EVENT = 0x100000,
	B2G_S_PRESOLVE = 0x200000,
	B2G_S_RELATIVE_VALID = 0x400000,
	B2G_S_LIVE = 0x40000000, /* slot holds a contact (device bookkeeping only) */
};

/* shape record (b2Shape geometry + material). Circles keep center in v[0]; capsules and
   segments keep their two points in v[0], v[1]; polygons use the full b2Polygon. */
typedef struct b2gShape
{
	int type;
	int bodyId;
	int enableHitEvents;
	int count;
	b2Vec2 v[B2_MAX_POLYGON_VERTICES];
	b2Vec2 n[B2_MAX_POLYGON_VERTICES];
	b2Vec2 centroid;
	float radius;
	float aabbMargin;
	float friction, restitution, rollingResistance, tangentSpeed;
	/* continuous collision (solver.c:183-376): filter, sensor flag, and the core circle
	   (centroid, 0.25 x minimum extent about it) used when the full shape starts overlapped */
	uint64_t categoryBits, maskBits;
	int groupIndex;
	int isSensor;
	b2Vec2 ccdCentroid;
	float ccdCoreRadius;
	int enableSensorEvents; /* the shape is seen by sensors (and a sensor reports events) */
	int proxyKey;			/* its broadphase proxy (proxy id << 2 | tree), -1 = none */
} b2gShape;

/* contact record (contact.h:103-142 b2ContactSim without ids kept on the host) */
typedef struct b2gContact
{
	int shapeIdA, shapeIdB;
	uint32_t simFlags;
	int bodySimIndexA, bodySimIndexB;
	float invMassA, invIA, invMassB, invIB;
	float friction, restitution, rollingResistance, tangentSpeed;
	b2Rot cachedRotationA, cachedRotationB;
	b2Transform cachedRelativePose;
	b2Manifold manifold;
	/* GJK simplex cache (contact.h b2ContactSim cache): vertex count and the vertex indices
	   on each shape; warm-starts the distance query of chain-segment manifolds */
	uint8_t cacheCount, cacheA[3], cacheB[3], cachePad;
} b2gContact;

/* new contact written by the host into the contact slot of its id */
typedef struct b2gContactInit
{
	int contactId;
	int shapeIdA, shapeIdB;
	uint32_t simFlags;
	float friction, restitution;
} b2gContactInit;

/* one contact constraint slot (contact_solver.c:1070-1100 b2ContactConstraintWide lane) */
typedef struct b2gContactLane
{
	int indexA, indexB; /* awake index + 1, 0 = none */
	float invMassA, invMassB, invIA, invIB;
	b2Vec2 normal;
	float friction, tangentSpeed, rollingResistance, rollingMass, rollingImpulse;
	float biasRate, massScale, impulseScale;
	b2Vec2 anchorA1, anchorB1;
	float normalMass1, tangentMass1, baseSeparation1, normalImpulse1, totalNormalImpulse1, tangentImpulse1;
	b2Vec2 anchorA2, anchorB2;
	float baseSeparation2, normalImpulse2, totalNormalImpulse2, tangentImpulse2, normalMass2, tangentMass2;
	float restitution, relativeVelocity1, relativeVelocity2;
	int groupFlags; /* bit 0: a lane of its 4-wide group has rolling resistance; bit 1: restitution */
	int pointCount;
} b2gContactLane;

/* joint record (joint.h:267-301 b2JointSim, revolute/prismatic/weld/wheel/distance) */
typedef struct b2gJoint
{
	int type;
	int bodyIdA, bodyIdB;
	int indexA, indexB; /* awake indices, -1 = static */
	b2Transform localFrameA, localFrameB;
	float invMassA, invMassB, invIA, invIB;
	float constraintHertz, constraintDampingRatio;
	float softBias, softMass, softImpulse; /* constraint softness */
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	/* per-type parameters */
	float p[16];
	/* per-type accumulated impulses and solver constants */
	float s[16];
	int enableSpring, enableLimit, enableMotor, jointId;
} b2gJoint;

/* step constants (b2StepContext, solver.h:155-237) */
typedef struct b2gStepParams
{
	float dt, inv_dt, h, inv_h;
	int subStepCount;
	float contactBiasRate, contactMassScale, contactImpulseScale;
	float staticBiasRate, staticMassScale, staticImpulseScale;
	float restitutionThreshold, maxLinearVelocity, contactSpeed, contactHertz, contactDampingRatio;
	float gravityX, gravityY;
	float jointHertzCap;
	int enableWarmStarting, enableContinuous, enableSleep, enableContactSoftening;
	float contactRecycleDistance;
} b2gStepParams;

/* per-step results the host reads back */
typedef struct b2gStepCounters
{
	int stateChangeCount;
	int enlargedBodyCount;
	int recycledContactCount;
	int pairCount;
	int pairOverflow;
	int fastBodyCount;
	int status;			/* nonzero: a device check failed (see B2G_STATUS_*) */
	int sensorHitCount; /* sensor shapes hit by continuous sweeps this step */
	int continuousSweeps; /* fast non-bullet bodies swept against static shapes */
	int continuousHits;	  /* sweeps that moved the body back to its time of impact */
	int pad;
	/* island to split before the next finalize: the largest (sleep time bits << 32 | island
	   id) over bodies that want to sleep in an island with removed constraints; 0 if none */
	unsigned long long splitKey;
} b2gStepCounters;

enum
{
	B2G_STATUS_OK = 0,
	B2G_STATUS_NAN = 1,
	B2G_STATUS_CAPACITY = 2,
};

/* ---- tape of differentiable stepping (box2d_gb300_diff.h) ----
   One world's recording, as b2Diff_DownloadTape returns it: a b2gTapeHeader, the world's
   shapes (b2gShape[shapeCount]), then stepCount step records. A step record is a
   b2gTapeStep followed by b2gTapeBody[bodyCount] (by body id), float[8 * awakeCount]
   (integration parameters by awake index, as the solver's), float[awakeCount] (time-of-
   impact fraction of the step's continuous sweep, 1 = none), int[slotCount] (contact id of
   each colored slot) and b2gContact[slotCount] (each contact after the narrowphase, in slot
   order); every part starts on a 16-byte boundary. */
typedef struct b2gTapeHeader
{
	int stepCount, shapeCount, bodyCount, contactCapacity;
	long long stepOffsets[1]; /* stepCount entries: byte offset of each step from the header */
} b2gTapeHeader;

typedef struct b2gTapeBody
{
	b2Transform xf; /* pose at the start of the step */
	b2Vec2 center;
	b2Vec2 localCenter;
	float vx, vy, w; /* velocity at the start of the step (awake bodies) */
	uint32_t flags;	 /* state flags (awake bodies) */
	int awakeIndex;	 /* -1: not awake */
	int type;
} b2gTapeBody;

typedef struct b2gTapeStep
{
	b2gStepParams params;
	int bodyCount, awakeCount, slotCount, jointCount;
	int colorOffsets[B2_GRAPH_COLOR_COUNT + 1];
	int bytes; /* the whole record */
	int pad[2];
} b2gTapeStep;

/* contact sim flag of a contact whose manifold was recycled this step (physics_world.c:508-560) */
#define B2G_S_RECYCLED 0x800000
/* the contact is in a sleeping or the disabled solver set: the narrowphase skips it
   (device bookkeeping only) */
#define B2G_S_ASLEEP 0x1000000

#ifdef __CUDACC__
#define B2G_TAPE_FN static inline __host__ __device__
#else
#define B2G_TAPE_FN static inline
#endif

B2G_TAPE_FN long long b2gTapeAlign( long long x ) { return ( x + 15 ) & ~15LL; }

/* byte offsets of a step record's parts */
B2G_TAPE_FN long long b2gTapeBodiesOffset( void ) { return b2gTapeAlign( (long long)sizeof( b2gTapeStep ) ); }
B2G_TAPE_FN long long b2gTapeParamsOffset( int bodyCount )
{
	return b2gTapeBodiesOffset() + b2gTapeAlign( (long long)bodyCount * (long long)sizeof( b2gTapeBody ) );
}
/* time-of-impact fraction of each awake body's continuous sweep (1: the body advanced to
   its solved pose), written by the step's finalize */
B2G_TAPE_FN long long b2gTapeToiOffset( int bodyCount, int awakeCount )
{
	return b2gTapeParamsOffset( bodyCount ) + b2gTapeAlign( 32LL * awakeCount );
}
B2G_TAPE_FN long long b2gTapeIdsOffset( int bodyCount, int awakeCount )
{
	return b2gTapeToiOffset( bodyCount, awakeCount ) + b2gTapeAlign( 4LL * awakeCount );
}
B2G_TAPE_FN long long b2gTapeContactsOffset( int bodyCount, int awakeCount, int slotCount )
{
	return b2gTapeIdsOffset( bodyCount, awakeCount ) + b2gTapeAlign( 4LL * slotCount );
}
B2G_TAPE_FN long long b2gTapeStepBytes( int bodyCount, int awakeCount, int slotCount )
{
	return b2gTapeContactsOffset( bodyCount, awakeCount, slotCount ) +
		   b2gTapeAlign( (long long)slotCount * (long long)sizeof( b2gContact ) );
}

typedef struct b2gDeviceWorld b2gDeviceWorld;

/* lifetime */
int b2gDev_Create( b2gDeviceWorld** out );
void b2gDev_Destroy( b2gDeviceWorld* dw );
const char* b2gDev_ErrorString( int code );

/* uploads of cold data (whole arrays; called when the host marks them dirty) */
int b2gDev_UploadShapes( b2gDeviceWorld* dw, const b2gShape* shapes, const float* aabbs, const float* fatAABBs, int count );
int b2gDev_UploadBodies( b2gDeviceWorld* dw, int bodyCount, const float* xf, const float* center, const float* localCenter,
						 const float* invMass, const float* invI, const float* minExtent, const float* maxExtent,
						 const float* sleepThreshold, const float* safetyFactor, const int* awakeIndex, const uint32_t* typeFlags,
						 const int* shapeStart, const int* shapeCount, const int* shapeList, int shapeListCount );
int b2gDev_UploadAwake( b2gDeviceWorld* dw, int awakeCount, const int* awakeBodyId, const float* stateV, const float* stateD,
						const float* params, const float* center0, const float* sleepTime );
int b2gDev_DownloadAwake( b2gDeviceWorld* dw, int awakeCount, float* stateV, float* stateD, float* params, float* center0 );
int b2gDev_DownloadBodies( b2gDeviceWorld* dw, int bodyCount, float* xf, float* center, uint32_t* typeFlags );
/* body transforms (4 floats), centers (2), flags and awake velocities (4) in one wait;
   the pointers refer to page-locked staging valid until the next call */
/* send the host-mirrored body state down behind the step's work, without waiting */
int b2gDev_PrefetchState( b2gDeviceWorld* dw, int bodyCount, int awakeCount );
/* whether the prefetched state is still the device's; put back after device work that
   changes no body state */
int b2gDev_PrefetchIsValid( b2gDeviceWorld* dw );
void b2gDev_PrefetchKeep( b2gDeviceWorld* dw, int valid );
int b2gDev_DownloadState( b2gDeviceWorld* dw, int bodyCount, int awakeCount, const float** xf, const float** center,
						  const uint32_t** flags, const float** stateV, const float** sleepTime );

/* islands and sleeping. Bodies woken inside a step are appended to the awake set: one
   record of 10 ints each (body id, awake index, the 8 body parameters as float bits); their
   velocity starts at zero and their flags are the body's (solver_set.c:35-76). Bodies put
   to sleep leave it: `slept` body ids, then `pairs` (destination, source) of the awake
   slots the swap-removals moved (sources at or past the new count). */
int b2gDev_WakeBodies( b2gDeviceWorld* dw, int newAwakeCount, const int* records, int count );
int b2gDev_SleepBodies( b2gDeviceWorld* dw, int newAwakeCount, const int* slept, int sleptCount, const int* pairs,
						int pairCount );
/* contacts that leave (asleep = 1) or rejoin (0) the set the narrowphase collides */
int b2gDev_SetContactsAsleep( b2gDeviceWorld* dw, const int* contactIds, int count, int asleep );
/* the colored contacts' awake body indices from the awake set (after bodies woke) */
int b2gDev_RefreshContactBodies( b2gDeviceWorld* dw );
/* the island table of the finalize: per awake index the island's index in the awake set,
   per awake island (island id, 1 if it has removed constraints); islandCount < 0 turns the
   island bookkeeping of the finalize off (sleeping disabled) */
int b2gDev_UploadIslands( b2gDeviceWorld* dw, const int* islandLocal, int awakeCount, const int* islandInfo, int islandCount );
/* after the solve's wait: the awake-island bits the finalize set and the split key (valid
   until the next solve) */
int b2gDev_IslandResults( b2gDeviceWorld* dw, const uint32_t** awakeIslandBits, int* islandCount,
						  unsigned long long* splitKey );
int b2gDev_DownloadShapeBoxes( b2gDeviceWorld* dw, int shapeCount, float* aabbs, float* fatAABBs );
int b2gDev_SetBodyVelocity( b2gDeviceWorld* dw, int awakeIndex, float vx, float vy, float w, int which );
int b2gDev_SetBodyForce( b2gDeviceWorld* dw, int awakeIndex, float fx, float fy, float torque );

/* contacts */
int b2gDev_ReserveContacts( b2gDeviceWorld* dw, int capacity );
int b2gDev_InitContacts( b2gDeviceWorld* dw, const b2gContactInit* inits, int count );
int b2gDev_KillContacts( b2gDeviceWorld* dw, const int* contactIds, int count );
int b2gDev_UploadColors( b2gDeviceWorld* dw, const int* colorContactIds, const int* colorContactOffsets,
						 int totalContacts );
/* the same from the colors' own id lists (listCount lists, counts[i] ids each) */
int b2gDev_UploadColorLists( b2gDeviceWorld* dw, const int* const* lists, const int* counts, int listCount, const int* offsets,
							 int total );
/* contact slots [0, count) to the host (slots the device never held read as zeros), and
   back (a world snapshot's restore) */
int b2gDev_DownloadContacts( b2gDeviceWorld* dw, b2gContact* out, int count );
int b2gDev_UploadContacts( b2gDeviceWorld* dw, const b2gContact* in, int count );
/* device addresses of the contact records and the color lists, the color offsets, the
   world's stream (cudaStream_t) and its CUDA device, for kernels outside world.cu */
void b2gDev_ContactView( b2gDeviceWorld* dw, const b2gContact** contacts, const int** colorIds, int* colorOffsets,
						 void** stream, int* device );
/* sensor.c:43-270 b2SensorQueryCallback for every sensor at the end of a step: the
   (sensor index, shape id) pairs whose shapes overlap (GJK distance with radii below
   10 FLT_EPSILON), unordered. sensorShapeIds[i] < 0 skips sensor i. Waits for the device;
   the returned array is valid until the next call. */
int b2gDev_SensorOverlaps( b2gDeviceWorld* dw, const int* sensorShapeIds, int sensorCount, int shapeCount,
						   const int** outPairs, int* outCount );
/* solver.c:321-335, :539-547: the (sensor shape, visitor shape) pairs continuous sweeps of
   the last step hit before their solid time of impact. Waits for the device. */
int b2gDev_SensorHits( b2gDeviceWorld* dw, const int** outPairs, int* outCount );
/* solver.c:1917-1989: sweep the fast bullet bodies (awake slots) against the static,
   kinematic and dynamic trees as last uploaded; per bullet shape a record (shape id,
   enlarged) and its fat box. Waits for the device; results valid until the next call. */
int b2gDev_SolveBullets( b2gDeviceWorld* dw, const b2gStepParams* params, int awakeCount, const int* bulletSims, int count,
						 const int** outRecs, const float** outBoxes, int* outCount );
/* the contact table of b2p_contacts built without allocating (noalloc.cu) */
int b2gDev_ContactTableNoAlloc( b2gDeviceWorld* dw, int capacity, int* out, int outCapacity );

/* joints */
int b2gDev_UploadJoints( b2gDeviceWorld* dw, const b2gJoint* joints, int count, const int* colorJointOffsets );
/* per body id, the bodies that a joint with collideConnected == false links it to (CSR:
   offsets has bodyCount + 1 entries); listCount 0 clears it. Read by continuous collision,
   as b2ShouldBodiesCollide (body.c:2076-2112). */
/* the counters of the last solve, as read back by it */
int b2gDev_LastCounters( b2gDeviceWorld* dw, b2gStepCounters* out );
int b2gDev_UploadJointPartners( b2gDeviceWorld* dw, const int* offsets, int bodyCount, const int* list, int listCount );
int b2gDev_DownloadJoints( b2gDeviceWorld* dw, b2gJoint* joints, int count );

/* broadphase: tree nodes as (aabb float4, child1, child2 / userData, flags) */
typedef struct b2gTreeNode
{
	b2AABB aabb;
	int child1; /* leaf: shape id */
	int child2; /* leaf: -1 */
	int isLeaf;
	int categoryNonZero; /* the node's category bits intersect the query mask (all ones) */
} b2gTreeNode;

/* host tree node (dynamic_tree.c b2TreeNode fields), uploaded as is */
typedef struct b2gHostTreeNode
{
	b2AABB aabb;
	uint64_t categoryBits;
	int child1, child2; /* internal nodes */
	uint64_t userData;	/* leaves: shape id */
	int parent;
	uint16_t height;
	uint16_t flags; /* 0x4: leaf */
} b2gHostTreeNode;

/* copy nodeCount host nodes to the device and convert them to query nodes on the
   device. The host array must stay unchanged until the next pair query returns. */
int b2gDev_UploadTree( b2gDeviceWorld* dw, int treeType, const b2gHostTreeNode* nodes, int nodeCount, int root,
					   int hostPinned );
/* the proxy enlargement of the last solve applied to the device's copies of the kinematic
   and dynamic trees (the first `recordCount` enlarged-proxy records); the device copies must
   hold the trees as the host left them before its own enlargement. Records an event after
   the trees' uploads, which b2gDev_WaitTreeUploads waits for (the host node arrays may then
   change). */
int b2gDev_EnlargeTrees( b2gDeviceWorld* dw, int recordCount );
int b2gDev_WaitTreeUploads( b2gDeviceWorld* dw );
/* create the enlargement's events and second stream and load its kernel ahead of use */
int b2gDev_PrepareEnlarge( b2gDeviceWorld* dw );
/* waits of this world block the calling thread (sleep) instead of spinning */
void b2gDev_SetBlockingSync( b2gDeviceWorld* dw, int on );

/* page-locked host memory (NULL on failure) for arrays uploaded every step */
void* b2gDev_HostAlloc( size_t bytes );
void b2gDev_HostFree( void* p );
/* query each moved proxy's fat AABB; pairs come back grouped per move in the reference's
   order (proxy list newest first). outPairs holds (shapeA, shapeB); outCounts per move */
int b2gDev_FindPairs( b2gDeviceWorld* dw, const int* moveProxyKeys, const float* moveBoxes, const int* moveShapeIds,
					  int moveCount, int** outPairs, int** outCounts, int* outTotal );

/* narrowphase over every live contact; returns the state-change list (contactId, flags)
   sorted by contact id */
int b2gDev_Collide( b2gDeviceWorld* dw, const b2gStepParams* params, int contactIdCapacity, const int** outChanges,
					int* outChangeCount, int* outRecycled );

/* Soft Step solver + body finalization; returns enlarged bodies (awake index, ascending) */
int b2gDev_Solve( b2gDeviceWorld* dw, const b2gStepParams* params, const int* activeColors, int activeColorCount,
				  const int* colorContactCounts, const int* colorJointCounts, int awakeCount, const int** outEnlarged,
				  int* outEnlargedCount, const float** outFatBoxes, int* outStatus );

/* the three waits of a step split in two: issue the work (or record it, see below), then
   collect the results after the world's wait (b2gDev_Synchronize) or a batch flush */
int b2gDev_FindPairsIssue( b2gDeviceWorld* dw, const int* keys, const float* boxes, const int* shapes, int count );
int b2gDev_FindPairsCollect( b2gDeviceWorld* dw, int** outPairs, int** outCounts, int* outTotal );
/* drop the issued query (its results are not collected; its moved flags are cleared) */
int b2gDev_FindPairsDiscard( b2gDeviceWorld* dw );
int b2gDev_CollideIssue( b2gDeviceWorld* dw, const b2gStepParams* params, int contactIdCapacity );
int b2gDev_CollideCollect( b2gDeviceWorld* dw, const int** outChanges, int* outChangeCount, int* outRecycled );
/* start the solve's component analysis from the touching contacts the narrowphase left,
   beside the host's contact-state pass (large worlds solved by components) */
int b2gDev_ComponentsEarly( b2gDeviceWorld* dw, int awakeCount );
int b2gDev_SolveIssue( b2gDeviceWorld* dw, const b2gStepParams* params, const int* activeColors, int activeColorCount,
					   int awakeCount );
int b2gDev_SolveCollect( b2gDeviceWorld* dw, const int** outEnlarged, int* outEnlargedCount, const float** outFatBoxes,
						 int* outStatus );
/* whether the world's solve runs as one CTA (the only solve a batch records) */
int b2gDev_SolveFitsOneBlock( b2gDeviceWorld* dw, int awakeCount );

/* batched stepping: while a world records, its uploads, downloads and kernels are kept;
   b2gDev_BatchFlush replays the records of many worlds with one launch per kernel kind and
   position, one upload, one download and one wait */
typedef struct b2gDevBatch b2gDevBatch;
int b2gDev_BatchCreate( b2gDevBatch** out );
void b2gDev_BatchDestroy( b2gDevBatch* batch );
int b2gDev_BatchRecord( b2gDeviceWorld* dw, int on );
/* whether the world's device work is being recorded for a batched flush */
int b2gDev_IsRecording( b2gDeviceWorld* dw );
/* device operations recorded since recording began */
int b2gDev_RecordedCount( b2gDeviceWorld* dw );
/* runs fn(ctx, i) for i in [0, count) on the caller's threads */
typedef void ( *b2gParallelFor )( void* pool, int count, void ( *fn )( void* ctx, int index ), void* ctx );
int b2gDev_BatchFlush( b2gDevBatch* batch, b2gDeviceWorld* const* worlds, int count, b2gParallelFor parallelFor, void* pool );
long long b2gDev_BatchLaunches( b2gDevBatch* batch );
void b2gDev_BatchPartTimes( b2gDevBatch* b, double* out, int reset );
void b2gDev_BatchTimes( b2gDevBatch* batch, double* assembleMs, double* waitMs, int reset );

/* bookkeeping for profiles */
int b2gDev_Synchronize( b2gDeviceWorld* dw );
int b2gDev_DeviceSynchronize( void );
void b2gDev_Timings( b2gDeviceWorld* dw, float* stageMs, long long* traffic, int reset );
void* b2gDev_Stream( b2gDeviceWorld* dw );

/* ---- differentiable stepping (adjoint.cu) ---- */
/* append one step record (the state after the narrowphase, before the solver) to a device
   arena that grows stream-ordered; *offset receives the record's offset in the arena */
int b2gDev_CaptureTape( b2gDeviceWorld* dw, const b2gStepParams* params, int bodyCount, int awakeCount, int jointCount,
						void** arena, long long* capacity, long long* used, long long* offset );
void b2gDev_FreeTapeArena( void* arena );
const b2gShape* b2gDev_ShapeArray( b2gDeviceWorld* dw, int* count );
int b2gDev_ContactCapacity( b2gDeviceWorld* dw );

typedef struct b2gAdjointWorld
{
	const void* arena;			   /* device tape arena of the world */
	const long long* stepOffsets; /* host: offset of each step record in the arena */
	const b2gShape* shapes;		   /* device shapes */
	int shapeCount, bodyCount, contactCapacity;
	int maxAwake, maxSlots, maxSubsteps; /* largest awake, slot and substep counts over the steps */
} b2gAdjointWorld;

/* reverse pass over stepCount recorded steps of every world (see box2d_gb300_diff.h for
   the host arrays); returns 0, a negative B2_DIFF_* code or a CUDA error. failure (5 ints,
   may be NULL) receives the first failing world's code, world, step, check and item. */
int b2gDev_AdjointRun( const b2gAdjointWorld* worlds, int worldCount, int stepCount, const int* bodyOffsets,
					   const int* shapeOffsets, const float* adjCenter, const float* adjRotation, const float* adjVelocity,
					   float* gradVelocity, float* gradCenter, float* gradFriction, float* ms, int* launches,
					   int* failure );
int b2gDev_DownloadArena( const void* arena, long long bytes, void* out );

#ifdef __cplusplus
}
#endif

#endif
