/*
 * Host world model of the GB300 step library. The host keeps the serial bookkeeping of
 * Box2D v3.2's step -- ids, body/shape/contact/joint records, the broadphase trees, the
 * move buffer, the shape-pair set and the graph colors -- in the exact array orders of
 * the reference (so contact ids and colors come out identical). All per-step numeric work
 * (pair query, narrowphase, solver, finalize) runs on the device; the host only reads
 * back compact change lists.
 */
#ifndef B2G_WORLD_H
#define B2G_WORLD_H

#include "../b2g_device_abi.h"
#include "b2g_host.h"

#define H_MAX_WORLDS 4096

enum
{
	H_STATIC_SET = 0,
	H_DISABLED_SET = 1,
	H_AWAKE_SET = 2,
	H_FIRST_SLEEPING_SET = 3,
};

/* constants.h B2_TIME_TO_SLEEP: seconds a body must be still before its island can sleep */
#define H_TIME_TO_SLEEP 0.5f

typedef struct h_body
{
	void* userData;
	int setIndex, localIndex; /* awake index for the awake set, static index otherwise */
	int headContactKey, contactCount;
	int headShapeId, shapeCount;
	int headJointKey, jointCount;
	int headChainId;
	int islandId, islandIndex; /* island of a non-static body and its index in the island */
	int bodyMoveIndex;		   /* its move event in the last step while the sleep pass runs */
	float mass, inertia;
	float sleepThreshold, sleepTime, safetyFactor;
	int id;
	uint32_t flags;
	b2BodyType type;
	uint16_t generation;
	/* cold simulation data (device is authoritative for transform/velocity after a step) */
	b2Transform transform;
	b2Vec2 center, localCenter;
	float invMass, invInertia, minExtent, maxExtent;
	float linearDamping, angularDamping, gravityScale;
	uint32_t simFlags;
	b2Vec2 linearVelocity;
	float angularVelocity;
	b2Vec2 force; /* external force and torque accumulated for the next step (cleared by it) */
	float torque;
} h_body;

typedef struct h_shape
{
	int id, bodyId, prevShapeId, nextShapeId;
	b2ShapeType type;
	b2SurfaceMaterial material;
	float density, aabbMargin;
	b2AABB aabb, fatAABB;
	b2Vec2 localCentroid;
	int proxyKey;
	b2Filter filter;
	void* userData;
	union
	{
		b2Capsule capsule;
		b2Circle circle;
		b2Polygon polygon;
		b2Segment segment;
		b2ChainSegment chainSegment;
	};
	uint16_t generation;
	int enableContactEvents, enableHitEvents, isSensor;
	int enableSensorEvents, sensorIndex; /* sensorIndex: its slot in the world's sensors, or -1 */
} h_shape;

/* a chain of segment shapes on one body (shape.h b2ChainShape) */
typedef struct h_chain
{
	int id, bodyId, nextChainId;
	int count; /* segment shapes */
	int* shapeIndices;
	uint16_t generation;
} h_chain;

/* a shape seen by a sensor (sensor.h b2Visitor) */
typedef struct h_visitor
{
	int shapeId;
	uint16_t generation;
} h_visitor;
typedef H_ARRAY( h_visitor ) h_visitorArray;

/* a sensor shape's overlaps (sensor.h b2Sensor): the previous and current step's sorted
   visitors, and the visitors continuous sweeps hit during the step */
typedef struct h_sensor
{
	int shapeId;
	h_visitorArray overlaps1, overlaps2, hits;
} h_sensor;

typedef struct h_contactEdge
{
	int bodyId, prevKey, nextKey;
} h_contactEdge;

typedef struct h_contact
{
	h_contactEdge edges[2];
	int setIndex, colorIndex, localIndex;
	int islandId, islandIndex;
	int shapeIdA, shapeIdB, contactId;
	uint32_t flags, generation;
} h_contact;

typedef struct h_jointEdge
{
	int bodyId, prevKey, nextKey;
} h_jointEdge;

typedef struct h_joint
{
	void* userData;
	int setIndex, colorIndex, localIndex;
	h_jointEdge edges[2];
	int islandId, islandIndex;
	int jointId;
	b2JointType type;
	uint16_t generation;
	int collideConnected;
} h_joint;

/* a contact or joint of an island with its two bodies (island.h b2ContactLink, b2JointLink) */
typedef struct h_link
{
	int id, bodyIdA, bodyIdB;
} h_link;
typedef H_ARRAY( h_link ) h_linkArray;

/* a persistent island (island.h b2Island): touching contacts and joints connect its bodies */
typedef struct h_island
{
	int setIndex, localIndex, islandId;
	int constraintRemoveCount;
	h_intArray bodies;
	h_linkArray contacts;
	h_linkArray joints;
} h_island;

/* a sleeping solver set (solver_set.h b2SolverSet, set index >= H_FIRST_SLEEPING_SET): the
   ids of its bodies, touching contacts, joints and islands, in the reference's array orders */
typedef struct h_sleepSet
{
	int setIndex; /* B2_NULL_INDEX when the slot is free */
	h_intArray bodyIds, contactIds, jointIds, islandIds;
} h_sleepSet;

typedef struct h_color
{
	h_bitSet bodySet;
	h_intArray contactIds; /* reference array order (add at end, swap-remove) */
	h_intArray jointIds;
} h_color;

typedef struct h_world
{
	int inUse;
	uint16_t worldId, generation;
	h_idPool bodyIdPool, shapeIdPool, contactIdPool, jointIdPool, chainIdPool;
	H_ARRAY( h_body ) bodies;
	H_ARRAY( h_shape ) shapes;
	H_ARRAY( h_contact ) contacts;
	H_ARRAY( h_joint ) joints;
	H_ARRAY( b2gJoint ) jointRecords; /* by joint id; device copy is authoritative */
	h_intArray awakeBodyIds;		  /* awake index -> body id */
	int staticCount;
	h_intArray staticBodyIds;  /* the static set's bodies, reference array order */
	int staticJointCount;	   /* joints of the static set (between two non-dynamic bodies) */
	h_intArray staticJointIds; /* those joints, reference array order */
	h_intArray awakeContactIds;		  /* non-touching contacts, reference array order */
	h_intArray disabledContactIds;	  /* non-touching contacts between sleeping bodies */
	/* islands and sleeping (island.c) */
	H_ARRAY( h_island ) islands;
	h_idPool islandIdPool;
	h_intArray awakeIslandIds; /* the awake set's islands, reference array order */
	H_ARRAY( h_sleepSet ) sets; /* by solver set id; slots below H_FIRST_SLEEPING_SET unused */
	h_idPool setIdPool;
	int splitIslandId;
	int islandsDirty;	  /* the finalize's island table must be sent again */
	int setChangeCount;	  /* islands put to sleep or woken since the world was created */
	int* sleepPerm;		  /* while the sleep pass runs: original awake index per awake slot */
	h_intArray pendingWake;	   /* device records (10 ints) of bodies woken inside the step */
	h_intArray pendingContacts; /* contacts whose solver set changed: collided or not */
	h_intArray sleptBodies;	   /* bodies put to sleep by the sleep pass in progress */
	int wokeInStep;			   /* a set woke inside the step: refresh the colored contacts */
	h_color colors[B2_GRAPH_COLOR_COUNT];
	h_tree trees[3];
	h_bitSet movedProxies[3];
	h_intArray moveArray;
	h_pairSet pairSet;
	/* settings */
	b2Vec2 gravity;
	float hitEventThreshold, restitutionThreshold, maxLinearSpeed, contactSpeed, contactHertz, contactDampingRatio;
	int enableSleep, enableWarmStarting, enableContactSoftening, enableContinuous, locked;
	/* sensors, in creation order (swap-removed) */
	H_ARRAY( h_chain ) chains; /* by chain id */
	H_ARRAY( h_sensor ) sensors;
	int sensorStep; /* stepIndex of the last sensor overlap pass */
	H_ARRAY( b2SensorBeginTouchEvent ) sensorBeginEvents;
	H_ARRAY( b2SensorEndTouchEvent ) sensorEndEvents[2];
	/* events */
	H_ARRAY( b2BodyMoveEvent ) moveEvents;
	H_ARRAY( b2ContactBeginTouchEvent ) beginEvents;
	H_ARRAY( b2ContactEndTouchEvent ) endEvents[2];
	int endEventArrayIndex;
	int stepIndex;
	int recycledContactCount;
	b2Profile profile;
	/* accumulated host-side time per step phase (ms), see H_PHASE_* */
	float hostMs[10];
	/* device mirror */
	b2gDeviceWorld* dev;
	int devReady;			/* device arrays hold the current world */
	int hostStateValid;		/* host body transforms/velocities match the device */
	/* the device's state arrays as downloaded after the last step (valid until the next
	   step's end): transforms and centers by body id, velocities and sleep times by awake
	   index */
	int mirrorValid;
	const float *mirrorXf, *mirrorCenter, *mirrorV, *mirrorSleep;
	const uint32_t* mirrorFlags;
	int jointsHostValid;	/* host joint records (impulses) match the device */
	int shapeBoxesValid;	/* host shape boxes (aabb) match the device */
	int moveEventsValid;	/* move event array matches the last step */
	int colorsDirty, jointsDirty;
	int uploadedTreeVersion[3];		 /* tree version last sent to the device */
	const void* uploadedTreeNodes[3]; /* node array it was sent from */
	H_ARRAY( b2gContactInit ) pendingInits;
	h_intArray pendingKills;
	h_intArray forcedBodies; /* bodies given a force or torque since the last step */
	int lastStatus;
	int continuousSweeps, continuousHits; /* accumulated device continuous-collision counters */
	struct h_tapeWorld* tape;			  /* differentiable-stepping recorder (diff.c), or NULL */
	/* the step in progress, between its phases (step.c) */
	b2gStepParams stepParams;
	float stepTimeStep;
	uint64_t stepTicks, stepT0;
	int stepPairsIssued, stepSolveIssued, stepSolveLate;
	/* the moved proxies' boxes and shapes sent with a pair query (reused buffers) */
	float* moveBoxes;
	int* moveShapes;
	int moveBufCap;
	/* the next step's pair query, issued at a step's end behind the state download; the next
	   step uses its results when nothing the query reads changed in between (the move keys
	   and boxes, the trees, the contacts), else drops it */
	int specIssued, specCount, specCap, specStale;
	int* specKeys;
	float* specBoxes;
	int specTreeVersion[3];
	void* rebuildWorker; /* host thread for the tree rebuild (step.c) */
} h_world;

h_world* h_worldFromId( b2WorldId id );
/* appends the step about to be solved to the world's tape when recording (diff.c) */
void h_tapeCapture( h_world* w, const b2gStepParams* params );
/* the step's phases (step.c): begin (issues the pair query), pairs (issues the narrowphase),
   collide (issues the solver), solve issue (a solve held back from a batch), finish */
int h_stepBegin( h_world* w, float timeStep, int subStepCount );
void h_stepPairs( h_world* w );
int h_stepCollide( h_world* w, int oneBlockOnly );
int h_stepSolveIssue( h_world* w );
void h_stepFinish( h_world* w );
void h_tapeDetach( h_world* w );

/* islands and solver sets (island.c: island.c, solver_set.c and the sleep pass of
   solver.c:2024-2080 in the reference) */
void h_islandsInit( h_world* w );
void h_islandsFree( h_world* w );
void h_createIslandForBody( h_world* w, int setIndex, h_body* body );
void h_linkContact( h_world* w, h_contact* contact );
void h_unlinkContact( h_world* w, h_contact* contact );
void h_linkJoint( h_world* w, h_joint* joint );
void h_unlinkJoint( h_world* w, h_joint* joint );
void h_removeBodyFromIsland( h_world* w, h_body* body );
void h_freeSleepingSet( h_world* w, int setIndex );
void h_splitIsland( h_world* w, int baseId );
void h_wakeSolverSet( h_world* w, int setIndex );
void h_trySleepIsland( h_world* w, int islandId );
void h_mergeSolverSets( h_world* w, int setId1, int setId2 );
int h_wakeBody( h_world* w, h_body* body );
int h_allocSleepingSet( h_world* w );
void h_removeJointFromGraph( h_world* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex );
void h_addJointToGraph( h_world* w, h_joint* joint );
/* per step: the split before the finalize, the finalize's island table, and the sleep pass
   over the finalize's awake-island bits and split candidate */
void h_stepIslands( h_world* w );
void h_sleepPass( h_world* w, const uint32_t* awakeIslandBits, uint64_t splitKey );
/* device work of sets that slept or woke: sent inside a step, or before the next one */
void h_flushSleepOps( h_world* w );
h_world* h_worldByIndex( int index );
/* the values b2World_GetStateHash mixes, in order, up to capacity; returns their count */
int h_stateHashWords( h_world* w, uint32_t* words, int capacity );

/* sensors (sensor.c): a new sensor shape's record; the overlap pass at the end of a step,
   its end events going to sensorEndEvents[endIndex]; records freed with the world */
void h_createSensor( h_world* w, h_shape* shape );
void h_overlapSensors( h_world* w, int endIndex );
void h_freeSensors( h_world* w );

/* geometry helpers (geometry.c) */
b2AABB h_computeFatShapeAABB( const h_shape* shape, b2Transform xf, float extra );
b2Vec2 h_getShapeCentroid( const h_shape* shape );
float h_computeShapeMargin( const h_shape* shape );
b2MassData h_computeShapeMass( const h_shape* shape );
void h_computeShapeExtent( const h_shape* shape, b2Vec2 localCenter, float* minExtent, float* maxExtent );

/* world.c internals used by step.c and joint.c */
void h_syncFromDevice( h_world* w );
/* the host records become authoritative: the device is refilled before the next step */
void h_markHostChanged( h_world* w );
/* the last step's move events, one per body awake at its finalize (solver.c:608-622) */
void h_buildMoveEvents( h_world* w );
void h_syncJointsFromDevice( h_world* w );
/* the shapes' tight boxes as the last finalize left them on the device */
void h_syncShapeBoxes( h_world* w );
/* frees every array of the world's simulation state; the device world, the rebuild worker
   and the tape stay (world.c) */
void h_freeWorldArrays( h_world* w );
/* drop the pair query issued at the last step's end, if any */
void h_dropSpeculativePairs( h_world* w );
/* the host thread pool (batch.c): fn(ctx, i) for i in [0, count) on up to `threads` threads,
   the caller among them; returns 0 without running anything when the pool is taken (by
   another thread, or by the caller itself inside a pool task): the caller then runs the
   loop alone */
int h_parallelFor( int threads, void ( *fn )( void*, int ), void* ctx, int count );
/* threads a step's host loops use: the online cores, at most 8 */
int h_hostThreads( void );
void h_ensureDevice( h_world* w );
void h_createContact( h_world* w, h_shape* a, h_shape* b );
void h_destroyContact( h_world* w, h_contact* c );
void h_addContactToGraph( h_world* w, h_contact* c );
void h_removeContactFromGraph( h_world* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex );
int h_assignJointColor( h_world* w, int bodyIdA, int bodyIdB, b2BodyType typeA, b2BodyType typeB );
int h_shouldBodiesCollide( h_world* w, h_body* a, h_body* b );
int h_canCollide( b2ShapeType a, b2ShapeType b );
int h_isPrimary( b2ShapeType a, b2ShapeType b );
void h_bufferMove( h_world* w, int proxyKey );
void h_fail( h_world* w, const char* what, int code );
void h_joinRebuild( h_world* w );
void h_stopRebuildWorker( h_world* w );

#define H_PROXY_TYPE( K ) ( (b2BodyType)( ( K ) & 3 ) )
#define H_PROXY_ID( K ) ( ( K ) >> 2 )
#define H_PROXY_KEY( ID, T ) ( ( ( ID ) << 2 ) | ( T ) )

/* host phases timed per step */
enum
{
	H_PHASE_TREE_UPLOAD = 0,
	H_PHASE_PAIR_QUERY = 1,	  /* device pair query call, includes its wait */
	H_PHASE_CONTACT_CREATE = 2,
	H_PHASE_TREE_REBUILD = 3,
	H_PHASE_COLLIDE = 4, /* device narrowphase call, includes its wait */
	H_PHASE_STATE_PASS = 5,
	H_PHASE_UPLOADS = 6, /* contact / color / joint uploads */
	H_PHASE_SOLVE = 7,	 /* device solver + finalize call, includes its wait */
	H_PHASE_ENLARGE = 8,
	H_PHASE_TAPE = 9, /* tape capture of differentiable stepping */
	H_PHASE_COUNT = 10,
};

#endif
