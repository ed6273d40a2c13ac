/*
 * box2d_gb300.h -- public C ABI of the GB300 step library.
 *
 * This header declares the subset of Box2D v3.2's public API (include/box2d/box2d.h,
 * types.h, collision.h, math_functions.h, id.h, base.h in the reference) that a program
 * needs to build worlds, step them and read results. Every struct below has the same
 * field order, types and size as the reference declaration it stands in for, so a
 * program compiled against the reference headers links against this library unchanged
 * (tests/test_abi.py compiles a layout probe against both headers where the reference
 * headers are present and requires identical sizes and offsets).
 *
 * float32 only: b2Pos is b2Vec2 and b2WorldTransform is b2Transform, as in the reference
 * when BOX2D_DOUBLE_PRECISION is off (math_functions.h:69-70).
 */
#ifndef BOX2D_GB300_H
#define BOX2D_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define B2G_API extern "C" __attribute__( ( visibility( "default" ) ) )
#define B2G_INLINE static inline
#define B2G_LITERAL( T ) T
#else
#define B2G_API __attribute__( ( visibility( "default" ) ) )
#define B2G_INLINE static inline
#define B2G_LITERAL( T ) ( T )
#endif

#define B2_NULL_INDEX ( -1 )
#define B2_MAX_POLYGON_VERTICES 8
#define B2_PI 3.14159265359f
#define B2_DEFAULT_CATEGORY_BITS 1
#define B2_DEFAULT_MASK_BITS UINT64_MAX
#define B2_GRAPH_COLOR_COUNT 24

/* ---- math types (math_functions.h:19-96) ---- */
typedef struct b2Vec2
{
	float x, y;
} b2Vec2;

typedef struct b2CosSin
{
	float cosine;
	float sine;
} b2CosSin;

typedef struct b2Rot
{
	float c, s;
} b2Rot;

typedef struct b2Transform
{
	b2Vec2 p;
	b2Rot q;
} b2Transform;

typedef b2Vec2 b2Pos;
typedef b2Transform b2WorldTransform;

typedef struct b2Mat22
{
	b2Vec2 cx, cy;
} b2Mat22;

typedef struct b2AABB
{
	b2Vec2 lowerBound;
	b2Vec2 upperBound;
} b2AABB;

typedef struct b2Plane
{
	b2Vec2 normal;
	float offset;
} b2Plane;

/* ---- ids (id.h:37-81) ---- */
typedef struct b2WorldId
{
	uint16_t index1;
	uint16_t generation;
} b2WorldId;

typedef struct b2BodyId
{
	int32_t index1;
	uint16_t world0;
	uint16_t generation;
} b2BodyId;

typedef struct b2ShapeId
{
	int32_t index1;
	uint16_t world0;
	uint16_t generation;
} b2ShapeId;

typedef struct b2JointId
{
	int32_t index1;
	uint16_t world0;
	uint16_t generation;
} b2JointId;

typedef struct b2ChainId
{
	int32_t index1;
	uint16_t world0;
	uint16_t generation;
} b2ChainId;

typedef struct b2ContactId
{
	int32_t index1;
	uint16_t world0;
	int16_t padding;
	uint32_t generation;
} b2ContactId;

#define B2_IS_NULL( id ) ( ( id ).index1 == 0 )
#define B2_IS_NON_NULL( id ) ( ( id ).index1 != 0 )

/* ---- geometry (collision.h) ---- */
typedef struct b2MassData
{
	float mass;
	b2Vec2 center;
	float rotationalInertia;
} b2MassData;

typedef struct b2Circle
{
	b2Vec2 center;
	float radius;
} b2Circle;

typedef struct b2Capsule
{
	b2Vec2 center1;
	b2Vec2 center2;
	float radius;
} b2Capsule;

typedef struct b2Polygon
{
	b2Vec2 vertices[B2_MAX_POLYGON_VERTICES];
	b2Vec2 normals[B2_MAX_POLYGON_VERTICES];
	b2Vec2 centroid;
	float radius;
	int count;
} b2Polygon;

typedef struct b2Segment
{
	b2Vec2 point1;
	b2Vec2 point2;
} b2Segment;

/* collision.h:184-197: a one-sided segment of a chain with its neighbors' far points */
typedef struct b2ChainSegment
{
	b2Vec2 ghost1;
	b2Segment segment;
	b2Vec2 ghost2;
	int chainId;
} b2ChainSegment;

typedef struct b2Hull
{
	b2Vec2 points[B2_MAX_POLYGON_VERTICES];
	int count;
} b2Hull;

typedef struct b2ManifoldPoint
{
	b2Vec2 anchorA;
	b2Vec2 anchorB;
	float separation;
	float baseSeparation;
	float normalImpulse;
	float tangentImpulse;
	float totalNormalImpulse;
	float normalVelocity;
	uint16_t id;
	bool persisted;
} b2ManifoldPoint;

typedef struct b2Manifold
{
	b2Vec2 normal;
	float rollingImpulse;
	b2ManifoldPoint points[2];
	int pointCount;
} b2Manifold;

typedef struct b2LocalManifoldPoint
{
	b2Vec2 point;
	float separation;
	uint16_t id;
} b2LocalManifoldPoint;

typedef struct b2LocalManifold
{
	b2Vec2 normal;
	b2LocalManifoldPoint points[2];
	int pointCount;
} b2LocalManifold;

/* ---- world / body / shape definitions (types.h) ---- */
typedef void b2TaskCallback( void* taskContext );
typedef void* b2EnqueueTaskCallback( b2TaskCallback* task, void* taskContext, void* userContext );
typedef void b2FinishTaskCallback( void* userTask, void* userContext );
typedef float b2FrictionCallback( float frictionA, uint64_t userMaterialIdA, float frictionB, uint64_t userMaterialIdB );
typedef float b2RestitutionCallback( float restitutionA, uint64_t userMaterialIdA, float restitutionB,
									 uint64_t userMaterialIdB );

typedef struct b2Capacity
{
	int staticShapeCount;
	int dynamicShapeCount;
	int staticBodyCount;
	int dynamicBodyCount;
	int contactCount;
} b2Capacity;

typedef struct b2WorldDef
{
	b2Vec2 gravity;
	float restitutionThreshold;
	float hitEventThreshold;
	float contactHertz;
	float contactDampingRatio;
	float contactSpeed;
	float maximumLinearSpeed;
	b2FrictionCallback* frictionCallback;
	b2RestitutionCallback* restitutionCallback;
	bool enableSleep;
	bool enableContinuous;
	bool enableContactSoftening;
	int workerCount;
	b2EnqueueTaskCallback* enqueueTask;
	b2FinishTaskCallback* finishTask;
	void* userTaskContext;
	void* userData;
	b2Capacity capacity;
	int internalValue;
} b2WorldDef;

typedef enum b2BodyType
{
	b2_staticBody = 0,
	b2_kinematicBody = 1,
	b2_dynamicBody = 2,
	b2_bodyTypeCount,
} b2BodyType;

typedef struct b2MotionLocks
{
	bool linearX;
	bool linearY;
	bool angularZ;
} b2MotionLocks;

typedef struct b2BodyDef
{
	b2BodyType type;
	b2Pos position;
	b2Rot rotation;
	b2Vec2 linearVelocity;
	float angularVelocity;
	float linearDamping;
	float angularDamping;
	float gravityScale;
	float sleepThreshold;
	float safetyFactor;
	const char* name;
	void* userData;
	b2MotionLocks motionLocks;
	bool enableSleep;
	bool isAwake;
	bool isBullet;
	bool isEnabled;
	bool allowFastRotation;
	bool enableContactRecycling;
	int internalValue;
} b2BodyDef;

typedef struct b2Filter
{
	uint64_t categoryBits;
	uint64_t maskBits;
	int groupIndex;
} b2Filter;

typedef enum b2ShapeType
{
	b2_circleShape,
	b2_capsuleShape,
	b2_segmentShape,
	b2_polygonShape,
	b2_chainSegmentShape,
	b2_shapeTypeCount
} b2ShapeType;

typedef struct b2SurfaceMaterial
{
	float friction;
	float restitution;
	float rollingResistance;
	float tangentSpeed;
	uint64_t userMaterialId;
	uint32_t customColor;
} b2SurfaceMaterial;

typedef struct b2ShapeDef
{
	void* userData;
	b2SurfaceMaterial material;
	float density;
	b2Filter filter;
	bool enableCustomFiltering;
	bool isSensor;
	bool enableSensorEvents;
	bool enableContactEvents;
	bool enableHitEvents;
	bool enablePreSolveEvents;
	bool invokeContactCreation;
	bool updateBodyMass;
	int internalValue;
} b2ShapeDef;

/* types.h:488-518 */
typedef struct b2ChainDef
{
	void* userData;
	const b2Vec2* points;
	int count;
	const b2SurfaceMaterial* materials;
	int materialCount;
	b2Filter filter;
	bool isLoop;
	bool enableSensorEvents;
	int internalValue;
} b2ChainDef;

typedef struct b2Profile
{
	float step;
	float pairs;
	float collide;
	float solve;
	float solverSetup;
	float constraints;
	float prepareConstraints;
	float integrateVelocities;
	float warmStart;
	float solveImpulses;
	float integratePositions;
	float relaxImpulses;
	float applyRestitution;
	float storeImpulses;
	float splitIslands;
	float transforms;
	float sensorHits;
	float jointEvents;
	float hitEvents;
	float refit;
	float bullets;
	float sleepIslands;
	float sensors;
} b2Profile;

typedef struct b2Counters
{
	int64_t byteCount;
	int bodyCount;
	int shapeCount;
	int contactCount;
	int jointCount;
	int islandCount;
	int stackUsed;
	int staticTreeHeight;
	int treeHeight;
	int taskCount;
	int colorCounts[24];
	int awakeContactCount;
	int recycledContactCount;
} b2Counters;

/* ---- joints (types.h b2JointDef family) ---- */
typedef enum b2JointType
{
	b2_distanceJoint,
	b2_filterJoint,
	b2_motorJoint,
	b2_moverJoint,
	b2_pogoJoint,
	b2_prismaticJoint,
	b2_revoluteJoint,
	b2_weldJoint,
	b2_wheelJoint,
} b2JointType;

typedef struct b2JointDef
{
	void* userData;
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Transform localFrameA;
	b2Transform localFrameB;
	float forceThreshold;
	float torqueThreshold;
	float constraintHertz;
	float constraintDampingRatio;
	float drawScale;
	bool collideConnected;
} b2JointDef;

typedef struct b2DistanceJointDef
{
	b2JointDef base;
	float length;
	bool enableSpring;
	float lowerSpringForce;
	float upperSpringForce;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float minLength;
	float maxLength;
	bool enableMotor;
	float maxMotorForce;
	float motorSpeed;
	int internalValue;
} b2DistanceJointDef;

typedef struct b2PrismaticJointDef
{
	b2JointDef base;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	float targetTranslation;
	bool enableLimit;
	float lowerTranslation;
	float upperTranslation;
	bool enableMotor;
	float maxMotorForce;
	float motorSpeed;
	int internalValue;
} b2PrismaticJointDef;

typedef struct b2RevoluteJointDef
{
	b2JointDef base;
	float targetAngle;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float lowerAngle;
	float upperAngle;
	bool enableMotor;
	float maxMotorTorque;
	float motorSpeed;
	int internalValue;
} b2RevoluteJointDef;

typedef struct b2WeldJointDef
{
	b2JointDef base;
	float linearHertz;
	float angularHertz;
	float linearDampingRatio;
	float angularDampingRatio;
	int internalValue;
} b2WeldJointDef;

typedef struct b2WheelJointDef
{
	b2JointDef base;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float lowerTranslation;
	float upperTranslation;
	bool enableMotor;
	float maxMotorTorque;
	float motorSpeed;
	int internalValue;
} b2WheelJointDef;

/* types.h:694-701: disables collision between two bodies, no constraint */
typedef struct b2FilterJointDef
{
	b2JointDef base;
	int internalValue;
} b2FilterJointDef;

/* types.h:710-747: relative velocity and spring control between two bodies */
typedef struct b2MotorJointDef
{
	b2JointDef base;
	b2Vec2 linearVelocity;
	float maxVelocityForce;
	float angularVelocity;
	float maxVelocityTorque;
	float linearHertz;
	float linearDampingRatio;
	float maxSpringForce;
	float angularHertz;
	float angularDampingRatio;
	float maxSpringTorque;
	int internalValue;
} b2MotorJointDef;

/* types.h:756-769: linear velocity control, x and y separately, no rotation */
typedef struct b2MoverJointDef
{
	b2JointDef base;
	b2Vec2 linearVelocity;
	b2Vec2 maxVelocityForce;
	int internalValue;
} b2MoverJointDef;

/* types.h:777-810: one-sided spring along a normal (character movers) */
typedef struct b2PogoJointDef
{
	b2JointDef base;
	b2Vec2 normal;
	float hertz;
	float dampingRatio;
	float restLength;
	float maxTensionForce;
	float maxCompressionForce;
	float impulse;
	float velocity;
	int internalValue;
} b2PogoJointDef;

/* ---- events (types.h) ---- */
typedef struct b2ContactBeginTouchEvent
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
	b2ContactId contactId;
} b2ContactBeginTouchEvent;

typedef struct b2ContactEndTouchEvent
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
	b2ContactId contactId;
} b2ContactEndTouchEvent;

typedef struct b2ContactHitEvent
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
	b2ContactId contactId;
	b2Pos point;
	b2Vec2 normal;
	float approachSpeed;
} b2ContactHitEvent;

typedef struct b2ContactEvents
{
	b2ContactBeginTouchEvent* beginEvents;
	b2ContactEndTouchEvent* endEvents;
	b2ContactHitEvent* hitEvents;
	int beginCount;
	int endCount;
	int hitCount;
} b2ContactEvents;

/* sensor events (types.h:1030-1073) */
typedef struct b2SensorBeginTouchEvent
{
	b2ShapeId sensorShapeId;
	b2ShapeId visitorShapeId;
} b2SensorBeginTouchEvent;

typedef struct b2SensorEndTouchEvent
{
	b2ShapeId sensorShapeId;
	b2ShapeId visitorShapeId;
} b2SensorEndTouchEvent;

typedef struct b2SensorEvents
{
	b2SensorBeginTouchEvent* beginEvents;
	b2SensorEndTouchEvent* endEvents;
	int beginCount;
	int endCount;
} b2SensorEvents;

typedef struct b2BodyMoveEvent
{
	void* userData;
	b2WorldTransform transform;
	b2BodyId bodyId;
	bool fellAsleep;
} b2BodyMoveEvent;

typedef struct b2BodyEvents
{
	b2BodyMoveEvent* moveEvents;
	int moveCount;
} b2BodyEvents;


/* ---- API: base (base.h:150-164) ---- */
B2G_API uint64_t b2GetTicks( void );
B2G_API float b2GetMilliseconds( uint64_t ticks );
B2G_API uint32_t b2Hash( uint32_t hash, const uint8_t* data, int count );

/* ---- API: math (math_functions.h, math_functions.c) ---- */
B2G_API float b2Atan2( float y, float x );
B2G_API b2CosSin b2ComputeCosSin( float radians );
B2G_API b2Rot b2MakeRot( float radians );

/* the reference's inline math, id helpers and constants */
#include "box2d_gb300_math.h"

/* ---- API: geometry (collision.h:160-230, geometry.c, hull.c) ---- */
B2G_API b2Hull b2ComputeHull( const b2Vec2* points, int count );
B2G_API b2Polygon b2MakePolygon( const b2Hull* hull, float radius );
B2G_API b2Polygon b2MakeOffsetPolygon( const b2Hull* hull, b2Vec2 position, b2Rot rotation );
B2G_API b2Polygon b2MakeSquare( float halfWidth );
B2G_API b2Polygon b2MakeBox( float halfWidth, float halfHeight );
B2G_API b2Polygon b2MakeRoundedBox( float halfWidth, float halfHeight, float radius );
B2G_API b2Polygon b2MakeOffsetBox( float halfWidth, float halfHeight, b2Vec2 center, b2Rot rotation );
B2G_API b2MassData b2ComputeCircleMass( const b2Circle* shape, float density );
B2G_API b2MassData b2ComputeCapsuleMass( const b2Capsule* shape, float density );
B2G_API b2MassData b2ComputePolygonMass( const b2Polygon* shape, float density );

/* ---- API: world (box2d.h:34-200) ---- */
B2G_API b2WorldDef b2DefaultWorldDef( void );
B2G_API b2BodyDef b2DefaultBodyDef( void );
B2G_API b2Filter b2DefaultFilter( void );
B2G_API b2ShapeDef b2DefaultShapeDef( void );
B2G_API b2SurfaceMaterial b2DefaultSurfaceMaterial( void );

B2G_API b2WorldId b2CreateWorld( const b2WorldDef* def );
B2G_API void b2DestroyWorld( b2WorldId worldId );
B2G_API bool b2World_IsValid( b2WorldId id );
B2G_API void b2World_Step( b2WorldId worldId, float timeStep, int subStepCount );
/* Step many independent worlds with the same time step and substeps, using up to
   threadCount host threads (no counterpart in the reference API). Each world ends exactly
   as a b2World_Step call on it would leave it. The worlds must be distinct; no other call
   may use them while the batch runs. */
B2G_API void b2World_StepBatch( const b2WorldId* worldIds, int worldCount, float timeStep, int subStepCount, int threadCount );
B2G_API b2BodyEvents b2World_GetBodyEvents( b2WorldId worldId );
B2G_API b2ContactEvents b2World_GetContactEvents( b2WorldId worldId );
B2G_API b2SensorEvents b2World_GetSensorEvents( b2WorldId worldId );
B2G_API void b2World_EnableSleeping( b2WorldId worldId, bool flag );
B2G_API bool b2World_IsSleepingEnabled( b2WorldId worldId );
B2G_API void b2World_EnableContinuous( b2WorldId worldId, bool flag );
B2G_API bool b2World_IsContinuousEnabled( b2WorldId worldId );
B2G_API void b2World_EnableWarmStarting( b2WorldId worldId, bool flag );
B2G_API void b2World_SetGravity( b2WorldId worldId, b2Vec2 gravity );
B2G_API b2Vec2 b2World_GetGravity( b2WorldId worldId );
B2G_API int b2World_GetAwakeBodyCount( b2WorldId worldId );
B2G_API b2Profile b2World_GetProfile( b2WorldId worldId );
B2G_API b2Counters b2World_GetCounters( b2WorldId worldId );
/* world_snapshot.c:1183 (box2d.h:235): FNV-1a 64 of the simulation state and bookkeeping */
B2G_API uint64_t b2World_GetStateHash( b2WorldId worldId );

/* ---- API: snapshots (world_snapshot.c; box2d.h:286-338) ----
   The world's simulation state at a step boundary as a caller-owned byte image. Call
   b2World_Snapshot with image == NULL for the size, then with a buffer of that size; it
   returns the size needed (nothing is written when capacity is smaller) and 0 inside a
   step. b2World_Restore rolls a world back to an image in place (ids held from that
   instant stay valid, ids minted later fail validation); a rejected image (bad magic,
   version, layout or checksum) leaves the world unchanged and returns false.
   b2CreateWorldFromSnapshot builds a new world from an image. Object user data is not
   stored and reads back as NULL. Images are for this library on the same machine type. */
B2G_API int b2World_Snapshot( b2WorldId worldId, uint8_t* image, int capacity );
B2G_API bool b2World_Restore( b2WorldId worldId, const uint8_t* image, int size );
B2G_API b2WorldId b2CreateWorldFromSnapshot( const uint8_t* image, int size, int workerCount );

/* ---- API: bodies (box2d.h:355-550) ---- */
B2G_API b2BodyId b2CreateBody( b2WorldId worldId, const b2BodyDef* def );
/* body.c:346 (box2d.h:359): its joints, contacts, shapes and chains go with it */
B2G_API void b2DestroyBody( b2BodyId bodyId );
B2G_API bool b2Body_IsValid( b2BodyId id );
B2G_API b2BodyType b2Body_GetType( b2BodyId bodyId );
B2G_API b2Pos b2Body_GetPosition( b2BodyId bodyId );
B2G_API b2Rot b2Body_GetRotation( b2BodyId bodyId );
B2G_API b2WorldTransform b2Body_GetTransform( b2BodyId bodyId );
B2G_API b2Vec2 b2Body_GetLocalPoint( b2BodyId bodyId, b2Pos worldPoint );
B2G_API b2Pos b2Body_GetWorldPoint( b2BodyId bodyId, b2Vec2 localPoint );
B2G_API b2Vec2 b2Body_GetLinearVelocity( b2BodyId bodyId );
B2G_API float b2Body_GetAngularVelocity( b2BodyId bodyId );
B2G_API void b2Body_SetLinearVelocity( b2BodyId bodyId, b2Vec2 linearVelocity );
B2G_API void b2Body_SetAngularVelocity( b2BodyId bodyId, float angularVelocity );
/* body.c:713, :842 and :935-1090 (box2d.h:396-490) */
B2G_API void b2Body_SetTransform( b2BodyId bodyId, b2Pos position, b2Rot rotation );
B2G_API void b2Body_SetTargetTransform( b2BodyId bodyId, b2WorldTransform target, float timeStep, bool wake );
B2G_API void b2Body_ApplyForce( b2BodyId bodyId, b2Vec2 force, b2Pos point, bool wake );
B2G_API void b2Body_ApplyForceToCenter( b2BodyId bodyId, b2Vec2 force, bool wake );
B2G_API void b2Body_ApplyTorque( b2BodyId bodyId, float torque, bool wake );
B2G_API void b2Body_ClearForces( b2BodyId bodyId );
B2G_API void b2Body_ApplyLinearImpulse( b2BodyId bodyId, b2Vec2 impulse, b2Pos point, bool wake );
B2G_API void b2Body_ApplyLinearImpulseToCenter( b2BodyId bodyId, b2Vec2 impulse, bool wake );
B2G_API void b2Body_ApplyAngularImpulse( b2BodyId bodyId, float impulse, bool wake );
B2G_API float b2Body_GetMass( b2BodyId bodyId );
B2G_API float b2Body_GetRotationalInertia( b2BodyId bodyId );
B2G_API b2Vec2 b2Body_GetLocalCenter( b2BodyId bodyId );
B2G_API b2Pos b2Body_GetWorldCenter( b2BodyId bodyId );
B2G_API bool b2Body_IsAwake( b2BodyId bodyId );
/* body.c b2Body_SetAwake (box2d.h:552): wake the body's sleeping set, or put its island
   to sleep */
B2G_API void b2Body_SetAwake( b2BodyId bodyId, bool awake );
/* body.c b2Body_GetSleepThreshold (box2d.h:567) */
B2G_API float b2Body_GetSleepThreshold( b2BodyId bodyId );

/* ---- API: shapes (box2d.h:659-724) ---- */
B2G_API b2ShapeId b2CreateCircleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Circle* circle );
B2G_API b2ShapeId b2CreateSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Segment* segment );
/* chains (shape.c:300-315, :439-640; box2d.h:860-900) */
B2G_API b2ChainDef b2DefaultChainDef( void );
B2G_API b2ChainId b2CreateChain( b2BodyId bodyId, const b2ChainDef* def );
B2G_API void b2DestroyChain( b2ChainId chainId );
B2G_API bool b2Chain_IsValid( b2ChainId id );
B2G_API int b2Chain_GetSegmentCount( b2ChainId chainId );
B2G_API int b2Chain_GetSegments( b2ChainId chainId, b2ShapeId* segmentArray, int capacity );
B2G_API b2ShapeId b2CreateChainSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2ChainSegment* chainSegment );
/* shape.c (box2d.h:689, :859) */
B2G_API bool b2Shape_IsValid( b2ShapeId id );
B2G_API b2AABB b2Shape_GetAABB( b2ShapeId shapeId );
B2G_API b2ShapeType b2Shape_GetType( b2ShapeId shapeId );
B2G_API b2ChainSegment b2Shape_GetChainSegment( b2ShapeId shapeId );
B2G_API b2ChainId b2Shape_GetParentChain( b2ShapeId shapeId );
B2G_API b2ShapeId b2CreateCapsuleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Capsule* capsule );
B2G_API b2ShapeId b2CreatePolygonShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Polygon* polygon );
/* shape.c:411 (box2d.h:686) */
B2G_API void b2DestroyShape( b2ShapeId shapeId, bool updateBodyMass );
B2G_API void b2Shape_SetFriction( b2ShapeId shapeId, float friction );
/* sensors (shape.c:1109, :1400-1415, :1780-1825; box2d.h:703-856) */
B2G_API bool b2Shape_IsSensor( b2ShapeId shapeId );
B2G_API void b2Shape_EnableSensorEvents( b2ShapeId shapeId, bool flag );
B2G_API bool b2Shape_AreSensorEventsEnabled( b2ShapeId shapeId );
B2G_API int b2Shape_GetSensorCapacity( b2ShapeId shapeId );
B2G_API int b2Shape_GetSensorData( b2ShapeId shapeId, b2ShapeId* visitorIds, int capacity );
B2G_API float b2Shape_GetFriction( b2ShapeId shapeId );
B2G_API int b2Body_GetShapeCount( b2BodyId bodyId );
B2G_API int b2Body_GetShapes( b2BodyId bodyId, b2ShapeId* shapeArray, int capacity );

/* ---- API: joints (box2d.h:760-1100) ---- */
B2G_API b2DistanceJointDef b2DefaultDistanceJointDef( void );
B2G_API b2PrismaticJointDef b2DefaultPrismaticJointDef( void );
B2G_API b2RevoluteJointDef b2DefaultRevoluteJointDef( void );
B2G_API b2WeldJointDef b2DefaultWeldJointDef( void );
B2G_API b2WheelJointDef b2DefaultWheelJointDef( void );
B2G_API b2JointId b2CreateDistanceJoint( b2WorldId worldId, const b2DistanceJointDef* def );
B2G_API b2JointId b2CreatePrismaticJoint( b2WorldId worldId, const b2PrismaticJointDef* def );
B2G_API b2JointId b2CreateRevoluteJoint( b2WorldId worldId, const b2RevoluteJointDef* def );
B2G_API b2JointId b2CreateWeldJoint( b2WorldId worldId, const b2WeldJointDef* def );
B2G_API b2JointId b2CreateWheelJoint( b2WorldId worldId, const b2WheelJointDef* def );
/* types.h:705, :751, :814 and box2d.h:1091, :1109, :1207 */
B2G_API b2FilterJointDef b2DefaultFilterJointDef( void );
B2G_API b2MotorJointDef b2DefaultMotorJointDef( void );
B2G_API b2PogoJointDef b2DefaultPogoJointDef( void );
/* types.h:773 and box2d.h b2CreateMoverJoint */
B2G_API b2MoverJointDef b2DefaultMoverJointDef( void );
B2G_API b2JointId b2CreateMoverJoint( b2WorldId worldId, const b2MoverJointDef* def );
B2G_API b2JointId b2CreateFilterJoint( b2WorldId worldId, const b2FilterJointDef* def );
B2G_API b2JointId b2CreateMotorJoint( b2WorldId worldId, const b2MotorJointDef* def );
B2G_API b2JointId b2CreatePogoJoint( b2WorldId worldId, const b2PogoJointDef* def );
/* joint.c:823 (box2d.h:919) */
B2G_API void b2DestroyJoint( b2JointId jointId );
/* joint.c (box2d.h:922) */
B2G_API bool b2Joint_IsValid( b2JointId id );
B2G_API b2JointType b2Joint_GetType( b2JointId jointId );
B2G_API float b2RevoluteJoint_GetAngle( b2JointId jointId );

#endif /* BOX2D_GB300_H */
