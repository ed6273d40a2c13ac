/*
 * Oracle for the GB300 Box2D step: a serial CPU restatement of Box2D v3.2's step
 * (b2World_Step, physics_world.c:845-1005) used ONLY as the test checker and as the
 * timed CPU baseline. It is test infrastructure: the product library never links it.
 *
 * Parity is pinned against the reference itself: oracle/ref/Makefile compiles the
 * reference sources into oracle/_ref/ and tests/golden/make_golden.py records per-step
 * state hashes, contact tables and colors from it; tests/test_oracle_pin.py checks the
 * oracle against those fixtures bit for bit.
 *
 * Floating point follows the reference's operation order exactly. Build with
 * -ffp-contract=off (the reference forces it, CMakeLists.txt:53-66).
 */
#ifndef O_CORE_H
#define O_CORE_H

#include "box2d_gb300.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define O_LINEAR_SLOP 0.005f
#define O_SPECULATIVE_DISTANCE ( 4.0f * O_LINEAR_SLOP )
#define O_AABB_MARGIN 0.05f
#define O_AABB_MARGIN_FRACTION 0.125f
#define O_HUGE 100000.0f
#define O_MAX_ROTATION ( 0.25f * B2_PI )
#define O_CONTACT_RECYCLE_DISTANCE ( 10.0f * O_LINEAR_SLOP )
#define O_CONTACT_RECYCLE_COS_ANGLE 0.98f
#define O_TIME_TO_SLEEP 0.5f
#define O_OVERFLOW_INDEX ( B2_GRAPH_COLOR_COUNT - 1 )
#define O_DYNAMIC_COLOR_COUNT ( B2_GRAPH_COLOR_COUNT - 4 )
#define O_MAX_WORLDS 128
#define O_SIMD_WIDTH 4

/* ---------------- scalar math, same operation order as math_functions.h ---------------- */
static inline float o_min( float a, float b ) { return a < b ? a : b; }
static inline float o_max( float a, float b ) { return a > b ? a : b; }
static inline float o_abs( float a ) { return a < 0 ? -a : a; }
static inline float o_clamp( float a, float lo, float hi ) { return a < lo ? lo : ( a > hi ? hi : a ); }
static inline int o_mini( int a, int b ) { return a < b ? a : b; }
static inline int o_maxi( int a, int b ) { return a > b ? a : b; }
static inline b2Vec2 o_v( float x, float y ) { b2Vec2 v = { x, y }; return v; }
static inline float o_dot( b2Vec2 a, b2Vec2 b ) { return a.x * b.x + a.y * b.y; }
static inline float o_cross( b2Vec2 a, b2Vec2 b ) { return a.x * b.y - a.y * b.x; }
static inline b2Vec2 o_crossVS( b2Vec2 v, float s ) { return o_v( s * v.y, -s * v.x ); }
static inline b2Vec2 o_crossSV( float s, b2Vec2 v ) { return o_v( -s * v.y, s * v.x ); }
static inline b2Vec2 o_leftPerp( b2Vec2 v ) { return o_v( -v.y, v.x ); }
static inline b2Vec2 o_rightPerp( b2Vec2 v ) { return o_v( v.y, -v.x ); }
static inline b2Vec2 o_add( b2Vec2 a, b2Vec2 b ) { return o_v( a.x + b.x, a.y + b.y ); }
static inline b2Vec2 o_sub( b2Vec2 a, b2Vec2 b ) { return o_v( a.x - b.x, a.y - b.y ); }
static inline b2Vec2 o_neg( b2Vec2 a ) { return o_v( -a.x, -a.y ); }
static inline b2Vec2 o_lerp( b2Vec2 a, b2Vec2 b, float t ) { return o_v( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y ); }
static inline b2Vec2 o_mulSV( float s, b2Vec2 v ) { return o_v( s * v.x, s * v.y ); }
static inline b2Vec2 o_mulAdd( b2Vec2 a, float s, b2Vec2 b ) { return o_v( a.x + s * b.x, a.y + s * b.y ); }
static inline b2Vec2 o_mulSub( b2Vec2 a, float s, b2Vec2 b ) { return o_v( a.x - s * b.x, a.y - s * b.y ); }
static inline b2Vec2 o_vmin( b2Vec2 a, b2Vec2 b ) { return o_v( o_min( a.x, b.x ), o_min( a.y, b.y ) ); }
static inline b2Vec2 o_vmax( b2Vec2 a, b2Vec2 b ) { return o_v( o_max( a.x, b.x ), o_max( a.y, b.y ) ); }
static inline float o_length( b2Vec2 v ) { return sqrtf( v.x * v.x + v.y * v.y ); }
static inline float o_lengthSq( b2Vec2 v ) { return v.x * v.x + v.y * v.y; }
static inline float o_distance( b2Vec2 a, b2Vec2 b )
{
	float dx = b.x - a.x, dy = b.y - a.y;
	return sqrtf( dx * dx + dy * dy );
}
static inline float o_distanceSq( b2Vec2 a, b2Vec2 b )
{
	b2Vec2 c = { b.x - a.x, b.y - a.y };
	return c.x * c.x + c.y * c.y;
}
static inline b2Vec2 o_normalize( b2Vec2 a )
{
	float ls = a.x * a.x + a.y * a.y;
	if ( ls > 1000.0f * FLT_MIN )
	{
		float s = 1.0f / sqrtf( ls );
		return o_v( s * a.x, s * a.y );
	}
	return o_v( 0.0f, 0.0f );
}
static inline b2Vec2 o_getLengthAndNormalize( float* length, b2Vec2 a )
{
	float ls = a.x * a.x + a.y * a.y;
	if ( ls > 1000.0f * FLT_MIN )
	{
		*length = sqrtf( ls );
		float s = 1.0f / *length;
		return o_v( s * a.x, s * a.y );
	}
	*length = 0.0f;
	return o_v( 0.0f, 0.0f );
}
static inline b2Rot o_normalizeRot( b2Rot q )
{
	float mag = sqrtf( q.s * q.s + q.c * q.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot r = { q.c * inv, q.s * inv };
	return r;
}
static inline b2Rot o_integrateRotation( b2Rot q1, float da )
{
	b2Rot q2 = { q1.c - da * q1.s, q1.s + da * q1.c };
	float mag = sqrtf( q2.s * q2.s + q2.c * q2.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot r = { q2.c * inv, q2.s * inv };
	return r;
}
static inline b2Rot o_nlerp( b2Rot q1, b2Rot q2, float t )
{
	float omt = 1.0f - t;
	b2Rot q = { omt * q1.c + t * q2.c, omt * q1.s + t * q2.s };
	return o_normalizeRot( q );
}
static inline b2Rot o_mulRot( b2Rot q, b2Rot r )
{
	b2Rot qr;
	qr.s = q.s * r.c + q.c * r.s;
	qr.c = q.c * r.c - q.s * r.s;
	return qr;
}
static inline b2Rot o_invMulRot( b2Rot a, b2Rot b )
{
	b2Rot r;
	r.s = a.c * b.s - a.s * b.c;
	r.c = a.c * b.c + a.s * b.s;
	return r;
}
static inline b2Rot o_invertRot( b2Rot a ) { b2Rot r = { a.c, -a.s }; return r; }
static inline b2Vec2 o_rotate( b2Rot q, b2Vec2 v ) { return o_v( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
static inline b2Vec2 o_invRotate( b2Rot q, b2Vec2 v ) { return o_v( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }
static inline b2Vec2 o_transformPoint( b2Transform t, b2Vec2 p )
{
	float x = ( t.q.c * p.x - t.q.s * p.y ) + t.p.x;
	float y = ( t.q.s * p.x + t.q.c * p.y ) + t.p.y;
	return o_v( x, y );
}
static inline b2Vec2 o_invTransformPoint( b2Transform t, b2Vec2 p )
{
	float vx = p.x - t.p.x, vy = p.y - t.p.y;
	return o_v( t.q.c * vx + t.q.s * vy, -t.q.s * vx + t.q.c * vy );
}
/* b2TransformWorldPoint (math_functions.h:577-582): rotation first, then offset */
static inline b2Vec2 o_transformWorldPoint( b2Transform t, b2Vec2 p )
{
	float rx = t.q.c * p.x - t.q.s * p.y;
	float ry = t.q.s * p.x + t.q.c * p.y;
	return o_v( t.p.x + rx, t.p.y + ry );
}
static inline b2Transform o_invMulTransforms( b2Transform A, b2Transform B )
{
	b2Transform C;
	C.q = o_invMulRot( A.q, B.q );
	b2Vec2 d = { B.p.x - A.p.x, B.p.y - A.p.y };
	C.p = o_invRotate( A.q, d );
	return C;
}
static inline float o_relativeCos( b2Rot a, b2Rot b ) { return a.c * b.c + a.s * b.s; }
static inline int o_aabbOverlaps( b2AABB a, b2AABB b )
{
	return !( b.lowerBound.x > a.upperBound.x || b.lowerBound.y > a.upperBound.y || a.lowerBound.x > b.upperBound.x ||
			  a.lowerBound.y > b.upperBound.y );
}
static inline int o_aabbContains( b2AABB a, b2AABB b )
{
	int s = 1;
	s = s && a.lowerBound.x <= b.lowerBound.x;
	s = s && a.lowerBound.y <= b.lowerBound.y;
	s = s && b.upperBound.x <= a.upperBound.x;
	s = s && b.upperBound.y <= a.upperBound.y;
	return s;
}
static inline b2AABB o_aabbUnion( b2AABB a, b2AABB b )
{
	b2AABB c;
	c.lowerBound.x = o_min( a.lowerBound.x, b.lowerBound.x );
	c.lowerBound.y = o_min( a.lowerBound.y, b.lowerBound.y );
	c.upperBound.x = o_max( a.upperBound.x, b.upperBound.x );
	c.upperBound.y = o_max( a.upperBound.y, b.upperBound.y );
	return c;
}
static inline b2Vec2 o_aabbCenter( b2AABB a )
{
	return o_v( 0.5f * ( a.lowerBound.x + a.upperBound.x ), 0.5f * ( a.lowerBound.y + a.upperBound.y ) );
}
static inline float o_perimeter( b2AABB a )
{
	float wx = a.upperBound.x - a.lowerBound.x;
	float wy = a.upperBound.y - a.lowerBound.y;
	return 2.0f * ( wx + wy );
}
static inline int o_enlargeAABB( b2AABB* a, b2AABB b )
{
	int changed = 0;
	if ( b.lowerBound.x < a->lowerBound.x ) { a->lowerBound.x = b.lowerBound.x; changed = 1; }
	if ( b.lowerBound.y < a->lowerBound.y ) { a->lowerBound.y = b.lowerBound.y; changed = 1; }
	if ( a->upperBound.x < b.upperBound.x ) { a->upperBound.x = b.upperBound.x; changed = 1; }
	if ( a->upperBound.y < b.upperBound.y ) { a->upperBound.y = b.upperBound.y; changed = 1; }
	return changed;
}
static inline int o_isValidFloat( float a ) { return !isnan( a ) && !isinf( a ); }

/* ---------------- growable arrays ---------------- */
#define O_ARRAY( T ) struct { T* data; int count; int capacity; }
#define o_reserve( a, n )                                                                                                      \
	do                                                                                                                           \
	{                                                                                                                            \
		if ( ( n ) > ( a ).capacity )                                                                                            \
		{                                                                                                                        \
			int nc_ = ( a ).capacity == 0 ? 8 : ( a ).capacity;                                                                  \
			while ( nc_ < ( n ) ) nc_ *= 2;                                                                                      \
			( a ).data = realloc( ( a ).data, (size_t)nc_ * sizeof( *( a ).data ) );                                            \
			( a ).capacity = nc_;                                                                                                \
		}                                                                                                                        \
	} while ( 0 )
#define o_push( a, v )                                                                                                         \
	do                                                                                                                           \
	{                                                                                                                            \
		o_reserve( a, ( a ).count + 1 );                                                                                         \
		( a ).data[( a ).count++] = ( v );                                                                                       \
	} while ( 0 )
#define o_free( a )                                                                                                            \
	do                                                                                                                           \
	{                                                                                                                            \
		free( ( a ).data );                                                                                                      \
		( a ).data = NULL;                                                                                                       \
		( a ).count = ( a ).capacity = 0;                                                                                        \
	} while ( 0 )
/* swap-remove; returns the index that moved into 'index' or -1 (container.h:136-150) */
#define o_removeSwap( a, index ) o_removeSwapHelper( ( a ).data, &( a ).count, ( index ), (int)sizeof( *( a ).data ) )
static inline int o_removeSwapHelper( void* data, int* count, int index, int size )
{
	( *count )--;
	if ( index != *count )
	{
		memcpy( (char*)data + (size_t)index * size, (char*)data + (size_t)( *count ) * size, size );
		return *count;
	}
	return -1;
}

typedef O_ARRAY( int ) o_intArray;

/* LIFO id pool (id_pool.c:19-38) */
typedef struct o_idPool
{
	o_intArray freeArray;
	int nextIndex;
} o_idPool;
static inline int o_allocId( o_idPool* p )
{
	if ( p->freeArray.count > 0 ) return p->freeArray.data[--p->freeArray.count];
	return p->nextIndex++;
}
static inline void o_freeId( o_idPool* p, int id ) { o_push( p->freeArray, id ); }

/* bit set */
typedef struct o_bitSet
{
	uint64_t* bits;
	int blockCount;
} o_bitSet;
static inline void o_bitGrow( o_bitSet* s, int bit )
{
	int need = bit / 64 + 1;
	if ( need > s->blockCount )
	{
		int nb = s->blockCount == 0 ? 16 : s->blockCount;
		while ( nb < need ) nb *= 2;
		s->bits = realloc( s->bits, (size_t)nb * 8 );
		memset( s->bits + s->blockCount, 0, (size_t)( nb - s->blockCount ) * 8 );
		s->blockCount = nb;
	}
}
static inline void o_bitSet1( o_bitSet* s, int bit ) { o_bitGrow( s, bit ); s->bits[bit / 64] |= ( 1ull << ( bit % 64 ) ); }
/* for parallel loops: the set must already hold `bit` */
static inline void o_bitSet1Atomic( o_bitSet* s, int bit )
{
	__atomic_fetch_or( s->bits + bit / 64, 1ull << ( bit % 64 ), __ATOMIC_RELAXED );
}
static inline void o_bitClear( o_bitSet* s, int bit )
{
	if ( bit / 64 < s->blockCount ) s->bits[bit / 64] &= ~( 1ull << ( bit % 64 ) );
}
static inline int o_bitGet( const o_bitSet* s, int bit )
{
	if ( bit / 64 >= s->blockCount ) return 0;
	return ( s->bits[bit / 64] >> ( bit % 64 ) ) & 1;
}
static inline void o_bitReset( o_bitSet* s, int bitCount )
{
	o_bitGrow( s, bitCount > 0 ? bitCount - 1 : 0 );
	memset( s->bits, 0, (size_t)s->blockCount * 8 );
}

/* open addressing set of uint64 pair keys (membership only; order never observed) */
typedef struct o_pairSet
{
	uint64_t* keys;
	int capacity;
	int count;
} o_pairSet;
void o_pairSetAdd( o_pairSet* s, uint64_t key );
int o_pairSetContains( const o_pairSet* s, uint64_t key );
void o_pairSetRemove( o_pairSet* s, uint64_t key );
void o_pairSetFree( o_pairSet* s );
#define O_SHAPE_PAIR_KEY( K1, K2 ) ( ( K1 ) < ( K2 ) ? (uint64_t)( K1 ) << 32 | (uint64_t)( K2 ) : (uint64_t)( K2 ) << 32 | (uint64_t)( K1 ) )

/* ---------------- dynamic tree (dynamic_tree.c) ---------------- */
enum
{
	O_NODE_ALLOCATED = 0x0001,
	O_NODE_ENLARGED = 0x0002,
	O_NODE_LEAF = 0x0004,
};

typedef struct o_treeNode
{
	b2AABB aabb;
	uint64_t categoryBits;
	int child1, child2; /* internal nodes */
	uint64_t userData;	/* leaves */
	int parent;			/* doubles as free-list next */
	uint16_t height;
	uint16_t flags;
} o_treeNode;

typedef struct o_tree
{
	o_treeNode* nodes;
	int root, nodeCount, nodeCapacity, freeList, proxyCount;
	int* leafIndices;
	b2Vec2* leafCenters;
	int rebuildCapacity;
} o_tree;

o_tree o_treeCreate( int proxyCapacity );
void o_treeDestroy( o_tree* t );
int o_treeCreateProxy( o_tree* t, b2AABB aabb, uint64_t categoryBits, uint64_t userData );
void o_treeDestroyProxy( o_tree* t, int proxyId );
void o_treeMoveProxy( o_tree* t, int proxyId, b2AABB aabb );
void o_treeEnlargeProxy( o_tree* t, int proxyId, b2AABB aabb );
int o_treeRebuild( o_tree* t, int fullBuild );
typedef int o_treeQueryFcn( int proxyId, uint64_t userData, void* ctx );
void o_treeQuery( const o_tree* t, b2AABB aabb, uint64_t maskBits, o_treeQueryFcn* fcn, void* ctx );
int o_treeHeight( const o_tree* t );

/* ---------------- world model ---------------- */
enum
{
	O_LOCK_X = 0x1,
	O_LOCK_Y = 0x2,
	O_LOCK_Z = 0x4,
	O_IS_FAST = 0x8,
	O_IS_BULLET = 0x10,
	O_SPEED_CAPPED = 0x20,
	O_HAD_TOI = 0x40,
	O_ALLOW_FAST_ROTATION = 0x80,
	O_ENLARGE_BOUNDS = 0x100,
	O_DYNAMIC_FLAG = 0x200,
	O_DIRTY_MASS = 0x400,
	O_ENABLE_SLEEP = 0x800,
	O_ENABLE_RECYCLING = 0x1000,
	O_TRANSIENT = O_IS_FAST | O_SPEED_CAPPED | O_HAD_TOI,
};

enum
{
	O_C_TOUCHING = 0x1,
	O_C_HIT_EVENT = 0x2,
	O_C_ENABLE_EVENTS = 0x4,
	O_C_RECYCLE = 0x8,
	O_S_TOUCHING = 0x10000,
	O_S_DISJOINT = 0x20000,
	O_S_STARTED = 0x40000,
	O_S_STOPPED = 0x80000,
	O_S_HIT_EVENT = 0x100000,
	O_S_PRESOLVE = 0x200000,
	O_S_RELATIVE_VALID = 0x400000,
};

enum
{
	O_STATIC_SET = 0,
	O_DISABLED_SET = 1,
	O_AWAKE_SET = 2,
};

typedef struct o_bodyState
{
	b2Vec2 linearVelocity;
	float angularVelocity;
	uint32_t flags;
	b2Vec2 deltaPosition;
	b2Rot deltaRotation;
} o_bodyState;

typedef struct o_bodySim
{
	b2Transform transform;
	b2Vec2 center;
	b2Rot rotation0;
	b2Vec2 center0;
	b2Vec2 localCenter;
	b2Vec2 force;
	float torque;
	float invMass, invInertia;
	float minExtent, maxExtent;
	float linearDamping, angularDamping, gravityScale;
	int bodyId;
	uint32_t flags;
} o_bodySim;

typedef struct o_body
{
	void* userData;
	int setIndex, localIndex;
	int headContactKey, contactCount;
	int headShapeId, shapeCount;
	int headJointKey, jointCount;
	float mass, inertia;
	float sleepThreshold, sleepTime, safetyFactor;
	int id;
	uint32_t flags;
	b2BodyType type;
	uint16_t generation;
} o_body;

typedef struct o_shape
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
	};
	uint16_t generation;
	int enableContactEvents, enableHitEvents, enlargedAABB, isSensor;
} o_shape;

typedef struct o_contactEdge
{
	int bodyId, prevKey, nextKey;
} o_contactEdge;

typedef struct o_contact
{
	o_contactEdge edges[2];
	int setIndex, colorIndex, localIndex;
	int shapeIdA, shapeIdB, contactId;
	uint32_t flags, generation;
} o_contact;

typedef struct o_contactSim
{
	int contactId;
	b2Rot cachedRotationA, cachedRotationB;
	b2Transform cachedRelativePose;
	int bodySimIndexA, bodySimIndexB;
	int shapeIdA, shapeIdB;
	float invMassA, invIA, invMassB, invIB;
	b2Manifold manifold;
	float friction, restitution, rollingResistance, tangentSpeed;
	uint32_t simFlags;
} o_contactSim;

typedef O_ARRAY( o_contactSim ) o_contactSimArray;

/* joints (joint.h) -- shared fields plus a per-type union */
typedef struct o_jointSim o_jointSim;
typedef O_ARRAY( o_jointSim ) o_jointSimArray;

typedef struct o_graphColor
{
	o_bitSet bodySet;
	o_contactSimArray contactSims;
	o_jointSimArray jointSims;
} o_graphColor;

typedef struct o_softness
{
	float biasRate, massScale, impulseScale;
} o_softness;

static inline o_softness o_makeSoft( float hertz, float zeta, float h )
{
	o_softness s = { 0.0f, 0.0f, 0.0f };
	if ( hertz == 0.0f ) return s;
	float omega = 2.0f * B2_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	s.biasRate = omega / a1;
	s.massScale = a2 * a3;
	s.impulseScale = a3;
	return s;
}

/* per-type joint solver data (joint.h:29-250) */
typedef struct o_distanceJoint
{
	float length, hertz, dampingRatio, lowerSpringForce, upperSpringForce, minLength, maxLength, maxMotorForce, motorSpeed;
	float impulse, lowerImpulse, upperImpulse, motorImpulse;
	int indexA, indexB;
	b2Vec2 anchorA, anchorB, deltaCenter;
	o_softness distanceSoftness;
	float axialMass;
	int enableSpring, enableLimit, enableMotor;
} o_distanceJoint;

typedef struct o_prismaticJoint
{
	b2Vec2 impulse;
	float springImpulse, motorImpulse, lowerImpulse, upperImpulse;
	float hertz, dampingRatio, targetTranslation, maxMotorForce, motorSpeed, lowerTranslation, upperTranslation;
	int indexA, indexB;
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	o_softness springSoftness;
	int enableSpring, enableLimit, enableMotor;
} o_prismaticJoint;

typedef struct o_revoluteJoint
{
	b2Vec2 linearImpulse;
	float springImpulse, motorImpulse, lowerImpulse, upperImpulse;
	float hertz, dampingRatio, targetAngle, maxMotorTorque, motorSpeed, lowerAngle, upperAngle;
	int indexA, indexB;
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	float axialMass;
	o_softness springSoftness;
	int enableSpring, enableMotor, enableLimit;
} o_revoluteJoint;

typedef struct o_weldJoint
{
	float linearHertz, linearDampingRatio, angularHertz, angularDampingRatio;
	o_softness linearSpring, angularSpring;
	b2Vec2 linearImpulse;
	float angularImpulse;
	int indexA, indexB;
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	float axialMass;
} o_weldJoint;

typedef struct o_wheelJoint
{
	float perpImpulse, motorImpulse, springImpulse, lowerImpulse, upperImpulse;
	float maxMotorTorque, motorSpeed, lowerTranslation, upperTranslation, hertz, dampingRatio;
	int indexA, indexB;
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	float perpMass, motorMass, axialMass;
	o_softness springSoftness;
	int enableSpring, enableMotor, enableLimit;
} o_wheelJoint;

/* joint.h b2MotorJoint */
typedef struct o_motorJoint
{
	b2Vec2 linearVelocity;
	float maxVelocityForce, angularVelocity, maxVelocityTorque;
	float linearHertz, linearDampingRatio, maxSpringForce, angularHertz, angularDampingRatio, maxSpringTorque;
	b2Vec2 linearVelocityImpulse;
	float angularVelocityImpulse;
	b2Vec2 linearSpringImpulse;
	float angularSpringImpulse;
	o_softness linearSpring, angularSpring;
	int indexA, indexB;
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	b2Vec2 linearMassCx, linearMassCy; /* b2Mat22 columns */
	float angularMass;
} o_motorJoint;

/* joint.h b2MoverJoint */
typedef struct o_moverJoint
{
	b2Vec2 linearVelocity, maxVelocityForce, linearVelocityImpulse;
	float linearMass;
	int indexA, indexB;
} o_moverJoint;

/* joint.h b2PogoJoint */
typedef struct o_pogoJoint
{
	b2Vec2 normal;
	float hertz, dampingRatio, restLength, maxTensionForce, maxCompressionForce;
	float impulse, velocity;
	int indexA, indexB;
	b2Transform frameA, frameB;
	b2Vec2 deltaCenter;
	float linearMass;
} o_pogoJoint;

struct o_jointSim
{
	int jointId, bodyIdA, bodyIdB;
	b2JointType type;
	b2Transform localFrameA, localFrameB;
	float invMassA, invMassB, invIA, invIB;
	float constraintHertz, constraintDampingRatio;
	o_softness constraintSoftness;
	float forceThreshold, torqueThreshold;
	union
	{
		o_distanceJoint distanceJoint;
		o_prismaticJoint prismaticJoint;
		o_revoluteJoint revoluteJoint;
		o_weldJoint weldJoint;
		o_wheelJoint wheelJoint;
		o_motorJoint motorJoint;
		o_pogoJoint pogoJoint;
		o_moverJoint moverJoint;
	};
};

typedef struct o_jointEdge
{
	int bodyId, prevKey, nextKey;
} o_jointEdge;

struct o_joint
{
	void* userData;
	int setIndex, colorIndex, localIndex;
	o_jointEdge edges[2];
	int jointId;
	b2JointType type;
	uint16_t generation;
	int collideConnected;
};

typedef struct o_stepContext
{
	float dt, inv_dt, h, inv_h;
	int subStepCount;
	o_softness contactSoftness, staticSoftness;
	float restitutionThreshold, maxLinearVelocity;
	int enableWarmStarting;
} o_stepContext;

typedef struct o_joint o_joint;
typedef O_ARRAY( o_joint ) o_jointArray;

typedef struct o_world
{
	int inUse;
	uint16_t worldId, generation;
	o_idPool bodyIdPool, shapeIdPool, contactIdPool, jointIdPool;
	O_ARRAY( o_body ) bodies;
	O_ARRAY( o_shape ) shapes;
	O_ARRAY( o_contact ) contacts;
	o_jointArray joints;
	/* awake set */
	O_ARRAY( o_bodySim ) awakeSims;
	O_ARRAY( o_bodyState ) awakeStates;
	o_contactSimArray awakeContactSims;
	/* static set */
	O_ARRAY( o_bodySim ) staticSims;
	o_graphColor colors[B2_GRAPH_COLOR_COUNT];
	/* broadphase (broad_phase.h:27-47) */
	o_tree trees[3];
	o_bitSet movedProxies[3];
	o_intArray moveArray;
	o_pairSet pairSet;
	/* settings */
	b2Vec2 gravity;
	float hitEventThreshold, restitutionThreshold, maxLinearSpeed, contactSpeed, contactHertz, contactDampingRatio,
		jointHertz, jointDampingRatio, contactRecycleDistance;
	int enableSleep, enableWarmStarting, enableContactSoftening, enableContinuous, enableSpeculative, locked;
	/* events */
	O_ARRAY( b2BodyMoveEvent ) moveEvents;
	O_ARRAY( b2ContactBeginTouchEvent ) beginEvents;
	O_ARRAY( b2ContactEndTouchEvent ) endEvents[2];
	int endEventArrayIndex;
	int stepIndex;
	int recycledContactCount;
	b2Profile profile;
	o_bitSet contactStateBits, enlargedSimBits;
	int continuousSweeps, continuousHits; /* fast bodies swept; sweeps that ended at a time of impact */
} o_world;

o_world* o_getWorld( int index );
o_world* o_worldFromId( b2WorldId id );

/* geometry helpers (shape.c / geometry.c) */
b2AABB o_computeFatShapeAABB( const o_shape* shape, b2Transform xf, float extra );
b2Vec2 o_getShapeCentroid( const o_shape* shape );
float o_computeShapeMargin( const o_shape* shape );
b2MassData o_computeShapeMass( const o_shape* shape );
void o_computeShapeExtent( const o_shape* shape, b2Vec2 localCenter, float* minExtent, float* maxExtent );
static inline float o_shapeRadius( const o_shape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape: return s->capsule.radius;
		case b2_circleShape: return s->circle.radius;
		case b2_polygonShape: return s->polygon.radius;
		default: return 0.0f;
	}
}

/* narrowphase (manifold.c) */
b2LocalManifold o_collideShapes( const o_shape* a, const o_shape* b, b2Transform xf );
int o_canCollide( b2ShapeType a, b2ShapeType b );
int o_isPrimary( b2ShapeType a, b2ShapeType b );

/* contacts */
void o_createContact( o_world* w, o_shape* a, o_shape* b );
void o_destroyContact( o_world* w, o_contact* c );

/* graph coloring (constraint_graph.c) */
void o_addContactToGraph( o_world* w, o_contactSim* sim, o_contact* c );
void o_removeContactFromGraph( o_world* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex );
int o_assignJointColor( o_world* w, int bodyIdA, int bodyIdB, b2BodyType typeA, b2BodyType typeB );

/* solver (solver.c, contact_solver.c) */
void o_solve( o_world* w, o_stepContext* ctx );
void o_updateBroadPhasePairs( o_world* w );
void o_collide( o_world* w, o_stepContext* ctx );
void o_bufferMove( o_world* w, int proxyKey );

/* fork-join loops (o_parallel.c): fcn( ctx, begin, end ) over [0, count), inline when the
   pool has one thread or count < minParallel */
typedef void o_rangeFcn( void* ctx, int begin, int end );
void o_parallelFor( int count, int minParallel, o_rangeFcn* fcn, void* ctx );
void o_setThreads( int n );

/* joints */
void o_prepareJoints( o_world* w, o_stepContext* ctx, o_jointSim* joints, int count );
void o_warmStartJoint( o_world* w, o_stepContext* ctx, o_jointSim* j );
void o_solveJoint( o_world* w, o_stepContext* ctx, o_jointSim* j, int useBias );
void o_prepareJoint( o_world* w, o_stepContext* ctx, o_jointSim* j );
int o_shouldBodiesCollide( o_world* w, o_body* a, o_body* b );

#define O_PROXY_TYPE( K ) ( (b2BodyType)( ( K ) & 3 ) )
#define O_PROXY_ID( K ) ( ( K ) >> 2 )
#define O_PROXY_KEY( ID, T ) ( ( ( ID ) << 2 ) | ( T ) )

#endif
