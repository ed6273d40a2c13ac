/*
 * Host-side internals of the GB300 step library (C17): float math in the reference's
 * operation order (math_functions.h), growable arrays, LIFO id pools (id_pool.c), bit sets,
 * the shape-pair set and the broadphase tree whose topology decides pair order
 * (dynamic_tree.c). The data-parallel stages run on the device (b2g_device_abi.h).
 */
#ifndef B2G_HOST_H
#define B2G_HOST_H

#include "box2d_gb300.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define H_LINEAR_SLOP 0.005f
#define H_SPECULATIVE_DISTANCE ( 4.0f * H_LINEAR_SLOP )
#define H_AABB_MARGIN 0.05f
#define H_AABB_MARGIN_FRACTION 0.125f
#define H_HUGE 100000.0f
#define H_MAX_ROTATION ( 0.25f * B2_PI )
#define H_CONTACT_RECYCLE_DISTANCE ( 10.0f * H_LINEAR_SLOP )
#define H_CONTACT_RECYCLE_COS_ANGLE 0.98f
#define H_TIME_TH_SLEEP 0.5f
#define H_OVERFLOW_INDEX ( B2_GRAPH_COLOR_COUNT - 1 )
#define H_DYNAMIC_COLOR_COUNT ( B2_GRAPH_COLOR_COUNT - 4 )
#define H_MAX_WORLDS 4096
#define H_SIMD_WIDTH 4

/* ---------------- scalar math, same operation order as math_functions.h ---------------- */
static inline float h_min( float a, float b ) { return a < b ? a : b; }
static inline float h_max( float a, float b ) { return a > b ? a : b; }
static inline float h_abs( float a ) { return a < 0 ? -a : a; }
static inline float h_clamp( float a, float lo, float hi ) { return a < lo ? lo : ( a > hi ? hi : a ); }
static inline int h_mini( int a, int b ) { return a < b ? a : b; }
static inline int h_maxi( int a, int b ) { return a > b ? a : b; }
static inline b2Vec2 h_v( float x, float y ) { b2Vec2 v = { x, y }; return v; }
static inline float h_dot( b2Vec2 a, b2Vec2 b ) { return a.x * b.x + a.y * b.y; }
static inline float h_cross( b2Vec2 a, b2Vec2 b ) { return a.x * b.y - a.y * b.x; }
static inline b2Vec2 h_crossVS( b2Vec2 v, float s ) { return h_v( s * v.y, -s * v.x ); }
static inline b2Vec2 h_crossSV( float s, b2Vec2 v ) { return h_v( -s * v.y, s * v.x ); }
static inline b2Vec2 h_leftPerp( b2Vec2 v ) { return h_v( -v.y, v.x ); }
static inline b2Vec2 h_rightPerp( b2Vec2 v ) { return h_v( v.y, -v.x ); }
static inline b2Vec2 h_add( b2Vec2 a, b2Vec2 b ) { return h_v( a.x + b.x, a.y + b.y ); }
static inline b2Vec2 h_sub( b2Vec2 a, b2Vec2 b ) { return h_v( a.x - b.x, a.y - b.y ); }
static inline b2Vec2 h_neg( b2Vec2 a ) { return h_v( -a.x, -a.y ); }
static inline b2Vec2 h_lerp( b2Vec2 a, b2Vec2 b, float t ) { return h_v( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y ); }
static inline b2Vec2 h_mulSV( float s, b2Vec2 v ) { return h_v( s * v.x, s * v.y ); }
static inline b2Vec2 h_mulAdd( b2Vec2 a, float s, b2Vec2 b ) { return h_v( a.x + s * b.x, a.y + s * b.y ); }
static inline b2Vec2 h_mulSub( b2Vec2 a, float s, b2Vec2 b ) { return h_v( a.x - s * b.x, a.y - s * b.y ); }
static inline b2Vec2 h_vmin( b2Vec2 a, b2Vec2 b ) { return h_v( h_min( a.x, b.x ), h_min( a.y, b.y ) ); }
static inline b2Vec2 h_vmax( b2Vec2 a, b2Vec2 b ) { return h_v( h_max( a.x, b.x ), h_max( a.y, b.y ) ); }
static inline float h_length( b2Vec2 v ) { return sqrtf( v.x * v.x + v.y * v.y ); }
static inline float h_lengthSq( b2Vec2 v ) { return v.x * v.x + v.y * v.y; }
static inline float h_distance( b2Vec2 a, b2Vec2 b )
{
	float dx = b.x - a.x, dy = b.y - a.y;
	return sqrtf( dx * dx + dy * dy );
}
static inline float h_distanceSq( b2Vec2 a, b2Vec2 b )
{
	b2Vec2 c = { b.x - a.x, b.y - a.y };
	return c.x * c.x + c.y * c.y;
}
static inline b2Vec2 h_normalize( b2Vec2 a )
{
	float ls = a.x * a.x + a.y * a.y;
	if ( ls > 1000.0f * FLT_MIN )
	{
		float s = 1.0f / sqrtf( ls );
		return h_v( s * a.x, s * a.y );
	}
	return h_v( 0.0f, 0.0f );
}
static inline b2Vec2 h_getLengthAndNormalize( float* length, b2Vec2 a )
{
	float ls = a.x * a.x + a.y * a.y;
	if ( ls > 1000.0f * FLT_MIN )
	{
		*length = sqrtf( ls );
		float s = 1.0f / *length;
		return h_v( s * a.x, s * a.y );
	}
	*length = 0.0f;
	return h_v( 0.0f, 0.0f );
}
static inline b2Rot h_normalizeRot( b2Rot q )
{
	float mag = sqrtf( q.s * q.s + q.c * q.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot r = { q.c * inv, q.s * inv };
	return r;
}
static inline b2Rot h_integrateRotation( b2Rot q1, float da )
{
	b2Rot q2 = { q1.c - da * q1.s, q1.s + da * q1.c };
	float mag = sqrtf( q2.s * q2.s + q2.c * q2.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot r = { q2.c * inv, q2.s * inv };
	return r;
}
static inline b2Rot h_nlerp( b2Rot q1, b2Rot q2, float t )
{
	float omt = 1.0f - t;
	b2Rot q = { omt * q1.c + t * q2.c, omt * q1.s + t * q2.s };
	return h_normalizeRot( q );
}
static inline b2Rot h_mulRot( b2Rot q, b2Rot r )
{
	b2Rot qr;
	qr.s = q.s * r.c + q.c * r.s;
	qr.c = q.c * r.c - q.s * r.s;
	return qr;
}
static inline b2Rot h_invMulRot( b2Rot a, b2Rot b )
{
	b2Rot r;
	r.s = a.c * b.s - a.s * b.c;
	r.c = a.c * b.c + a.s * b.s;
	return r;
}
static inline b2Rot h_invertRot( b2Rot a ) { b2Rot r = { a.c, -a.s }; return r; }
static inline b2Vec2 h_rotate( b2Rot q, b2Vec2 v ) { return h_v( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
static inline b2Vec2 h_invRotate( b2Rot q, b2Vec2 v ) { return h_v( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }
static inline b2Vec2 h_transformPoint( b2Transform t, b2Vec2 p )
{
	float x = ( t.q.c * p.x - t.q.s * p.y ) + t.p.x;
	float y = ( t.q.s * p.x + t.q.c * p.y ) + t.p.y;
	return h_v( x, y );
}
static inline b2Vec2 h_invTransformPoint( b2Transform t, b2Vec2 p )
{
	float vx = p.x - t.p.x, vy = p.y - t.p.y;
	return h_v( t.q.c * vx + t.q.s * vy, -t.q.s * vx + t.q.c * vy );
}
/* b2TransformWorldPoint (math_functions.h:577-582): rotation first, then offset */
static inline b2Vec2 h_transformWorldPoint( b2Transform t, b2Vec2 p )
{
	float rx = t.q.c * p.x - t.q.s * p.y;
	float ry = t.q.s * p.x + t.q.c * p.y;
	return h_v( t.p.x + rx, t.p.y + ry );
}
static inline b2Transform h_invMulTransforms( b2Transform A, b2Transform B )
{
	b2Transform C;
	C.q = h_invMulRot( A.q, B.q );
	b2Vec2 d = { B.p.x - A.p.x, B.p.y - A.p.y };
	C.p = h_invRotate( A.q, d );
	return C;
}
static inline float h_relativeCos( b2Rot a, b2Rot b ) { return a.c * b.c + a.s * b.s; }
static inline int h_aabbOverlaps( b2AABB a, b2AABB b )
{
	return !( b.lowerBound.x > a.upperBound.x || b.lowerBound.y > a.upperBound.y || a.lowerBound.x > b.upperBound.x ||
			  a.lowerBound.y > b.upperBound.y );
}
static inline int h_aabbContains( b2AABB a, b2AABB b )
{
	int s = 1;
	s = s && a.lowerBound.x <= b.lowerBound.x;
	s = s && a.lowerBound.y <= b.lowerBound.y;
	s = s && b.upperBound.x <= a.upperBound.x;
	s = s && b.upperBound.y <= a.upperBound.y;
	return s;
}
static inline b2AABB h_aabbUnion( b2AABB a, b2AABB b )
{
	b2AABB c;
	c.lowerBound.x = h_min( a.lowerBound.x, b.lowerBound.x );
	c.lowerBound.y = h_min( a.lowerBound.y, b.lowerBound.y );
	c.upperBound.x = h_max( a.upperBound.x, b.upperBound.x );
	c.upperBound.y = h_max( a.upperBound.y, b.upperBound.y );
	return c;
}
static inline b2Vec2 h_aabbCenter( b2AABB a )
{
	return h_v( 0.5f * ( a.lowerBound.x + a.upperBound.x ), 0.5f * ( a.lowerBound.y + a.upperBound.y ) );
}
static inline float h_perimeter( b2AABB a )
{
	float wx = a.upperBound.x - a.lowerBound.x;
	float wy = a.upperBound.y - a.lowerBound.y;
	return 2.0f * ( wx + wy );
}
static inline int h_enlargeAABB( b2AABB* a, b2AABB b )
{
	int changed = 0;
	if ( b.lowerBound.x < a->lowerBound.x ) { a->lowerBound.x = b.lowerBound.x; changed = 1; }
	if ( b.lowerBound.y < a->lowerBound.y ) { a->lowerBound.y = b.lowerBound.y; changed = 1; }
	if ( a->upperBound.x < b.upperBound.x ) { a->upperBound.x = b.upperBound.x; changed = 1; }
	if ( a->upperBound.y < b.upperBound.y ) { a->upperBound.y = b.upperBound.y; changed = 1; }
	return changed;
}
static inline int h_isValidFloat( float a ) { return !isnan( a ) && !isinf( a ); }

/* ---------------- growable arrays ---------------- */
#define H_ARRAY( T ) struct { T* data; int count; int capacity; }
#define h_reserve( a, n )                                                                                                      \
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
#define h_push( a, v )                                                                                                         \
	do                                                                                                                           \
	{                                                                                                                            \
		h_reserve( a, ( a ).count + 1 );                                                                                         \
		( a ).data[( a ).count++] = ( v );                                                                                       \
	} while ( 0 )
#define h_free( a )                                                                                                            \
	do                                                                                                                           \
	{                                                                                                                            \
		free( ( a ).data );                                                                                                      \
		( a ).data = NULL;                                                                                                       \
		( a ).count = ( a ).capacity = 0;                                                                                        \
	} while ( 0 )
/* swap-remove; returns the index that moved into 'index' or -1 (container.h:136-150) */
#define h_removeSwap( a, index ) h_removeSwapHelper( ( a ).data, &( a ).count, ( index ), (int)sizeof( *( a ).data ) )
static inline int h_removeSwapHelper( void* data, int* count, int index, int size )
{
	( *count )--;
	if ( index != *count )
	{
		memcpy( (char*)data + (size_t)index * size, (char*)data + (size_t)( *count ) * size, size );
		return *count;
	}
	return -1;
}

typedef H_ARRAY( int ) h_intArray;

/* LIFO id pool (id_pool.c:19-38) */
typedef struct h_idPool
{
	h_intArray freeArray;
	int nextIndex;
} h_idPool;
static inline int h_allocId( h_idPool* p )
{
	if ( p->freeArray.count > 0 ) return p->freeArray.data[--p->freeArray.count];
	return p->nextIndex++;
}
static inline void h_freeId( h_idPool* p, int id ) { h_push( p->freeArray, id ); }

/* bit set */
typedef struct h_bitSet
{
	uint64_t* bits;
	int blockCount;
} h_bitSet;
static inline void h_bitGrow( h_bitSet* s, int bit )
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
static inline void h_bitSet1( h_bitSet* s, int bit ) { h_bitGrow( s, bit ); s->bits[bit / 64] |= ( 1ull << ( bit % 64 ) ); }
static inline void h_bitClear( h_bitSet* s, int bit )
{
	if ( bit / 64 < s->blockCount ) s->bits[bit / 64] &= ~( 1ull << ( bit % 64 ) );
}
static inline int h_bitGet( const h_bitSet* s, int bit )
{
	if ( bit / 64 >= s->blockCount ) return 0;
	return ( s->bits[bit / 64] >> ( bit % 64 ) ) & 1;
}
static inline void h_bitReset( h_bitSet* s, int bitCount )
{
	h_bitGrow( s, bitCount > 0 ? bitCount - 1 : 0 );
	memset( s->bits, 0, (size_t)s->blockCount * 8 );
}

/* open addressing set of uint64 pair keys (membership only; order never observed) */
typedef struct h_pairSet
{
	uint64_t* keys;
	int capacity;
	int count;
} h_pairSet;
void h_pairSetAdd( h_pairSet* s, uint64_t key );
int h_pairSetContains( const h_pairSet* s, uint64_t key );
/* start loading the slot a lookup of `key` probes first (a hint; no effect on results) */
void h_pairSetPrefetch( const h_pairSet* s, uint64_t key );
void h_pairSetRemove( h_pairSet* s, uint64_t key );
void h_pairSetFree( h_pairSet* s );
#define H_SHAPE_PAIR_KEY( K1, K2 ) ( ( K1 ) < ( K2 ) ? (uint64_t)( K1 ) << 32 | (uint64_t)( K2 ) : (uint64_t)( K2 ) << 32 | (uint64_t)( K1 ) )

/* ---------------- dynamic tree (dynamic_tree.c) ---------------- */
enum
{
	H_NODE_ALLOCATED = 0x0001,
	H_NODE_ENLARGED = 0x0002,
	H_NODE_LEAF = 0x0004,
};

typedef struct h_treeNode
{
	b2AABB aabb;
	uint64_t categoryBits;
	int child1, child2; /* internal nodes */
	uint64_t userData;	/* leaves */
	int parent;			/* doubles as free-list next */
	uint16_t height;
	uint16_t flags;
} h_treeNode;

typedef struct h_tree
{
	h_treeNode* nodes;
	int root, nodeCount, nodeCapacity, freeList, proxyCount;
	int version; /* bumped by every change of the node array */
	int pinned;	 /* nodes live in page-locked memory */
	int* leafIndices;
	b2Vec2* leafCenters;
	int rebuildCapacity;
} h_tree;

/* node array storage, provided by the library (page-locked above a size threshold) */
void* h_nodeAlloc( size_t bytes, int* pinned );
void h_nodeFree( void* p, int pinned );

h_tree h_treeCreate( int proxyCapacity );
void h_treeDestroy( h_tree* t );
int h_treeCreateProxy( h_tree* t, b2AABB aabb, uint64_t categoryBits, uint64_t userData );
void h_treeDestroyProxy( h_tree* t, int proxyId );
void h_treeMoveProxy( h_tree* t, int proxyId, b2AABB aabb );
void h_treeEnlargeProxy( h_tree* t, int proxyId, b2AABB aabb );
/* h_treeEnlargeProxy of each proxy in turn, without touching the version (the caller bumps it) */
void h_treeEnlargeProxies( h_tree* t, const int* proxyIds, const b2AABB* boxes, int count );
/* h_treeEnlargeProxy for threads that enlarge different proxies of one tree at once (the
   result is that of the enlargements one after another); the caller bumps the version */
void h_treeEnlargeProxyShared( h_tree* t, int proxyId, b2AABB aabb );
int h_treeRebuild( h_tree* t, int fullBuild );
typedef int h_treeQueryFcn( int proxyId, uint64_t userData, void* ctx );
void h_treeQuery( const h_tree* t, b2AABB aabb, uint64_t maskBits, h_treeQueryFcn* fcn, void* ctx );
int h_treeHeight( const h_tree* t );



/* soft constraint coefficients (solver.h:239-281 b2MakeSoft) */
typedef struct h_softness
{
	float biasRate, massScale, impulseScale;
} h_softness;

static inline h_softness h_makeSoft( float hertz, float zeta, float h )
{
	h_softness s = { 0.0f, 0.0f, 0.0f };
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

#endif
