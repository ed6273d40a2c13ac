/*
 * Device float math of the GB300 step kernels, in the operation order of the reference's
 * math_functions.h so that results match the CPU step bit for bit when the kernels are
 * compiled with --fmad=false, IEEE division and square root, and no flush-to-zero.
 * min/max are written as selects (a < b ? a : b), never fminf/fmaxf, to keep the
 * reference's signed-zero and operand-order behaviour.
 */
#pragma once

#include "../b2g_device_abi.h"

#include <float.h>
#include <math.h>

#define D_LINEAR_SLOP 0.005f
#define D_SPECULATIVE_DISTANCE ( 4.0f * D_LINEAR_SLOP )
#define D_HUGE 100000.0f
#define D_MAX_ROTATION ( 0.25f * B2_PI )
#define D_CONTACT_RECYCLE_COS_ANGLE 0.98f
#define D_TIME_TO_SLEEP 0.5f /* constants.h B2_TIME_TO_SLEEP */

/* ---------------- scalar math, same operation order as math_functions.h ---------------- */
static __device__ __forceinline__ float d_min( float a, float b ) { return a < b ? a : b; }
static __device__ __forceinline__ float d_max( float a, float b ) { return a > b ? a : b; }
static __device__ __forceinline__ float d_abs( float a ) { return a < 0 ? -a : a; }
static __device__ __forceinline__ float d_clamp( float a, float lo, float hi ) { return a < lo ? lo : ( a > hi ? hi : a ); }
static __device__ __forceinline__ int d_mini( int a, int b ) { return a < b ? a : b; }
static __device__ __forceinline__ int d_maxi( int a, int b ) { return a > b ? a : b; }
static __device__ __forceinline__ b2Vec2 d_v( float x, float y ) { b2Vec2 v = { x, y }; return v; }
static __device__ __forceinline__ float d_dot( b2Vec2 a, b2Vec2 b ) { return a.x * b.x + a.y * b.y; }
static __device__ __forceinline__ float d_cross( b2Vec2 a, b2Vec2 b ) { return a.x * b.y - a.y * b.x; }
static __device__ __forceinline__ b2Vec2 d_crossVS( b2Vec2 v, float s ) { return d_v( s * v.y, -s * v.x ); }
static __device__ __forceinline__ b2Vec2 d_crossSV( float s, b2Vec2 v ) { return d_v( -s * v.y, s * v.x ); }
static __device__ __forceinline__ b2Vec2 d_leftPerp( b2Vec2 v ) { return d_v( -v.y, v.x ); }
static __device__ __forceinline__ b2Vec2 d_rightPerp( b2Vec2 v ) { return d_v( v.y, -v.x ); }
static __device__ __forceinline__ b2Vec2 d_add( b2Vec2 a, b2Vec2 b ) { return d_v( a.x + b.x, a.y + b.y ); }
static __device__ __forceinline__ b2Vec2 d_sub( b2Vec2 a, b2Vec2 b ) { return d_v( a.x - b.x, a.y - b.y ); }
static __device__ __forceinline__ b2Vec2 d_neg( b2Vec2 a ) { return d_v( -a.x, -a.y ); }
static __device__ __forceinline__ b2Vec2 d_lerp( b2Vec2 a, b2Vec2 b, float t ) { return d_v( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y ); }
static __device__ __forceinline__ b2Vec2 d_mulSV( float s, b2Vec2 v ) { return d_v( s * v.x, s * v.y ); }
static __device__ __forceinline__ b2Vec2 d_mulAdd( b2Vec2 a, float s, b2Vec2 b ) { return d_v( a.x + s * b.x, a.y + s * b.y ); }
static __device__ __forceinline__ b2Vec2 d_mulSub( b2Vec2 a, float s, b2Vec2 b ) { return d_v( a.x - s * b.x, a.y - s * b.y ); }
static __device__ __forceinline__ b2Vec2 d_vmin( b2Vec2 a, b2Vec2 b ) { return d_v( d_min( a.x, b.x ), d_min( a.y, b.y ) ); }
static __device__ __forceinline__ b2Vec2 d_vmax( b2Vec2 a, b2Vec2 b ) { return d_v( d_max( a.x, b.x ), d_max( a.y, b.y ) ); }
static __device__ __forceinline__ float d_length( b2Vec2 v ) { return sqrtf( v.x * v.x + v.y * v.y ); }
static __device__ __forceinline__ float d_lengthSq( b2Vec2 v ) { return v.x * v.x + v.y * v.y; }
static __device__ __forceinline__ float d_distance( b2Vec2 a, b2Vec2 b )
{
	float dx = b.x - a.x, dy = b.y - a.y;
	return sqrtf( dx * dx + dy * dy );
}
static __device__ __forceinline__ float d_distanceSq( b2Vec2 a, b2Vec2 b )
{
	b2Vec2 c = { b.x - a.x, b.y - a.y };
	return c.x * c.x + c.y * c.y;
}
static __device__ __forceinline__ b2Vec2 d_normalize( b2Vec2 a )
{
	float ls = a.x * a.x + a.y * a.y;
	if ( ls > 1000.0f * FLT_MIN )
	{
		float s = 1.0f / sqrtf( ls );
		return d_v( s * a.x, s * a.y );
	}
	return d_v( 0.0f, 0.0f );
}
static __device__ __forceinline__ b2Vec2 d_getLengthAndNormalize( float* length, b2Vec2 a )
{
	float ls = a.x * a.x + a.y * a.y;
	if ( ls > 1000.0f * FLT_MIN )
	{
		*length = sqrtf( ls );
		float s = 1.0f / *length;
		return d_v( s * a.x, s * a.y );
	}
	*length = 0.0f;
	return d_v( 0.0f, 0.0f );
}
static __device__ __forceinline__ b2Rot d_normalizeRot( b2Rot q )
{
	float mag = sqrtf( q.s * q.s + q.c * q.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot r = { q.c * inv, q.s * inv };
	return r;
}
static __device__ __forceinline__ b2Rot d_integrateRotation( b2Rot q1, float da )
{
	b2Rot q2 = { q1.c - da * q1.s, q1.s + da * q1.c };
	float mag = sqrtf( q2.s * q2.s + q2.c * q2.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot r = { q2.c * inv, q2.s * inv };
	return r;
}
static __device__ __forceinline__ b2Rot d_nlerp( b2Rot q1, b2Rot q2, float t )
{
	float omt = 1.0f - t;
	b2Rot q = { omt * q1.c + t * q2.c, omt * q1.s + t * q2.s };
	return d_normalizeRot( q );
}
static __device__ __forceinline__ b2Rot d_mulRot( b2Rot q, b2Rot r )
{
	b2Rot qr;
	qr.s = q.s * r.c + q.c * r.s;
	qr.c = q.c * r.c - q.s * r.s;
	return qr;
}
static __device__ __forceinline__ b2Rot d_invMulRot( b2Rot a, b2Rot b )
{
	b2Rot r;
	r.s = a.c * b.s - a.s * b.c;
	r.c = a.c * b.c + a.s * b.s;
	return r;
}
static __device__ __forceinline__ b2Rot d_invertRot( b2Rot a ) { b2Rot r = { a.c, -a.s }; return r; }
static __device__ __forceinline__ b2Vec2 d_rotate( b2Rot q, b2Vec2 v ) { return d_v( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
static __device__ __forceinline__ b2Vec2 d_invRotate( b2Rot q, b2Vec2 v ) { return d_v( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }
static __device__ __forceinline__ b2Vec2 d_transformPoint( b2Transform t, b2Vec2 p )
{
	float x = ( t.q.c * p.x - t.q.s * p.y ) + t.p.x;
	float y = ( t.q.s * p.x + t.q.c * p.y ) + t.p.y;
	return d_v( x, y );
}
static __device__ __forceinline__ b2Vec2 d_invTransformPoint( b2Transform t, b2Vec2 p )
{
	float vx = p.x - t.p.x, vy = p.y - t.p.y;
	return d_v( t.q.c * vx + t.q.s * vy, -t.q.s * vx + t.q.c * vy );
}
/* b2TransformWorldPoint (math_functions.h:577-582): rotation first, then offset */
static __device__ __forceinline__ b2Vec2 d_transformWorldPoint( b2Transform t, b2Vec2 p )
{
	float rx = t.q.c * p.x - t.q.s * p.y;
	float ry = t.q.s * p.x + t.q.c * p.y;
	return d_v( t.p.x + rx, t.p.y + ry );
}
static __device__ __forceinline__ b2Transform d_invMulTransforms( b2Transform A, b2Transform B )
{
	b2Transform C;
	C.q = d_invMulRot( A.q, B.q );
	b2Vec2 d = { B.p.x - A.p.x, B.p.y - A.p.y };
	C.p = d_invRotate( A.q, d );
	return C;
}
static __device__ __forceinline__ float d_relativeCos( b2Rot a, b2Rot b ) { return a.c * b.c + a.s * b.s; }
static __device__ __forceinline__ int d_aabbOverlaps( b2AABB a, b2AABB b )
{
	return !( b.lowerBound.x > a.upperBound.x || b.lowerBound.y > a.upperBound.y || a.lowerBound.x > b.upperBound.x ||
			  a.lowerBound.y > b.upperBound.y );
}
static __device__ __forceinline__ int d_aabbContains( b2AABB a, b2AABB b )
{
	int s = 1;
	s = s && a.lowerBound.x <= b.lowerBound.x;
	s = s && a.lowerBound.y <= b.lowerBound.y;
	s = s && b.upperBound.x <= a.upperBound.x;
	s = s && b.upperBound.y <= a.upperBound.y;
	return s;
}
static __device__ __forceinline__ b2AABB d_aabbUnion( b2AABB a, b2AABB b )
{
	b2AABB c;
	c.lowerBound.x = d_min( a.lowerBound.x, b.lowerBound.x );
	c.lowerBound.y = d_min( a.lowerBound.y, b.lowerBound.y );
	c.upperBound.x = d_max( a.upperBound.x, b.upperBound.x );
	c.upperBound.y = d_max( a.upperBound.y, b.upperBound.y );
	return c;
}
static __device__ __forceinline__ b2Vec2 d_aabbCenter( b2AABB a )
{
	return d_v( 0.5f * ( a.lowerBound.x + a.upperBound.x ), 0.5f * ( a.lowerBound.y + a.upperBound.y ) );
}
static __device__ __forceinline__ float d_perimeter( b2AABB a )
{
	float wx = a.upperBound.x - a.lowerBound.x;
	float wy = a.upperBound.y - a.lowerBound.y;
	return 2.0f * ( wx + wy );
}
static __device__ __forceinline__ int d_enlargeAABB( b2AABB* a, b2AABB b )
{
	int changed = 0;
	if ( b.lowerBound.x < a->lowerBound.x ) { a->lowerBound.x = b.lowerBound.x; changed = 1; }
	if ( b.lowerBound.y < a->lowerBound.y ) { a->lowerBound.y = b.lowerBound.y; changed = 1; }
	if ( a->upperBound.x < b.upperBound.x ) { a->upperBound.x = b.upperBound.x; changed = 1; }
	if ( a->upperBound.y < b.upperBound.y ) { a->upperBound.y = b.upperBound.y; changed = 1; }
	return changed;
}

/* a tree node box against a query box packed as (lower x, lower y, upper x, upper y) */
static __device__ __forceinline__ bool d_overlaps( b2AABB a, float4 b )
{
	return !( b.x > a.upperBound.x || b.y > a.upperBound.y || a.lowerBound.x > b.z || a.lowerBound.y > b.w );
}

static __device__ __forceinline__ int d_isValidFloat( float a ) { return !isnan( a ) && !isinf( a ); }

