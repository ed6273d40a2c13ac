/*
 * box2d_gb300_math.h -- the inline vector, rotation and transform helpers of Box2D v3.2's
 * public math header (include/box2d/math_functions.h:105-840), the id helpers of id.h:83-160
 * and the small constants callers use (base.h:163, constants.h:18-40), written for the GB300
 * step library's public ABI. Included by box2d_gb300.h; callers do not include it directly.
 *
 * The reference defines these in its headers, so a program built against the reference
 * compiles them into itself. They are reproduced here with the same names, signatures and
 * floating-point operation order (a caller that builds scene inputs with them must get the
 * same bits as with the reference's headers), float32 only (b2Pos is b2Vec2).
 */
#ifndef BOX2D_GB300_MATH_H
#define BOX2D_GB300_MATH_H

#include <float.h>
#include <math.h>

/* ---- constants ---- */
#define B2_HASH_INIT 5381
#define B2_MAX_WORKERS 32
#define B2_MAX_TASKS 256
#ifndef B2_MAX_WORLDS
#define B2_MAX_WORLDS 128
#endif
#define B2_NAME_LENGTH 10
#ifndef B2_INLINE
#define B2_INLINE static inline
#endif

/* ---- ids ---- */
#ifdef __cplusplus
#define B2G_NULL_ID {}
#else
#define B2G_NULL_ID { 0 }
#endif

static const b2WorldId b2_nullWorldId = B2G_NULL_ID;
static const b2BodyId b2_nullBodyId = B2G_NULL_ID;
static const b2ShapeId b2_nullShapeId = B2G_NULL_ID;
static const b2ChainId b2_nullChainId = B2G_NULL_ID;
static const b2JointId b2_nullJointId = B2G_NULL_ID;
static const b2ContactId b2_nullContactId = B2G_NULL_ID;

#define B2_ID_EQUALS( a, b ) ( ( a ).index1 == ( b ).index1 && ( a ).world0 == ( b ).world0 && ( a ).generation == ( b ).generation )

/* pack an id into an integer (index1 high, then world, then generation) and back */
B2G_INLINE uint32_t b2StoreWorldId( b2WorldId id )
{
	return ( (uint32_t)id.index1 << 16 ) | (uint32_t)id.generation;
}
B2G_INLINE b2WorldId b2LoadWorldId( uint32_t x )
{
	b2WorldId id = { (uint16_t)( x >> 16 ), (uint16_t)x };
	return id;
}
#define B2G_ID64_FUNCS( T, STORE, LOAD )                                                                                        \
	B2G_INLINE uint64_t STORE( T id )                                                                                           \
	{                                                                                                                           \
		return ( (uint64_t)(uint32_t)id.index1 << 32 ) | ( (uint64_t)id.world0 << 16 ) | (uint64_t)id.generation;              \
	}                                                                                                                           \
	B2G_INLINE T LOAD( uint64_t x )                                                                                             \
	{                                                                                                                           \
		T id = { (int32_t)( x >> 32 ), (uint16_t)( x >> 16 ), (uint16_t)x };                                                    \
		return id;                                                                                                              \
	}
B2G_ID64_FUNCS( b2BodyId, b2StoreBodyId, b2LoadBodyId )
B2G_ID64_FUNCS( b2ShapeId, b2StoreShapeId, b2LoadShapeId )
B2G_ID64_FUNCS( b2ChainId, b2StoreChainId, b2LoadChainId )
B2G_ID64_FUNCS( b2JointId, b2StoreJointId, b2LoadJointId )
#undef B2G_ID64_FUNCS

/* ---- constant values ---- */
static const b2Vec2 b2Vec2_zero = { 0.0f, 0.0f };
static const b2Rot b2Rot_identity = { 1.0f, 0.0f };
static const b2Transform b2Transform_identity = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };
static const b2Mat22 b2Mat22_zero = { { 0.0f, 0.0f }, { 0.0f, 0.0f } };
static const b2Pos b2Pos_zero = { 0.0f, 0.0f };
static const b2WorldTransform b2WorldTransform_identity = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };

/* ---- scalars ---- */
B2G_INLINE int b2MinInt( int a, int b ) { return a < b ? a : b; }
B2G_INLINE int b2MaxInt( int a, int b ) { return a > b ? a : b; }
B2G_INLINE int b2AbsInt( int a ) { return a < 0 ? -a : a; }
B2G_INLINE int b2ClampInt( int a, int lower, int upper ) { return a < lower ? lower : ( a > upper ? upper : a ); }
B2G_INLINE int b2CeilingInt( int numerator, int denominator ) { return ( numerator + denominator - 1 ) / denominator; }
B2G_INLINE float b2MinFloat( float a, float b ) { return a < b ? a : b; }
B2G_INLINE float b2MaxFloat( float a, float b ) { return a > b ? a : b; }
B2G_INLINE float b2AbsFloat( float a ) { return a < 0.0f ? -a : a; }
B2G_INLINE float b2ClampFloat( float a, float lower, float upper ) { return a < lower ? lower : ( a > upper ? upper : a ); }

/* ---- vectors ---- */
B2G_INLINE b2Vec2 b2G_v( float x, float y )
{
	b2Vec2 v = { x, y };
	return v;
}
B2G_INLINE float b2Dot( b2Vec2 a, b2Vec2 b ) { return a.x * b.x + a.y * b.y; }
B2G_INLINE float b2Cross( b2Vec2 a, b2Vec2 b ) { return a.x * b.y - a.y * b.x; }
B2G_INLINE b2Vec2 b2CrossVS( b2Vec2 v, float s ) { return b2G_v( s * v.y, -s * v.x ); }
B2G_INLINE b2Vec2 b2CrossSV( float s, b2Vec2 v ) { return b2G_v( -s * v.y, s * v.x ); }
B2G_INLINE b2Vec2 b2LeftPerp( b2Vec2 v ) { return b2G_v( -v.y, v.x ); }
B2G_INLINE b2Vec2 b2RightPerp( b2Vec2 v ) { return b2G_v( v.y, -v.x ); }
B2G_INLINE b2Vec2 b2Add( b2Vec2 a, b2Vec2 b ) { return b2G_v( a.x + b.x, a.y + b.y ); }
B2G_INLINE b2Vec2 b2Sub( b2Vec2 a, b2Vec2 b ) { return b2G_v( a.x - b.x, a.y - b.y ); }
B2G_INLINE b2Vec2 b2Neg( b2Vec2 a ) { return b2G_v( -a.x, -a.y ); }
B2G_INLINE b2Vec2 b2Lerp( b2Vec2 a, b2Vec2 b, float t )
{
	return b2G_v( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y );
}
B2G_INLINE b2Vec2 b2Mul( b2Vec2 a, b2Vec2 b ) { return b2G_v( a.x * b.x, a.y * b.y ); }
B2G_INLINE b2Vec2 b2MulSV( float s, b2Vec2 v ) { return b2G_v( s * v.x, s * v.y ); }
B2G_INLINE b2Vec2 b2MulAdd( b2Vec2 a, float s, b2Vec2 b ) { return b2G_v( a.x + s * b.x, a.y + s * b.y ); }
B2G_INLINE b2Vec2 b2MulSub( b2Vec2 a, float s, b2Vec2 b ) { return b2G_v( a.x - s * b.x, a.y - s * b.y ); }
B2G_INLINE b2Vec2 b2Abs( b2Vec2 a ) { return b2G_v( b2AbsFloat( a.x ), b2AbsFloat( a.y ) ); }
B2G_INLINE b2Vec2 b2Min( b2Vec2 a, b2Vec2 b ) { return b2G_v( b2MinFloat( a.x, b.x ), b2MinFloat( a.y, b.y ) ); }
B2G_INLINE b2Vec2 b2Max( b2Vec2 a, b2Vec2 b ) { return b2G_v( b2MaxFloat( a.x, b.x ), b2MaxFloat( a.y, b.y ) ); }
B2G_INLINE b2Vec2 b2Clamp( b2Vec2 v, b2Vec2 a, b2Vec2 b )
{
	return b2G_v( b2ClampFloat( v.x, a.x, b.x ), b2ClampFloat( v.y, a.y, b.y ) );
}
B2G_INLINE float b2Length( b2Vec2 v ) { return sqrtf( v.x * v.x + v.y * v.y ); }
B2G_INLINE float b2LengthSquared( b2Vec2 v ) { return v.x * v.x + v.y * v.y; }
B2G_INLINE float b2Distance( b2Vec2 a, b2Vec2 b )
{
	float dx = b.x - a.x, dy = b.y - a.y;
	return sqrtf( dx * dx + dy * dy );
}
B2G_INLINE float b2DistanceSquared( b2Vec2 a, b2Vec2 b )
{
	float dx = b.x - a.x, dy = b.y - a.y;
	return dx * dx + dy * dy;
}
/* unit vector, or zero below a tiny length */
B2G_INLINE b2Vec2 b2Normalize( b2Vec2 a )
{
	float lengthSquared = a.x * a.x + a.y * a.y;
	if ( !( lengthSquared > 1000.0f * FLT_MIN ) ) return b2G_v( 0.0f, 0.0f );
	float s = 1.0f / sqrtf( lengthSquared );
	return b2G_v( s * a.x, s * a.y );
}
B2G_INLINE bool b2IsNormalized( b2Vec2 a )
{
	return b2AbsFloat( 1.0f - b2Dot( a, a ) ) < 100.0f * FLT_EPSILON;
}
B2G_INLINE b2Vec2 b2GetLengthAndNormalize( float* length, b2Vec2 a )
{
	float lengthSquared = a.x * a.x + a.y * a.y;
	if ( !( lengthSquared > 1000.0f * FLT_MIN ) )
	{
		*length = 0.0f;
		return b2G_v( 0.0f, 0.0f );
	}
	*length = sqrtf( lengthSquared );
	float s = 1.0f / *length;
	return b2G_v( s * a.x, s * a.y );
}

/* ---- rotations ---- */
B2G_INLINE b2Rot b2G_unitRot( float c, float s )
{
	float mag = sqrtf( s * s + c * c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2Rot q = { c * inv, s * inv };
	return q;
}
B2G_INLINE b2Rot b2NormalizeRot( b2Rot q ) { return b2G_unitRot( q.c, q.s ); }
/* first-order rotation update by deltaAngle, renormalized */
B2G_INLINE b2Rot b2IntegrateRotation( b2Rot q1, float deltaAngle )
{
	return b2G_unitRot( q1.c - deltaAngle * q1.s, q1.s + deltaAngle * q1.c );
}
B2G_INLINE b2Rot b2MakeRotFromUnitVector( b2Vec2 unitVector )
{
	b2Rot q = { unitVector.x, unitVector.y };
	return q;
}
B2G_INLINE bool b2IsNormalizedRot( b2Rot q )
{
	float qq = q.s * q.s + q.c * q.c;
	return 1.0f - 0.0006f < qq && qq < 1.0f + 0.0006f;
}
B2G_INLINE b2Rot b2InvertRot( b2Rot a )
{
	b2Rot r = { a.c, -a.s };
	return r;
}
/* normalized linear interpolation of rotations */
B2G_INLINE b2Rot b2NLerp( b2Rot q1, b2Rot q2, float t )
{
	float omt = 1.0f - t;
	return b2G_unitRot( omt * q1.c + t * q2.c, omt * q1.s + t * q2.s );
}
B2G_INLINE float b2ComputeAngularVelocity( b2Rot q1, b2Rot q2, float inv_h )
{
	return inv_h * ( q2.s * q1.c - q2.c * q1.s );
}
B2G_INLINE float b2Rot_GetAngle( b2Rot q ) { return b2Atan2( q.s, q.c ); }
B2G_INLINE b2Vec2 b2Rot_GetXAxis( b2Rot q ) { return b2G_v( q.c, q.s ); }
B2G_INLINE b2Vec2 b2Rot_GetYAxis( b2Rot q ) { return b2G_v( -q.s, q.c ); }
/* q * r */
B2G_INLINE b2Rot b2MulRot( b2Rot q, b2Rot r )
{
	b2Rot qr;
	qr.s = q.s * r.c + q.c * r.s;
	qr.c = q.c * r.c - q.s * r.s;
	return qr;
}
/* inverse(a) * b */
B2G_INLINE b2Rot b2InvMulRot( b2Rot a, b2Rot b )
{
	b2Rot r;
	r.s = a.c * b.s - a.s * b.c;
	r.c = a.c * b.c + a.s * b.s;
	return r;
}
B2G_INLINE float b2RelativeAngle( b2Rot a, b2Rot b )
{
	float s = a.c * b.s - a.s * b.c;
	float c = a.c * b.c + a.s * b.s;
	return b2Atan2( s, c );
}
/* angle wrapped into [-pi, pi]: subtract the nearest multiple of 2 pi, found in double by
   the add-and-subtract-2^52*1.5 rounding trick */
B2G_INLINE float b2UnwindAngle( float radians )
{
	double a = (double)b2ClampFloat( radians, -1.0e6f, 1.0e6f );
	double twoPi = 2.0f * B2_PI;
	double shifter = 6755399441055744.0;
	double k = ( a / twoPi + shifter ) - shifter;
	return (float)( a - k * twoPi );
}
B2G_INLINE b2Vec2 b2RotateVector( b2Rot q, b2Vec2 v ) { return b2G_v( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
B2G_INLINE b2Vec2 b2InvRotateVector( b2Rot q, b2Vec2 v ) { return b2G_v( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }

/* ---- transforms ---- */
B2G_INLINE b2Vec2 b2TransformPoint( b2Transform t, const b2Vec2 p )
{
	float x = ( t.q.c * p.x - t.q.s * p.y ) + t.p.x;
	float y = ( t.q.s * p.x + t.q.c * p.y ) + t.p.y;
	return b2G_v( x, y );
}
B2G_INLINE b2Vec2 b2InvTransformPoint( b2Transform t, const b2Vec2 p )
{
	float vx = p.x - t.p.x, vy = p.y - t.p.y;
	return b2G_v( t.q.c * vx + t.q.s * vy, -t.q.s * vx + t.q.c * vy );
}
B2G_INLINE b2Transform b2MulTransforms( b2Transform A, b2Transform B )
{
	b2Transform C;
	C.q = b2MulRot( A.q, B.q );
	C.p = b2Add( b2RotateVector( A.q, B.p ), A.p );
	return C;
}
B2G_INLINE b2Transform b2InvMulTransforms( b2Transform A, b2Transform B )
{
	b2Transform C;
	C.q = b2InvMulRot( A.q, B.q );
	C.p = b2InvRotateVector( A.q, b2Sub( B.p, A.p ) );
	return C;
}
B2G_INLINE b2Pos b2ToPos( b2Vec2 v ) { return v; }
B2G_INLINE b2Vec2 b2ToVec2( b2Pos p ) { return p; }
B2G_INLINE float b2RoundDownFloat( double x ) { return (float)x; }
B2G_INLINE float b2RoundUpFloat( double x ) { return (float)x; }
B2G_INLINE b2Vec2 b2SubPos( b2Pos a, b2Pos b ) { return b2G_v( a.x - b.x, a.y - b.y ); }
B2G_INLINE b2Pos b2OffsetPos( b2Pos p, b2Vec2 d ) { return b2G_v( p.x + d.x, p.y + d.y ); }
B2G_INLINE b2Pos b2LerpPosition( b2Pos a, b2Pos b, float t ) { return b2Lerp( a, b, t ); }
B2G_INLINE b2Pos b2TransformWorldPoint( b2WorldTransform t, b2Vec2 p )
{
	float rx = t.q.c * p.x - t.q.s * p.y;
	float ry = t.q.s * p.x + t.q.c * p.y;
	return b2G_v( t.p.x + rx, t.p.y + ry );
}
B2G_INLINE b2Vec2 b2InvTransformWorldPoint( b2WorldTransform t, b2Pos p ) { return b2InvTransformPoint( t, p ); }
B2G_INLINE b2Transform b2InvMulWorldTransforms( b2WorldTransform A, b2WorldTransform B ) { return b2InvMulTransforms( A, B ); }
B2G_INLINE b2WorldTransform b2MulWorldTransforms( b2WorldTransform A, b2Transform B )
{
	b2WorldTransform C;
	C.q = b2MulRot( A.q, B.q );
	C.p = b2OffsetPos( A.p, b2RotateVector( A.q, B.p ) );
	return C;
}
B2G_INLINE b2Transform b2ToRelativeTransform( b2WorldTransform t, b2Pos base )
{
	b2Transform r;
	r.q = t.q;
	r.p = b2G_v( t.p.x - base.x, t.p.y - base.y );
	return r;
}
B2G_INLINE b2WorldTransform b2MakeWorldTransform( b2Transform t ) { return t; }

/* ---- 2x2 matrices ---- */
B2G_INLINE b2Vec2 b2MulMV( b2Mat22 A, b2Vec2 v )
{
	return b2G_v( A.cx.x * v.x + A.cy.x * v.y, A.cx.y * v.x + A.cy.y * v.y );
}
B2G_INLINE b2Mat22 b2GetInverse22( b2Mat22 A )
{
	float a = A.cx.x, b = A.cy.x, c = A.cx.y, d = A.cy.y;
	float det = a * d - b * c;
	if ( det != 0.0f ) det = 1.0f / det;
	b2Mat22 B = { { det * d, -det * c }, { -det * b, det * a } };
	return B;
}
/* solve A x = b by Cramer's rule (zero determinant gives zero) */
B2G_INLINE b2Vec2 b2Solve22( b2Mat22 A, b2Vec2 b )
{
	float a11 = A.cx.x, a12 = A.cy.x, a21 = A.cx.y, a22 = A.cy.y;
	float det = a11 * a22 - a12 * a21;
	if ( det != 0.0f ) det = 1.0f / det;
	return b2G_v( det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) );
}

/* ---- boxes, planes, springs ---- */
B2G_INLINE bool b2AABB_Contains( b2AABB a, b2AABB b )
{
	return a.lowerBound.x <= b.lowerBound.x && a.lowerBound.y <= b.lowerBound.y && b.upperBound.x <= a.upperBound.x &&
		   b.upperBound.y <= a.upperBound.y;
}
B2G_INLINE b2Vec2 b2AABB_Center( b2AABB a )
{
	return b2G_v( 0.5f * ( a.lowerBound.x + a.upperBound.x ), 0.5f * ( a.lowerBound.y + a.upperBound.y ) );
}
B2G_INLINE b2Vec2 b2AABB_Extents( b2AABB a )
{
	return b2G_v( 0.5f * ( a.upperBound.x - a.lowerBound.x ), 0.5f * ( a.upperBound.y - a.lowerBound.y ) );
}
B2G_INLINE b2AABB b2AABB_Union( b2AABB a, b2AABB b )
{
	b2AABB c;
	c.lowerBound = b2Min( a.lowerBound, b.lowerBound );
	c.upperBound = b2Max( a.upperBound, b.upperBound );
	return c;
}
B2G_INLINE bool b2AABB_Overlaps( b2AABB a, b2AABB b )
{
	return !( b.lowerBound.x > a.upperBound.x || b.lowerBound.y > a.upperBound.y || a.lowerBound.x > b.upperBound.x ||
			  a.lowerBound.y > b.upperBound.y );
}
B2G_INLINE b2AABB b2MakeAABB( const b2Vec2* points, int count, float radius )
{
	b2AABB a = { points[0], points[0] };
	for ( int i = 1; i < count; ++i )
	{
		a.lowerBound = b2Min( a.lowerBound, points[i] );
		a.upperBound = b2Max( a.upperBound, points[i] );
	}
	b2Vec2 r = { radius, radius };
	a.lowerBound = b2Sub( a.lowerBound, r );
	a.upperBound = b2Add( a.upperBound, r );
	return a;
}
B2G_INLINE float b2PlaneSeparation( b2Plane plane, b2Vec2 point ) { return b2Dot( plane.normal, point ) - plane.offset; }
/* implicit spring-damper velocity update (one step of a damped harmonic oscillator) */
B2G_INLINE float b2SpringDamper( float hertz, float dampingRatio, float position, float velocity, float timeStep )
{
	float omega = 2.0f * B2_PI * hertz;
	float omegaH = omega * timeStep;
	return ( velocity - omega * omegaH * position ) / ( 1.0f + 2.0f * dampingRatio * omegaH + omegaH * omegaH );
}

#endif
