/*
 * Oracle (test checker only): FP64 tangent-linear model of recorded GB300 steps, the
 * reference for the adjoint of box2d_gb300_diff.h.
 *
 * Input is one world's tape as b2Diff_DownloadTape returns it. The recorded trajectory is
 * replayed on the host in float, operation for operation as the step computes it
 * (contact_solver.c:1573-2331, solver.c:66-162 and :583-600, contact.c:519-698,
 * physics_world.c:508-560), so every branch (clamp, speculative or soft contact, friction
 * cone, speed cap, clip and edge choice) is the recorded one; each float carries one tangent
 * in double, propagated forward from a direction in (initial velocity, friction) space.
 * Every step's replay must land bit for bit on the next recorded step.
 *
 * Nothing of the product's differentiation code is used here: the dual numbers, the vector
 * math and the polygon contact (manifold.c:511-1028) are this file's own, restated from the
 * reference; only the tape's record layout (b2g_device_abi.h) is shared.
 */
#include "../box2d_gb300/csrc/b2g_device_abi.h"

#include <float.h>
#include <math.h>
#include <string.h>

#include <vector>

/* ---- dual numbers: the float value as the step computes it, one double tangent ----
   Every value operation is the plain float operation in the order the expression is
   written (this file is compiled with -ffp-contract=off), so the value of a computation
   equals the step's float result bit for bit; the tangent follows the chain rule in
   double. */
struct T1
{
	float v;
	double d[1];
	static T1 make( float x )
	{
		T1 r;
		r.v = x;
		r.d[0] = 0.0;
		return r;
	}
};

static inline T1 t_num( float v, double d )
{
	T1 r;
	r.v = v;
	r.d[0] = d;
	return r;
}
static inline T1 operator+( const T1& a, const T1& b ) { return t_num( a.v + b.v, a.d[0] + b.d[0] ); }
static inline T1 operator-( const T1& a, const T1& b ) { return t_num( a.v - b.v, a.d[0] - b.d[0] ); }
static inline T1 operator-( const T1& a ) { return t_num( -a.v, -a.d[0] ); }
static inline T1 operator*( const T1& a, const T1& b )
{
	return t_num( a.v * b.v, a.d[0] * (double)b.v + (double)a.v * b.d[0] );
}
static inline T1 operator/( const T1& a, const T1& b )
{
	float q = a.v / b.v;
	return t_num( q, ( a.d[0] - (double)q * b.d[0] ) / (double)b.v );
}
static inline T1 operator+( float a, const T1& b ) { return t_num( a + b.v, b.d[0] ); }
static inline T1 operator+( const T1& a, float b ) { return t_num( a.v + b, a.d[0] ); }
static inline T1 operator-( float a, const T1& b ) { return t_num( a - b.v, -b.d[0] ); }
static inline T1 operator-( const T1& a, float b ) { return t_num( a.v - b, a.d[0] ); }
static inline T1 operator*( float a, const T1& b ) { return t_num( a * b.v, (double)a * b.d[0] ); }
static inline T1 operator*( const T1& a, float b ) { return t_num( a.v * b, a.d[0] * (double)b ); }
static inline T1 operator/( float a, const T1& b )
{
	float q = a / b.v;
	return t_num( q, -(double)q * b.d[0] / (double)b.v );
}
static inline T1 operator/( const T1& a, float b ) { return t_num( a.v / b, a.d[0] / (double)b ); }
static inline T1 t_sqrt( const T1& a )
{
	float r = sqrtf( a.v );
	return t_num( r, r > 0.0f ? a.d[0] / ( 2.0 * (double)r ) : 0.0 );
}

struct V1
{
	T1 x, y;
};
struct R1
{
	T1 c, s;
};
struct t_xf
{
	V1 p;
	R1 q;
};

static inline T1 t_c( float x ) { return T1::make( x ); }
static inline T1 t_v( float x, double d ) { return t_num( x, d ); }
static inline V1 t_v2( T1 x, T1 y )
{
	V1 r = { x, y };
	return r;
}
static inline V1 t_vec( b2Vec2 a ) { return t_v2( t_c( a.x ), t_c( a.y ) ); }
static inline V1 t_add( V1 a, V1 b ) { return t_v2( a.x + b.x, a.y + b.y ); }
static inline V1 t_sub( V1 a, V1 b ) { return t_v2( a.x - b.x, a.y - b.y ); }
static inline T1 t_dot( V1 a, V1 b ) { return a.x * b.x + a.y * b.y; }
static inline T1 t_cross( V1 a, V1 b ) { return a.x * b.y - a.y * b.x; }
/* math_functions.h b2RotateVector, b2InvRotateVector, b2InvMulRot, b2TransformPoint, b2Lerp */
static inline V1 t_rotate( R1 q, V1 v ) { return t_v2( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
static inline V1 t_invRotate( R1 q, V1 v ) { return t_v2( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }
static inline R1 t_invMulRot( R1 a, R1 b )
{
	R1 r = { a.c * b.c + a.s * b.s, a.c * b.s - a.s * b.c };
	return r;
}
static inline V1 t_transformPoint( const t_xf& t, V1 p )
{
	return t_v2( ( t.q.c * p.x - t.q.s * p.y ) + t.p.x, ( t.q.s * p.x + t.q.c * p.y ) + t.p.y );
}
static inline V1 t_lerp( V1 a, V1 b, float t )
{
	return t_v2( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y );
}
static inline V1 t_lerpT( V1 a, V1 b, T1 t ) { return t_v2( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y ); }
static inline V1 t_mulAdd( V1 a, T1 s, V1 b ) { return t_v2( a.x + s * b.x, a.y + s * b.y ); }
static inline T1 t_max( const T1& a, const T1& b ) { return a.v > b.v ? a : b; }
static inline T1 t_min( const T1& a, const T1& b ) { return a.v < b.v ? a : b; }
static inline T1 t_clamp( const T1& a, float lo, float hi ) { return a.v < lo ? t_c( lo ) : ( a.v > hi ? t_c( hi ) : a ); }

/* ---- polygon contact in duals (manifold.c:511-1028 b2CollidePolygons with its clip and
   edge search, contact.c:519-545 and physics_world.c:568-569 for the world anchors) ----
   Written here for the checker alone: the value path is the reference's float operation
   order, so the recorded feature ids, edge choices and clip branches come out again, and
   the tangents are the Jacobian of the manifold with respect to both poses. */
#define T_LINEAR_SLOP 0.005f
#define T_SPECULATIVE_DISTANCE ( 4.0f * T_LINEAR_SLOP )
#define T_MAKE_ID( A, B ) ( (uint16_t)( (uint8_t)( A ) << 8 | (uint8_t)( B ) ) )

struct t_polygon
{
	int count;
	float radius;
	V1 v[B2_MAX_POLYGON_VERTICES], n[B2_MAX_POLYGON_VERTICES];
};

struct t_local
{
	int count;
	V1 normal;
	V1 point[2];
	T1 separation[2];
	uint16_t id[2];
};

/* the contact geometry the solver reads: world normal, anchors relative to the centers of
   mass, separations and feature ids */
struct t_geometry
{
	int count;
	V1 normal;
	V1 anchorA[2], anchorB[2];
	T1 separation[2];
	uint16_t id[2];
};

/* manifold.c:646-682 */
static T1 t_findMaxSeparation( int* edgeIndex, const t_polygon& poly1, const t_polygon& poly2 )
{
	int bestIndex = 0;
	T1 maxSeparation = t_c( -FLT_MAX );
	for ( int i = 0; i < poly1.count; ++i )
	{
		V1 n = poly1.n[i];
		V1 v1 = poly1.v[i];
		T1 si = t_c( FLT_MAX );
		for ( int j = 0; j < poly2.count; ++j )
		{
			T1 sij = t_dot( n, t_sub( poly2.v[j], v1 ) );
			if ( sij.v < si.v ) si = sij;
		}
		if ( si.v > maxSeparation.v )
		{
			maxSeparation = si;
			bestIndex = i;
		}
	}
	*edgeIndex = bestIndex;
	return maxSeparation;
}

/* manifold.c:511-643 */
static t_local t_clipPolygons( const t_polygon& polyA, const t_polygon& polyB, int edgeA, int edgeB, bool flip )
{
	t_local m;
	memset( &m, 0, sizeof( m ) );
	const t_polygon* poly1 = flip ? &polyB : &polyA;
	const t_polygon* poly2 = flip ? &polyA : &polyB;
	int i11 = flip ? edgeB : edgeA;
	int i12 = i11 + 1 < poly1->count ? i11 + 1 : 0;
	int i21 = flip ? edgeA : edgeB;
	int i22 = i21 + 1 < poly2->count ? i21 + 1 : 0;
	V1 normal = poly1->n[i11];
	V1 v11 = poly1->v[i11], v12 = poly1->v[i12];
	V1 v21 = poly2->v[i21], v22 = poly2->v[i22];
	V1 tangent = t_v2( -1.0f * normal.y, 1.0f * normal.x );
	T1 lower1 = t_c( 0.0f );
	T1 upper1 = t_dot( t_sub( v12, v11 ), tangent );
	T1 upper2 = t_dot( t_sub( v21, v11 ), tangent );
	T1 lower2 = t_dot( t_sub( v22, v11 ), tangent );
	if ( upper2.v < lower1.v || upper1.v < lower2.v ) return m;
	V1 vLower;
	if ( lower2.v < lower1.v && ( upper2 - lower2 ).v > FLT_EPSILON )
		vLower = t_lerpT( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = v22;
	V1 vUpper;
	if ( upper2.v > upper1.v && ( upper2 - lower2 ).v > FLT_EPSILON )
		vUpper = t_lerpT( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = v21;
	T1 separationLower = t_dot( t_sub( vLower, v11 ), normal );
	T1 separationUpper = t_dot( t_sub( vUpper, v11 ), normal );
	float r1 = poly1->radius, r2 = poly2->radius;
	vLower = t_mulAdd( vLower, 0.5f * ( r1 - r2 - separationLower ), normal );
	vUpper = t_mulAdd( vUpper, 0.5f * ( r1 - r2 - separationUpper ), normal );
	float radius = r1 + r2;
	m.count = 2;
	if ( flip == false )
	{
		m.normal = normal;
		m.point[0] = vLower;
		m.separation[0] = separationLower - radius;
		m.id[0] = T_MAKE_ID( i11, i22 );
		m.point[1] = vUpper;
		m.separation[1] = separationUpper - radius;
		m.id[1] = T_MAKE_ID( i12, i21 );
	}
	else
	{
		m.normal = t_v2( -normal.x, -normal.y );
		m.point[0] = vUpper;
		m.separation[0] = separationUpper - radius;
		m.id[0] = T_MAKE_ID( i21, i12 );
		m.point[1] = vLower;
		m.separation[1] = separationLower - radius;
		m.id[1] = T_MAKE_ID( i22, i11 );
	}
	return m;
}

/* distance.c:33-106 b2SegmentDistance */
struct t_segmentDistance
{
	T1 fraction1, fraction2, distanceSquared;
};

static t_segmentDistance t_segDistance( V1 p1, V1 q1, V1 p2, V1 q2 )
{
	t_segmentDistance res;
	V1 d1 = t_sub( q1, p1 ), d2 = t_sub( q2, p2 ), r = t_sub( p1, p2 );
	T1 dd1 = t_dot( d1, d1 ), dd2 = t_dot( d2, d2 ), rd1 = t_dot( r, d1 ), rd2 = t_dot( r, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	T1 f1 = t_c( 0.0f ), f2 = t_c( 0.0f );
	if ( dd1.v < epsSqr || dd2.v < epsSqr )
	{
		if ( dd1.v >= epsSqr ) f1 = t_clamp( -rd1 / dd1, 0.0f, 1.0f );
		else if ( dd2.v >= epsSqr ) f2 = t_clamp( rd2 / dd2, 0.0f, 1.0f );
	}
	else
	{
		T1 d12 = t_dot( d1, d2 );
		T1 denom = dd1 * dd2 - d12 * d12;
		if ( denom.v != 0.0f ) f1 = t_clamp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
		f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2.v < 0.0f )
		{
			f2 = t_c( 0.0f );
			f1 = t_clamp( -rd1 / dd1, 0.0f, 1.0f );
		}
		else if ( f2.v > 1.0f )
		{
			f2 = t_c( 1.0f );
			f1 = t_clamp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
		}
	}
	V1 closest1 = t_mulAdd( p1, f1, d1 );
	V1 closest2 = t_mulAdd( p2, f2, d2 );
	V1 dc = t_sub( closest2, closest1 );
	res.fraction1 = f1;
	res.fraction2 = f2;
	res.distanceSquared = dc.x * dc.x + dc.y * dc.y;
	return res;
}

/* manifold.c:702-1028, in frame A after the relative transform */
static t_local t_collidePolygons( const t_polygon& polyA, const t_polygon& polyB, const t_xf& xf )
{
	t_local empty;
	memset( &empty, 0, sizeof( empty ) );
	V1 origin = polyA.v[0];
	t_xf xfs = { t_sub( xf.p, origin ), xf.q };
	t_polygon A, B;
	A.count = polyA.count;
	A.radius = polyA.radius;
	A.v[0] = t_v2( t_c( 0.0f ), t_c( 0.0f ) );
	A.n[0] = polyA.n[0];
	for ( int i = 1; i < A.count; ++i )
	{
		A.v[i] = t_sub( polyA.v[i], origin );
		A.n[i] = polyA.n[i];
	}
	B.count = polyB.count;
	B.radius = polyB.radius;
	for ( int i = 0; i < B.count; ++i )
	{
		B.v[i] = t_transformPoint( xfs, polyB.v[i] );
		B.n[i] = t_rotate( xfs.q, polyB.n[i] );
	}
	int edgeA = 0;
	T1 separationA = t_findMaxSeparation( &edgeA, A, B );
	int edgeB = 0;
	T1 separationB = t_findMaxSeparation( &edgeB, B, A );
	float radius = A.radius + B.radius;
	if ( separationA.v > T_SPECULATIVE_DISTANCE + radius || separationB.v > T_SPECULATIVE_DISTANCE + radius ) return empty;
	bool flip;
	if ( separationA.v >= separationB.v )
	{
		flip = false;
		V1 search = A.n[edgeA];
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < B.count; ++i )
		{
			float d = t_dot( search, B.n[i] ).v;
			if ( d < minDot )
			{
				minDot = d;
				edgeB = i;
			}
		}
	}
	else
	{
		flip = true;
		V1 search = B.n[edgeB];
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < A.count; ++i )
		{
			float d = t_dot( search, A.n[i] ).v;
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}
	t_local m = empty;
	if ( separationA.v > 0.1f * T_LINEAR_SLOP || separationB.v > 0.1f * T_LINEAR_SLOP )
	{
		int i11 = edgeA, i12 = edgeA + 1 < A.count ? edgeA + 1 : 0;
		int i21 = edgeB, i22 = edgeB + 1 < B.count ? edgeB + 1 : 0;
		V1 v11 = A.v[i11], v12 = A.v[i12], v21 = B.v[i21], v22 = B.v[i22];
		t_segmentDistance res = t_segDistance( v11, v12, v21, v22 );
		T1 distance = t_sqrt( res.distanceSquared );
		T1 separation = distance - radius;
		if ( ( distance - radius ).v > T_SPECULATIVE_DISTANCE ) return m;
		m = t_clipPolygons( A, B, edgeA, edgeB, flip );
		float minSeparation = FLT_MAX;
		for ( int i = 0; i < m.count; ++i ) minSeparation = minSeparation < m.separation[i].v ? minSeparation : m.separation[i].v;
		if ( ( separation + 0.1f * T_LINEAR_SLOP ).v < minSeparation )
		{
			float f1 = res.fraction1.v, f2 = res.fraction2.v;
			bool hit = ( f1 == 0.0f || f1 == 1.0f ) && ( f2 == 0.0f || f2 == 1.0f );
			if ( hit )
			{
				V1 va = f1 == 0.0f ? v11 : v12;
				V1 vb = f2 == 0.0f ? v21 : v22;
				int ia = f1 == 0.0f ? i11 : i12;
				int ib = f2 == 0.0f ? i21 : i22;
				V1 normal = t_sub( vb, va );
				T1 invDistance = 1.0f / distance;
				normal.x = normal.x * invDistance;
				normal.y = normal.y * invDistance;
				V1 c1 = t_mulAdd( va, t_c( A.radius ), normal );
				V1 c2 = t_mulAdd( vb, t_c( -B.radius ), normal );
				m.count = 1;
				m.normal = normal;
				m.point[0] = t_lerp( c1, c2, 0.5f );
				m.separation[0] = distance - radius;
				m.id[0] = T_MAKE_ID( ia, ib );
			}
		}
	}
	else
	{
		m = t_clipPolygons( A, B, edgeA, edgeB, flip );
	}
	for ( int i = 0; i < m.count; ++i ) m.point[i] = t_add( m.point[i], origin );
	return m;
}

static t_polygon t_polygonOf( const b2gShape* s )
{
	t_polygon p;
	p.count = s->count;
	p.radius = s->radius;
	for ( int i = 0; i < s->count; ++i )
	{
		p.v[i] = t_vec( s->v[i] );
		p.n[i] = t_vec( s->n[i] );
	}
	return p;
}

/* manifold.c:16-34 b2MakeCapsule: a capsule (or a segment, radius 0) as a two-vertex
   polygon; shape-local constants, in float */
static t_polygon t_capsulePolygon( b2Vec2 p1, b2Vec2 p2, float radius )
{
	t_polygon p;
	memset( &p, 0, sizeof( p ) );
	float dx = p2.x - p1.x, dy = p2.y - p1.y;
	float lengthSquared = dx * dx + dy * dy;
	float ax = 0.0f, ay = 0.0f;
	if ( lengthSquared > 1000.0f * FLT_MIN )
	{
		float s = 1.0f / sqrtf( lengthSquared );
		ax = s * dx;
		ay = s * dy;
	}
	/* right perpendicular of the axis, then its negation */
	b2Vec2 n0 = { ay, -ax }, n1 = { -ay, ax };
	p.count = 2;
	p.radius = radius;
	p.v[0] = t_vec( p1 );
	p.v[1] = t_vec( p2 );
	p.n[0] = t_vec( n0 );
	p.n[1] = t_vec( n1 );
	return p;
}

/* math_functions.h b2Normalize / b2GetLengthAndNormalize */
static V1 t_normalize( V1 a )
{
	T1 lengthSquared = a.x * a.x + a.y * a.y;
	if ( lengthSquared.v > 1000.0f * FLT_MIN )
	{
		T1 s = 1.0f / t_sqrt( lengthSquared );
		return t_v2( s * a.x, s * a.y );
	}
	return t_v2( t_c( 0.0f ), t_c( 0.0f ) );
}

static V1 t_lengthAndNormalize( T1* length, V1 a )
{
	T1 lengthSquared = a.x * a.x + a.y * a.y;
	if ( lengthSquared.v > 1000.0f * FLT_MIN )
	{
		*length = t_sqrt( lengthSquared );
		T1 s = 1.0f / *length;
		return t_v2( s * a.x, s * a.y );
	}
	*length = t_c( 0.0f );
	return t_v2( t_c( 0.0f ), t_c( 0.0f ) );
}

static t_local t_emptyLocal( void )
{
	t_local m;
	memset( &m, 0, sizeof( m ) );
	return m;
}

/* manifold.c:36-66 */
static t_local t_collideCircles( V1 centerA, float radiusA, V1 centerB, float radiusB, const t_xf& xf )
{
	t_local m = t_emptyLocal();
	V1 pointA = centerA;
	V1 pointB = t_transformPoint( xf, centerB );
	T1 distance;
	V1 normal = t_lengthAndNormalize( &distance, t_sub( pointB, pointA ) );
	T1 separation = distance - radiusA - radiusB;
	if ( separation.v > T_SPECULATIVE_DISTANCE ) return m;
	V1 cA = t_v2( pointA.x + radiusA * normal.x, pointA.y + radiusA * normal.y );
	V1 cB = t_v2( pointB.x + ( -radiusB ) * normal.x, pointB.y + ( -radiusB ) * normal.y );
	m.normal = normal;
	m.point[0] = t_lerp( cA, cB, 0.5f );
	m.separation[0] = separation;
	m.id[0] = 0;
	m.count = 1;
	return m;
}

/* manifold.c:127-230 */
static t_local t_collidePolygonAndCircle( const t_polygon& poly, V1 centerB, float radiusB, const t_xf& xf )
{
	t_local m = t_emptyLocal();
	V1 center = t_transformPoint( xf, centerB );
	float radiusA = poly.radius;
	float radius = radiusA + radiusB;
	int normalIndex = 0;
	T1 separation = t_c( -FLT_MAX );
	for ( int i = 0; i < poly.count; ++i )
	{
		T1 s = t_dot( poly.n[i], t_sub( center, poly.v[i] ) );
		if ( s.v > separation.v )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation.v > radius + T_SPECULATIVE_DISTANCE ) return m;
	int i1 = normalIndex, i2 = i1 + 1 < poly.count ? i1 + 1 : 0;
	V1 v1 = poly.v[i1], v2 = poly.v[i2];
	T1 u1 = t_dot( t_sub( center, v1 ), t_sub( v2, v1 ) );
	T1 u2 = t_dot( t_sub( center, v2 ), t_sub( v1, v2 ) );
	for ( int k = 0; k < 2; ++k )
	{
		/* the circle center closest to vertex 1, then vertex 2, and safely outside */
		T1 u = k == 0 ? u1 : u2;
		if ( !( u.v < 0.0f && separation.v > FLT_EPSILON ) ) continue;
		V1 v = k == 0 ? v1 : v2;
		V1 normal = t_normalize( t_sub( center, v ) );
		T1 sep = t_dot( t_sub( center, v ), normal );
		if ( sep.v > radius + T_SPECULATIVE_DISTANCE ) return m;
		V1 cA = t_v2( v.x + radiusA * normal.x, v.y + radiusA * normal.y );
		V1 cB = t_v2( center.x - radiusB * normal.x, center.y - radiusB * normal.y );
		m.normal = normal;
		m.point[0] = t_lerp( cA, cB, 0.5f );
		m.separation[0] = t_dot( t_sub( cB, cA ), normal );
		m.id[0] = 0;
		m.count = 1;
		return m;
	}
	V1 normal = poly.n[normalIndex];
	m.normal = normal;
	T1 depth = radiusA - t_dot( t_sub( center, v1 ), normal );
	V1 cA = t_v2( center.x + depth * normal.x, center.y + depth * normal.y );
	V1 cB = t_v2( center.x - radiusB * normal.x, center.y - radiusB * normal.y );
	m.point[0] = t_lerp( cA, cB, 0.5f );
	m.separation[0] = separation - radius;
	m.id[0] = 0;
	m.count = 1;
	return m;
}

/* contact.c:519-545 and :619-623: the manifold in frame A, then world anchors, then
   anchors relative to the centers of mass (physics_world.c:568-569); polygons and circles,
   a mixed pair with the polygon as shape A */
static t_geometry t_polygonContact( const b2gShape* shapeA, const b2gShape* shapeB, const t_xf& xfA, const t_xf& xfB, b2Vec2 lcA,
								   b2Vec2 lcB )
{
	t_xf rel;
	rel.q = t_invMulRot( xfA.q, xfB.q );
	rel.p = t_invRotate( xfA.q, t_v2( xfB.p.x - xfA.p.x, xfB.p.y - xfA.p.y ) );
	t_local local;
	if ( shapeA->type == b2_polygonShape && shapeB->type == b2_polygonShape )
		local = t_collidePolygons( t_polygonOf( shapeA ), t_polygonOf( shapeB ), rel );
	else if ( shapeA->type == b2_polygonShape && shapeB->type == b2_capsuleShape )
		local = t_collidePolygons( t_polygonOf( shapeA ), t_capsulePolygon( shapeB->v[0], shapeB->v[1], shapeB->radius ), rel );
	else if ( shapeA->type == b2_segmentShape )
		local = t_collidePolygons( t_capsulePolygon( shapeA->v[0], shapeA->v[1], 0.0f ), t_polygonOf( shapeB ), rel );
	else if ( shapeA->type == b2_polygonShape )
		local = t_collidePolygonAndCircle( t_polygonOf( shapeA ), t_vec( shapeB->v[0] ), shapeB->radius, rel );
	else
		local = t_collideCircles( t_vec( shapeA->v[0] ), shapeA->radius, t_vec( shapeB->v[0] ), shapeB->radius, rel );
	t_geometry g;
	memset( &g, 0, sizeof( g ) );
	g.count = local.count;
	g.normal = t_rotate( xfA.q, local.normal );
	V1 originDelta = t_v2( xfA.p.x - xfB.p.x, xfA.p.y - xfB.p.y );
	V1 centerOffsetA = t_rotate( xfA.q, t_vec( lcA ) );
	V1 centerOffsetB = t_rotate( xfB.q, t_vec( lcB ) );
	for ( int i = 0; i < local.count; ++i )
	{
		V1 anchorA = t_rotate( xfA.q, local.point[i] );
		V1 anchorB = t_add( anchorA, originDelta );
		g.anchorA[i] = t_sub( anchorA, centerOffsetA );
		g.anchorB[i] = t_sub( anchorB, centerOffsetB );
		g.separation[i] = local.separation[i];
		g.id[i] = local.id[i];
	}
	return g;
}

/* body state of the substep loop */
struct t_body
{
	T1 vx, vy, w;
	uint32_t flags;
	T1 dpx, dpy, dqc, dqs;
};

/* contact constraint lane (the fields of b2gContactLane the stages read) */
struct t_lane
{
	int indexA, indexB;
	float invMassA, invMassB, invIA, invIB;
	V1 normal;
	T1 friction;
	float tangentSpeed, restitution;
	float biasRate, massScale, impulseScale;
	V1 anchorA[2], anchorB[2];
	T1 normalMass[2], tangentMass[2], baseSeparation[2], normalImpulse[2], tangentImpulse[2], totalNormalImpulse[2];
	T1 relativeVelocity[2];
	T1 rollingImpulse;
	float rollingMass, rollingResistance;
	int groupFlags;
	int pointCount;
};

/* manifold state carried by contact id between steps */
struct t_manifold
{
	V1 normal;
	V1 anchorA[2], anchorB[2];
	T1 baseSeparation[2], separation[2], normalImpulse[2], tangentImpulse[2];
	T1 rollingImpulse;
	R1 cachedA, cachedB;
	uint16_t id[2];
	int pointCount;
	bool valid;
};

static t_body t_static( void )
{
	t_body b;
	b.vx = t_c( 0.0f );
	b.vy = t_c( 0.0f );
	b.w = t_c( 0.0f );
	b.flags = 0;
	b.dpx = t_c( 0.0f );
	b.dpy = t_c( 0.0f );
	b.dqc = t_c( 1.0f );
	b.dqs = t_c( 0.0f );
	return b;
}

/* ---------------- stages (the device's operation order) ---------------- */

static void t_apply( const t_lane& c, t_body* A, t_body* B, V1 rA, V1 rB, T1 Px, T1 Py )
{
	A->vx = A->vx - c.invMassA * Px;
	A->vy = A->vy - c.invMassA * Py;
	A->w = A->w - c.invIA * ( rA.x * Py - rA.y * Px );
	B->vx = B->vx + c.invMassB * Px;
	B->vy = B->vy + c.invMassB * Py;
	B->w = B->w + c.invIB * ( rB.x * Py - rB.y * Px );
}

static void t_warmStart( t_lane& c, t_body* A, t_body* B )
{
	T1 tx = c.normal.y, ty = 0.0f - c.normal.x;
	for ( int p = 0; p < 2; ++p )
	{
		V1 rA = c.anchorA[p], rB = c.anchorB[p];
		T1 Px = c.normalImpulse[p] * c.normal.x + c.tangentImpulse[p] * tx;
		T1 Py = c.normalImpulse[p] * c.normal.y + c.tangentImpulse[p] * ty;
		A->w = A->w - c.invIA * ( rA.x * Py - rA.y * Px );
		A->vx = A->vx - c.invMassA * Px;
		A->vy = A->vy - c.invMassA * Py;
		B->w = B->w + c.invIB * ( rB.x * Py - rB.y * Px );
		B->vx = B->vx + c.invMassB * Px;
		B->vy = B->vy + c.invMassB * Py;
		c.totalNormalImpulse[p] = c.totalNormalImpulse[p] + c.normalImpulse[p];
	}
	/* contact_solver.c:1863-1864 */
	A->w = A->w - c.invIA * c.rollingImpulse;
	B->w = B->w + c.invIB * c.rollingImpulse;
}

static void t_normalPoint( t_lane& c, int p, t_body* A, t_body* B, T1 dpx, T1 dpy, float biasRate, float massScale, float impulseScale,
						   float inv_h, float contactSpeed, T1* total )
{
	V1 rA = c.anchorA[p], rB = c.anchorB[p];
	T1 rsAx = A->dqc * rA.x - A->dqs * rA.y;
	T1 rsAy = A->dqs * rA.x + A->dqc * rA.y;
	T1 rsBx = B->dqc * rB.x - B->dqs * rB.y;
	T1 rsBy = B->dqs * rB.x + B->dqc * rB.y;
	T1 dsx = dpx + ( rsBx - rsAx );
	T1 dsy = dpy + ( rsBy - rsAy );
	T1 s = ( c.normal.x * dsx + c.normal.y * dsy ) + c.baseSeparation[p];
	bool mask = s.v > 0.0f;
	T1 specBias = s * inv_h;
	T1 softBias = t_max( biasRate * s, t_c( contactSpeed ) );
	T1 bias = mask ? specBias : softBias;
	float pointMassScale = mask ? 1.0f : massScale;
	float pointImpulseScale = mask ? 0.0f : impulseScale;
	T1 dvx = ( B->vx - B->w * rB.y ) - ( A->vx - A->w * rA.y );
	T1 dvy = ( B->vy + B->w * rB.x ) - ( A->vy + A->w * rA.x );
	T1 vn = dvx * c.normal.x + dvy * c.normal.y;
	T1 negImpulse = c.normalMass[p] * ( pointMassScale * vn + bias ) + pointImpulseScale * c.normalImpulse[p];
	T1 newImpulse = t_max( c.normalImpulse[p] - negImpulse, t_c( 0.0f ) );
	T1 impulse = newImpulse - c.normalImpulse[p];
	c.normalImpulse[p] = newImpulse;
	c.totalNormalImpulse[p] = c.totalNormalImpulse[p] + impulse;
	*total = *total + newImpulse;
	t_apply( c, A, B, rA, rB, impulse * c.normal.x, impulse * c.normal.y );
}

static void t_frictionPoint( t_lane& c, int p, t_body* A, t_body* B )
{
	V1 rA = c.anchorA[p], rB = c.anchorB[p];
	T1 tx = c.normal.y;
	T1 ty = 0.0f - c.normal.x;
	T1 dvx = ( B->vx - B->w * rB.y ) - ( A->vx - A->w * rA.y );
	T1 dvy = ( B->vy + B->w * rB.x ) - ( A->vy + A->w * rA.x );
	T1 vt = dvx * tx + dvy * ty;
	vt = vt - c.tangentSpeed;
	T1 negImpulse = c.tangentMass[p] * vt;
	T1 maxFriction = c.friction * c.normalImpulse[p];
	T1 newImpulse = c.tangentImpulse[p] - negImpulse;
	newImpulse = t_max( 0.0f - maxFriction, t_min( newImpulse, maxFriction ) );
	T1 impulse = newImpulse - c.tangentImpulse[p];
	c.tangentImpulse[p] = newImpulse;
	t_apply( c, A, B, rA, rB, impulse * tx, impulse * ty );
}

static void t_solve( t_lane& c, t_body* A, t_body* B, float inv_h, float contactSpeedNeg, bool useBias )
{
	float biasRate, massScale, impulseScale;
	if ( useBias )
	{
		biasRate = c.massScale * c.biasRate;
		massScale = c.massScale;
		impulseScale = c.impulseScale;
	}
	else
	{
		biasRate = 0.0f;
		massScale = 1.0f;
		impulseScale = 0.0f;
	}
	T1 dpx = B->dpx - A->dpx, dpy = B->dpy - A->dpy;
	T1 total = t_c( 0.0f );
	t_normalPoint( c, 0, A, B, dpx, dpy, biasRate, massScale, impulseScale, inv_h, contactSpeedNeg, &total );
	t_normalPoint( c, 1, A, B, dpx, dpy, biasRate, massScale, impulseScale, inv_h, contactSpeedNeg, &total );
	if ( useBias == false )
	{
		/* rolling resistance (contact_solver.c:2021-2031) */
		if ( c.groupFlags & 1 )
		{
			T1 deltaLambda = c.rollingMass * ( A->w - B->w );
			T1 lambda = c.rollingImpulse;
			T1 maxLambda = c.rollingResistance * total;
			T1 nb = -maxLambda;
			c.rollingImpulse = t_max( nb, t_min( lambda + deltaLambda, maxLambda ) );
			deltaLambda = c.rollingImpulse - lambda;
			A->w = A->w - c.invIA * deltaLambda;
			B->w = B->w + c.invIB * deltaLambda;
		}
		t_frictionPoint( c, 0, A, B );
		t_frictionPoint( c, 1, A, B );
	}
}

static void t_restitution( t_lane& c, t_body* A, t_body* B, float threshold )
{
	if ( ( c.groupFlags & 2 ) == 0 ) return;
	for ( int p = 0; p < 2; ++p )
	{
		V1 rA = c.anchorA[p], rB = c.anchorB[p];
		bool mask = ( c.relativeVelocity[p].v + threshold > 0.0f ) || ( c.totalNormalImpulse[p].v == 0.0f ) || ( c.restitution == 0.0f );
		T1 mass = mask ? t_c( 0.0f ) : c.normalMass[p];
		T1 dvx = ( B->vx - B->w * rB.y ) - ( A->vx - A->w * rA.y );
		T1 dvy = ( B->vy + B->w * rB.x ) - ( A->vy + A->w * rA.x );
		T1 vn = dvx * c.normal.x + dvy * c.normal.y;
		T1 negImpulse = mass * ( vn + c.restitution * c.relativeVelocity[p] );
		T1 newImpulse = t_max( c.normalImpulse[p] - negImpulse, t_c( 0.0f ) );
		T1 deltaImpulse = newImpulse - c.normalImpulse[p];
		c.normalImpulse[p] = newImpulse;
		c.totalNormalImpulse[p] = c.totalNormalImpulse[p] + deltaImpulse;
		t_apply( c, A, B, rA, rB, deltaImpulse * c.normal.x, deltaImpulse * c.normal.y );
	}
}

static void t_integrateVelocities( const b2gStepParams& P, t_body* b, const float* pr )
{
	float h = P.h;
	float linearDamping = 1.0f / ( 1.0f + h * pr[3] );
	float angularDamping = 1.0f / ( 1.0f + h * pr[4] );
	float invMass = pr[6];
	float gravityScale = invMass > 0.0f ? pr[5] : 0.0f;
	float lvdx = ( h * invMass ) * pr[0] + ( h * gravityScale ) * P.gravityX;
	float lvdy = ( h * invMass ) * pr[1] + ( h * gravityScale ) * P.gravityY;
	float avd = h * pr[7] * pr[2];
	b->vx = lvdx + linearDamping * b->vx;
	b->vy = lvdy + linearDamping * b->vy;
	b->w = avd + angularDamping * b->w;
}

static void t_integratePositions( const b2gStepParams& P, t_body* b )
{
	float h = P.h;
	float maxLinearSpeed = P.maxLinearVelocity;
	float maxAngularSpeed = ( 0.25f * B2_PI ) * P.inv_dt;
	float maxLinearSq = maxLinearSpeed * maxLinearSpeed;
	float maxAngularSq = maxAngularSpeed * maxAngularSpeed;
	uint32_t flags = b->flags;
	T1 vx = ( flags & B2G_LOCK_X ) ? t_c( 0.0f ) : b->vx;
	T1 vy = ( flags & B2G_LOCK_Y ) ? t_c( 0.0f ) : b->vy;
	T1 w = ( flags & B2G_LOCK_Z ) ? t_c( 0.0f ) : b->w;
	if ( ( vx * vx + vy * vy ).v > maxLinearSq )
	{
		T1 ratio = maxLinearSpeed / t_sqrt( vx * vx + vy * vy );
		vx = ratio * vx;
		vy = ratio * vy;
		flags |= B2G_SPEED_CAPPED;
	}
	if ( ( w * w ).v > maxAngularSq && ( flags & B2G_ALLOW_FAST_ROTATION ) == 0 )
	{
		T1 aw = w.v < 0.0f ? -w : w;
		T1 ratio = maxAngularSpeed / aw;
		w = w * ratio;
		flags |= B2G_SPEED_CAPPED;
	}
	b->dpx = b->dpx + h * vx;
	b->dpy = b->dpy + h * vy;
	T1 da = h * w;
	T1 q2c = b->dqc - da * b->dqs, q2s = b->dqs + da * b->dqc;
	T1 mag = t_sqrt( q2s * q2s + q2c * q2c );
	T1 inv = mag.v > 0.0f ? 1.0f / mag : t_c( 0.0f );
	b->dqc = q2c * inv;
	b->dqs = q2s * inv;
	b->vx = vx;
	b->vy = vy;
	b->w = w;
	b->flags = flags;
}

static void t_makeSoft( float hertz, float zeta, float h, float* biasRate, float* massScale, float* impulseScale )
{
	if ( hertz == 0.0f )
	{
		*biasRate = 0.0f;
		*massScale = 0.0f;
		*impulseScale = 0.0f;
		return;
	}
	float omega = 2.0f * B2_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	*biasRate = omega / a1;
	*massScale = a2 * a3;
	*impulseScale = a3;
}

/* contact_solver.c:1573-1809 for one colored slot; v0 are the awake bodies' velocities at
   the step's start */
static t_lane t_prepare( const b2gStepParams& P, const b2gContact* cs, const t_manifold& m, T1 friction, const std::vector<t_body>& v0 )
{
	t_lane c;
	memset( &c, 0, sizeof( c ) );
	float warmStartScale = P.enableWarmStarting ? 1.0f : 0.0f;
	int indexA = cs->bodySimIndexA, indexB = cs->bodySimIndexB;
	c.indexA = indexA + 1;
	c.indexB = indexB + 1;
	t_body zero = t_static();
	const t_body& A = indexA != -1 ? v0[indexA] : zero;
	const t_body& B = indexB != -1 ? v0[indexB] : zero;
	float mA = cs->invMassA, iA = cs->invIA, mB = cs->invMassB, iB = cs->invIB;
	c.invMassA = mA;
	c.invMassB = mB;
	c.invIA = iA;
	c.invIB = iB;
	{
		/* contact_solver.c:1675-1678, :1708-1709 */
		float k = iA + iB;
		c.rollingMass = k > 0.0f ? 1.0f / k : 0.0f;
		c.rollingResistance = cs->rollingResistance;
		c.rollingImpulse = warmStartScale * m.rollingImpulse;
	}
	float biasRate = P.contactBiasRate, massScale = P.contactMassScale, impulseScale = P.contactImpulseScale;
	if ( indexA == -1 || indexB == -1 )
	{
		biasRate = P.staticBiasRate;
		massScale = P.staticMassScale;
		impulseScale = P.staticImpulseScale;
	}
	else if ( P.enableContactSoftening )
	{
		float contactHertz = ( P.contactHertz < 0.125f * P.inv_h ) ? P.contactHertz : 0.125f * P.inv_h;
		float ratio = 1.0f;
		if ( mA < mB ) ratio = ( 0.5f > mA / mB ) ? 0.5f : mA / mB;
		else if ( mB < mA ) ratio = ( 0.5f > mB / mA ) ? 0.5f : mB / mA;
		t_makeSoft( ratio * contactHertz, ratio * P.contactDampingRatio, P.h, &biasRate, &massScale, &impulseScale );
	}
	V1 normal = m.normal;
	c.normal = normal;
	c.friction = friction;
	c.tangentSpeed = cs->tangentSpeed;
	c.restitution = cs->restitution;
	c.biasRate = biasRate;
	c.massScale = massScale;
	c.impulseScale = impulseScale;
	c.pointCount = m.pointCount;
	V1 tangent = t_v2( normal.y, -normal.x );
	for ( int p = 0; p < 2; ++p )
	{
		if ( p >= m.pointCount )
		{
			c.anchorA[p] = t_v2( t_c( 0.0f ), t_c( 0.0f ) );
			c.anchorB[p] = c.anchorA[p];
			c.baseSeparation[p] = t_c( 0.0f );
			c.normalImpulse[p] = t_c( 0.0f );
			c.tangentImpulse[p] = t_c( 0.0f );
			c.totalNormalImpulse[p] = t_c( 0.0f );
			c.normalMass[p] = t_c( 0.0f );
			c.tangentMass[p] = t_c( 0.0f );
			c.relativeVelocity[p] = t_c( 0.0f );
			continue;
		}
		V1 rA = m.anchorA[p], rB = m.anchorB[p];
		c.anchorA[p] = rA;
		c.anchorB[p] = rB;
		c.baseSeparation[p] = m.separation[p] - t_dot( t_sub( rB, rA ), normal );
		c.normalImpulse[p] = warmStartScale * m.normalImpulse[p];
		c.tangentImpulse[p] = warmStartScale * m.tangentImpulse[p];
		c.totalNormalImpulse[p] = t_c( 0.0f );
		T1 rnA = t_cross( rA, normal ), rnB = t_cross( rB, normal );
		T1 kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		c.normalMass[p] = kNormal.v > 0.0f ? 1.0f / kNormal : t_c( 0.0f );
		T1 rtA = t_cross( rA, tangent ), rtB = t_cross( rB, tangent );
		T1 kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		c.tangentMass[p] = kTangent.v > 0.0f ? 1.0f / kTangent : t_c( 0.0f );
		V1 vrA = t_v2( A.vx - A.w * rA.y, A.vy + A.w * rA.x );
		V1 vrB = t_v2( B.vx - B.w * rB.y, B.vy + B.w * rB.x );
		c.relativeVelocity[p] = t_dot( normal, t_sub( vrB, vrA ) );
	}
	return c;
}

/* pose of a body as a dual transform: p = c - R(q) lc */
struct t_pose
{
	V1 c;
	R1 q;
};

static t_xf t_transform( const t_pose& b, b2Vec2 lc, b2Transform recorded )
{
	t_xf xf;
	xf.q = b.q;
	V1 off = t_rotate( b.q, t_vec( lc ) );
	xf.p = t_v2( b.c.x - off.x, b.c.y - off.y );
	/* the primal is the recorded transform (the step stores p, not c - R(q) lc) */
	xf.p.x.v = recorded.p.x;
	xf.p.y.v = recorded.p.y;
	return xf;
}

static t_manifold t_invalid( void )
{
	t_manifold m;
	memset( &m, 0, sizeof( m ) );
	m.valid = false;
	return m;
}

static inline bool t_same( float a, float b ) { return memcmp( &a, &b, 4 ) == 0; }

/* colored-slot group flags of the wide path: bit 0 rolling resistance, bit 1 restitution in
   the slot's 4-wide group (contact_solver.c:2021, :2131) */
static int t_groupFlags( const b2gTapeStep* h, const b2gContact* contacts, int slot )
{
	int color = 0;
	while ( h->colorOffsets[color + 1] <= slot ) color += 1;
	int begin = h->colorOffsets[color], end = h->colorOffsets[color + 1];
	int g0 = begin + ( ( slot - begin ) / 4 ) * 4;
	int flags = 0;
	for ( int k = g0; k < g0 + 4 && k < end; ++k )
	{
		flags |= contacts[k].rollingResistance != 0.0f ? 1 : 0;
		flags |= contacts[k].restitution != 0.0f ? 2 : 0;
	}
	return flags;
}

extern "C" __attribute__( ( visibility( "default" ) ) ) int b2t_tangent( const void* tape, long long bytes, const float* dirVelocity,
																		  const float* dirFriction, double* centerTangent,
																		  double* velocityTangent )
{
	const unsigned char* base = (const unsigned char*)tape;
	if ( bytes < 16 ) return -4;
	const b2gTapeHeader* H = (const b2gTapeHeader*)base;
	const int stepCount = H->stepCount, bodyCount = H->bodyCount, cap = H->contactCapacity;
	const long long headerBytes = b2gTapeAlign( 16 + 8LL * stepCount );
	const b2gShape* shapes = (const b2gShape*)( base + headerBytes );
	/* tangents of the state at the start of the current step, by body id */
	std::vector<double> dC( 2 * bodyCount, 0.0 ), dQ( 2 * bodyCount, 0.0 ), dV( 3 * bodyCount, 0.0 );
	for ( int b = 0; b < bodyCount; ++b )
		for ( int k = 0; k < 3; ++k ) dV[3 * b + k] = dirVelocity[3 * b + k];
	std::vector<t_manifold> carry( cap > 0 ? cap : 1, t_invalid() ), next( cap > 0 ? cap : 1, t_invalid() );
	for ( int n = 0; n < stepCount; ++n )
	{
		const unsigned char* rec = base + H->stepOffsets[n];
		const b2gTapeStep* h = (const b2gTapeStep*)rec;
		const int nb = h->bodyCount, na = h->awakeCount, nc = h->slotCount;
		if ( nb != bodyCount || h->jointCount > 0 || h->colorOffsets[B2_GRAPH_COLOR_COUNT] > h->colorOffsets[B2G_OVERFLOW_INDEX] )
			return -1;
		const b2gStepParams& P = h->params;
		const b2gTapeBody* bodies = (const b2gTapeBody*)( rec + b2gTapeBodiesOffset() );
		const float* params = (const float*)( rec + b2gTapeParamsOffset( nb ) );
		const float* toi = (const float*)( rec + b2gTapeToiOffset( nb, na ) );
		const int* ids = (const int*)( rec + b2gTapeIdsOffset( nb, na ) );
		const b2gContact* contacts = (const b2gContact*)( rec + b2gTapeContactsOffset( nb, na, nc ) );
		std::vector<t_pose> pose( nb );
		std::vector<int> awakeBody( na > 0 ? na : 1 );
		std::vector<t_body> v0( na > 0 ? na : 1 );
		for ( int b = 0; b < nb; ++b )
		{
			const b2gTapeBody& T = bodies[b];
			pose[b].c = t_v2( t_v( T.center.x, dC[2 * b] ), t_v( T.center.y, dC[2 * b + 1] ) );
			pose[b].q.c = t_v( T.xf.q.c, dQ[2 * b] );
			pose[b].q.s = t_v( T.xf.q.s, dQ[2 * b + 1] );
			if ( T.awakeIndex >= 0 )
			{
				t_body& s = v0[T.awakeIndex];
				s = t_static();
				s.vx = t_v( T.vx, dV[3 * b] );
				s.vy = t_v( T.vy, dV[3 * b + 1] );
				s.w = t_v( T.w, dV[3 * b + 2] );
				s.flags = T.flags;
				awakeBody[T.awakeIndex] = b;
			}
		}
		/* ---- narrowphase (contact.c:519-698, physics_world.c:508-560) ---- */
		std::vector<t_manifold> man( nc > 0 ? nc : 1 );
		std::vector<t_lane> lanes( nc > 0 ? nc : 1 );
		for ( int s = 0; s < nc; ++s )
		{
			const b2gContact* cs = contacts + s;
			const b2Manifold& rm = cs->manifold;
			const b2gShape* shapeA = shapes + cs->shapeIdA;
			const b2gShape* shapeB = shapes + cs->shapeIdB;
			int bA = shapeA->bodyId, bB = shapeB->bodyId;
			const t_manifold& old = carry[ids[s]];
			t_manifold m = t_invalid();
			m.valid = true;
			m.pointCount = rm.pointCount;
			if ( cs->simFlags & B2G_S_RECYCLED )
			{
				if ( old.valid == false || old.pointCount != rm.pointCount ) return -2;
				m = old;
				R1 qA = pose[bA].q, qB = pose[bB].q;
				R1 iA = { old.cachedA.c, -old.cachedA.s }, iB = { old.cachedB.c, -old.cachedB.s };
				R1 dqA = { qA.c * iA.c - qA.s * iA.s, qA.s * iA.c + qA.c * iA.s };
				R1 dqB = { qB.c * iB.c - qB.s * iB.s, qB.s * iB.c + qB.c * iB.s };
				V1 dc = t_v2( pose[bB].c.x - pose[bA].c.x, pose[bB].c.y - pose[bA].c.y );
				for ( int p = 0; p < m.pointCount; ++p )
				{
					V1 rA = t_rotate( dqA, old.anchorA[p] );
					V1 rB = t_rotate( dqB, old.anchorB[p] );
					V1 dp = t_add( dc, t_sub( rB, rA ) );
					m.separation[p] = old.baseSeparation[p] + t_dot( dp, old.normal );
					if ( t_same( m.separation[p].v, rm.points[p].separation ) == false ) return -2;
				}
			}
			else if ( rm.pointCount > 0 )
			{
				bool polyA = shapeA->type == b2_polygonShape, polyB = shapeB->type == b2_polygonShape;
				bool circleA = shapeA->type == b2_circleShape, circleB = shapeB->type == b2_circleShape;
				bool capsuleB = shapeB->type == b2_capsuleShape, segmentA = shapeA->type == b2_segmentShape;
				if ( !( ( polyA && ( polyB || circleB || capsuleB ) ) || ( segmentA && polyB ) || ( circleA && circleB ) ) ) return -1;
				t_xf xfA = t_transform( pose[bA], bodies[bA].localCenter, bodies[bA].xf );
				t_xf xfB = t_transform( pose[bB], bodies[bB].localCenter, bodies[bB].xf );
				t_geometry g = t_polygonContact( shapeA, shapeB, xfA, xfB, bodies[bA].localCenter, bodies[bB].localCenter );
				if ( g.count != rm.pointCount || t_same( g.normal.x.v, rm.normal.x ) == false || t_same( g.normal.y.v, rm.normal.y ) == false )
					return -2;
				m.normal = g.normal;
				for ( int p = 0; p < g.count; ++p )
				{
					if ( g.id[p] != rm.points[p].id || t_same( g.separation[p].v, rm.points[p].separation ) == false ||
						 t_same( g.anchorA[p].x.v, rm.points[p].anchorA.x ) == false ||
						 t_same( g.anchorB[p].y.v, rm.points[p].anchorB.y ) == false )
						return -2;
					m.anchorA[p] = g.anchorA[p];
					m.anchorB[p] = g.anchorB[p];
					m.separation[p] = g.separation[p];
					m.baseSeparation[p] = g.separation[p];
					m.id[p] = g.id[p];
					m.normalImpulse[p] = t_c( 0.0f );
					m.tangentImpulse[p] = t_c( 0.0f );
					if ( old.valid )
					{
						for ( int j = 0; j < old.pointCount; ++j )
						{
							if ( old.id[j] == g.id[p] )
							{
								m.normalImpulse[p] = old.normalImpulse[j];
								m.tangentImpulse[p] = old.tangentImpulse[j];
								break;
							}
						}
					}
					if ( t_same( m.normalImpulse[p].v, rm.points[p].normalImpulse ) == false ||
						 t_same( m.tangentImpulse[p].v, rm.points[p].tangentImpulse ) == false )
						return -2;
				}
				m.cachedA = pose[bA].q;
				m.cachedB = pose[bB].q;
				/* the old manifold's rolling impulse (contact.c:609-612) */
				m.rollingImpulse = old.valid ? old.rollingImpulse : t_c( 0.0f );
			}
			if ( t_same( m.rollingImpulse.v, rm.rollingImpulse ) == false ) return -2;
			/* friction = sqrt(fA fB) (b2MixFriction) */
			T1 fA = t_v( shapeA->friction, dirFriction[cs->shapeIdA] ), fB = t_v( shapeB->friction, dirFriction[cs->shapeIdB] );
			T1 friction = t_sqrt( fA * fB );
			if ( t_same( friction.v, cs->friction ) == false ) return -2;
			man[s] = m;
			lanes[s] = t_prepare( P, cs, m, friction, v0 );
			lanes[s].groupFlags = t_groupFlags( h, contacts, s );
		}
		/* ---- substeps (solver.c:1010-1198), colors in order ---- */
		std::vector<t_body> sb( v0 );
		for ( int i = 0; i < na; ++i )
		{
			sb[i].dpx = t_c( 0.0f );
			sb[i].dpy = t_c( 0.0f );
			sb[i].dqc = t_c( 1.0f );
			sb[i].dqs = t_c( 0.0f );
		}
		const float contactSpeedNeg = -P.contactSpeed;
		bool restitution = false;
		for ( int s = 0; s < nc; ++s ) restitution = restitution || ( lanes[s].groupFlags & 2 ) != 0;
		for ( int sub = 0; sub < P.subStepCount; ++sub )
		{
			for ( int i = 0; i < na; ++i ) t_integrateVelocities( P, &sb[i], params + 8 * i );
			for ( int stage = 0; stage < 3; ++stage )
			{
				if ( stage == 2 )
					for ( int i = 0; i < na; ++i ) t_integratePositions( P, &sb[i] );
				for ( int c = 0; c < B2G_OVERFLOW_INDEX; ++c )
				{
					for ( int s = h->colorOffsets[c]; s < h->colorOffsets[c + 1]; ++s )
					{
						t_lane& L = lanes[s];
						t_body sA = t_static(), sBd = t_static();
						t_body* A = L.indexA ? &sb[L.indexA - 1] : &sA;
						t_body* B = L.indexB ? &sb[L.indexB - 1] : &sBd;
						t_body a0 = *A, b0 = *B;
						if ( stage == 0 ) t_warmStart( L, A, B );
						else t_solve( L, A, B, P.inv_h, contactSpeedNeg, stage == 1 );
						/* static and non-dynamic bodies keep their state (contact_solver.c:1526-1562) */
						if ( L.indexA == 0 || ( a0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *A = a0;
						if ( L.indexB == 0 || ( b0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *B = b0;
					}
				}
			}
		}
		if ( restitution )
		{
			for ( int c = 0; c < B2G_OVERFLOW_INDEX; ++c )
			{
				for ( int s = h->colorOffsets[c]; s < h->colorOffsets[c + 1]; ++s )
				{
					t_lane& L = lanes[s];
					t_body sA = t_static(), sBd = t_static();
					t_body* A = L.indexA ? &sb[L.indexA - 1] : &sA;
					t_body* B = L.indexB ? &sb[L.indexB - 1] : &sBd;
					t_body a0 = *A, b0 = *B;
					t_restitution( L, A, B, P.restitutionThreshold );
					if ( L.indexA == 0 || ( a0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *A = a0;
					if ( L.indexB == 0 || ( b0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *B = b0;
				}
			}
		}
		/* ---- store impulses: the manifold the next step reads ---- */
		for ( int k = 0; k < cap; ++k ) next[k] = t_invalid();
		for ( int s = 0; s < nc; ++s )
		{
			t_manifold m = man[s];
			for ( int p = 0; p < m.pointCount; ++p )
			{
				m.normalImpulse[p] = lanes[s].normalImpulse[p];
				m.tangentImpulse[p] = lanes[s].tangentImpulse[p];
			}
			m.rollingImpulse = lanes[s].rollingImpulse;
			next[ids[s]] = m;
		}
		carry.swap( next );
		/* ---- finalize (solver.c:583-600) and the next step's start ---- */
		const b2gTapeBody* nextBodies = NULL;
		if ( n + 1 < stepCount ) nextBodies = (const b2gTapeBody*)( base + H->stepOffsets[n + 1] + b2gTapeBodiesOffset() );
		for ( int i = 0; i < na; ++i )
		{
			int b = awakeBody[i];
			const t_body& s = sb[i];
			V1 c2 = t_v2( pose[b].c.x + s.dpx, pose[b].c.y + s.dpy );
			R1 r = { s.dqc * pose[b].q.c - s.dqs * pose[b].q.s, s.dqs * pose[b].q.c + s.dqc * pose[b].q.s };
			T1 mag = t_sqrt( r.s * r.s + r.c * r.c );
			T1 inv = mag.v > 0.0f ? 1.0f / mag : t_c( 0.0f );
			R1 q2 = { r.c * inv, r.s * inv };
			float t = toi[i];
			if ( t < 1.0f )
			{
				/* solver.c:495-512 with the recorded fraction: the sweep is relative to the start center */
				V1 base = pose[b].c;
				V1 c1 = t_sub( base, base ), cs2 = t_sub( c2, base );
				V1 ct = t_lerp( c1, cs2, t );
				float omt = 1.0f - t;
				R1 qt = { omt * pose[b].q.c + t * q2.c, omt * pose[b].q.s + t * q2.s };
				T1 m2 = t_sqrt( qt.s * qt.s + qt.c * qt.c );
				T1 i2 = m2.v > 0.0f ? 1.0f / m2 : t_c( 0.0f );
				q2 = { qt.c * i2, qt.s * i2 };
				c2 = t_add( base, ct );
			}
			if ( nextBodies != NULL )
			{
				const b2gTapeBody& T2 = nextBodies[b];
				bool ok = t_same( c2.x.v, T2.center.x ) && t_same( c2.y.v, T2.center.y ) && t_same( q2.c.v, T2.xf.q.c ) &&
						  t_same( q2.s.v, T2.xf.q.s );
				if ( T2.awakeIndex >= 0 ) ok = ok && t_same( s.vx.v, T2.vx ) && t_same( s.vy.v, T2.vy ) && t_same( s.w.v, T2.w );
				if ( ok == false ) return -2;
			}
			dC[2 * b] = c2.x.d[0];
			dC[2 * b + 1] = c2.y.d[0];
			dQ[2 * b] = q2.c.d[0];
			dQ[2 * b + 1] = q2.s.d[0];
			dV[3 * b] = s.vx.d[0];
			dV[3 * b + 1] = s.vy.d[0];
			dV[3 * b + 2] = s.w.d[0];
		}
	}
	for ( int b = 0; b < bodyCount; ++b )
	{
		centerTangent[2 * b] = dC[2 * b];
		centerTangent[2 * b + 1] = dC[2 * b + 1];
		if ( velocityTangent )
			for ( int k = 0; k < 3; ++k ) velocityTangent[3 * b + k] = dV[3 * b + k];
	}
	return 0;
}
