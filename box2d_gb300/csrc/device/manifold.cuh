/*
 * Device contact manifolds (circles, capsules, segments, polygons) for the narrowphase
 * kernel. Same algorithms and operation order as manifold.c / distance.c:33-106 of the
 * reference; one thread computes one contact's manifold in shape A's frame.
 */
#pragma once

#include "math.cuh"
#include "ccd.cuh"

#define D_MAKE_ID( A, B ) ( (uint16_t)( ( (uint8_t)( A ) << 8 ) | (uint8_t)( B ) ) )

static __device__ b2LocalManifold d_emptyManifold( void )
{
	b2LocalManifold m;
	memset( &m, 0, sizeof( m ) );
	return m;
}

/* manifold.c:16-34 */
static __device__ b2Polygon d_makeCapsule( b2Vec2 p1, b2Vec2 p2, float radius )
{
	b2Polygon s;
	memset( &s, 0, sizeof( s ) );
	s.vertices[0] = p1;
	s.vertices[1] = p2;
	s.centroid = d_lerp( p1, p2, 0.5f );
	b2Vec2 axis = d_normalize( d_sub( p2, p1 ) );
	b2Vec2 normal = d_rightPerp( axis );
	s.normals[0] = normal;
	s.normals[1] = d_neg( normal );
	s.count = 2;
	s.radius = radius;
	return s;
}

/* manifold.c:36-65 */
static __device__ b2LocalManifold d_collideCircles( const b2Circle* a, const b2Circle* b, b2Transform xf )
{
	b2LocalManifold m = d_emptyManifold();
	b2Vec2 pA = a->center;
	b2Vec2 pB = d_transformPoint( xf, b->center );
	float distance;
	b2Vec2 normal = d_getLengthAndNormalize( &distance, d_sub( pB, pA ) );
	float rA = a->radius, rB = b->radius;
	float separation = distance - rA - rB;
	if ( separation > D_SPECULATIVE_DISTANCE ) return m;
	b2Vec2 cA = d_mulAdd( pA, rA, normal );
	b2Vec2 cB = d_mulAdd( pB, -rB, normal );
	m.normal = normal;
	m.points[0].point = d_lerp( cA, cB, 0.5f );
	m.points[0].separation = separation;
	m.points[0].id = 0;
	m.pointCount = 1;
	return m;
}

/* manifold.c:68-125 */
static __device__ b2LocalManifold d_collideCapsuleAndCircle( const b2Capsule* a, const b2Circle* b, b2Transform xf )
{
	b2LocalManifold m = d_emptyManifold();
	b2Vec2 pB = d_transformPoint( xf, b->center );
	b2Vec2 p1 = a->center1, p2 = a->center2;
	b2Vec2 e = d_sub( p2, p1 );
	b2Vec2 pA;
	float s1 = d_dot( d_sub( pB, p1 ), e );
	float s2 = d_dot( d_sub( p2, pB ), e );
	if ( s1 < 0.0f ) pA = p1;
	else if ( s2 < 0.0f ) pA = p2;
	else
	{
		float s = s1 / d_dot( e, e );
		pA = d_mulAdd( p1, s, e );
	}
	float distance;
	b2Vec2 normal = d_getLengthAndNormalize( &distance, d_sub( pB, pA ) );
	float rA = a->radius, rB = b->radius;
	float separation = distance - rA - rB;
	if ( separation > D_SPECULATIVE_DISTANCE ) return m;
	b2Vec2 cA = d_mulAdd( pA, rA, normal );
	b2Vec2 cB = d_mulAdd( pB, -rB, normal );
	m.normal = normal;
	m.points[0].point = d_lerp( cA, cB, 0.5f );
	m.points[0].separation = separation;
	m.points[0].id = 0;
	m.pointCount = 1;
	return m;
}

/* manifold.c:127-233 */
static __device__ b2LocalManifold d_collidePolygonAndCircle( const b2Polygon* a, const b2Circle* b, b2Transform xf )
{
	b2LocalManifold m = d_emptyManifold();
	b2Vec2 center = d_transformPoint( xf, b->center );
	float rA = a->radius, rB = b->radius;
	float radius = rA + rB;
	int normalIndex = 0;
	float separation = -FLT_MAX;
	int n = a->count;
	for ( int i = 0; i < n; ++i )
	{
		float s = d_dot( a->normals[i], d_sub( center, a->vertices[i] ) );
		if ( s > separation )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation > radius + D_SPECULATIVE_DISTANCE ) return m;
	int i1 = normalIndex;
	int i2 = i1 + 1 < n ? i1 + 1 : 0;
	b2Vec2 v1 = a->vertices[i1], v2 = a->vertices[i2];
	float u1 = d_dot( d_sub( center, v1 ), d_sub( v2, v1 ) );
	float u2 = d_dot( d_sub( center, v2 ), d_sub( v1, v2 ) );
	if ( u1 < 0.0f && separation > FLT_EPSILON )
	{
		b2Vec2 normal = d_normalize( d_sub( center, v1 ) );
		separation = d_dot( d_sub( center, v1 ), normal );
		if ( separation > radius + D_SPECULATIVE_DISTANCE ) return m;
		b2Vec2 cA = d_mulAdd( v1, rA, normal );
		b2Vec2 cB = d_mulSub( center, rB, normal );
		m.normal = normal;
		m.points[0].point = d_lerp( cA, cB, 0.5f );
		m.points[0].separation = d_dot( d_sub( cB, cA ), normal );
		m.points[0].id = 0;
		m.pointCount = 1;
	}
	else if ( u2 < 0.0f && separation > FLT_EPSILON )
	{
		b2Vec2 normal = d_normalize( d_sub( center, v2 ) );
		separation = d_dot( d_sub( center, v2 ), normal );
		if ( separation > radius + D_SPECULATIVE_DISTANCE ) return m;
		b2Vec2 cA = d_mulAdd( v2, rA, normal );
		b2Vec2 cB = d_mulSub( center, rB, normal );
		m.normal = normal;
		m.points[0].point = d_lerp( cA, cB, 0.5f );
		m.points[0].separation = d_dot( d_sub( cB, cA ), normal );
		m.points[0].id = 0;
		m.pointCount = 1;
	}
	else
	{
		b2Vec2 normal = a->normals[normalIndex];
		m.normal = normal;
		b2Vec2 cA = d_mulAdd( center, rA - d_dot( d_sub( center, v1 ), normal ), normal );
		b2Vec2 cB = d_mulSub( center, rB, normal );
		m.points[0].point = d_lerp( cA, cB, 0.5f );
		m.points[0].separation = separation - radius;
		m.points[0].id = 0;
		m.pointCount = 1;
	}
	return m;
}

/* manifold.c:237-496 */
static __device__ b2LocalManifold d_collideCapsules( const b2Capsule* capA, const b2Capsule* capB, b2Transform xf )
{
	b2Vec2 origin = capA->center1;
	b2Transform xfs = { d_sub( xf.p, origin ), xf.q };
	b2Vec2 p1 = { 0.0f, 0.0f };
	b2Vec2 q1 = d_sub( capA->center2, origin );
	b2Vec2 p2 = d_transformPoint( xfs, capB->center1 );
	b2Vec2 q2 = d_transformPoint( xfs, capB->center2 );
	b2Vec2 d1 = d_sub( q1, p1 ), d2 = d_sub( q2, p2 );
	float dd1 = d_dot( d1, d1 ), dd2 = d_dot( d2, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	b2Vec2 r = d_sub( p1, p2 );
	float rd1 = d_dot( r, d1 ), rd2 = d_dot( r, d2 );
	float d12 = d_dot( d1, d2 );
	float denom = dd1 * dd2 - d12 * d12;
	float f1 = 0.0f;
	if ( denom != 0.0f ) f1 = d_clamp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
	float f2 = ( d12 * f1 + rd2 ) / dd2;
	if ( f2 < 0.0f )
	{
		f2 = 0.0f;
		f1 = d_clamp( -rd1 / dd1, 0.0f, 1.0f );
	}
	else if ( f2 > 1.0f )
	{
		f2 = 1.0f;
		f1 = d_clamp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
	}
	b2Vec2 closest1 = d_mulAdd( p1, f1, d1 );
	b2Vec2 closest2 = d_mulAdd( p2, f2, d2 );
	float distanceSquared = d_distanceSq( closest1, closest2 );
	b2LocalManifold m = d_emptyManifold();
	float rA = capA->radius, rB = capB->radius;
	float radius = rA + rB;
	float maxDistance = radius + D_SPECULATIVE_DISTANCE;
	if ( distanceSquared > maxDistance * maxDistance ) return m;
	float distance = sqrtf( distanceSquared );
	float length1, length2;
	b2Vec2 u1 = d_getLengthAndNormalize( &length1, d1 );
	b2Vec2 u2 = d_getLengthAndNormalize( &length2, d2 );
	float fp2 = d_dot( d_sub( p2, p1 ), u1 );
	float fq2 = d_dot( d_sub( q2, p1 ), u1 );
	int outsideA = ( fp2 <= 0.0f && fq2 <= 0.0f ) || ( fp2 >= length1 && fq2 >= length1 );
	float fp1 = d_dot( d_sub( p1, p2 ), u2 );
	float fq1 = d_dot( d_sub( q1, p2 ), u2 );
	int outsideB = ( fp1 <= 0.0f && fq1 <= 0.0f ) || ( fp1 >= length2 && fq1 >= length2 );
	if ( outsideA == 0 && outsideB == 0 )
	{
		b2Vec2 normalA;
		float separationA;
		{
			normalA = d_leftPerp( u1 );
			float ss1 = d_dot( d_sub( p2, p1 ), normalA );
			float ss2 = d_dot( d_sub( q2, p1 ), normalA );
			float s1p = ss1 < ss2 ? ss1 : ss2;
			float s1n = -ss1 < -ss2 ? -ss1 : -ss2;
			if ( s1p > s1n ) separationA = s1p;
			else
			{
				separationA = s1n;
				normalA = d_neg( normalA );
			}
		}
		b2Vec2 normalB;
		float separationB;
		{
			normalB = d_leftPerp( u2 );
			float ss1 = d_dot( d_sub( p1, p2 ), normalB );
			float ss2 = d_dot( d_sub( q1, p2 ), normalB );
			float s1p = ss1 < ss2 ? ss1 : ss2;
			float s1n = -ss1 < -ss2 ? -ss1 : -ss2;
			if ( s1p > s1n ) separationB = s1p;
			else
			{
				separationB = s1n;
				normalB = d_neg( normalB );
			}
		}
		if ( separationA + 0.1f * D_LINEAR_SLOP >= separationB )
		{
			m.normal = normalA;
			b2Vec2 cp = p2, cq = q2;
			if ( fp2 < 0.0f && fq2 > 0.0f ) cp = d_lerp( p2, q2, ( 0.0f - fp2 ) / ( fq2 - fp2 ) );
			else if ( fq2 < 0.0f && fp2 > 0.0f ) cq = d_lerp( q2, p2, ( 0.0f - fq2 ) / ( fp2 - fq2 ) );
			if ( fp2 > length1 && fq2 < length1 ) cp = d_lerp( p2, q2, ( fp2 - length1 ) / ( fp2 - fq2 ) );
			else if ( fq2 > length1 && fp2 < length1 ) cq = d_lerp( q2, p2, ( fq2 - length1 ) / ( fq2 - fp2 ) );
			float sp = d_dot( d_sub( cp, p1 ), normalA );
			float sq = d_dot( d_sub( cq, p1 ), normalA );
			if ( sp <= distance + D_LINEAR_SLOP || sq <= distance + D_LINEAR_SLOP )
			{
				m.points[0].point = d_mulAdd( cp, 0.5f * ( rA - rB - sp ), normalA );
				m.points[0].separation = sp - radius;
				m.points[0].id = D_MAKE_ID( 0, 0 );
				m.points[1].point = d_mulAdd( cq, 0.5f * ( rA - rB - sq ), normalA );
				m.points[1].separation = sq - radius;
				m.points[1].id = D_MAKE_ID( 0, 1 );
				m.pointCount = 2;
			}
		}
		else
		{
			m.normal = d_neg( normalB );
			b2Vec2 cp = p1, cq = q1;
			if ( fp1 < 0.0f && fq1 > 0.0f ) cp = d_lerp( p1, q1, ( 0.0f - fp1 ) / ( fq1 - fp1 ) );
			else if ( fq1 < 0.0f && fp1 > 0.0f ) cq = d_lerp( q1, p1, ( 0.0f - fq1 ) / ( fp1 - fq1 ) );
			if ( fp1 > length2 && fq1 < length2 ) cp = d_lerp( p1, q1, ( fp1 - length2 ) / ( fp1 - fq1 ) );
			else if ( fq1 > length2 && fp1 < length2 ) cq = d_lerp( q1, p1, ( fq1 - length2 ) / ( fq1 - fp1 ) );
			float sp = d_dot( d_sub( cp, p2 ), normalB );
			float sq = d_dot( d_sub( cq, p2 ), normalB );
			if ( sp <= distance + D_LINEAR_SLOP || sq <= distance + D_LINEAR_SLOP )
			{
				m.points[0].point = d_mulAdd( cp, 0.5f * ( rB - rA - sp ), normalB );
				m.points[0].separation = sp - radius;
				m.points[0].id = D_MAKE_ID( 0, 0 );
				m.points[1].point = d_mulAdd( cq, 0.5f * ( rB - rA - sq ), normalB );
				m.points[1].separation = sq - radius;
				m.points[1].id = D_MAKE_ID( 1, 0 );
				m.pointCount = 2;
			}
		}
	}
	if ( m.pointCount == 0 )
	{
		b2Vec2 normal = d_sub( closest2, closest1 );
		if ( d_dot( normal, normal ) > epsSqr ) normal = d_normalize( normal );
		else normal = d_leftPerp( u1 );
		b2Vec2 c1 = d_mulAdd( closest1, rA, normal );
		b2Vec2 c2 = d_mulAdd( closest2, -rB, normal );
		int i1 = f1 == 0.0f ? 0 : 1;
		int i2 = f2 == 0.0f ? 0 : 1;
		m.normal = normal;
		m.points[0].point = d_lerp( c1, c2, 0.5f );
		m.points[0].separation = sqrtf( distanceSquared ) - radius;
		m.points[0].id = D_MAKE_ID( i1, i2 );
		m.pointCount = 1;
	}
	for ( int i = 0; i < m.pointCount; ++i ) m.points[i].point = d_add( m.points[i].point, origin );
	return m;
}

/* distance.c:33-106 */
typedef struct d_segDist
{
	b2Vec2 closest1, closest2;
	float fraction1, fraction2, distanceSquared;
} d_segDist;

static __device__ d_segDist d_segmentDistance( b2Vec2 p1, b2Vec2 q1, b2Vec2 p2, b2Vec2 q2 )
{
	d_segDist res;
	memset( &res, 0, sizeof( res ) );
	b2Vec2 d1 = d_sub( q1, p1 ), d2 = d_sub( q2, p2 ), r = d_sub( p1, p2 );
	float dd1 = d_dot( d1, d1 ), dd2 = d_dot( d2, d2 ), rd1 = d_dot( r, d1 ), rd2 = d_dot( r, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	if ( dd1 < epsSqr || dd2 < epsSqr )
	{
		if ( dd1 >= epsSqr )
		{
			res.fraction1 = d_clamp( -rd1 / dd1, 0.0f, 1.0f );
			res.fraction2 = 0.0f;
		}
		else if ( dd2 >= epsSqr )
		{
			res.fraction1 = 0.0f;
			res.fraction2 = d_clamp( rd2 / dd2, 0.0f, 1.0f );
		}
	}
	else
	{
		float d12 = d_dot( d1, d2 );
		float denom = dd1 * dd2 - d12 * d12;
		float f1 = 0.0f;
		if ( denom != 0.0f ) f1 = d_clamp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
		float f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2 < 0.0f )
		{
			f2 = 0.0f;
			f1 = d_clamp( -rd1 / dd1, 0.0f, 1.0f );
		}
		else if ( f2 > 1.0f )
		{
			f2 = 1.0f;
			f1 = d_clamp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
		}
		res.fraction1 = f1;
		res.fraction2 = f2;
	}
	res.closest1 = d_mulAdd( p1, res.fraction1, d1 );
	res.closest2 = d_mulAdd( p2, res.fraction2, d2 );
	res.distanceSquared = d_distanceSq( res.closest1, res.closest2 );
	return res;
}

/* manifold.c:511-643 */
static __device__ b2LocalManifold d_clipPolygons( const b2Polygon* polyA, const b2Polygon* polyB, int edgeA, int edgeB, int flip )
{
	b2LocalManifold m = d_emptyManifold();
	const b2Polygon *poly1, *poly2;
	int i11, i12, i21, i22;
	if ( flip )
	{
		poly1 = polyB;
		poly2 = polyA;
		i11 = edgeB;
		i12 = edgeB + 1 < polyB->count ? edgeB + 1 : 0;
		i21 = edgeA;
		i22 = edgeA + 1 < polyA->count ? edgeA + 1 : 0;
	}
	else
	{
		poly1 = polyA;
		poly2 = polyB;
		i11 = edgeA;
		i12 = edgeA + 1 < polyA->count ? edgeA + 1 : 0;
		i21 = edgeB;
		i22 = edgeB + 1 < polyB->count ? edgeB + 1 : 0;
	}
	b2Vec2 normal = poly1->normals[i11];
	b2Vec2 v11 = poly1->vertices[i11], v12 = poly1->vertices[i12];
	b2Vec2 v21 = poly2->vertices[i21], v22 = poly2->vertices[i22];
	b2Vec2 tangent = d_crossSV( 1.0f, normal );
	float lower1 = 0.0f;
	float upper1 = d_dot( d_sub( v12, v11 ), tangent );
	float upper2 = d_dot( d_sub( v21, v11 ), tangent );
	float lower2 = d_dot( d_sub( v22, v11 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 ) return m;
	b2Vec2 vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON ) vLower = d_lerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else vLower = v22;
	b2Vec2 vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON ) vUpper = d_lerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else vUpper = v21;
	float separationLower = d_dot( d_sub( vLower, v11 ), normal );
	float separationUpper = d_dot( d_sub( vUpper, v11 ), normal );
	float r1 = poly1->radius, r2 = poly2->radius;
	vLower = d_mulAdd( vLower, 0.5f * ( r1 - r2 - separationLower ), normal );
	vUpper = d_mulAdd( vUpper, 0.5f * ( r1 - r2 - separationUpper ), normal );
	float radius = r1 + r2;
	if ( flip == 0 )
	{
		m.normal = normal;
		m.points[0].point = vLower;
		m.points[0].separation = separationLower - radius;
		m.points[0].id = D_MAKE_ID( i11, i22 );
		m.points[1].point = vUpper;
		m.points[1].separation = separationUpper - radius;
		m.points[1].id = D_MAKE_ID( i12, i21 );
		m.pointCount = 2;
	}
	else
	{
		m.normal = d_neg( normal );
		m.points[0].point = vUpper;
		m.points[0].separation = separationUpper - radius;
		m.points[0].id = D_MAKE_ID( i21, i12 );
		m.points[1].point = vLower;
		m.points[1].separation = separationLower - radius;
		m.points[1].id = D_MAKE_ID( i22, i11 );
		m.pointCount = 2;
	}
	return m;
}

/* manifold.c:646-682 */
static __device__ float d_findMaxSeparation( int* edgeIndex, const b2Polygon* poly1, const b2Polygon* poly2 )
{
	int count1 = poly1->count, count2 = poly2->count;
	int bestIndex = 0;
	float maxSeparation = -FLT_MAX;
	for ( int i = 0; i < count1; ++i )
	{
		b2Vec2 n = poly1->normals[i];
		b2Vec2 v1 = poly1->vertices[i];
		float si = FLT_MAX;
		for ( int j = 0; j < count2; ++j )
		{
			float sij = d_dot( n, d_sub( poly2->vertices[j], v1 ) );
			if ( sij < si ) si = sij;
		}
		if ( si > maxSeparation )
		{
			maxSeparation = si;
			bestIndex = i;
		}
	}
	*edgeIndex = bestIndex;
	return maxSeparation;
}

/* manifold.c:702-1028 */
static __device__ b2LocalManifold d_collidePolygons( const b2Polygon* polygonA, const b2Polygon* polygonB, b2Transform xf )
{
	b2Vec2 origin = polygonA->vertices[0];
	b2Transform xfs = { d_sub( xf.p, origin ), xf.q };
	b2Polygon A, B;
	A.count = polygonA->count;
	A.radius = polygonA->radius;
	A.vertices[0] = d_v( 0.0f, 0.0f );
	A.normals[0] = polygonA->normals[0];
	for ( int i = 1; i < A.count; ++i )
	{
		A.vertices[i] = d_sub( polygonA->vertices[i], origin );
		A.normals[i] = polygonA->normals[i];
	}
	B.count = polygonB->count;
	B.radius = polygonB->radius;
	for ( int i = 0; i < B.count; ++i )
	{
		B.vertices[i] = d_transformPoint( xfs, polygonB->vertices[i] );
		B.normals[i] = d_rotate( xfs.q, polygonB->normals[i] );
	}
	int edgeA = 0;
	float separationA = d_findMaxSeparation( &edgeA, &A, &B );
	int edgeB = 0;
	float separationB = d_findMaxSeparation( &edgeB, &B, &A );
	float radius = A.radius + B.radius;
	if ( separationA > D_SPECULATIVE_DISTANCE + radius || separationB > D_SPECULATIVE_DISTANCE + radius )
		return d_emptyManifold();
	int flip;
	if ( separationA >= separationB )
	{
		flip = 0;
		b2Vec2 search = A.normals[edgeA];
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < B.count; ++i )
		{
			float d = d_dot( search, B.normals[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeB = i;
			}
		}
	}
	else
	{
		flip = 1;
		b2Vec2 search = B.normals[edgeB];
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < A.count; ++i )
		{
			float d = d_dot( search, A.normals[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}
	b2LocalManifold m = d_emptyManifold();
	if ( separationA > 0.1f * D_LINEAR_SLOP || separationB > 0.1f * D_LINEAR_SLOP )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < A.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < B.count ? edgeB + 1 : 0;
		b2Vec2 v11 = A.vertices[i11], v12 = A.vertices[i12], v21 = B.vertices[i21], v22 = B.vertices[i22];
		d_segDist res = d_segmentDistance( v11, v12, v21, v22 );
		float distance = sqrtf( res.distanceSquared );
		float separation = distance - radius;
		if ( distance - radius > D_SPECULATIVE_DISTANCE ) return m;
		m = d_clipPolygons( &A, &B, edgeA, edgeB, flip );
		float minSeparation = FLT_MAX;
		for ( int i = 0; i < m.pointCount; ++i ) minSeparation = d_min( minSeparation, m.points[i].separation );
		if ( separation + 0.1f * D_LINEAR_SLOP < minSeparation )
		{
			int hit = 0;
			b2Vec2 va = v11, vb = v21;
			int ia = i11, ib = i21;
			if ( res.fraction1 == 0.0f && res.fraction2 == 0.0f )
			{
				hit = 1;
			}
			else if ( res.fraction1 == 0.0f && res.fraction2 == 1.0f )
			{
				hit = 1;
				vb = v22;
				ib = i22;
			}
			else if ( res.fraction1 == 1.0f && res.fraction2 == 0.0f )
			{
				hit = 1;
				va = v12;
				ia = i12;
			}
			else if ( res.fraction1 == 1.0f && res.fraction2 == 1.0f )
			{
				hit = 1;
				va = v12;
				ia = i12;
				vb = v22;
				ib = i22;
			}
			if ( hit )
			{
				b2Vec2 normal = d_sub( vb, va );
				float invDistance = 1.0f / distance;
				normal.x *= invDistance;
				normal.y *= invDistance;
				b2Vec2 c1 = d_mulAdd( va, A.radius, normal );
				b2Vec2 c2 = d_mulAdd( vb, -B.radius, normal );
				m.normal = normal;
				m.points[0].point = d_lerp( c1, c2, 0.5f );
				m.points[0].separation = distance - radius;
				m.points[0].id = D_MAKE_ID( ia, ib );
				m.pointCount = 1;
			}
		}
	}
	else
	{
		m = d_clipPolygons( &A, &B, edgeA, edgeB, flip );
	}
	for ( int i = 0; i < m.pointCount; ++i ) m.points[i].point = d_add( m.points[i].point, origin );
	return m;
}


/* build a b2Polygon from a device shape record */
static __device__ b2Polygon d_shapePolygon( const b2gShape* s )
{
	b2Polygon p;
	for ( int i = 0; i < B2_MAX_POLYGON_VERTICES; ++i )
	{
		p.vertices[i] = s->v[i];
		p.normals[i] = s->n[i];
	}
	p.centroid = s->centroid;
	p.radius = s->radius;
	p.count = s->count;
	return p;
}


/* ---- chain segments (manifold.c:1042-1641): one-sided segments with ghost vertices that
   smooth the collision across the chain's joints. A chain segment keeps its points in v[0],
   v[1] and its ghost vertices in v[2] (before point 1) and v[3] (after point 2). ---- */

/* manifold.c:1042-1122 */
static __device__ b2LocalManifold d_collideChainSegmentAndCircle( const b2gShape* seg, const b2Circle* circleB, b2Transform xf )
{
	b2LocalManifold manifold = d_emptyManifold();
	b2Vec2 pB = d_transformPoint( xf, circleB->center );
	b2Vec2 p1 = seg->v[0], p2 = seg->v[1];
	b2Vec2 e = d_sub( p2, p1 );
	float offset = d_dot( d_rightPerp( e ), d_sub( pB, p1 ) );
	if ( offset < 0.0f ) return manifold;
	float u = d_dot( e, d_sub( p2, pB ) );
	float v = d_dot( e, d_sub( pB, p1 ) );
	b2Vec2 pA;
	if ( v <= 0.0f )
	{
		b2Vec2 prevEdge = d_sub( p1, seg->v[2] );
		float uPrev = d_dot( prevEdge, d_sub( pB, p1 ) );
		if ( uPrev <= 0.0f ) return manifold;
		pA = p1;
	}
	else if ( u <= 0.0f )
	{
		b2Vec2 nextEdge = d_sub( seg->v[3], p2 );
		float vNext = d_dot( nextEdge, d_sub( pB, p2 ) );
		if ( vNext > 0.0f ) return manifold;
		pA = p2;
	}
	else
	{
		float ee = d_dot( e, e );
		pA = d_v( u * p1.x + v * p2.x, u * p1.y + v * p2.y );
		pA = ee > 0.0f ? d_mulSV( 1.0f / ee, pA ) : p1;
	}
	float distance;
	b2Vec2 normal = d_getLengthAndNormalize( &distance, d_sub( pB, pA ) );
	float radius = circleB->radius;
	float separation = distance - radius;
	if ( separation > D_SPECULATIVE_DISTANCE ) return manifold;
	b2Vec2 cA = pA;
	b2Vec2 cB = d_mulAdd( pB, -radius, normal );
	manifold.normal = normal;
	manifold.points[0].point = d_lerp( cA, cB, 0.5f );
	manifold.points[0].separation = separation;
	manifold.points[0].id = 0;
	manifold.pointCount = 1;
	return manifold;
}

/* manifold.c:1131-1196: two-point manifold from the overlap of edge (a1, a2) with the
   incident edge (b1, b2) along `normal` */
static __device__ b2LocalManifold d_clipSegments( b2Vec2 a1, b2Vec2 a2, b2Vec2 b1, b2Vec2 b2, b2Vec2 normal, float ra, float rb,
												  uint16_t id1, uint16_t id2 )
{
	b2LocalManifold manifold = d_emptyManifold();
	b2Vec2 tangent = d_leftPerp( normal );
	float lower1 = 0.0f;
	float upper1 = d_dot( d_sub( a2, a1 ), tangent );
	float upper2 = d_dot( d_sub( b1, a1 ), tangent );
	float lower2 = d_dot( d_sub( b2, a1 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 ) return manifold;
	b2Vec2 vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON ) vLower = d_lerp( b2, b1, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else vLower = b2;
	b2Vec2 vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON ) vUpper = d_lerp( b2, b1, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else vUpper = b1;
	float separationLower = d_dot( d_sub( vLower, a1 ), normal );
	float separationUpper = d_dot( d_sub( vUpper, a1 ), normal );
	vLower = d_mulAdd( vLower, 0.5f * ( ra - rb - separationLower ), normal );
	vUpper = d_mulAdd( vUpper, 0.5f * ( ra - rb - separationUpper ), normal );
	float radius = ra + rb;
	manifold.normal = normal;
	manifold.points[0].point = vLower;
	manifold.points[0].separation = separationLower - radius;
	manifold.points[0].id = id1;
	manifold.points[1].point = vUpper;
	manifold.points[1].separation = separationUpper - radius;
	manifold.points[1].id = id2;
	manifold.pointCount = 2;
	return manifold;
}

enum
{
	D_NORMAL_SKIP = 0,
	D_NORMAL_ADMIT = 1,
	D_NORMAL_SNAP = 2,
};

struct d_chainParams
{
	b2Vec2 edge1, normal0, normal2;
	bool convex1, convex2;
};

/* manifold.c:1219-1259: where a normal falls on the Gauss map of the segment's vertices */
static __device__ int d_classifyNormal( const d_chainParams& params, b2Vec2 normal )
{
	const float sinTol = 0.01f;
	if ( d_dot( normal, params.edge1 ) <= 0.0f )
	{
		if ( params.convex1 ) return d_cross( normal, params.normal0 ) > sinTol ? D_NORMAL_SKIP : D_NORMAL_ADMIT;
		return D_NORMAL_SNAP;
	}
	if ( params.convex2 ) return d_cross( params.normal2, normal ) > sinTol ? D_NORMAL_SKIP : D_NORMAL_ADMIT;
	return D_NORMAL_SNAP;
}

/* manifold.c:1261-1641 */
static __device__ b2LocalManifold d_collideChainSegmentAndPolygon( const b2gShape* seg, const b2Polygon* polygonB, b2Transform xf,
																   d_simplexCache* cache )
{
	b2LocalManifold manifold = d_emptyManifold();
	b2Vec2 centroidB = d_transformPoint( xf, polygonB->centroid );
	float radiusB = polygonB->radius;
	b2Vec2 p1 = seg->v[0], p2 = seg->v[1];
	b2Vec2 edge1 = d_normalize( d_sub( p2, p1 ) );
	d_chainParams sp;
	sp.edge1 = edge1;
	const float convexTol = 0.01f;
	b2Vec2 edge0 = d_normalize( d_sub( p1, seg->v[2] ) );
	sp.normal0 = d_rightPerp( edge0 );
	sp.convex1 = d_cross( edge0, edge1 ) >= convexTol;
	b2Vec2 edge2 = d_normalize( d_sub( seg->v[3], p2 ) );
	sp.normal2 = d_rightPerp( edge2 );
	sp.convex2 = d_cross( edge1, edge2 ) >= convexTol;
	b2Vec2 normal1 = d_rightPerp( edge1 );
	bool behind1 = d_dot( normal1, d_sub( centroidB, p1 ) ) < 0.0f;
	bool behind0 = true, behind2 = true;
	if ( sp.convex1 ) behind0 = d_dot( sp.normal0, d_sub( centroidB, p1 ) ) < 0.0f;
	if ( sp.convex2 ) behind2 = d_dot( sp.normal2, d_sub( centroidB, p2 ) ) < 0.0f;
	if ( behind1 && behind0 && behind2 ) return manifold;

	int count = polygonB->count;
	b2Vec2 vertices[B2_MAX_POLYGON_VERTICES];
	b2Vec2 normals[B2_MAX_POLYGON_VERTICES];
	for ( int i = 0; i < count; ++i )
	{
		vertices[i] = d_transformPoint( xf, polygonB->vertices[i] );
		normals[i] = d_rotate( xf.q, polygonB->normals[i] );
	}
	d_proxy proxyA, proxyB;
	proxyA.points[0] = p1;
	proxyA.points[1] = p2;
	proxyA.count = 2;
	proxyA.radius = 0.0f;
	for ( int i = 0; i < count; ++i ) proxyB.points[i] = vertices[i];
	proxyB.count = count;
	proxyB.radius = 0.0f;
	b2Transform identity = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };
	b2Vec2 outA, outB;
	float outDistance = d_shapeDistanceWitness( &proxyA, &proxyB, identity, cache, &outA, &outB );
	if ( outDistance > radiusB + D_SPECULATIVE_DISTANCE ) return manifold;

	b2Vec2 n0 = sp.convex1 ? sp.normal0 : normal1;
	b2Vec2 n2 = sp.convex2 ? sp.normal2 : normal1;
	int incidentIndex = -1;
	int incidentNormal = -1;
	if ( behind1 == false && outDistance > 0.1f * D_LINEAR_SLOP )
	{
		if ( cache->count == 1 )
		{
			/* vertex-vertex */
			b2Vec2 pA = outA, pB = outB;
			b2Vec2 normal = d_normalize( d_sub( pB, pA ) );
			int type = d_classifyNormal( sp, normal );
			if ( type == D_NORMAL_SKIP ) return manifold;
			if ( type == D_NORMAL_ADMIT )
			{
				manifold.normal = normal;
				manifold.points[0].point = pA;
				manifold.points[0].separation = outDistance - radiusB;
				manifold.points[0].id = D_MAKE_ID( cache->indexA[0], cache->indexB[0] );
				manifold.pointCount = 1;
				return manifold;
			}
			incidentIndex = cache->indexB[0];
		}
		else
		{
			/* vertex-edge */
			int ia1 = cache->indexA[0], ia2 = cache->indexA[1];
			int ib1 = cache->indexB[0], ib2 = cache->indexB[1];
			if ( ia1 == ia2 )
			{
				b2Vec2 normalB = d_sub( outA, outB );
				float dot1 = d_dot( normalB, normals[ib1] );
				float dot2 = d_dot( normalB, normals[ib2] );
				int ib = dot1 > dot2 ? ib1 : ib2;
				normalB = normals[ib];
				int type = d_classifyNormal( sp, d_neg( normalB ) );
				if ( type == D_NORMAL_SKIP ) return manifold;
				if ( type == D_NORMAL_ADMIT )
				{
					ib1 = ib;
					ib2 = ib < count - 1 ? ib + 1 : 0;
					b2Vec2 b1 = vertices[ib1], b2 = vertices[ib2];
					dot1 = d_dot( normalB, d_sub( p1, b1 ) );
					dot2 = d_dot( normalB, d_sub( p2, b1 ) );
					if ( dot1 < dot2 )
					{
						if ( d_dot( n0, normalB ) < d_dot( normal1, normalB ) ) return manifold;
					}
					else
					{
						if ( d_dot( n2, normalB ) < d_dot( normal1, normalB ) ) return manifold;
					}
					manifold = d_clipSegments( b1, b2, p1, p2, normalB, radiusB, 0.0f, D_MAKE_ID( ib1, 1 ), D_MAKE_ID( ib2, 0 ) );
					if ( manifold.pointCount == 2 ) manifold.normal = d_neg( normalB );
					return manifold;
				}
				incidentNormal = ib;
			}
			else
			{
				float dot1 = d_dot( normal1, d_sub( vertices[ib1], p1 ) );
				float dot2 = d_dot( normal1, d_sub( vertices[ib2], p2 ) );
				incidentIndex = dot1 < dot2 ? ib1 : ib2;
			}
		}
	}
	else
	{
		/* separating axes: the segment normal, the convex neighbors' normals, the polygon's */
		float edgeSeparation = FLT_MAX;
		for ( int i = 0; i < count; ++i )
		{
			float s = d_dot( normal1, d_sub( vertices[i], p1 ) );
			if ( s < edgeSeparation )
			{
				edgeSeparation = s;
				incidentIndex = i;
			}
		}
		if ( sp.convex1 )
		{
			float s0 = FLT_MAX;
			for ( int i = 0; i < count; ++i )
			{
				float s = d_dot( sp.normal0, d_sub( vertices[i], p1 ) );
				if ( s < s0 ) s0 = s;
			}
			if ( s0 > edgeSeparation )
			{
				edgeSeparation = s0;
				incidentIndex = -1;
			}
		}
		if ( sp.convex2 )
		{
			float s2 = FLT_MAX;
			for ( int i = 0; i < count; ++i )
			{
				float s = d_dot( sp.normal2, d_sub( vertices[i], p2 ) );
				if ( s < s2 ) s2 = s;
			}
			if ( s2 > edgeSeparation )
			{
				edgeSeparation = s2;
				incidentIndex = -1;
			}
		}
		float polygonSeparation = -FLT_MAX;
		int referenceIndex = -1;
		for ( int i = 0; i < count; ++i )
		{
			b2Vec2 n = normals[i];
			if ( d_classifyNormal( sp, d_neg( n ) ) != D_NORMAL_ADMIT ) continue;
			b2Vec2 pv = vertices[i];
			float s = d_min( d_dot( n, d_sub( p2, pv ) ), d_dot( n, d_sub( p1, pv ) ) );
			if ( s > polygonSeparation )
			{
				polygonSeparation = s;
				referenceIndex = i;
			}
		}
		if ( polygonSeparation > edgeSeparation )
		{
			int ia1 = referenceIndex;
			int ia2 = ia1 < count - 1 ? ia1 + 1 : 0;
			b2Vec2 a1 = vertices[ia1], a2 = vertices[ia2];
			b2Vec2 n = normals[ia1];
			float dot1 = d_dot( n, d_sub( p1, a1 ) );
			float dot2 = d_dot( n, d_sub( p2, a1 ) );
			if ( dot1 < dot2 )
			{
				if ( d_dot( n0, n ) < d_dot( normal1, n ) ) return manifold;
			}
			else
			{
				if ( d_dot( n2, n ) < d_dot( normal1, n ) ) return manifold;
			}
			manifold = d_clipSegments( a1, a2, p1, p2, normals[ia1], radiusB, 0.0f, D_MAKE_ID( ia1, 1 ), D_MAKE_ID( ia2, 0 ) );
			if ( manifold.pointCount == 2 ) manifold.normal = d_neg( normals[ia1] );
			return manifold;
		}
		if ( incidentIndex == -1 ) return manifold;
	}

	/* the segment normal: clip the polygon edge most anti-parallel to it */
	b2Vec2 b1, b2;
	int ib1, ib2;
	if ( incidentNormal != -1 )
	{
		ib1 = incidentNormal;
		ib2 = ib1 < count - 1 ? ib1 + 1 : 0;
		b1 = vertices[ib1];
		b2 = vertices[ib2];
	}
	else
	{
		int i2 = incidentIndex;
		int i1 = i2 > 0 ? i2 - 1 : count - 1;
		float d1 = d_dot( normal1, normals[i1] );
		float d2 = d_dot( normal1, normals[i2] );
		if ( d1 < d2 )
		{
			ib1 = i1;
			ib2 = i2;
		}
		else
		{
			ib1 = i2;
			ib2 = i2 < count - 1 ? i2 + 1 : 0;
		}
		b1 = vertices[ib1];
		b2 = vertices[ib2];
	}
	return d_clipSegments( p1, p2, b1, b2, normal1, 0.0f, radiusB, D_MAKE_ID( 0, ib2 ), D_MAKE_ID( 1, ib1 ) );
}

/* dispatch in the primary order of the contact register table (contact.c:188-206):
   circle 0, capsule 1, segment 2, polygon 3, chain segment 4 (always shape A). `cache` is
   the contact's GJK simplex cache, read and updated by the chain-segment manifolds. */
static __device__ b2LocalManifold d_collideShapes( const b2gShape* a, const b2gShape* b, b2Transform xf, d_simplexCache* cache )
{
	int ta = a->type, tb = b->type;
	if ( ta == b2_chainSegmentShape )
	{
		if ( tb == b2_circleShape )
		{
			b2Circle cb = { b->v[0], b->radius };
			return d_collideChainSegmentAndCircle( a, &cb, xf );
		}
		if ( tb == b2_capsuleShape )
		{
			b2Polygon pb = d_makeCapsule( b->v[0], b->v[1], b->radius );
			return d_collideChainSegmentAndPolygon( a, &pb, xf, cache );
		}
		if ( tb == b2_polygonShape )
		{
			b2Polygon pb = d_shapePolygon( b );
			return d_collideChainSegmentAndPolygon( a, &pb, xf, cache );
		}
		return d_emptyManifold();
	}
	if ( ta == b2_circleShape && tb == b2_circleShape )
	{
		b2Circle ca = { a->v[0], a->radius }, cb = { b->v[0], b->radius };
		return d_collideCircles( &ca, &cb, xf );
	}
	if ( ta == b2_capsuleShape && tb == b2_circleShape )
	{
		b2Capsule ca = { a->v[0], a->v[1], a->radius };
		b2Circle cb = { b->v[0], b->radius };
		return d_collideCapsuleAndCircle( &ca, &cb, xf );
	}
	if ( ta == b2_capsuleShape && tb == b2_capsuleShape )
	{
		b2Capsule ca = { a->v[0], a->v[1], a->radius }, cb = { b->v[0], b->v[1], b->radius };
		return d_collideCapsules( &ca, &cb, xf );
	}
	if ( ta == b2_polygonShape && tb == b2_circleShape )
	{
		b2Polygon pa = d_shapePolygon( a );
		b2Circle cb = { b->v[0], b->radius };
		return d_collidePolygonAndCircle( &pa, &cb, xf );
	}
	if ( ta == b2_polygonShape && tb == b2_capsuleShape )
	{
		b2Polygon pa = d_shapePolygon( a );
		b2Polygon pb = d_makeCapsule( b->v[0], b->v[1], b->radius );
		return d_collidePolygons( &pa, &pb, xf );
	}
	if ( ta == b2_polygonShape && tb == b2_polygonShape )
	{
		b2Polygon pa = d_shapePolygon( a );
		b2Polygon pb = d_shapePolygon( b );
		return d_collidePolygons( &pa, &pb, xf );
	}
	if ( ta == b2_segmentShape && tb == b2_circleShape )
	{
		b2Capsule ca = { a->v[0], a->v[1], 0.0f };
		b2Circle cb = { b->v[0], b->radius };
		return d_collideCapsuleAndCircle( &ca, &cb, xf );
	}
	if ( ta == b2_segmentShape && tb == b2_capsuleShape )
	{
		b2Capsule ca = { a->v[0], a->v[1], 0.0f };
		b2Capsule cb = { b->v[0], b->v[1], b->radius };
		return d_collideCapsules( &ca, &cb, xf );
	}
	if ( ta == b2_segmentShape && tb == b2_polygonShape )
	{
		b2Polygon pa = d_makeCapsule( a->v[0], a->v[1], 0.0f );
		b2Polygon pb = d_shapePolygon( b );
		return d_collidePolygons( &pa, &pb, xf );
	}
	return d_emptyManifold();
}
