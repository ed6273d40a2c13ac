/*
 * Polygon-polygon manifold (manifold.c:511-1028 b2ClipPolygons / b2FindMaxSeparation /
 * b2CollidePolygons, distance.c:33-106 b2SegmentDistance), and the circle-circle and
 * polygon-circle manifolds (manifold.c:36-66, :127-230), over a dual scalar, for the
 * Jacobian of a contact's manifold with respect to the two body poses. The operation order
 * is the forward narrowphase's, so the primal reproduces its float result and the same
 * reference edge, incident edge, flip and clip branches are taken; the tangents are the
 * derivative of that branch. Shared by the device adjoint and the host tangent-linear
 * checker.
 */
#pragma once

#include "diff_scalar.h"

#include <float.h>
#include <stdint.h>

#define B2D_LINEAR_SLOP 0.005f
#define B2D_SPECULATIVE_DISTANCE ( 4.0f * B2D_LINEAR_SLOP )
#define B2D_MAX_VERTS 8

template <class S> struct b2dPoly
{
	b2dVec2<S> v[B2D_MAX_VERTS];
	b2dVec2<S> n[B2D_MAX_VERTS];
	float radius;
	int count;
};

template <class S> struct b2dManifoldPoint
{
	b2dVec2<S> point;
	S separation;
	uint16_t id;
};

template <class S> struct b2dManifold
{
	b2dVec2<S> normal;
	b2dManifoldPoint<S> points[2];
	int count;
};

#define B2D_MAKE_ID( A, B ) ( (uint16_t)( ( (uint8_t)( A ) << 8 ) | (uint8_t)( B ) ) )

template <class S> B2D_HD b2dVec2<S> b2dV( S x, S y )
{
	b2dVec2<S> r = { x, y };
	return r;
}
template <class S> B2D_HD b2dVec2<S> b2dSub( b2dVec2<S> a, b2dVec2<S> b ) { return b2dV( a.x - b.x, a.y - b.y ); }
template <class S> B2D_HD b2dVec2<S> b2dAdd( b2dVec2<S> a, b2dVec2<S> b ) { return b2dV( a.x + b.x, a.y + b.y ); }
template <class S> B2D_HD S b2dDot( b2dVec2<S> a, b2dVec2<S> b ) { return a.x * b.x + a.y * b.y; }
template <class S> B2D_HD b2dVec2<S> b2dNeg( b2dVec2<S> a ) { return b2dV( -a.x, -a.y ); }
/* b2CrossSV( 1.0f, v ): the unit factor is exact */
template <class S> B2D_HD b2dVec2<S> b2dLeftPerp( b2dVec2<S> v ) { return b2dV( -v.y, v.x ); }
template <class S> B2D_HD b2dVec2<S> b2dLerp( b2dVec2<S> a, b2dVec2<S> b, S t )
{
	S omt = 1.0f - t;
	return b2dV( omt * a.x + t * b.x, omt * a.y + t * b.y );
}
/* b2Lerp with a float fraction */
template <class S> B2D_HD b2dVec2<S> b2dLerpF( b2dVec2<S> a, b2dVec2<S> b, float t )
{
	float omt = 1.0f - t;
	return b2dV( omt * a.x + t * b.x, omt * a.y + t * b.y );
}
template <class S> B2D_HD b2dVec2<S> b2dMulAdd( b2dVec2<S> a, S s, b2dVec2<S> b ) { return b2dV( a.x + s * b.x, a.y + s * b.y ); }
template <class S> B2D_HD b2dVec2<S> b2dMulAddF( b2dVec2<S> a, float s, b2dVec2<S> b )
{
	return b2dV( a.x + s * b.x, a.y + s * b.y );
}
template <class S> B2D_HD b2dVec2<S> b2dRotate( b2dRot<S> q, b2dVec2<S> v ) { return b2dV( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
template <class S> B2D_HD b2dVec2<S> b2dInvRotate( b2dRot<S> q, b2dVec2<S> v )
{
	return b2dV( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y );
}
template <class S> B2D_HD b2dVec2<S> b2dTransformPoint( b2dXf<S> t, b2dVec2<S> p )
{
	return b2dV( ( t.q.c * p.x - t.q.s * p.y ) + t.p.x, ( t.q.s * p.x + t.q.c * p.y ) + t.p.y );
}
template <class S> B2D_HD b2dXf<S> b2dInvMulTransforms( b2dXf<S> A, b2dXf<S> B )
{
	b2dXf<S> C;
	C.q.s = A.q.c * B.q.s - A.q.s * B.q.c;
	C.q.c = A.q.c * B.q.c + A.q.s * B.q.s;
	b2dVec2<S> d = b2dV( B.p.x - A.p.x, B.p.y - A.p.y );
	C.p = b2dInvRotate( A.q, d );
	return C;
}

template <class S> struct b2dSegDist
{
	b2dVec2<S> closest1, closest2;
	S fraction1, fraction2, distanceSquared;
};

/* distance.c:33-106 */
template <class S> B2D_HD b2dSegDist<S> b2dSegmentDistance( b2dVec2<S> p1, b2dVec2<S> q1, b2dVec2<S> p2, b2dVec2<S> q2 )
{
	const S zero = S::make( 0.0f );
	b2dSegDist<S> res;
	res.fraction1 = zero;
	res.fraction2 = zero;
	b2dVec2<S> d1 = b2dSub( q1, p1 ), d2 = b2dSub( q2, p2 ), r = b2dSub( p1, p2 );
	S dd1 = b2dDot( d1, d1 ), dd2 = b2dDot( d2, d2 ), rd1 = b2dDot( r, d1 ), rd2 = b2dDot( r, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	if ( dd1.v < epsSqr || dd2.v < epsSqr )
	{
		if ( dd1.v >= epsSqr )
		{
			res.fraction1 = b2dClamp( -rd1 / dd1, 0.0f, 1.0f );
			res.fraction2 = zero;
		}
		else if ( dd2.v >= epsSqr )
		{
			res.fraction1 = zero;
			res.fraction2 = b2dClamp( rd2 / dd2, 0.0f, 1.0f );
		}
	}
	else
	{
		S d12 = b2dDot( d1, d2 );
		S denom = dd1 * dd2 - d12 * d12;
		S f1 = zero;
		if ( denom.v != 0.0f ) f1 = b2dClamp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
		S f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2.v < 0.0f )
		{
			f2 = zero;
			f1 = b2dClamp( -rd1 / dd1, 0.0f, 1.0f );
		}
		else if ( f2.v > 1.0f )
		{
			f2 = S::make( 1.0f );
			f1 = b2dClamp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
		}
		res.fraction1 = f1;
		res.fraction2 = f2;
	}
	res.closest1 = b2dMulAdd( p1, res.fraction1, d1 );
	res.closest2 = b2dMulAdd( p2, res.fraction2, d2 );
	b2dVec2<S> c = b2dV( res.closest2.x - res.closest1.x, res.closest2.y - res.closest1.y );
	res.distanceSquared = c.x * c.x + c.y * c.y;
	return res;
}

/* manifold.c:511-643 */
template <class S>
B2D_HD b2dManifold<S> b2dClipPolygons( const b2dPoly<S>* polyA, const b2dPoly<S>* polyB, int edgeA, int edgeB, int flip )
{
	b2dManifold<S> m;
	m.count = 0;
	const b2dPoly<S>*poly1, *poly2;
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
	b2dVec2<S> normal = poly1->n[i11];
	b2dVec2<S> v11 = poly1->v[i11], v12 = poly1->v[i12];
	b2dVec2<S> v21 = poly2->v[i21], v22 = poly2->v[i22];
	b2dVec2<S> tangent = b2dLeftPerp( normal );
	S lower1 = S::make( 0.0f );
	S upper1 = b2dDot( b2dSub( v12, v11 ), tangent );
	S upper2 = b2dDot( b2dSub( v21, v11 ), tangent );
	S lower2 = b2dDot( b2dSub( v22, v11 ), tangent );
	if ( upper2.v < lower1.v || upper1.v < lower2.v )
	{
		m.normal = normal;
		return m;
	}
	b2dVec2<S> vLower;
	if ( lower2.v < lower1.v && ( upper2 - lower2 ).v > FLT_EPSILON ) vLower = b2dLerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else vLower = v22;
	b2dVec2<S> vUpper;
	if ( upper2.v > upper1.v && ( upper2 - lower2 ).v > FLT_EPSILON ) vUpper = b2dLerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else vUpper = v21;
	S separationLower = b2dDot( b2dSub( vLower, v11 ), normal );
	S separationUpper = b2dDot( b2dSub( vUpper, v11 ), normal );
	float r1 = poly1->radius, r2 = poly2->radius;
	vLower = b2dMulAdd( vLower, 0.5f * ( ( r1 - r2 ) - separationLower ), normal );
	vUpper = b2dMulAdd( vUpper, 0.5f * ( ( r1 - r2 ) - separationUpper ), normal );
	float radius = r1 + r2;
	if ( flip == 0 )
	{
		m.normal = normal;
		m.points[0].point = vLower;
		m.points[0].separation = separationLower - radius;
		m.points[0].id = B2D_MAKE_ID( i11, i22 );
		m.points[1].point = vUpper;
		m.points[1].separation = separationUpper - radius;
		m.points[1].id = B2D_MAKE_ID( i12, i21 );
		m.count = 2;
	}
	else
	{
		m.normal = b2dNeg( normal );
		m.points[0].point = vUpper;
		m.points[0].separation = separationUpper - radius;
		m.points[0].id = B2D_MAKE_ID( i21, i12 );
		m.points[1].point = vLower;
		m.points[1].separation = separationLower - radius;
		m.points[1].id = B2D_MAKE_ID( i22, i11 );
		m.count = 2;
	}
	return m;
}

/* manifold.c:646-682; only the primal decides */
template <class S> B2D_HD float b2dFindMaxSeparation( int* edgeIndex, const b2dPoly<S>* poly1, const b2dPoly<S>* poly2 )
{
	int bestIndex = 0;
	float maxSeparation = -FLT_MAX;
	for ( int i = 0; i < poly1->count; ++i )
	{
		float nx = poly1->n[i].x.v, ny = poly1->n[i].y.v;
		float v1x = poly1->v[i].x.v, v1y = poly1->v[i].y.v;
		float si = FLT_MAX;
		for ( int j = 0; j < poly2->count; ++j )
		{
			float dx = poly2->v[j].x.v - v1x, dy = poly2->v[j].y.v - v1y;
			float sij = nx * dx + ny * dy;
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

/* manifold.c:702-1028 b2CollidePolygons: polygon A in its own frame, B placed by xf */
template <class S> B2D_HD b2dManifold<S> b2dCollidePolygons( const b2dPoly<S>* polygonA, const b2dPoly<S>* polygonB, b2dXf<S> xf )
{
	b2dVec2<S> origin = polygonA->v[0];
	b2dXf<S> xfs;
	xfs.p = b2dSub( xf.p, origin );
	xfs.q = xf.q;
	b2dPoly<S> A, B;
	A.count = polygonA->count;
	A.radius = polygonA->radius;
	A.v[0] = b2dV( S::make( 0.0f ), S::make( 0.0f ) );
	A.n[0] = polygonA->n[0];
	for ( int i = 1; i < A.count; ++i )
	{
		A.v[i] = b2dSub( polygonA->v[i], origin );
		A.n[i] = polygonA->n[i];
	}
	B.count = polygonB->count;
	B.radius = polygonB->radius;
	for ( int i = 0; i < B.count; ++i )
	{
		B.v[i] = b2dTransformPoint( xfs, polygonB->v[i] );
		B.n[i] = b2dRotate( xfs.q, polygonB->n[i] );
	}
	b2dManifold<S> m;
	m.count = 0;
	m.normal = b2dV( S::make( 0.0f ), S::make( 0.0f ) );
	int edgeA = 0;
	float separationA = b2dFindMaxSeparation( &edgeA, &A, &B );
	int edgeB = 0;
	float separationB = b2dFindMaxSeparation( &edgeB, &B, &A );
	float radius = A.radius + B.radius;
	if ( separationA > B2D_SPECULATIVE_DISTANCE + radius || separationB > B2D_SPECULATIVE_DISTANCE + radius ) return m;
	int flip;
	if ( separationA >= separationB )
	{
		flip = 0;
		float sx = A.n[edgeA].x.v, sy = A.n[edgeA].y.v;
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < B.count; ++i )
		{
			float d = sx * B.n[i].x.v + sy * B.n[i].y.v;
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
		float sx = B.n[edgeB].x.v, sy = B.n[edgeB].y.v;
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < A.count; ++i )
		{
			float d = sx * A.n[i].x.v + sy * A.n[i].y.v;
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}
	if ( separationA > 0.1f * B2D_LINEAR_SLOP || separationB > 0.1f * B2D_LINEAR_SLOP )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < A.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < B.count ? edgeB + 1 : 0;
		b2dVec2<S> v11 = A.v[i11], v12 = A.v[i12], v21 = B.v[i21], v22 = B.v[i22];
		b2dSegDist<S> res = b2dSegmentDistance( v11, v12, v21, v22 );
		S distance = b2dSqrt( res.distanceSquared );
		S separation = distance - radius;
		if ( ( distance - radius ).v > B2D_SPECULATIVE_DISTANCE ) return m;
		m = b2dClipPolygons( &A, &B, edgeA, edgeB, flip );
		float minSeparation = FLT_MAX;
		for ( int i = 0; i < m.count; ++i )
			minSeparation = minSeparation < m.points[i].separation.v ? minSeparation : m.points[i].separation.v;
		if ( separation.v + 0.1f * B2D_LINEAR_SLOP < minSeparation )
		{
			int hit = 0;
			b2dVec2<S> va = v11, vb = v21;
			int ia = i11, ib = i21;
			float f1 = res.fraction1.v, f2 = res.fraction2.v;
			if ( f1 == 0.0f && f2 == 0.0f )
			{
				hit = 1;
			}
			else if ( f1 == 0.0f && f2 == 1.0f )
			{
				hit = 1;
				vb = v22;
				ib = i22;
			}
			else if ( f1 == 1.0f && f2 == 0.0f )
			{
				hit = 1;
				va = v12;
				ia = i12;
			}
			else if ( f1 == 1.0f && f2 == 1.0f )
			{
				hit = 1;
				va = v12;
				ia = i12;
				vb = v22;
				ib = i22;
			}
			if ( hit )
			{
				b2dVec2<S> normal = b2dSub( vb, va );
				S invDistance = 1.0f / distance;
				normal.x = normal.x * invDistance;
				normal.y = normal.y * invDistance;
				b2dVec2<S> c1 = b2dMulAddF( va, A.radius, normal );
				b2dVec2<S> c2 = b2dMulAddF( vb, -B.radius, normal );
				m.normal = normal;
				m.points[0].point = b2dLerpF( c1, c2, 0.5f );
				m.points[0].separation = distance - radius;
				m.points[0].id = B2D_MAKE_ID( ia, ib );
				m.count = 1;
			}
		}
	}
	else
	{
		m = b2dClipPolygons( &A, &B, edgeA, edgeB, flip );
	}
	for ( int i = 0; i < m.count; ++i ) m.points[i].point = b2dAdd( m.points[i].point, origin );
	return m;
}

template <class S> B2D_HD b2dVec2<S> b2dMulSubF( b2dVec2<S> a, float s, b2dVec2<S> b )
{
	return b2dV( a.x - s * b.x, a.y - s * b.y );
}

/* math_functions.h b2Normalize and b2GetLengthAndNormalize */
template <class S> B2D_HD b2dVec2<S> b2dNormalize( b2dVec2<S> a )
{
	S lengthSquared = a.x * a.x + a.y * a.y;
	if ( lengthSquared.v > 1000.0f * FLT_MIN )
	{
		S s = 1.0f / b2dSqrt( lengthSquared );
		return b2dV( s * a.x, s * a.y );
	}
	return b2dV( S::make( 0.0f ), S::make( 0.0f ) );
}

template <class S> B2D_HD b2dVec2<S> b2dGetLengthAndNormalize( S* length, b2dVec2<S> a )
{
	S lengthSquared = a.x * a.x + a.y * a.y;
	if ( lengthSquared.v > 1000.0f * FLT_MIN )
	{
		*length = b2dSqrt( lengthSquared );
		S s = 1.0f / *length;
		return b2dV( s * a.x, s * a.y );
	}
	*length = S::make( 0.0f );
	return b2dV( S::make( 0.0f ), S::make( 0.0f ) );
}

/* manifold.c:36-66 b2CollideCircles: circle A in its own frame, B placed by xf */
template <class S>
B2D_HD b2dManifold<S> b2dCollideCircles( b2dVec2<S> centerA, float radiusA, b2dVec2<S> centerB, float radiusB, b2dXf<S> xf )
{
	b2dManifold<S> m;
	m.count = 0;
	m.normal = b2dV( S::make( 0.0f ), S::make( 0.0f ) );
	b2dVec2<S> pointA = centerA;
	b2dVec2<S> pointB = b2dTransformPoint( xf, centerB );
	S distance;
	b2dVec2<S> normal = b2dGetLengthAndNormalize( &distance, b2dSub( pointB, pointA ) );
	S separation = distance - radiusA - radiusB;
	if ( separation.v > B2D_SPECULATIVE_DISTANCE ) return m;
	b2dVec2<S> cA = b2dMulAddF( pointA, radiusA, normal );
	b2dVec2<S> cB = b2dMulAddF( pointB, -radiusB, normal );
	m.normal = normal;
	m.points[0].point = b2dLerpF( cA, cB, 0.5f );
	m.points[0].separation = separation;
	m.points[0].id = 0;
	m.count = 1;
	return m;
}

/* manifold.c:127-230 b2CollidePolygonAndCircle: polygon A in its own frame, circle B placed
   by xf */
template <class S>
B2D_HD b2dManifold<S> b2dCollidePolygonAndCircle( const b2dPoly<S>* polygonA, b2dVec2<S> centerB, float radiusB, b2dXf<S> xf )
{
	b2dManifold<S> m;
	m.count = 0;
	m.normal = b2dV( S::make( 0.0f ), S::make( 0.0f ) );
	const float speculativeDistance = B2D_SPECULATIVE_DISTANCE;
	b2dVec2<S> center = b2dTransformPoint( xf, centerB );
	float radiusA = polygonA->radius;
	float radius = radiusA + radiusB;
	int normalIndex = 0;
	S separation = S::make( -FLT_MAX );
	for ( int i = 0; i < polygonA->count; ++i )
	{
		S s = b2dDot( polygonA->n[i], b2dSub( center, polygonA->v[i] ) );
		if ( s.v > separation.v )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation.v > radius + speculativeDistance ) return m;
	int vertIndex1 = normalIndex;
	int vertIndex2 = vertIndex1 + 1 < polygonA->count ? vertIndex1 + 1 : 0;
	b2dVec2<S> v1 = polygonA->v[vertIndex1];
	b2dVec2<S> v2 = polygonA->v[vertIndex2];
	S u1 = b2dDot( b2dSub( center, v1 ), b2dSub( v2, v1 ) );
	S u2 = b2dDot( b2dSub( center, v2 ), b2dSub( v1, v2 ) );
	if ( ( u1.v < 0.0f && separation.v > FLT_EPSILON ) || ( u2.v < 0.0f && separation.v > FLT_EPSILON ) )
	{
		/* the circle center is closest to a vertex and safely outside the polygon */
		b2dVec2<S> v = u1.v < 0.0f ? v1 : v2;
		b2dVec2<S> normal = b2dNormalize( b2dSub( center, v ) );
		S sep = b2dDot( b2dSub( center, v ), normal );
		if ( sep.v > radius + speculativeDistance ) return m;
		b2dVec2<S> cA = b2dMulAddF( v, radiusA, normal );
		b2dVec2<S> cB = b2dMulSubF( center, radiusB, normal );
		m.normal = normal;
		m.points[0].point = b2dLerpF( cA, cB, 0.5f );
		m.points[0].separation = b2dDot( b2dSub( cB, cA ), normal );
		m.points[0].id = 0;
		m.count = 1;
		return m;
	}
	b2dVec2<S> normal = polygonA->n[normalIndex];
	m.normal = normal;
	b2dVec2<S> cA = b2dMulAdd( center, radiusA - b2dDot( b2dSub( center, v1 ), normal ), normal );
	b2dVec2<S> cB = b2dMulSubF( center, radiusB, normal );
	m.points[0].point = b2dLerpF( cA, cB, 0.5f );
	m.points[0].separation = separation - radius;
	m.points[0].id = 0;
	m.count = 1;
	return m;
}

/* a polygon shape's local geometry as dual constants */
template <class S>
B2D_HD void b2dMakePoly( b2dPoly<S>* p, const float* verts, const float* normals, int count, float radius )
{
	p->count = count;
	p->radius = radius;
	for ( int i = 0; i < count; ++i )
	{
		p->v[i] = b2dV( S::make( verts[2 * i] ), S::make( verts[2 * i + 1] ) );
		p->n[i] = b2dV( S::make( normals[2 * i] ), S::make( normals[2 * i + 1] ) );
	}
}

/* contact manifold in world orientation (contact.c:519-698 b2UpdateContact): normal, and
   per point the anchors relative to each body's center of mass and the separation */
template <class S> struct b2dContactGeometry
{
	b2dVec2<S> normal;
	b2dVec2<S> anchorA[2], anchorB[2];
	S separation[2];
	uint16_t id[2];
	int count;
};

/* the world geometry of a manifold computed in frame A */
template <class S>
B2D_HD b2dContactGeometry<S> b2dContactFromLocal( const b2dManifold<S>& local, b2dXf<S> xfA, b2dXf<S> xfB, float lcAx, float lcAy,
												   float lcBx, float lcBy );

template <class S>
B2D_HD b2dContactGeometry<S> b2dContactManifold( const b2dPoly<S>* polyA, const b2dPoly<S>* polyB, b2dXf<S> xfA, b2dXf<S> xfB,
												  float lcAx, float lcAy, float lcBx, float lcBy )
{
	b2dXf<S> rel = b2dInvMulTransforms( xfA, xfB );
	return b2dContactFromLocal( b2dCollidePolygons( polyA, polyB, rel ), xfA, xfB, lcAx, lcAy, lcBx, lcBy );
}

/* a polygon (A) and a circle (B, center in its body frame) */
template <class S>
B2D_HD b2dContactGeometry<S> b2dContactPolygonCircle( const b2dPoly<S>* polyA, b2dVec2<S> centerB, float radiusB, b2dXf<S> xfA,
													   b2dXf<S> xfB, float lcAx, float lcAy, float lcBx, float lcBy )
{
	b2dXf<S> rel = b2dInvMulTransforms( xfA, xfB );
	return b2dContactFromLocal( b2dCollidePolygonAndCircle( polyA, centerB, radiusB, rel ), xfA, xfB, lcAx, lcAy, lcBx, lcBy );
}

/* two circles */
template <class S>
B2D_HD b2dContactGeometry<S> b2dContactCircles( b2dVec2<S> centerA, float radiusA, b2dVec2<S> centerB, float radiusB, b2dXf<S> xfA,
												 b2dXf<S> xfB, float lcAx, float lcAy, float lcBx, float lcBy )
{
	b2dXf<S> rel = b2dInvMulTransforms( xfA, xfB );
	return b2dContactFromLocal( b2dCollideCircles( centerA, radiusA, centerB, radiusB, rel ), xfA, xfB, lcAx, lcAy, lcBx, lcBy );
}

template <class S>
B2D_HD b2dContactGeometry<S> b2dContactFromLocal( const b2dManifold<S>& local, b2dXf<S> xfA, b2dXf<S> xfB, float lcAx, float lcAy,
												   float lcBx, float lcBy )
{
	b2dContactGeometry<S> g;
	g.count = local.count;
	g.normal = b2dRotate( xfA.q, local.normal );
	b2dVec2<S> originDelta = b2dV( xfA.p.x - xfB.p.x, xfA.p.y - xfB.p.y );
	b2dVec2<S> lcA = b2dV( S::make( lcAx ), S::make( lcAy ) ), lcB = b2dV( S::make( lcBx ), S::make( lcBy ) );
	b2dVec2<S> centerOffsetA = b2dRotate( xfA.q, lcA );
	b2dVec2<S> centerOffsetB = b2dRotate( xfB.q, lcB );
	for ( int i = 0; i < local.count; ++i )
	{
		b2dVec2<S> anchorA = b2dRotate( xfA.q, local.points[i].point );
		b2dVec2<S> anchorB = b2dAdd( anchorA, originDelta );
		g.anchorA[i] = b2dSub( anchorA, centerOffsetA );
		g.anchorB[i] = b2dSub( anchorB, centerOffsetB );
		g.separation[i] = local.points[i].separation;
		g.id[i] = local.points[i].id;
	}
	return g;
}
