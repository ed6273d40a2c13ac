/*
 * Oracle (test checker and CPU baseline only): continuous collision of fast non-bullet
 * bodies against static shapes (b2SolveContinuous and b2ContinuousQueryCallback,
 * solver.c:183-550), with the time of impact by conservative advancement on separating
 * axes (b2TimeOfImpact, distance.c:953-1430) over the GJK distance (b2ShapeDistance,
 * distance.c:138-612). Bullets are not restated; they are advanced like slow bodies and
 * counted so tests can refuse a run that needed them.
 */
#include "o_core.h"

#include <float.h>

int o_continuousSkipped = 0;

typedef struct o_proxy
{
	b2Vec2 points[B2_MAX_POLYGON_VERTICES];
	int count;
	float radius;
} o_proxy;

typedef struct o_sweep
{
	b2Vec2 localCenter, c1, c2;
	b2Rot q1, q2;
} o_sweep;

typedef struct o_simplexVertex
{
	b2Vec2 wA, wB, w;
	float a;
	int indexA, indexB;
} o_simplexVertex;

typedef struct o_simplex
{
	o_simplexVertex v1, v2, v3;
	int count;
} o_simplex;

typedef struct o_simplexCache
{
	int count;
	int indexA[3], indexB[3];
} o_simplexCache;

/* b2MakeProxy (distance.c:108-119) */
static o_proxy o_makeProxy( const b2Vec2* points, int count, float radius )
{
	o_proxy p;
	memset( &p, 0, sizeof( p ) );
	count = count < B2_MAX_POLYGON_VERTICES ? count : B2_MAX_POLYGON_VERTICES;
	for ( int i = 0; i < count; ++i ) p.points[i] = points[i];
	p.count = count;
	p.radius = radius;
	return p;
}

/* b2MakeShapeDistanceProxy (shape.c:1055-1076) */
static o_proxy o_shapeProxy( const o_shape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape: return o_makeProxy( &s->capsule.center1, 2, s->capsule.radius );
		case b2_circleShape: return o_makeProxy( &s->circle.center, 1, s->circle.radius );
		case b2_polygonShape: return o_makeProxy( s->polygon.vertices, s->polygon.count, s->polygon.radius );
		case b2_segmentShape: return o_makeProxy( &s->segment.point1, 2, 0.0f );
		default:
		{
			o_proxy empty;
			memset( &empty, 0, sizeof( empty ) );
			return empty;
		}
	}
}

/* b2GetSweepTransform (distance.c:14-30) */
static b2Transform o_sweepTransform( const o_sweep* sweep, float time )
{
	b2Transform xf;
	xf.p = o_add( o_mulSV( 1.0f - time, sweep->c1 ), o_mulSV( time, sweep->c2 ) );
	b2Rot q = { ( 1.0f - time ) * sweep->q1.c + time * sweep->q2.c, ( 1.0f - time ) * sweep->q1.s + time * sweep->q2.s };
	xf.q = o_normalizeRot( q );
	xf.p = o_sub( xf.p, o_rotate( xf.q, sweep->localCenter ) );
	return xf;
}

static int o_findSupport( const o_proxy* proxy, b2Vec2 direction )
{
	int bestIndex = 0;
	float bestValue = o_dot( proxy->points[0], direction );
	for ( int i = 1; i < proxy->count; ++i )
	{
		float value = o_dot( proxy->points[i], direction );
		if ( value > bestValue )
		{
			bestIndex = i;
			bestValue = value;
		}
	}
	return bestIndex;
}

static o_simplexVertex* o_vertex( o_simplex* s, int i ) { return i == 0 ? &s->v1 : ( i == 1 ? &s->v2 : &s->v3 ); }

static o_simplex o_simplexFromCache( const o_simplexCache* cache, const o_proxy* proxyA, const o_proxy* proxyB )
{
	o_simplex s;
	memset( &s, 0, sizeof( s ) );
	s.count = cache->count;
	for ( int i = 0; i < s.count; ++i )
	{
		o_simplexVertex* v = o_vertex( &s, i );
		v->indexA = cache->indexA[i];
		v->indexB = cache->indexB[i];
		v->wA = proxyA->points[v->indexA];
		v->wB = proxyB->points[v->indexB];
		v->w = o_sub( v->wA, v->wB );
		v->a = -1.0f;
	}
	if ( s.count == 0 )
	{
		o_simplexVertex* v = &s.v1;
		v->indexA = 0;
		v->indexB = 0;
		v->wA = proxyA->points[0];
		v->wB = proxyB->points[0];
		v->w = o_sub( v->wA, v->wB );
		v->a = 1.0f;
		s.count = 1;
	}
	return s;
}

static o_simplexCache o_makeCache( o_simplex* s )
{
	o_simplexCache c;
	memset( &c, 0, sizeof( c ) );
	c.count = s->count;
	for ( int i = 0; i < s->count; ++i )
	{
		c.indexA[i] = o_vertex( s, i )->indexA;
		c.indexB[i] = o_vertex( s, i )->indexB;
	}
	return c;
}

static void o_witnessPoints( const o_simplex* s, b2Vec2* a, b2Vec2* b )
{
	switch ( s->count )
	{
		case 1:
			*a = s->v1.wA;
			*b = s->v1.wB;
			break;
		case 2:
			*a = o_v( s->v1.a * s->v1.wA.x + s->v2.a * s->v2.wA.x, s->v1.a * s->v1.wA.y + s->v2.a * s->v2.wA.y );
			*b = o_v( s->v1.a * s->v1.wB.x + s->v2.a * s->v2.wB.x, s->v1.a * s->v1.wB.y + s->v2.a * s->v2.wB.y );
			break;
		case 3:
			*a = o_v( s->v1.a * s->v1.wA.x + s->v2.a * s->v2.wA.x + s->v3.a * s->v3.wA.x,
					  s->v1.a * s->v1.wA.y + s->v2.a * s->v2.wA.y + s->v3.a * s->v3.wA.y );
			*b = *a;
			break;
		default:
			*a = o_v( 0.0f, 0.0f );
			*b = o_v( 0.0f, 0.0f );
			break;
	}
}

/* b2SolveSimplex2 (distance.c:274-307): closest point of a segment simplex, returns the
   direction towards the origin */
static b2Vec2 o_solveSimplex2( o_simplex* s )
{
	b2Vec2 w1 = s->v1.w, w2 = s->v2.w;
	b2Vec2 e12 = o_sub( w2, w1 );
	float d12_2 = -o_dot( w1, e12 );
	if ( d12_2 <= 0.0f )
	{
		s->v1.a = 1.0f;
		s->count = 1;
		return o_neg( w1 );
	}
	float d12_1 = o_dot( w2, e12 );
	if ( d12_1 <= 0.0f )
	{
		s->v2.a = 1.0f;
		s->count = 1;
		s->v1 = s->v2;
		return o_neg( w2 );
	}
	float inv_d12 = 1.0f / ( d12_1 + d12_2 );
	s->v1.a = d12_1 * inv_d12;
	s->v2.a = d12_2 * inv_d12;
	s->count = 2;
	return o_crossSV( o_cross( o_add( w1, w2 ), e12 ), e12 );
}

/* b2SolveSimplex3 (distance.c:309-419) */
static b2Vec2 o_solveSimplex3( o_simplex* s )
{
	b2Vec2 w1 = s->v1.w, w2 = s->v2.w, w3 = s->v3.w;
	b2Vec2 e12 = o_sub( w2, w1 );
	float w1e12 = o_dot( w1, e12 ), w2e12 = o_dot( w2, e12 );
	float d12_1 = w2e12, d12_2 = -w1e12;
	b2Vec2 e13 = o_sub( w3, w1 );
	float w1e13 = o_dot( w1, e13 ), w3e13 = o_dot( w3, e13 );
	float d13_1 = w3e13, d13_2 = -w1e13;
	b2Vec2 e23 = o_sub( w3, w2 );
	float w2e23 = o_dot( w2, e23 ), w3e23 = o_dot( w3, e23 );
	float d23_1 = w3e23, d23_2 = -w2e23;
	float n123 = o_cross( e12, e13 );
	float d123_1 = n123 * o_cross( w2, w3 );
	float d123_2 = n123 * o_cross( w3, w1 );
	float d123_3 = n123 * o_cross( w1, w2 );
	if ( d12_2 <= 0.0f && d13_2 <= 0.0f )
	{
		s->v1.a = 1.0f;
		s->count = 1;
		return o_neg( w1 );
	}
	if ( d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f )
	{
		float inv_d12 = 1.0f / ( d12_1 + d12_2 );
		s->v1.a = d12_1 * inv_d12;
		s->v2.a = d12_2 * inv_d12;
		s->count = 2;
		return o_crossSV( o_cross( o_add( w1, w2 ), e12 ), e12 );
	}
	if ( d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f )
	{
		float inv_d13 = 1.0f / ( d13_1 + d13_2 );
		s->v1.a = d13_1 * inv_d13;
		s->v3.a = d13_2 * inv_d13;
		s->count = 2;
		s->v2 = s->v3;
		return o_crossSV( o_cross( o_add( w1, w3 ), e13 ), e13 );
	}
	if ( d12_1 <= 0.0f && d23_2 <= 0.0f )
	{
		s->v2.a = 1.0f;
		s->count = 1;
		s->v1 = s->v2;
		return o_neg( w2 );
	}
	if ( d13_1 <= 0.0f && d23_1 <= 0.0f )
	{
		s->v3.a = 1.0f;
		s->count = 1;
		s->v1 = s->v3;
		return o_neg( w3 );
	}
	if ( d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f )
	{
		float inv_d23 = 1.0f / ( d23_1 + d23_2 );
		s->v2.a = d23_1 * inv_d23;
		s->v3.a = d23_2 * inv_d23;
		s->count = 2;
		s->v1 = s->v3;
		return o_crossSV( o_cross( o_add( w2, w3 ), e23 ), e23 );
	}
	float inv_d123 = 1.0f / ( d123_1 + d123_2 + d123_3 );
	s->v1.a = d123_1 * inv_d123;
	s->v2.a = d123_2 * inv_d123;
	s->v3.a = d123_3 * inv_d123;
	s->count = 3;
	return o_v( 0.0f, 0.0f );
}

typedef struct o_distanceOutput
{
	b2Vec2 pointA, pointB, normal;
	float distance;
} o_distanceOutput;

/* b2ShapeDistance without radii (distance.c:424-612): GJK in the frame of proxy A, with
   proxy B placed by `transform`; updates the simplex cache */
static o_distanceOutput o_shapeDistance( const o_proxy* proxyA, const o_proxy* proxyB, b2Transform transform,
										 o_simplexCache* cache )
{
	o_distanceOutput output;
	memset( &output, 0, sizeof( output ) );
	o_proxy localB;
	memset( &localB, 0, sizeof( localB ) );
	localB.count = proxyB->count;
	localB.radius = proxyB->radius;
	for ( int i = 0; i < localB.count; ++i ) localB.points[i] = o_transformPoint( transform, proxyB->points[i] );
	o_simplex simplex = o_simplexFromCache( cache, proxyA, &localB );
	b2Vec2 nonUnitNormal = o_v( 0.0f, 0.0f );
	int saveA[3], saveB[3];
	const int maxIterations = 20;
	int iteration = 0;
	while ( iteration < maxIterations )
	{
		int saveCount = simplex.count;
		for ( int i = 0; i < saveCount; ++i )
		{
			saveA[i] = o_vertex( &simplex, i )->indexA;
			saveB[i] = o_vertex( &simplex, i )->indexB;
		}
		b2Vec2 d = o_v( 0.0f, 0.0f );
		switch ( simplex.count )
		{
			case 1: d = o_neg( simplex.v1.w ); break;
			case 2: d = o_solveSimplex2( &simplex ); break;
			case 3: d = o_solveSimplex3( &simplex ); break;
			default: break;
		}
		if ( simplex.count == 3 )
		{
			*cache = o_makeCache( &simplex );
			o_witnessPoints( &simplex, &output.pointA, &output.pointB );
			output.distance = 0.0f;
			return output;
		}
		if ( o_dot( d, d ) < 1000.0f * FLT_MIN )
		{
			*cache = o_makeCache( &simplex );
			o_witnessPoints( &simplex, &output.pointA, &output.pointB );
			output.distance = 0.0f;
			return output;
		}
		nonUnitNormal = d;
		o_simplexVertex* vertex = o_vertex( &simplex, simplex.count );
		vertex->indexA = o_findSupport( proxyA, d );
		vertex->wA = proxyA->points[vertex->indexA];
		vertex->indexB = o_findSupport( &localB, o_neg( d ) );
		vertex->wB = localB.points[vertex->indexB];
		vertex->w = o_sub( vertex->wA, vertex->wB );
		++iteration;
		int duplicate = 0;
		for ( int i = 0; i < saveCount; ++i )
		{
			if ( vertex->indexA == saveA[i] && vertex->indexB == saveB[i] )
			{
				duplicate = 1;
				break;
			}
		}
		if ( duplicate ) break;
		simplex.count += 1;
	}
	b2Vec2 normal = o_normalize( nonUnitNormal );
	o_witnessPoints( &simplex, &output.pointA, &output.pointB );
	output.normal = normal;
	output.distance = o_distance( output.pointA, output.pointB );
	*cache = o_makeCache( &simplex );
	return output;
}

enum
{
	O_SEP_POINTS = 0,
	O_SEP_FACE_A = 1,
	O_SEP_FACE_B = 2,
};

typedef struct o_separation
{
	const o_proxy *proxyA, *proxyB;
	o_sweep sweepA, sweepB;
	b2Vec2 localPoint, axis;
	int type;
} o_separation;

/* b2MakeSeparationFunction (distance.c:953-1027) */
static o_separation o_makeSeparation( const o_simplexCache* cache, const o_proxy* proxyA, const o_sweep* sweepA,
									  const o_proxy* proxyB, const o_sweep* sweepB, float t1 )
{
	o_separation f;
	memset( &f, 0, sizeof( f ) );
	f.proxyA = proxyA;
	f.proxyB = proxyB;
	f.sweepA = *sweepA;
	f.sweepB = *sweepB;
	b2Transform xfA = o_sweepTransform( sweepA, t1 );
	b2Transform xfB = o_sweepTransform( sweepB, t1 );
	if ( cache->count == 1 )
	{
		f.type = O_SEP_POINTS;
		b2Vec2 pointA = o_transformPoint( xfA, proxyA->points[cache->indexA[0]] );
		b2Vec2 pointB = o_transformPoint( xfB, proxyB->points[cache->indexB[0]] );
		f.axis = o_normalize( o_sub( pointB, pointA ) );
		f.localPoint = o_v( 0.0f, 0.0f );
		return f;
	}
	if ( cache->indexA[0] == cache->indexA[1] )
	{
		f.type = O_SEP_FACE_B;
		b2Vec2 localPointB1 = proxyB->points[cache->indexB[0]];
		b2Vec2 localPointB2 = proxyB->points[cache->indexB[1]];
		f.axis = o_crossVS( o_sub( localPointB2, localPointB1 ), 1.0f );
		f.axis = o_normalize( f.axis );
		b2Vec2 normal = o_rotate( xfB.q, f.axis );
		f.localPoint = o_v( 0.5f * ( localPointB1.x + localPointB2.x ), 0.5f * ( localPointB1.y + localPointB2.y ) );
		b2Vec2 pointB = o_transformPoint( xfB, f.localPoint );
		b2Vec2 pointA = o_transformPoint( xfA, proxyA->points[cache->indexA[0]] );
		float s = o_dot( o_sub( pointA, pointB ), normal );
		if ( s < 0.0f ) f.axis = o_neg( f.axis );
		return f;
	}
	f.type = O_SEP_FACE_A;
	b2Vec2 localPointA1 = proxyA->points[cache->indexA[0]];
	b2Vec2 localPointA2 = proxyA->points[cache->indexA[1]];
	f.axis = o_crossVS( o_sub( localPointA2, localPointA1 ), 1.0f );
	f.axis = o_normalize( f.axis );
	b2Vec2 normal = o_rotate( xfA.q, f.axis );
	f.localPoint = o_v( 0.5f * ( localPointA1.x + localPointA2.x ), 0.5f * ( localPointA1.y + localPointA2.y ) );
	b2Vec2 pointA = o_transformPoint( xfA, f.localPoint );
	b2Vec2 pointB = o_transformPoint( xfB, proxyB->points[cache->indexB[0]] );
	float s = o_dot( o_sub( pointB, pointA ), normal );
	if ( s < 0.0f ) f.axis = o_neg( f.axis );
	return f;
}

/* b2FindMinSeparation (distance.c:1029-1095) */
static float o_findMinSeparation( const o_separation* f, int* indexA, int* indexB, float t )
{
	b2Transform xfA = o_sweepTransform( &f->sweepA, t );
	b2Transform xfB = o_sweepTransform( &f->sweepB, t );
	switch ( f->type )
	{
		case O_SEP_POINTS:
		{
			b2Vec2 axisA = o_invRotate( xfA.q, f->axis );
			b2Vec2 axisB = o_invRotate( xfB.q, o_neg( f->axis ) );
			*indexA = o_findSupport( f->proxyA, axisA );
			*indexB = o_findSupport( f->proxyB, axisB );
			b2Vec2 pointA = o_transformPoint( xfA, f->proxyA->points[*indexA] );
			b2Vec2 pointB = o_transformPoint( xfB, f->proxyB->points[*indexB] );
			return o_dot( o_sub( pointB, pointA ), f->axis );
		}
		case O_SEP_FACE_A:
		{
			b2Vec2 normal = o_rotate( xfA.q, f->axis );
			b2Vec2 pointA = o_transformPoint( xfA, f->localPoint );
			b2Vec2 axisB = o_invRotate( xfB.q, o_neg( normal ) );
			*indexA = -1;
			*indexB = o_findSupport( f->proxyB, axisB );
			b2Vec2 pointB = o_transformPoint( xfB, f->proxyB->points[*indexB] );
			return o_dot( o_sub( pointB, pointA ), normal );
		}
		default:
		{
			b2Vec2 normal = o_rotate( xfB.q, f->axis );
			b2Vec2 pointB = o_transformPoint( xfB, f->localPoint );
			b2Vec2 axisA = o_invRotate( xfA.q, o_neg( normal ) );
			*indexB = -1;
			*indexA = o_findSupport( f->proxyA, axisA );
			b2Vec2 pointA = o_transformPoint( xfA, f->proxyA->points[*indexA] );
			return o_dot( o_sub( pointA, pointB ), normal );
		}
	}
}

/* b2EvaluateSeparation (distance.c:1097-1145) */
static float o_evaluateSeparation( const o_separation* f, int indexA, int indexB, float t )
{
	b2Transform xfA = o_sweepTransform( &f->sweepA, t );
	b2Transform xfB = o_sweepTransform( &f->sweepB, t );
	switch ( f->type )
	{
		case O_SEP_POINTS:
		{
			b2Vec2 pointA = o_transformPoint( xfA, f->proxyA->points[indexA] );
			b2Vec2 pointB = o_transformPoint( xfB, f->proxyB->points[indexB] );
			return o_dot( o_sub( pointB, pointA ), f->axis );
		}
		case O_SEP_FACE_A:
		{
			b2Vec2 normal = o_rotate( xfA.q, f->axis );
			b2Vec2 pointA = o_transformPoint( xfA, f->localPoint );
			b2Vec2 pointB = o_transformPoint( xfB, f->proxyB->points[indexB] );
			return o_dot( o_sub( pointB, pointA ), normal );
		}
		default:
		{
			b2Vec2 normal = o_rotate( xfB.q, f->axis );
			b2Vec2 pointB = o_transformPoint( xfB, f->localPoint );
			b2Vec2 pointA = o_transformPoint( xfA, f->proxyA->points[indexA] );
			return o_dot( o_sub( pointA, pointB ), normal );
		}
	}
}

/* b2TimeOfImpact (distance.c:1148-1430); only the fraction is used by the step */
static float o_timeOfImpact( const o_proxy* proxyA, const o_sweep* sweepA, const o_proxy* proxyB, const o_sweep* sweepB,
							 float maxFraction )
{
	float fraction = maxFraction;
	float tMax = maxFraction;
	float totalRadius = proxyA->radius + proxyB->radius;
	float target = o_max( O_LINEAR_SLOP, totalRadius - O_LINEAR_SLOP );
	float tolerance = 0.25f * O_LINEAR_SLOP;
	float t1 = 0.0f;
	const int maxIterations = 20;
	int distanceIterations = 0;
	o_simplexCache cache;
	memset( &cache, 0, sizeof( cache ) );
	for ( ;; )
	{
		b2Transform xfA = o_sweepTransform( sweepA, t1 );
		b2Transform xfB = o_sweepTransform( sweepB, t1 );
		o_distanceOutput d = o_shapeDistance( proxyA, proxyB, o_invMulTransforms( xfA, xfB ), &cache );
		distanceIterations += 1;
		if ( d.distance <= 0.0f )
		{
			fraction = 0.0f; /* overlapped */
			break;
		}
		if ( d.distance <= target + tolerance )
		{
			fraction = t1; /* hit */
			break;
		}
		o_separation fcn = o_makeSeparation( &cache, proxyA, sweepA, proxyB, sweepB, t1 );
		int done = 0;
		float t2 = tMax;
		int pushBackIterations = 0;
		for ( ;; )
		{
			int indexA, indexB;
			float s2 = o_findMinSeparation( &fcn, &indexA, &indexB, t2 );
			if ( s2 > target + tolerance )
			{
				fraction = tMax; /* separated */
				done = 1;
				break;
			}
			if ( s2 > target - tolerance )
			{
				t1 = t2;
				break;
			}
			float s1 = o_evaluateSeparation( &fcn, indexA, indexB, t1 );
			if ( s1 < target - tolerance )
			{
				fraction = t1; /* failed */
				done = 1;
				break;
			}
			if ( s1 <= target + tolerance )
			{
				fraction = t1; /* hit */
				done = 1;
				break;
			}
			int rootIterationCount = 0;
			float a1 = t1, a2 = t2;
			for ( ;; )
			{
				float t;
				if ( rootIterationCount & 1 ) t = a1 + ( target - s1 ) * ( a2 - a1 ) / ( s2 - s1 );
				else t = 0.5f * ( a1 + a2 );
				rootIterationCount += 1;
				float s = o_evaluateSeparation( &fcn, indexA, indexB, t );
				if ( o_abs( s - target ) < tolerance )
				{
					t2 = t;
					break;
				}
				if ( s > target )
				{
					a1 = t;
					s1 = s;
				}
				else
				{
					a2 = t;
					s2 = s;
				}
				if ( rootIterationCount == 50 ) break;
			}
			pushBackIterations += 1;
			if ( pushBackIterations == B2_MAX_POLYGON_VERTICES ) break;
		}
		if ( done ) break;
		if ( distanceIterations == maxIterations )
		{
			fraction = t1; /* failed */
			break;
		}
	}
	return fraction;
}

typedef struct o_continuousContext
{
	o_world* w;
	o_bodySim* fastSim;
	o_shape* fastShape;
	o_sweep sweep;
	b2Vec2 base;
	float fraction;
} o_continuousContext;

#define O_CORE_FRACTION 0.25f

static int o_shouldShapesCollideCcd( b2Filter a, b2Filter b )
{
	if ( a.groupIndex == b.groupIndex && a.groupIndex != 0 ) return a.groupIndex > 0;
	return ( a.maskBits & b.categoryBits ) != 0 && ( a.categoryBits & b.maskBits ) != 0;
}

/* sweep of a body relative to `base` (body.h:237-247 b2MakeRelativeSweep) */
static o_sweep o_relativeSweep( const o_bodySim* sim, b2Vec2 base )
{
	o_sweep s;
	s.c1 = o_sub( sim->center0, base );
	s.c2 = o_sub( sim->center, base );
	s.q1 = sim->rotation0;
	s.q2 = sim->transform.q;
	s.localCenter = sim->localCenter;
	return s;
}

/* b2ContinuousQueryCallback (solver.c:183-376) for static shapes; chain segments, sensors
   and custom filters do not exist on this path */
static int o_continuousQuery( int proxyId, uint64_t userData, void* context )
{
	(void)proxyId;
	int shapeId = (int)userData;
	o_continuousContext* c = context;
	o_world* w = c->w;
	o_shape* fastShape = c->fastShape;
	if ( shapeId == fastShape->id ) return 1;
	o_shape* shape = w->shapes.data + shapeId;
	if ( shape->bodyId == fastShape->bodyId ) return 1;
	if ( shape->isSensor ) return 1;
	if ( o_shouldShapesCollideCcd( fastShape->filter, shape->filter ) == 0 ) return 1;
	o_body* body = w->bodies.data + shape->bodyId;
	o_bodySim* bodySim = body->setIndex == O_AWAKE_SET ? w->awakeSims.data + body->localIndex : w->staticSims.data + body->localIndex;
	if ( bodySim->flags & O_IS_BULLET ) return 1;
	o_body* fastBody = w->bodies.data + c->fastSim->bodyId;
	if ( o_shouldBodiesCollide( w, fastBody, body ) == 0 ) return 1;
	o_proxy proxyA = o_shapeProxy( shape );
	o_proxy proxyB = o_shapeProxy( fastShape );
	o_sweep sweepA = o_relativeSweep( bodySim, c->base );
	float f = o_timeOfImpact( &proxyA, &sweepA, &proxyB, &c->sweep, c->fraction );
	float hitFraction = c->fraction;
	int didHit = 0;
	if ( 0.0f < f && f < c->fraction )
	{
		hitFraction = f;
		didHit = 1;
	}
	else if ( 0.0f == f )
	{
		/* fall back to a small circle around the fast shape's centroid */
		b2Vec2 centroid = o_getShapeCentroid( fastShape );
		float minExtent, maxExtent;
		o_computeShapeExtent( fastShape, centroid, &minExtent, &maxExtent );
		proxyB = o_makeProxy( &centroid, 1, O_CORE_FRACTION * minExtent );
		f = o_timeOfImpact( &proxyA, &sweepA, &proxyB, &c->sweep, c->fraction );
		if ( 0.0f < f && f < c->fraction )
		{
			hitFraction = f;
			didHit = 1;
		}
	}
	if ( didHit )
	{
		c->fastSim->flags |= O_HAD_TOI;
		c->fraction = hitFraction;
	}
	return 1;
}

static b2AABB o_offsetAABB( b2AABB box, b2Vec2 origin )
{
	b2AABB r;
	r.lowerBound.x = (float)( origin.x + (double)box.lowerBound.x );
	r.lowerBound.y = (float)( origin.y + (double)box.lowerBound.y );
	r.upperBound.x = (float)( origin.x + (double)box.upperBound.x );
	r.upperBound.y = (float)( origin.y + (double)box.upperBound.y );
	return r;
}

/* b2SolveContinuous (solver.c:384-550) for a fast non-bullet body */
void o_solveContinuous( o_world* w, int simIndex )
{
	o_bodySim* fastSim = w->awakeSims.data + simIndex;
	if ( fastSim->flags & O_IS_BULLET )
	{
		/* bullets sweep against dynamic bodies too: not part of this path */
		fastSim->center0 = fastSim->center;
		fastSim->rotation0 = fastSim->transform.q;
		__atomic_fetch_add( &o_continuousSkipped, 1, __ATOMIC_RELAXED );
		return;
	}
	__atomic_fetch_add( &w->continuousSweeps, 1, __ATOMIC_RELAXED );
	b2Vec2 base = fastSim->center0;
	o_continuousContext c;
	memset( &c, 0, sizeof( c ) );
	c.w = w;
	c.fastSim = fastSim;
	c.sweep = o_relativeSweep( fastSim, base );
	c.base = base;
	c.fraction = 1.0f;
	b2Transform xf2;
	xf2.q = c.sweep.q2;
	xf2.p = o_sub( c.sweep.c2, o_rotate( c.sweep.q2, c.sweep.localCenter ) );
	o_body* fastBody = w->bodies.data + fastSim->bodyId;
	int shapeId = fastBody->headShapeId;
	while ( shapeId != B2_NULL_INDEX )
	{
		o_shape* fastShape = w->shapes.data + shapeId;
		shapeId = fastShape->nextShapeId;
		c.fastShape = fastShape;
		b2AABB box1 = fastShape->aabb;
		b2AABB box2 = o_offsetAABB( o_computeFatShapeAABB( fastShape, xf2, 0.0f ), base );
		fastShape->aabb = box2;
		if ( fastShape->isSensor ) continue;
		b2AABB sweptBox = o_aabbUnion( box1, box2 );
		o_treeQuery( w->trees + b2_staticBody, sweptBox, B2_DEFAULT_MASK_BITS, o_continuousQuery, &c );
	}
	if ( c.fraction < 1.0f )
	{
		__atomic_fetch_add( &w->continuousHits, 1, __ATOMIC_RELAXED );
		b2Rot q = o_nlerp( c.sweep.q1, c.sweep.q2, c.fraction );
		b2Vec2 cc = o_lerp( c.sweep.c1, c.sweep.c2, c.fraction );
		b2Vec2 origin = o_sub( cc, o_rotate( q, c.sweep.localCenter ) );
		fastSim->transform.q = q;
		fastSim->transform.p = o_add( base, origin );
		fastSim->center = o_add( base, cc );
		fastSim->rotation0 = q;
		fastSim->center0 = fastSim->center;
		w->moveEvents.data[simIndex].transform = fastSim->transform;
		shapeId = fastBody->headShapeId;
		while ( shapeId != B2_NULL_INDEX )
		{
			o_shape* shape = w->shapes.data + shapeId;
			b2AABB aabb = o_computeFatShapeAABB( shape, fastSim->transform, O_SPECULATIVE_DISTANCE );
			shape->aabb = aabb;
			if ( o_aabbContains( shape->fatAABB, aabb ) == 0 )
			{
				float margin = shape->aabbMargin;
				b2AABB fat = { { aabb.lowerBound.x - margin, aabb.lowerBound.y - margin },
							   { aabb.upperBound.x + margin, aabb.upperBound.y + margin } };
				shape->fatAABB = fat;
				shape->enlargedAABB = 1;
			}
			shapeId = shape->nextShapeId;
		}
	}
	else
	{
		fastSim->rotation0 = fastSim->transform.q;
		fastSim->center0 = fastSim->center;
		shapeId = fastBody->headShapeId;
		while ( shapeId != B2_NULL_INDEX )
		{
			o_shape* shape = w->shapes.data + shapeId;
			if ( o_aabbContains( shape->fatAABB, shape->aabb ) == 0 )
			{
				float margin = shape->aabbMargin;
				b2AABB fat = { { shape->aabb.lowerBound.x - margin, shape->aabb.lowerBound.y - margin },
							   { shape->aabb.upperBound.x + margin, shape->aabb.upperBound.y + margin } };
				shape->fatAABB = fat;
				shape->enlargedAABB = 1;
			}
			shapeId = shape->nextShapeId;
		}
	}
}
