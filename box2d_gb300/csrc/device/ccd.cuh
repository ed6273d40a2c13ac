/*
 * Device continuous collision: the time of impact of a fast body's shape against a static
 * shape by conservative advancement on separating axes (distance.c:953-1430 b2TimeOfImpact)
 * over the GJK distance (distance.c:138-612 b2ShapeDistance), with the reference's
 * operation order. Every loop is bounded (20 distance iterations, 8 push-backs, 50 root
 * iterations). Used by the finalize kernel for fast non-bullet bodies (solver.c:384-550).
 */
#pragma once

#include "math.cuh"

#define D_CORE_FRACTION 0.25f

typedef struct d_proxy
{
	b2Vec2 points[B2_MAX_POLYGON_VERTICES];
	int count;
	float radius;
} d_proxy;

typedef struct d_sweep
{
	b2Vec2 localCenter, c1, c2;
	b2Rot q1, q2;
} d_sweep;

typedef struct d_simplexVertex
{
	b2Vec2 wA, wB, w;
	float a;
	int indexA, indexB;
} d_simplexVertex;

typedef struct d_simplex
{
	d_simplexVertex v[3];
	int count;
} d_simplex;

typedef struct d_simplexCache
{
	int count;
	int indexA[3], indexB[3];
} d_simplexCache;

/* b2MakeShapeDistanceProxy (shape.c:1055-1076) over the device shape record */
static __device__ d_proxy d_shapeProxy( const b2gShape* s )
{
	d_proxy p;
	p.count = 0;
	p.radius = 0.0f;
	switch ( s->type )
	{
		case b2_capsuleShape:
			p.points[0] = s->v[0];
			p.points[1] = s->v[1];
			p.count = 2;
			p.radius = s->radius;
			break;
		case b2_circleShape:
			p.points[0] = s->v[0];
			p.count = 1;
			p.radius = s->radius;
			break;
		case b2_polygonShape:
			for ( int i = 0; i < s->count; ++i ) p.points[i] = s->v[i];
			p.count = s->count;
			p.radius = s->radius;
			break;
		case b2_segmentShape:
		case b2_chainSegmentShape:
			p.points[0] = s->v[0];
			p.points[1] = s->v[1];
			p.count = 2;
			p.radius = 0.0f;
			break;
		default:
			break;
	}
	return p;
}

/* distance.c:14-30 b2GetSweepTransform */
static __device__ b2Transform d_sweepTransform( const d_sweep* sweep, float time )
{
	b2Transform xf;
	xf.p = d_add( d_mulSV( 1.0f - time, sweep->c1 ), d_mulSV( time, sweep->c2 ) );
	b2Rot q = { ( 1.0f - time ) * sweep->q1.c + time * sweep->q2.c, ( 1.0f - time ) * sweep->q1.s + time * sweep->q2.s };
	xf.q = d_normalizeRot( q );
	xf.p = d_sub( xf.p, d_rotate( xf.q, sweep->localCenter ) );
	return xf;
}

static __device__ int d_findSupport( const d_proxy* proxy, b2Vec2 direction )
{
	int bestIndex = 0;
	float bestValue = d_dot( proxy->points[0], direction );
	for ( int i = 1; i < proxy->count; ++i )
	{
		float value = d_dot( proxy->points[i], direction );
		if ( value > bestValue )
		{
			bestIndex = i;
			bestValue = value;
		}
	}
	return bestIndex;
}

static __device__ void d_witnessPoints( const d_simplex* s, b2Vec2* a, b2Vec2* b )
{
	const d_simplexVertex* v = s->v;
	if ( s->count == 1 )
	{
		*a = v[0].wA;
		*b = v[0].wB;
	}
	else if ( s->count == 2 )
	{
		*a = d_v( v[0].a * v[0].wA.x + v[1].a * v[1].wA.x, v[0].a * v[0].wA.y + v[1].a * v[1].wA.y );
		*b = d_v( v[0].a * v[0].wB.x + v[1].a * v[1].wB.x, v[0].a * v[0].wB.y + v[1].a * v[1].wB.y );
	}
	else if ( s->count == 3 )
	{
		*a = d_v( v[0].a * v[0].wA.x + v[1].a * v[1].wA.x + v[2].a * v[2].wA.x,
				  v[0].a * v[0].wA.y + v[1].a * v[1].wA.y + v[2].a * v[2].wA.y );
		*b = *a;
	}
	else
	{
		*a = d_v( 0.0f, 0.0f );
		*b = d_v( 0.0f, 0.0f );
	}
}

/* distance.c:274-307 */
static __device__ b2Vec2 d_solveSimplex2( d_simplex* s )
{
	b2Vec2 w1 = s->v[0].w, w2 = s->v[1].w;
	b2Vec2 e12 = d_sub( w2, w1 );
	float d12_2 = -d_dot( w1, e12 );
	if ( d12_2 <= 0.0f )
	{
		s->v[0].a = 1.0f;
		s->count = 1;
		return d_neg( w1 );
	}
	float d12_1 = d_dot( w2, e12 );
	if ( d12_1 <= 0.0f )
	{
		s->v[1].a = 1.0f;
		s->count = 1;
		s->v[0] = s->v[1];
		return d_neg( w2 );
	}
	float inv_d12 = 1.0f / ( d12_1 + d12_2 );
	s->v[0].a = d12_1 * inv_d12;
	s->v[1].a = d12_2 * inv_d12;
	s->count = 2;
	return d_crossSV( d_cross( d_add( w1, w2 ), e12 ), e12 );
}

/* distance.c:309-419 */
static __device__ b2Vec2 d_solveSimplex3( d_simplex* s )
{
	b2Vec2 w1 = s->v[0].w, w2 = s->v[1].w, w3 = s->v[2].w;
	b2Vec2 e12 = d_sub( w2, w1 );
	float w1e12 = d_dot( w1, e12 ), w2e12 = d_dot( w2, e12 );
	float d12_1 = w2e12, d12_2 = -w1e12;
	b2Vec2 e13 = d_sub( w3, w1 );
	float w1e13 = d_dot( w1, e13 ), w3e13 = d_dot( w3, e13 );
	float d13_1 = w3e13, d13_2 = -w1e13;
	b2Vec2 e23 = d_sub( w3, w2 );
	float w2e23 = d_dot( w2, e23 ), w3e23 = d_dot( w3, e23 );
	float d23_1 = w3e23, d23_2 = -w2e23;
	float n123 = d_cross( e12, e13 );
	float d123_1 = n123 * d_cross( w2, w3 );
	float d123_2 = n123 * d_cross( w3, w1 );
	float d123_3 = n123 * d_cross( w1, w2 );
	if ( d12_2 <= 0.0f && d13_2 <= 0.0f )
	{
		s->v[0].a = 1.0f;
		s->count = 1;
		return d_neg( w1 );
	}
	if ( d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f )
	{
		float inv_d12 = 1.0f / ( d12_1 + d12_2 );
		s->v[0].a = d12_1 * inv_d12;
		s->v[1].a = d12_2 * inv_d12;
		s->count = 2;
		return d_crossSV( d_cross( d_add( w1, w2 ), e12 ), e12 );
	}
	if ( d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f )
	{
		float inv_d13 = 1.0f / ( d13_1 + d13_2 );
		s->v[0].a = d13_1 * inv_d13;
		s->v[2].a = d13_2 * inv_d13;
		s->count = 2;
		s->v[1] = s->v[2];
		return d_crossSV( d_cross( d_add( w1, w3 ), e13 ), e13 );
	}
	if ( d12_1 <= 0.0f && d23_2 <= 0.0f )
	{
		s->v[1].a = 1.0f;
		s->count = 1;
		s->v[0] = s->v[1];
		return d_neg( w2 );
	}
	if ( d13_1 <= 0.0f && d23_1 <= 0.0f )
	{
		s->v[2].a = 1.0f;
		s->count = 1;
		s->v[0] = s->v[2];
		return d_neg( w3 );
	}
	if ( d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f )
	{
		float inv_d23 = 1.0f / ( d23_1 + d23_2 );
		s->v[1].a = d23_1 * inv_d23;
		s->v[2].a = d23_2 * inv_d23;
		s->count = 2;
		s->v[0] = s->v[2];
		return d_crossSV( d_cross( d_add( w2, w3 ), e23 ), e23 );
	}
	float inv_d123 = 1.0f / ( d123_1 + d123_2 + d123_3 );
	s->v[0].a = d123_1 * inv_d123;
	s->v[1].a = d123_2 * inv_d123;
	s->v[2].a = d123_3 * inv_d123;
	s->count = 3;
	return d_v( 0.0f, 0.0f );
}

/* distance.c:424-612 without radii: the distance in the frame of proxy A, with proxy B
   placed by `transform`, and the witness points on both (when pointA is not null); the
   simplex cache is updated */
static __device__ float d_shapeDistanceWitness( const d_proxy* proxyA, const d_proxy* proxyB, b2Transform transform,
												 d_simplexCache* cache, b2Vec2* pointA, b2Vec2* pointB )
{
	d_proxy localB;
	localB.count = proxyB->count;
	localB.radius = proxyB->radius;
	for ( int i = 0; i < localB.count; ++i ) localB.points[i] = d_transformPoint( transform, proxyB->points[i] );
	d_simplex s;
	s.count = cache->count;
	for ( int i = 0; i < s.count; ++i )
	{
		d_simplexVertex* v = s.v + i;
		v->indexA = cache->indexA[i];
		v->indexB = cache->indexB[i];
		v->wA = proxyA->points[v->indexA];
		v->wB = localB.points[v->indexB];
		v->w = d_sub( v->wA, v->wB );
		v->a = -1.0f;
	}
	if ( s.count == 0 )
	{
		d_simplexVertex* v = s.v;
		v->indexA = 0;
		v->indexB = 0;
		v->wA = proxyA->points[0];
		v->wB = localB.points[0];
		v->w = d_sub( v->wA, v->wB );
		v->a = 1.0f;
		s.count = 1;
	}
	int saveA[3], saveB[3];
	int iteration = 0;
	float distance = 0.0f;
	bool overlapped = false;
	while ( iteration < 20 )
	{
		int saveCount = s.count;
		for ( int i = 0; i < saveCount; ++i )
		{
			saveA[i] = s.v[i].indexA;
			saveB[i] = s.v[i].indexB;
		}
		b2Vec2 d = d_v( 0.0f, 0.0f );
		if ( s.count == 1 ) d = d_neg( s.v[0].w );
		else if ( s.count == 2 ) d = d_solveSimplex2( &s );
		else if ( s.count == 3 ) d = d_solveSimplex3( &s );
		if ( s.count == 3 || d_dot( d, d ) < 1000.0f * FLT_MIN )
		{
			overlapped = true;
			break;
		}
		d_simplexVertex* vertex = s.v + s.count;
		vertex->indexA = d_findSupport( proxyA, d );
		vertex->wA = proxyA->points[vertex->indexA];
		vertex->indexB = d_findSupport( &localB, d_neg( d ) );
		vertex->wB = localB.points[vertex->indexB];
		vertex->w = d_sub( vertex->wA, vertex->wB );
		++iteration;
		bool duplicate = false;
		for ( int i = 0; i < saveCount; ++i )
		{
			if ( vertex->indexA == saveA[i] && vertex->indexB == saveB[i] )
			{
				duplicate = true;
				break;
			}
		}
		if ( duplicate ) break;
		s.count += 1;
	}
	if ( overlapped == false || pointA != nullptr )
	{
		b2Vec2 wA, wB;
		d_witnessPoints( &s, &wA, &wB );
		if ( overlapped == false ) distance = d_distance( wA, wB );
		if ( pointA != nullptr )
		{
			*pointA = wA;
			*pointB = wB;
		}
	}
	cache->count = s.count;
	for ( int i = 0; i < s.count; ++i )
	{
		cache->indexA[i] = s.v[i].indexA;
		cache->indexB[i] = s.v[i].indexB;
	}
	return distance;
}

static __device__ float d_shapeDistance( const d_proxy* proxyA, const d_proxy* proxyB, b2Transform transform, d_simplexCache* cache )
{
	return d_shapeDistanceWitness( proxyA, proxyB, transform, cache, nullptr, nullptr );
}

enum
{
	D_SEP_POINTS = 0,
	D_SEP_FACE_A = 1,
	D_SEP_FACE_B = 2,
};

typedef struct d_separation
{
	const d_proxy *proxyA, *proxyB;
	d_sweep sweepA, sweepB;
	b2Vec2 localPoint, axis;
	int type;
} d_separation;

/* distance.c:953-1027 b2MakeSeparationFunction */
static __device__ d_separation d_makeSeparation( const d_simplexCache* cache, const d_proxy* proxyA, const d_sweep* sweepA,
												 const d_proxy* proxyB, const d_sweep* sweepB, float t1 )
{
	d_separation f;
	f.proxyA = proxyA;
	f.proxyB = proxyB;
	f.sweepA = *sweepA;
	f.sweepB = *sweepB;
	b2Transform xfA = d_sweepTransform( sweepA, t1 );
	b2Transform xfB = d_sweepTransform( sweepB, t1 );
	if ( cache->count == 1 )
	{
		f.type = D_SEP_POINTS;
		b2Vec2 pointA = d_transformPoint( xfA, proxyA->points[cache->indexA[0]] );
		b2Vec2 pointB = d_transformPoint( xfB, proxyB->points[cache->indexB[0]] );
		f.axis = d_normalize( d_sub( pointB, pointA ) );
		f.localPoint = d_v( 0.0f, 0.0f );
		return f;
	}
	if ( cache->indexA[0] == cache->indexA[1] )
	{
		f.type = D_SEP_FACE_B;
		b2Vec2 b1 = proxyB->points[cache->indexB[0]];
		b2Vec2 b2 = proxyB->points[cache->indexB[1]];
		f.axis = d_normalize( d_crossVS( d_sub( b2, b1 ), 1.0f ) );
		b2Vec2 normal = d_rotate( xfB.q, f.axis );
		f.localPoint = d_v( 0.5f * ( b1.x + b2.x ), 0.5f * ( b1.y + b2.y ) );
		b2Vec2 pointB = d_transformPoint( xfB, f.localPoint );
		b2Vec2 pointA = d_transformPoint( xfA, proxyA->points[cache->indexA[0]] );
		float s = d_dot( d_sub( pointA, pointB ), normal );
		if ( s < 0.0f ) f.axis = d_neg( f.axis );
		return f;
	}
	f.type = D_SEP_FACE_A;
	b2Vec2 a1 = proxyA->points[cache->indexA[0]];
	b2Vec2 a2 = proxyA->points[cache->indexA[1]];
	f.axis = d_normalize( d_crossVS( d_sub( a2, a1 ), 1.0f ) );
	b2Vec2 normal = d_rotate( xfA.q, f.axis );
	f.localPoint = d_v( 0.5f * ( a1.x + a2.x ), 0.5f * ( a1.y + a2.y ) );
	b2Vec2 pointA = d_transformPoint( xfA, f.localPoint );
	b2Vec2 pointB = d_transformPoint( xfB, proxyB->points[cache->indexB[0]] );
	float s = d_dot( d_sub( pointB, pointA ), normal );
	if ( s < 0.0f ) f.axis = d_neg( f.axis );
	return f;
}

/* distance.c:1029-1095 b2FindMinSeparation */
static __device__ float d_findMinSeparation( const d_separation* f, int* indexA, int* indexB, float t )
{
	b2Transform xfA = d_sweepTransform( &f->sweepA, t );
	b2Transform xfB = d_sweepTransform( &f->sweepB, t );
	if ( f->type == D_SEP_POINTS )
	{
		b2Vec2 axisA = d_invRotate( xfA.q, f->axis );
		b2Vec2 axisB = d_invRotate( xfB.q, d_neg( f->axis ) );
		*indexA = d_findSupport( f->proxyA, axisA );
		*indexB = d_findSupport( f->proxyB, axisB );
		b2Vec2 pointA = d_transformPoint( xfA, f->proxyA->points[*indexA] );
		b2Vec2 pointB = d_transformPoint( xfB, f->proxyB->points[*indexB] );
		return d_dot( d_sub( pointB, pointA ), f->axis );
	}
	if ( f->type == D_SEP_FACE_A )
	{
		b2Vec2 normal = d_rotate( xfA.q, f->axis );
		b2Vec2 pointA = d_transformPoint( xfA, f->localPoint );
		b2Vec2 axisB = d_invRotate( xfB.q, d_neg( normal ) );
		*indexA = -1;
		*indexB = d_findSupport( f->proxyB, axisB );
		b2Vec2 pointB = d_transformPoint( xfB, f->proxyB->points[*indexB] );
		return d_dot( d_sub( pointB, pointA ), normal );
	}
	b2Vec2 normal = d_rotate( xfB.q, f->axis );
	b2Vec2 pointB = d_transformPoint( xfB, f->localPoint );
	b2Vec2 axisA = d_invRotate( xfA.q, d_neg( normal ) );
	*indexB = -1;
	*indexA = d_findSupport( f->proxyA, axisA );
	b2Vec2 pointA = d_transformPoint( xfA, f->proxyA->points[*indexA] );
	return d_dot( d_sub( pointA, pointB ), normal );
}

/* distance.c:1097-1145 b2EvaluateSeparation */
static __device__ float d_evaluateSeparation( const d_separation* f, int indexA, int indexB, float t )
{
	b2Transform xfA = d_sweepTransform( &f->sweepA, t );
	b2Transform xfB = d_sweepTransform( &f->sweepB, t );
	if ( f->type == D_SEP_POINTS )
	{
		b2Vec2 pointA = d_transformPoint( xfA, f->proxyA->points[indexA] );
		b2Vec2 pointB = d_transformPoint( xfB, f->proxyB->points[indexB] );
		return d_dot( d_sub( pointB, pointA ), f->axis );
	}
	if ( f->type == D_SEP_FACE_A )
	{
		b2Vec2 normal = d_rotate( xfA.q, f->axis );
		b2Vec2 pointA = d_transformPoint( xfA, f->localPoint );
		b2Vec2 pointB = d_transformPoint( xfB, f->proxyB->points[indexB] );
		return d_dot( d_sub( pointB, pointA ), normal );
	}
	b2Vec2 normal = d_rotate( xfB.q, f->axis );
	b2Vec2 pointB = d_transformPoint( xfB, f->localPoint );
	b2Vec2 pointA = d_transformPoint( xfA, f->proxyA->points[indexA] );
	return d_dot( d_sub( pointA, pointB ), normal );
}

/* distance.c:1148-1430 b2TimeOfImpact; only the fraction is used by the step */
static __device__ float d_timeOfImpact( const d_proxy* proxyA, const d_sweep* sweepA, const d_proxy* proxyB, const d_sweep* sweepB,
										float maxFraction )
{
	float fraction = maxFraction;
	float tMax = maxFraction;
	float totalRadius = proxyA->radius + proxyB->radius;
	float target = d_max( D_LINEAR_SLOP, totalRadius - D_LINEAR_SLOP );
	float tolerance = 0.25f * D_LINEAR_SLOP;
	float t1 = 0.0f;
	int distanceIterations = 0;
	d_simplexCache cache;
	cache.count = 0;
	for ( ;; )
	{
		b2Transform xfA = d_sweepTransform( sweepA, t1 );
		b2Transform xfB = d_sweepTransform( sweepB, t1 );
		float distance = d_shapeDistance( proxyA, proxyB, d_invMulTransforms( xfA, xfB ), &cache );
		distanceIterations += 1;
		if ( distance <= 0.0f )
		{
			fraction = 0.0f; /* overlapped */
			break;
		}
		if ( distance <= target + tolerance )
		{
			fraction = t1; /* hit */
			break;
		}
		d_separation fcn = d_makeSeparation( &cache, proxyA, sweepA, proxyB, sweepB, t1 );
		bool done = false;
		float t2 = tMax;
		int pushBackIterations = 0;
		for ( ;; )
		{
			int indexA, indexB;
			float s2 = d_findMinSeparation( &fcn, &indexA, &indexB, t2 );
			if ( s2 > target + tolerance )
			{
				fraction = tMax; /* separated */
				done = true;
				break;
			}
			if ( s2 > target - tolerance )
			{
				t1 = t2;
				break;
			}
			float s1 = d_evaluateSeparation( &fcn, indexA, indexB, t1 );
			if ( s1 < target - tolerance )
			{
				fraction = t1; /* failed */
				done = true;
				break;
			}
			if ( s1 <= target + tolerance )
			{
				fraction = t1; /* hit */
				done = true;
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
				float s = d_evaluateSeparation( &fcn, indexA, indexB, t );
				if ( d_abs( s - target ) < tolerance )
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
		if ( distanceIterations == 20 )
		{
			fraction = t1; /* failed */
			break;
		}
	}
	return fraction;
}

/* body.h:237-247 b2MakeRelativeSweep */
static __device__ d_sweep d_relativeSweep( b2Vec2 center0, b2Rot q0, b2Vec2 center, b2Rot q, b2Vec2 localCenter, b2Vec2 base )
{
	d_sweep s;
	s.c1 = d_sub( center0, base );
	s.c2 = d_sub( center, base );
	s.q1 = q0;
	s.q2 = q;
	s.localCenter = localCenter;
	return s;
}

/* b2OffsetAABB: the box lifted by `origin`, each bound rounded once from double */
static __device__ float4 d_offsetAABB( float4 box, b2Vec2 origin )
{
	return make_float4( __double2float_rn( __dadd_rn( (double)origin.x, (double)box.x ) ),
						__double2float_rn( __dadd_rn( (double)origin.y, (double)box.y ) ),
						__double2float_rn( __dadd_rn( (double)origin.x, (double)box.z ) ),
						__double2float_rn( __dadd_rn( (double)origin.y, (double)box.w ) ) );
}

#define D_CCD_STACK 128

/* what the continuous sweep of one fast body reads */
struct d_ccdWorld
{
	const b2gTreeNode* staticTree;
	int staticRoot;
	/* for bullets (solver.c:443-447): the kinematic and dynamic trees after this step's
	   enlargement, or null */
	const b2gTreeNode* kinematicTree;
	int kinematicRoot;
	const b2gTreeNode* dynamicTree;
	int dynamicRoot;
	const b2gShape* shapes;
	const float4* xf;
	const float2* center;
	const float2* localCenter;
	const uint32_t* bodyFlags;
	const int* partnerOffsets; /* per body: joint partners that must not collide (NULL: none) */
	const int* partnerList;
	/* sensors hit by the sweeps: (sensor shape, visitor shape), counted in *sensorHitCount */
	int2* sensorHits;
	int sensorHitCap;
	int* sensorHitCount;
};

#define D_MAX_SENSOR_HITS 8

/* solver.c:164-177: the sensors one fast body's sweep hits, with their fractions */
struct d_sensorHits
{
	int sensor[D_MAX_SENSOR_HITS], visitor[D_MAX_SENSOR_HITS];
	float fraction[D_MAX_SENSOR_HITS];
	int count;
};

/* shape.c b2ShouldShapesCollide */
static __device__ bool d_shouldShapesCollide( const b2gShape* a, const b2gShape* b )
{
	if ( a->groupIndex == b->groupIndex && a->groupIndex != 0 ) return a->groupIndex > 0;
	return ( a->maskBits & b->categoryBits ) != 0 && ( a->categoryBits & b->maskBits ) != 0;
}

/* body.c:2076-2112 b2ShouldBodiesCollide for a dynamic body: false when a joint that does
   not collide its bodies connects the two */
static __device__ bool d_jointAllowsCollision( const d_ccdWorld& cw, int bodyA, int bodyB )
{
	if ( cw.partnerOffsets == nullptr ) return true;
	int end = cw.partnerOffsets[bodyA + 1];
	for ( int k = cw.partnerOffsets[bodyA]; k < end; ++k )
		if ( cw.partnerList[k] == bodyB ) return false;
	return true;
}

/* the fast shape's centroid at the sweep's start and end (in the base frame) and the core
   distance (B2_CORE_FRACTION of the fast body's minimum extent) */
struct d_fastShape
{
	b2Vec2 centroid1, centroid2;
	float coreDistance;
};

/* solver.c:183-376 b2ContinuousQueryCallback for one static candidate; returns the new
   fraction (unchanged when there is no hit) */
static __device__ float d_continuousCandidate( const d_ccdWorld& cw, int shapeId, int fastShapeId, const b2gShape* fastShape,
											   const d_sweep& fastSweep, b2Vec2 base, float fraction, bool* hit,
											   const d_fastShape& fast, d_sensorHits* hits )
{
	if ( shapeId == fastShapeId ) return fraction;
	const b2gShape* shape = cw.shapes + shapeId;
	if ( shape->bodyId == fastShape->bodyId ) return fraction;
	/* a sensor is swept only for its events, when both shapes want them */
	bool isSensor = shape->isSensor != 0;
	if ( isSensor && ( shape->enableSensorEvents == 0 || fastShape->enableSensorEvents == 0 ) ) return fraction;
	if ( d_shouldShapesCollide( fastShape, shape ) == false ) return fraction;
	int bodyId = shape->bodyId;
	if ( cw.bodyFlags[bodyId] & B2G_IS_BULLET ) return fraction;
	if ( d_jointAllowsCollision( cw, fastShape->bodyId, bodyId ) == false ) return fraction;
	if ( shape->type == b2_chainSegmentShape )
	{
		/* solver.c:258-281: early out on fast movement parallel to, or from behind, a chain */
		float4 xb = cw.xf[bodyId];
		b2Transform transform = { { xb.x - base.x, xb.y - base.y }, { xb.z, xb.w } };
		b2Vec2 p1 = d_transformPoint( transform, shape->v[0] );
		b2Vec2 p2 = d_transformPoint( transform, shape->v[1] );
		float length;
		b2Vec2 e = d_getLengthAndNormalize( &length, d_sub( p2, p1 ) );
		if ( length > D_LINEAR_SLOP )
		{
			float separation1 = d_cross( d_sub( fast.centroid1, p1 ), e );
			float separation2 = d_cross( d_sub( fast.centroid2, p1 ), e );
			if ( separation1 < 0.0f || ( separation1 - separation2 < fast.coreDistance && separation2 > fast.coreDistance ) )
				return fraction;
		}
	}
	d_proxy proxyA = d_shapeProxy( shape );
	d_proxy proxyB = d_shapeProxy( fastShape );
	/* the candidate's sweep is at rest: a static body's, and (for bullets) a kinematic or
	   non-bullet dynamic body's, whose center0 and rotation0 the finalize set to its pose */
	float2 c = cw.center[bodyId];
	float4 x = cw.xf[bodyId];
	float2 lc = cw.localCenter[bodyId];
	b2Rot q = { x.z, x.w };
	d_sweep sweepA = d_relativeSweep( d_v( c.x, c.y ), q, d_v( c.x, c.y ), q, d_v( lc.x, lc.y ), base );
	float f = d_timeOfImpact( &proxyA, &sweepA, &proxyB, &fastSweep, fraction );
	if ( isSensor )
	{
		/* solver.c:319-335: a sensor hit no later than the solid hit so far; it never
		   moves the body */
		if ( f <= fraction && hits->count < D_MAX_SENSOR_HITS )
		{
			hits->sensor[hits->count] = shapeId;
			hits->visitor[hits->count] = fastShapeId;
			hits->fraction[hits->count] = f;
			hits->count += 1;
		}
		return fraction;
	}
	if ( 0.0f < f && f < fraction )
	{
		*hit = true;
		return f;
	}
	if ( 0.0f == f )
	{
		/* fall back to a small circle around the fast shape's centroid */
		proxyB.points[0] = fastShape->ccdCentroid;
		proxyB.count = 1;
		proxyB.radius = fastShape->ccdCoreRadius;
		f = d_timeOfImpact( &proxyA, &sweepA, &proxyB, &fastSweep, fraction );
		if ( 0.0f < f && f < fraction )
		{
			*hit = true;
			return f;
		}
	}
	return fraction;
}

/* dynamic_tree.c b2DynamicTree_Query over one tree with the swept box, visiting
   overlapping leaves in the reference's order (children pushed child1 then child2) */
static __device__ float d_continuousQuery( const d_ccdWorld& cw, const b2gTreeNode* tree, int root, float4 box, int fastShapeId,
										   const b2gShape* fastShape, const d_sweep& fastSweep, b2Vec2 base, float fraction,
										   bool* hit, bool* overflow, const d_fastShape& fast, d_sensorHits* hits )
{
	if ( tree == nullptr || root < 0 ) return fraction;
	int2 stack[D_CCD_STACK];
	int sp = 0;
	{
		const b2gTreeNode r = tree[root];
		if ( d_overlaps( r.aabb, box ) == false || r.categoryNonZero == 0 ) return fraction;
		stack[sp++] = r.isLeaf ? make_int2( ~root, r.child1 ) : make_int2( r.child1, r.child2 );
	}
	while ( sp > 0 )
	{
		int2 e = stack[--sp];
		if ( e.x < 0 )
		{
			fraction = d_continuousCandidate( cw, e.y, fastShapeId, fastShape, fastSweep, base, fraction, hit, fast, hits );
			continue;
		}
		const b2gTreeNode c1 = tree[e.x];
		const b2gTreeNode c2 = tree[e.y];
		bool hit1 = d_overlaps( c1.aabb, box ) && c1.categoryNonZero != 0;
		bool hit2 = d_overlaps( c2.aabb, box ) && c2.categoryNonZero != 0;
		if ( sp + 2 > D_CCD_STACK )
		{
			*overflow = true;
			break;
		}
		if ( hit1 ) stack[sp++] = c1.isLeaf ? make_int2( ~e.x, c1.child1 ) : make_int2( c1.child1, c1.child2 );
		if ( hit2 ) stack[sp++] = c2.isLeaf ? make_int2( ~e.y, c2.child1 ) : make_int2( c2.child1, c2.child2 );
	}
	return fraction;
}
