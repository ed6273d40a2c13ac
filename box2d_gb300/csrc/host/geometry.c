/*
 * Geometry helpers of the public API -- hull, polygon construction, mass properties,
 * fat AABBs and shape extents (geometry.c, hull.c, shape.c in the reference). These run
 * at body/shape creation, not per step.
 */
#include "b2g_world.h"

#include <stdio.h>
#include <time.h>

/* math_functions.c:96-136 */
float b2Atan2( float y, float x )
{
	if ( x == 0.0f && y == 0.0f ) return 0.0f;
	float ax = h_abs( x ), ay = h_abs( y );
	float mx = h_max( ay, ax ), mn = h_min( ay, ax );
	float a = mn / mx;
	float s = a * a;
	float c = s * a;
	float q = s * s;
	float r = 0.024840285f * q + 0.18681418f;
	float t = -0.094097948f * q - 0.33213072f;
	r = r * s + t;
	r = r * c + a;
	if ( ay > ax ) r = 1.57079637f - r;
	if ( x < 0 ) r = 3.14159274f - r;
	if ( y < 0 ) r = -r;
	return r;
}

/* math_functions.h:531-545 b2UnwindAngle */
static float h_unwindAngle( float radians )
{
	float x = h_clamp( radians, -1.0e6f, 1.0e6f );
	double twoPi = 2.0f * B2_PI;
	double roundToNearest = 6755399441055744.0;
	double a = x;
	double k = ( a / twoPi + roundToNearest ) - roundToNearest;
	return (float)( a - k * twoPi );
}

/* math_functions.c:142-183 (Bhaskara approximation) */
b2CosSin b2ComputeCosSin( float radians )
{
	float x = h_unwindAngle( radians );
	float pi2 = B2_PI * B2_PI;
	float c;
	if ( x < -0.5f * B2_PI )
	{
		float y = x + B2_PI;
		float y2 = y * y;
		c = -( pi2 - 4.0f * y2 ) / ( pi2 + y2 );
	}
	else if ( x > 0.5f * B2_PI )
	{
		float y = x - B2_PI;
		float y2 = y * y;
		c = -( pi2 - 4.0f * y2 ) / ( pi2 + y2 );
	}
	else
	{
		float y2 = x * x;
		c = ( pi2 - 4.0f * y2 ) / ( pi2 + y2 );
	}
	float s;
	if ( x < 0.0f )
	{
		float y = x + B2_PI;
		s = -16.0f * y * ( B2_PI - y ) / ( 5.0f * pi2 - 4.0f * y * ( B2_PI - y ) );
	}
	else
	{
		s = 16.0f * x * ( B2_PI - x ) / ( 5.0f * pi2 - 4.0f * x * ( B2_PI - x ) );
	}
	float mag = sqrtf( s * s + c * c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	b2CosSin cs = { c * inv, s * inv };
	return cs;
}

b2Rot b2MakeRot( float radians )
{
	b2CosSin cs = b2ComputeCosSin( radians );
	b2Rot q = { cs.cosine, cs.sine };
	return q;
}

uint64_t b2GetTicks( void )
{
	struct timespec ts;
	clock_gettime( CLOCK_MONOTONIC, &ts );
	return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

float b2GetMilliseconds( uint64_t ticks )
{
	return (float)( (double)( b2GetTicks() - ticks ) * 1.0e-6 );
}

/* timer.c:662-671 djb2 */
uint32_t b2Hash( uint32_t hash, const uint8_t* data, int count )
{
	uint32_t result = hash;
	for ( int i = 0; i < count; i++ ) result = ( result << 5 ) + result + data[i];
	return result;
}

/* hull.c quickhull */
static b2Hull h_recurseHull( b2Vec2 p1, b2Vec2 p2, b2Vec2* ps, int count )
{
	b2Hull hull;
	hull.count = 0;
	if ( count == 0 ) return hull;
	b2Vec2 e = h_normalize( h_sub( p2, p1 ) );
	b2Vec2 right[B2_MAX_POLYGON_VERTICES];
	int rightCount = 0;
	int bestIndex = 0;
	float bestDistance = h_cross( h_sub( ps[bestIndex], p1 ), e );
	if ( bestDistance > 0.0f ) right[rightCount++] = ps[bestIndex];
	for ( int i = 1; i < count; ++i )
	{
		float d = h_cross( h_sub( ps[i], p1 ), e );
		if ( d > bestDistance )
		{
			bestIndex = i;
			bestDistance = d;
		}
		if ( d > 0.0f ) right[rightCount++] = ps[i];
	}
	if ( bestDistance < 2.0f * H_LINEAR_SLOP ) return hull;
	b2Vec2 best = ps[bestIndex];
	b2Hull h1 = h_recurseHull( p1, best, right, rightCount );
	b2Hull h2 = h_recurseHull( best, p2, right, rightCount );
	for ( int i = 0; i < h1.count; ++i ) hull.points[hull.count++] = h1.points[i];
	hull.points[hull.count++] = best;
	for ( int i = 0; i < h2.count; ++i ) hull.points[hull.count++] = h2.points[i];
	return hull;
}

b2Hull b2ComputeHull( const b2Vec2* points, int count )
{
	b2Hull hull;
	memset( &hull, 0, sizeof( hull ) );
	if ( count < 3 || count > B2_MAX_POLYGON_VERTICES ) return hull;
	b2AABB aabb = { { FLT_MAX, FLT_MAX }, { -FLT_MAX, -FLT_MAX } };
	b2Vec2 ps[B2_MAX_POLYGON_VERTICES];
	int n = 0;
	const float tolSqr = 16.0f * H_LINEAR_SLOP * H_LINEAR_SLOP;
	for ( int i = 0; i < count; ++i )
	{
		aabb.lowerBound = h_vmin( aabb.lowerBound, points[i] );
		aabb.upperBound = h_vmax( aabb.upperBound, points[i] );
		b2Vec2 vi = points[i];
		int unique = 1;
		for ( int j = 0; j < i; ++j )
		{
			if ( h_distanceSq( vi, points[j] ) < tolSqr )
			{
				unique = 0;
				break;
			}
		}
		if ( unique ) ps[n++] = vi;
	}
	if ( n < 3 ) return hull;
	b2Vec2 c = h_aabbCenter( aabb );
	int f1 = 0;
	float dsq1 = h_distanceSq( c, ps[f1] );
	for ( int i = 1; i < n; ++i )
	{
		float dsq = h_distanceSq( c, ps[i] );
		if ( dsq > dsq1 )
		{
			f1 = i;
			dsq1 = dsq;
		}
	}
	b2Vec2 p1 = ps[f1];
	ps[f1] = ps[n - 1];
	n = n - 1;
	int f2 = 0;
	float dsq2 = h_distanceSq( p1, ps[f2] );
	for ( int i = 1; i < n; ++i )
	{
		float dsq = h_distanceSq( p1, ps[i] );
		if ( dsq > dsq2 )
		{
			f2 = i;
			dsq2 = dsq;
		}
	}
	b2Vec2 p2 = ps[f2];
	ps[f2] = ps[n - 1];
	n = n - 1;
	b2Vec2 right[B2_MAX_POLYGON_VERTICES - 2], left[B2_MAX_POLYGON_VERTICES - 2];
	int rightCount = 0, leftCount = 0;
	b2Vec2 e = h_normalize( h_sub( p2, p1 ) );
	for ( int i = 0; i < n; ++i )
	{
		float d = h_cross( h_sub( ps[i], p1 ), e );
		if ( d >= 2.0f * H_LINEAR_SLOP ) right[rightCount++] = ps[i];
		else if ( d <= -2.0f * H_LINEAR_SLOP ) left[leftCount++] = ps[i];
	}
	b2Hull h1 = h_recurseHull( p1, p2, right, rightCount );
	b2Hull h2 = h_recurseHull( p2, p1, left, leftCount );
	if ( h1.count == 0 && h2.count == 0 ) return hull;
	hull.points[hull.count++] = p1;
	for ( int i = 0; i < h1.count; ++i ) hull.points[hull.count++] = h1.points[i];
	hull.points[hull.count++] = p2;
	for ( int i = 0; i < h2.count; ++i ) hull.points[hull.count++] = h2.points[i];
	int searching = 1;
	while ( searching && hull.count > 2 )
	{
		searching = 0;
		for ( int i = 0; i < hull.count; ++i )
		{
			int i1 = i, i2 = ( i + 1 ) % hull.count, i3 = ( i + 2 ) % hull.count;
			b2Vec2 s1 = hull.points[i1], s2 = hull.points[i2], s3 = hull.points[i3];
			b2Vec2 r = h_normalize( h_sub( s3, s1 ) );
			float d = h_cross( h_sub( s2, s1 ), r );
			if ( d <= 2.0f * H_LINEAR_SLOP )
			{
				for ( int j = i2; j < hull.count - 1; ++j ) hull.points[j] = hull.points[j + 1];
				hull.count -= 1;
				searching = 1;
				break;
			}
		}
	}
	if ( hull.count < 3 ) hull.count = 0;
	return hull;
}

/* geometry.c:20-46 */
static b2Vec2 h_polygonCentroid( const b2Vec2* v, int count )
{
	b2Vec2 center = { 0.0f, 0.0f };
	float area = 0.0f;
	b2Vec2 origin = v[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		b2Vec2 e1 = h_sub( v[i], origin );
		b2Vec2 e2 = h_sub( v[i + 1], origin );
		float a = 0.5f * h_cross( e1, e2 );
		center = h_mulAdd( center, a * inv3, h_add( e1, e2 ) );
		area += a;
	}
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	return h_add( origin, center );
}

b2Polygon b2MakeBox( float hx, float hy )
{
	b2Polygon s;
	memset( &s, 0, sizeof( s ) );
	s.count = 4;
	s.vertices[0] = h_v( -hx, -hy );
	s.vertices[1] = h_v( hx, -hy );
	s.vertices[2] = h_v( hx, hy );
	s.vertices[3] = h_v( -hx, hy );
	s.normals[0] = h_v( 0.0f, -1.0f );
	s.normals[1] = h_v( 1.0f, 0.0f );
	s.normals[2] = h_v( 0.0f, 1.0f );
	s.normals[3] = h_v( -1.0f, 0.0f );
	return s;
}

b2Polygon b2MakeSquare( float h ) { return b2MakeBox( h, h ); }

b2Polygon b2MakeRoundedBox( float hx, float hy, float radius )
{
	b2Polygon s = b2MakeBox( hx, hy );
	s.radius = radius;
	return s;
}

b2Polygon b2MakeOffsetBox( float hx, float hy, b2Vec2 center, b2Rot rotation )
{
	b2Transform xf = { center, rotation };
	b2Polygon s;
	memset( &s, 0, sizeof( s ) );
	s.count = 4;
	s.vertices[0] = h_transformPoint( xf, h_v( -hx, -hy ) );
	s.vertices[1] = h_transformPoint( xf, h_v( hx, -hy ) );
	s.vertices[2] = h_transformPoint( xf, h_v( hx, hy ) );
	s.vertices[3] = h_transformPoint( xf, h_v( -hx, hy ) );
	s.normals[0] = h_rotate( xf.q, h_v( 0.0f, -1.0f ) );
	s.normals[1] = h_rotate( xf.q, h_v( 1.0f, 0.0f ) );
	s.normals[2] = h_rotate( xf.q, h_v( 0.0f, 1.0f ) );
	s.normals[3] = h_rotate( xf.q, h_v( -1.0f, 0.0f ) );
	s.centroid = xf.p;
	return s;
}

static b2Polygon h_makeOffsetRoundedPolygon( const b2Hull* hull, b2Vec2 position, b2Rot rotation, float radius, int transformed )
{
	if ( hull->count < 3 ) return b2MakeSquare( 0.5f );
	b2Transform xf = { position, rotation };
	b2Polygon s;
	memset( &s, 0, sizeof( s ) );
	s.count = hull->count;
	s.radius = radius;
	for ( int i = 0; i < s.count; ++i ) s.vertices[i] = transformed ? h_transformPoint( xf, hull->points[i] ) : hull->points[i];
	for ( int i = 0; i < s.count; ++i )
	{
		int i2 = i + 1 < s.count ? i + 1 : 0;
		b2Vec2 edge = h_sub( s.vertices[i2], s.vertices[i] );
		s.normals[i] = h_normalize( h_crossVS( edge, 1.0f ) );
	}
	s.centroid = h_polygonCentroid( s.vertices, s.count );
	return s;
}

b2Polygon b2MakePolygon( const b2Hull* hull, float radius )
{
	b2Rot q = { 1.0f, 0.0f };
	return h_makeOffsetRoundedPolygon( hull, h_v( 0.0f, 0.0f ), q, radius, 0 );
}

b2Polygon b2MakeOffsetPolygon( const b2Hull* hull, b2Vec2 position, b2Rot rotation )
{
	return h_makeOffsetRoundedPolygon( hull, position, rotation, 0.0f, 1 );
}

/* geometry.c:236-330 */
b2MassData b2ComputeCircleMass( const b2Circle* shape, float density )
{
	float rr = shape->radius * shape->radius;
	b2MassData m;
	m.mass = density * B2_PI * rr;
	m.center = shape->center;
	m.rotationalInertia = m.mass * 0.5f * rr;
	return m;
}

b2MassData b2ComputeCapsuleMass( const b2Capsule* shape, float density )
{
	float radius = shape->radius;
	float rr = radius * radius;
	b2Vec2 p1 = shape->center1, p2 = shape->center2;
	float length = h_length( h_sub( p2, p1 ) );
	float ll = length * length;
	float circleMass = density * ( B2_PI * radius * radius );
	float boxMass = density * ( 2.0f * radius * length );
	b2MassData m;
	m.mass = circleMass + boxMass;
	m.center.x = 0.5f * ( p1.x + p2.x );
	m.center.y = 0.5f * ( p1.y + p2.y );
	float lc = 4.0f * radius / ( 3.0f * B2_PI );
	float h = 0.5f * length;
	float circleInertia = circleMass * ( 0.5f * rr + h * h + 2.0f * h * lc );
	float boxInertia = boxMass * ( 4.0f * rr + ll ) / 12.0f;
	m.rotationalInertia = circleInertia + boxInertia;
	return m;
}

b2MassData b2ComputePolygonMass( const b2Polygon* shape, float density )
{
	if ( shape->count == 1 )
	{
		b2Circle c = { shape->vertices[0], shape->radius };
		return b2ComputeCircleMass( &c, density );
	}
	if ( shape->count == 2 )
	{
		b2Capsule c = { shape->vertices[0], shape->vertices[1], shape->radius };
		return b2ComputeCapsuleMass( &c, density );
	}
	b2Vec2 vertices[B2_MAX_POLYGON_VERTICES];
	memset( vertices, 0, sizeof( vertices ) );
	int count = shape->count;
	float radius = shape->radius;
	if ( radius > 0.0f )
	{
		float sqrt2 = 1.412f;
		for ( int i = 0; i < count; ++i )
		{
			int j = i == 0 ? count - 1 : i - 1;
			b2Vec2 mid = h_normalize( h_add( shape->normals[j], shape->normals[i] ) );
			vertices[i] = h_mulAdd( shape->vertices[i], sqrt2 * radius, mid );
		}
	}
	else
	{
		for ( int i = 0; i < count; ++i ) vertices[i] = shape->vertices[i];
	}
	b2Vec2 center = { 0.0f, 0.0f };
	float area = 0.0f, rotationalInertia = 0.0f;
	b2Vec2 r = vertices[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		b2Vec2 e1 = h_sub( vertices[i], r );
		b2Vec2 e2 = h_sub( vertices[i + 1], r );
		float D = h_cross( e1, e2 );
		float triangleArea = 0.5f * D;
		area += triangleArea;
		center = h_mulAdd( center, triangleArea * inv3, h_add( e1, e2 ) );
		float ex1 = e1.x, ey1 = e1.y, ex2 = e2.x, ey2 = e2.y;
		float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
		float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
		rotationalInertia += ( 0.25f * inv3 * D ) * ( intx2 + inty2 );
	}
	b2MassData m;
	m.mass = density * area;
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	m.center = h_add( r, center );
	m.rotationalInertia = density * rotationalInertia;
	m.rotationalInertia -= m.mass * h_dot( center, center );
	return m;
}

/* geometry.c:400-506: built in double, narrowed to float once */
static b2AABB h_fatBox( double lx, double ly, double ux, double uy, double r )
{
	b2AABB a = { { (float)( lx - r ), (float)( ly - r ) }, { (float)( ux + r ), (float)( uy + r ) } };
	return a;
}

b2AABB h_computeFatShapeAABB( const h_shape* shape, b2Transform xf, float extra )
{
	switch ( shape->type )
	{
		case b2_circleShape:
		{
			b2Vec2 c = h_transformWorldPoint( xf, shape->circle.center );
			double r = (double)shape->circle.radius + (double)extra;
			return h_fatBox( c.x, c.y, c.x, c.y, r );
		}
		case b2_capsuleShape:
		{
			b2Vec2 v1 = h_transformWorldPoint( xf, shape->capsule.center1 );
			b2Vec2 v2 = h_transformWorldPoint( xf, shape->capsule.center2 );
			double r = (double)shape->capsule.radius + (double)extra;
			return h_fatBox( v1.x < v2.x ? v1.x : v2.x, v1.y < v2.y ? v1.y : v2.y, v1.x > v2.x ? v1.x : v2.x,
							 v1.y > v2.y ? v1.y : v2.y, r );
		}
		case b2_polygonShape:
		{
			const b2Polygon* p = &shape->polygon;
			b2Vec2 v = h_transformWorldPoint( xf, p->vertices[0] );
			double lx = v.x, ly = v.y, ux = v.x, uy = v.y;
			for ( int i = 1; i < p->count; ++i )
			{
				v = h_transformWorldPoint( xf, p->vertices[i] );
				lx = v.x < lx ? v.x : lx;
				ly = v.y < ly ? v.y : ly;
				ux = v.x > ux ? v.x : ux;
				uy = v.y > uy ? v.y : uy;
			}
			double r = (double)p->radius + (double)extra;
			return h_fatBox( lx, ly, ux, uy, r );
		}
		case b2_segmentShape:
		case b2_chainSegmentShape:
		{
			const b2Segment* seg = shape->type == b2_segmentShape ? &shape->segment : &shape->chainSegment.segment;
			b2Vec2 v1 = h_transformWorldPoint( xf, seg->point1 );
			b2Vec2 v2 = h_transformWorldPoint( xf, seg->point2 );
			double e = (double)extra;
			return h_fatBox( v1.x < v2.x ? v1.x : v2.x, v1.y < v2.y ? v1.y : v2.y, v1.x > v2.x ? v1.x : v2.x,
							 v1.y > v2.y ? v1.y : v2.y, e );
		}
		default:
		{
			b2AABB z = { { 0, 0 }, { 0, 0 } };
			return z;
		}
	}
}

/* shape.c:705-722 */
b2Vec2 h_getShapeCentroid( const h_shape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape: return h_lerp( s->capsule.center1, s->capsule.center2, 0.5f );
		case b2_circleShape: return s->circle.center;
		case b2_polygonShape: return s->polygon.centroid;
		case b2_segmentShape: return h_lerp( s->segment.point1, s->segment.point2, 0.5f );
		case b2_chainSegmentShape: return h_lerp( s->chainSegment.segment.point1, s->chainSegment.segment.point2, 0.5f );
		default: return h_v( 0.0f, 0.0f );
	}
}

/* shape.c:36-83 */
float h_computeShapeMargin( const h_shape* s )
{
	float margin = 0.0f;
	switch ( s->type )
	{
		case b2_capsuleShape:
			margin = 0.5f * h_distance( s->capsule.center2, s->capsule.center1 ) + s->capsule.radius;
			break;
		case b2_circleShape:
			margin = s->circle.radius;
			break;
		case b2_polygonShape:
		{
			float maxSq = 0.0f;
			for ( int i = 0; i < s->polygon.count; ++i )
				maxSq = h_max( maxSq, h_distanceSq( s->polygon.vertices[i], s->polygon.centroid ) );
			margin = sqrtf( maxSq );
		}
		break;
		case b2_segmentShape:
			margin = 0.5f * h_distance( s->segment.point1, s->segment.point2 );
			break;
		case b2_chainSegmentShape:
			margin = 0.5f * h_distance( s->chainSegment.segment.point1, s->chainSegment.segment.point2 );
			break;
		default:
			return H_AABB_MARGIN;
	}
	return h_min( H_AABB_MARGIN, H_AABB_MARGIN_FRACTION * margin );
}

b2MassData h_computeShapeMass( const h_shape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape: return b2ComputeCapsuleMass( &s->capsule, s->density );
		case b2_circleShape: return b2ComputeCircleMass( &s->circle, s->density );
		case b2_polygonShape: return b2ComputePolygonMass( &s->polygon, s->density );
		default:
		{
			b2MassData z;
			memset( &z, 0, sizeof( z ) );
			return z;
		}
	}
}

/* shape.c:826-895 */
void h_computeShapeExtent( const h_shape* s, b2Vec2 lc, float* minExtent, float* maxExtent )
{
	*minExtent = 0.0f;
	*maxExtent = 0.0f;
	switch ( s->type )
	{
		case b2_capsuleShape:
		{
			float r = s->capsule.radius;
			*minExtent = r;
			b2Vec2 c1 = h_sub( s->capsule.center1, lc ), c2 = h_sub( s->capsule.center2, lc );
			*maxExtent = sqrtf( h_max( h_lengthSq( c1 ), h_lengthSq( c2 ) ) ) + r;
		}
		break;
		case b2_circleShape:
		{
			float r = s->circle.radius;
			*minExtent = r;
			*maxExtent = h_length( h_sub( s->circle.center, lc ) ) + r;
		}
		break;
		case b2_polygonShape:
		{
			const b2Polygon* p = &s->polygon;
			float mn = H_HUGE, maxSq = 0.0f;
			for ( int i = 0; i < p->count; ++i )
			{
				b2Vec2 v = p->vertices[i];
				float planeOffset = h_dot( p->normals[i], h_sub( v, p->centroid ) );
				mn = h_min( mn, planeOffset );
				maxSq = h_max( maxSq, h_lengthSq( h_sub( v, lc ) ) );
			}
			*minExtent = mn + p->radius;
			*maxExtent = sqrtf( maxSq ) + p->radius;
		}
		break;
		case b2_segmentShape:
		{
			b2Vec2 c1 = h_sub( s->segment.point1, lc ), c2 = h_sub( s->segment.point2, lc );
			*maxExtent = sqrtf( h_max( h_lengthSq( c1 ), h_lengthSq( c2 ) ) );
		}
		break;
		case b2_chainSegmentShape:
		{
			b2Vec2 c1 = h_sub( s->chainSegment.segment.point1, lc ), c2 = h_sub( s->chainSegment.segment.point2, lc );
			*maxExtent = sqrtf( h_max( h_lengthSq( c1 ), h_lengthSq( c2 ) ) );
		}
		break;
		default:
			break;
	}
}
