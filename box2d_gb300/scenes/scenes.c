/*
 * Scene builders for the benchmark configurations and parity tests, written only
 * against the public Box2D C API. The same file is compiled against three libraries:
 * the GB300 library (box2d_gb300.h), the CPU oracle, and -- in the development
 * container only -- the reference itself, so one scene definition drives all three.
 *
 * Random numbers: XorShift32 with seed 12345 mapped to [0, 32767], the generator of
 * shared/utils.h:29-65 in the reference; normal variates from sums of that stream's draws.
 * Every draw is its own statement: C leaves the evaluation order of function arguments
 * and initializer lists unspecified, and gcc orders them differently on x86-64 and
 * aarch64, which would build different worlds on the two machines.
 *
 * Exported entry points (prefix b2s_) keep a small table of live scenes and read body
 * state through b2Body_* getters, so they never touch library internals.
 */
#ifdef B2S_REFERENCE_HEADERS
#include "box2d/box2d.h"
#else
#include "box2d_gb300.h"
#endif

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define B2S_EXPORT __attribute__( ( visibility( "default" ) ) )

typedef struct b2sRng
{
	uint32_t state;
} b2sRng;

static int b2sRandomInt( b2sRng* r )
{
	uint32_t x = r->state;
	x ^= x << 13;
	x ^= x >> 17;
	x ^= x << 5;
	r->state = x;
	return (int)( x % ( 32767 + 1 ) );
}

static float b2sRandomFloatRange( b2sRng* r, float lo, float hi )
{
	float v = (float)( b2sRandomInt( r ) & 32767 );
	v /= 32767;
	v = ( hi - lo ) * v + lo;
	return v;
}

static int b2sRandomIntRange( b2sRng* r, int lo, int hi )
{
	return lo + b2sRandomInt( r ) % ( hi - lo + 1 );
}

/* approximately normal variate: Irwin-Hall sum of four uniform draws, centred and scaled
   to unit variance. Plain float arithmetic only, so no libm routine (whose last-bit
   rounding may differ between platforms) can change a scene. */
static float b2sRandomNormal( b2sRng* r, float sigma )
{
	float sum = 0.0f;
	for ( int k = 0; k < 4; ++k )
		sum += b2sRandomFloatRange( r, 0.0f, 1.0f );
	return sigma * ( ( sum - 2.0f ) * 1.7320508f );
}

typedef struct b2sScene
{
	int inUse;
	b2WorldId worldId;
	b2BodyId* bodies;
	int bodyCount, bodyCapacity;
	int dynamicCount;
	float targetX, targetY;
	int flags; /* creation flags: 1 no continuous, 2 no warm starting, 4 no contact recycling (ramp) */
	uint8_t* image;		  /* the last b2s_snapshot image */
	int imageSize;
	b2BodyId* imageBodies; /* the scene's body list when that image was taken */
	int imageBodyCount;
} b2sScene;

#define B2S_MAX_SCENES 4096
static b2sScene b2s_scenes[B2S_MAX_SCENES];

static void b2sAddBody( b2sScene* s, b2BodyId id, int dynamic )
{
	if ( s->bodyCount == s->bodyCapacity )
	{
		s->bodyCapacity = s->bodyCapacity ? 2 * s->bodyCapacity : 256;
		s->bodies = realloc( s->bodies, (size_t)s->bodyCapacity * sizeof( b2BodyId ) );
	}
	s->bodies[s->bodyCount++] = id;
	s->dynamicCount += dynamic;
}

static b2BodyId b2sBody( b2sScene* s, b2BodyType type, float x, float y )
{
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = type;
	bd.position.x = x;
	bd.position.y = y;
	b2BodyId id = b2CreateBody( s->worldId, &bd );
	b2sAddBody( s, id, type == b2_dynamicBody );
	return id;
}

/* Large pyramid (benchmark scene large_pyramid, shared/benchmarks.c:89-131).
   ground 0: b2MakeBox(100, 1) at y = -1 as in the reference scene;
   ground 1: one 200 m static segment at y = 0. */
static void b2sLargePyramid( b2sScene* s, int baseCount, int groundKind )
{
	b2World_EnableSleeping( s->worldId, false );
	{
		b2ShapeDef sd = b2DefaultShapeDef();
		if ( groundKind == 0 )
		{
			b2BodyId g = b2sBody( s, b2_staticBody, 0.0f, -1.0f );
			b2Polygon box = b2MakeBox( 100.0f, 1.0f );
			b2CreatePolygonShape( g, &sd, &box );
		}
		else
		{
			b2BodyId g = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
			b2Segment seg = { { -100.0f, 0.0f }, { 100.0f, 0.0f } };
			b2CreateSegmentShape( g, &sd, &seg );
		}
	}
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	float a = 0.5f;
	b2Polygon box = b2MakeSquare( a );
	float shift = 1.0f * a;
	for ( int i = 0; i < baseCount; ++i )
	{
		float y = ( 2.0f * i + 1.0f ) * shift;
		for ( int j = i; j < baseCount; ++j )
		{
			float x = ( i + 1.0f ) * shift + 2.0f * ( j - i ) * shift - a * baseCount;
			b2BodyId id = b2sBody( s, b2_dynamicBody, x, y );
			b2CreatePolygonShape( id, &sd, &box );
		}
	}
}

/* Many pyramids with rain: a grid of gridN x gridN pyramids of pyramidRows rows of
   0.5 m boxes, 12 m apart; each grid row stands on its own span of one static ground
   body (rows 7 m apart); rainCount circles of radius U(0.1, 0.3) start 30-60 m above the
   top row. */
static void b2sManyPyramidsRain( b2sScene* s, int gridN, int pyramidRows, int rainCount, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	float extent = 0.25f;
	float spacing = 12.0f;
	float rowDelta = 2.0f * extent * pyramidRows + 2.0f;
	float width = spacing * gridN;
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	b2ShapeDef sd = b2DefaultShapeDef();
	for ( int r = 0; r < gridN; ++r )
	{
		float gy = r * rowDelta;
		b2Segment seg = { { -0.5f * width - 2.0f, gy }, { 0.5f * width + 2.0f, gy } };
		b2CreateSegmentShape( ground, &sd, &seg );
	}
	b2Polygon box = b2MakeSquare( extent );
	for ( int r = 0; r < gridN; ++r )
	{
		float baseY = r * rowDelta;
		for ( int c = 0; c < gridN; ++c )
		{
			float centerX = -0.5f * width + ( c + 0.5f ) * spacing;
			for ( int i = 0; i < pyramidRows; ++i )
			{
				float y = ( 2.0f * i + 1.0f ) * extent + baseY;
				for ( int j = i; j < pyramidRows; ++j )
				{
					float x = ( i + 1.0f ) * extent + 2.0f * ( j - i ) * extent + centerX - extent * pyramidRows;
					b2BodyId id = b2sBody( s, b2_dynamicBody, x, y );
					b2CreatePolygonShape( id, &sd, &box );
				}
			}
		}
	}
	float topY = ( gridN - 1 ) * rowDelta + 2.0f * extent * pyramidRows;
	for ( int k = 0; k < rainCount; ++k )
	{
		float x = b2sRandomFloatRange( rng, -0.5f * width, 0.5f * width );
		float y = topY + b2sRandomFloatRange( rng, 30.0f, 60.0f );
		float radius = b2sRandomFloatRange( rng, 0.1f, 0.3f );
		b2BodyId id = b2sBody( s, b2_dynamicBody, x, y );
		b2Circle circle = { { 0.0f, 0.0f }, radius };
		b2CreateCircleShape( id, &sd, &circle );
	}
}

/* Reference many_pyramids (shared/benchmarks.c:157-195): rowCount x columnCount pyramids of
   10 rows of 1 m boxes, 20 stacked ground segments. */
static void b2sManyPyramidsReference( b2sScene* s, int rowCount, int columnCount )
{
	b2World_EnableSleeping( s->worldId, false );
	int baseCount = 10;
	float extent = 0.5f;
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	float groundDeltaY = 2.0f * extent * ( baseCount + 1.0f );
	float groundWidth = 2.0f * extent * columnCount * ( baseCount + 1.0f );
	b2ShapeDef sd = b2DefaultShapeDef();
	float groundY = 0.0f;
	for ( int i = 0; i < rowCount; ++i )
	{
		b2Segment seg = { { -0.5f * groundWidth, groundY }, { 0.5f * groundWidth, groundY } };
		b2CreateSegmentShape( ground, &sd, &seg );
		groundY += groundDeltaY;
	}
	float baseWidth = 2.0f * extent * baseCount;
	float baseY = 0.0f;
	b2Polygon box = b2MakeSquare( extent );
	for ( int i = 0; i < rowCount; ++i )
	{
		for ( int j = 0; j < columnCount; ++j )
		{
			float centerX = -0.5f * groundWidth + j * ( baseWidth + 2.0f * extent ) + 2.0f * extent;
			for ( int r = 0; r < baseCount; ++r )
			{
				float y = ( 2.0f * r + 1.0f ) * extent + baseY;
				for ( int q = r; q < baseCount; ++q )
				{
					float x = ( r + 1.0f ) * extent + 2.0f * ( q - r ) * extent + centerX - 0.5f;
					b2BodyId id = b2sBody( s, b2_dynamicBody, x, y );
					b2CreatePolygonShape( id, &sd, &box );
				}
			}
		}
		baseY += groundDeltaY;
	}
}

/* Joint grid: n x n circles of radius 0.4 joined to the upper and left neighbours by
   revolute joints (shared/benchmarks.c:20-87). pinAll != 0 makes the whole top row static
   (the reference pins 7 bodies of it); grid circles use category 2 / mask ~2 so they do not
   collide with each other. mixedCount shapes (capsule, convex polygon or segment) with
   velocities N(0, 2) are dropped on the grid. */
static void b2sJointGrid( b2sScene* s, int n, int pinAll, int mixedCount, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId* grid = malloc( (size_t)n * n * sizeof( b2BodyId ) );
	int index = 0;
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.filter.categoryBits = 2;
	sd.filter.maskBits = ~(uint64_t)2;
	b2Circle circle = { { 0.0f, 0.0f }, 0.4f };
	b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
	jd.base.drawScale = 0.4f;
	for ( int k = 0; k < n; ++k )
	{
		for ( int i = 0; i < n; ++i )
		{
			int isStatic = pinAll ? ( i == 0 ) : ( k >= n / 2 - 3 && k <= n / 2 + 3 && i == 0 );
			b2BodyId body = b2sBody( s, isStatic ? b2_staticBody : b2_dynamicBody, (float)k, -(float)i );
			b2CreateCircleShape( body, &sd, &circle );
			if ( i > 0 )
			{
				jd.base.bodyIdA = grid[index - 1];
				jd.base.bodyIdB = body;
				jd.base.localFrameA.p.x = 0.0f;
				jd.base.localFrameA.p.y = -0.5f;
				jd.base.localFrameB.p.x = 0.0f;
				jd.base.localFrameB.p.y = 0.5f;
				b2CreateRevoluteJoint( s->worldId, &jd );
			}
			if ( k > 0 )
			{
				jd.base.bodyIdA = grid[index - n];
				jd.base.bodyIdB = body;
				jd.base.localFrameA.p.x = 0.5f;
				jd.base.localFrameA.p.y = 0.0f;
				jd.base.localFrameB.p.x = -0.5f;
				jd.base.localFrameB.p.y = 0.0f;
				b2CreateRevoluteJoint( s->worldId, &jd );
			}
			grid[index++] = body;
		}
	}
	free( grid );
	b2ShapeDef md = b2DefaultShapeDef();
	for ( int m = 0; m < mixedCount; ++m )
	{
		float x = b2sRandomFloatRange( rng, 0.0f, (float)( n - 1 ) );
		float y = b2sRandomFloatRange( rng, 2.0f, 2.0f + 0.3f * (float)n );
		b2BodyId body = b2sBody( s, b2_dynamicBody, x, y );
		int kind = b2sRandomIntRange( rng, 0, 2 );
		if ( kind == 0 )
		{
			float length = b2sRandomFloatRange( rng, 0.5f, 1.5f );
			float radius = b2sRandomFloatRange( rng, 0.1f, 0.25f );
			b2Capsule cap = { { -0.5f * length, 0.0f }, { 0.5f * length, 0.0f }, radius };
			b2CreateCapsuleShape( body, &md, &cap );
		}
		else if ( kind == 1 )
		{
			int count = b2sRandomIntRange( rng, 3, 8 );
			float radius = b2sRandomFloatRange( rng, 0.3f, 0.6f );
			b2Vec2 pts[8];
			for ( int v = 0; v < count; ++v )
			{
				float angle = 2.0f * 3.14159265359f * v / count + b2sRandomFloatRange( rng, -0.2f, 0.2f );
				b2CosSin cs = b2ComputeCosSin( angle );
				pts[v].x = radius * cs.cosine;
				pts[v].y = radius * cs.sine;
			}
			float rounding = b2sRandomFloatRange( rng, 0.0f, 0.05f );
			b2Hull hull = b2ComputeHull( pts, count );
			b2Polygon poly = hull.count >= 3 ? b2MakePolygon( &hull, rounding ) : b2MakeBox( 0.3f, 0.3f );
			b2CreatePolygonShape( body, &md, &poly );
		}
		else
		{
			float length = b2sRandomFloatRange( rng, 0.5f, 1.5f );
			b2Segment seg = { { -0.5f * length, 0.0f }, { 0.5f * length, 0.0f } };
			b2CreateSegmentShape( body, &md, &seg );
		}
		/* one draw per statement: argument and initializer evaluation order is unspecified */
		b2Vec2 v;
		v.x = b2sRandomNormal( rng, 2.0f );
		v.y = b2sRandomNormal( rng, 2.0f );
		b2Body_SetLinearVelocity( body, v );
	}
}

/* One world of the batched configuration: U{10..400} bodies (boxes of half-extent
   U(0.2, 0.8), circles of radius U(0.1, 0.5), capsules), dropped from heights U(1, 20)
   into a static container of three segments, velocities N(0, 1), friction U(0.2, 0.9),
   restitution U(0, 0.3). bodyCount <= 0 draws the count. */
static void b2sBatchWorld( b2sScene* s, int bodyCount, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	if ( bodyCount <= 0 ) bodyCount = b2sRandomIntRange( rng, 10, 400 );
	float halfWidth = 2.0f + 0.1f * (float)bodyCount;
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	b2ShapeDef gd = b2DefaultShapeDef();
	b2Segment floorSeg = { { -halfWidth, 0.0f }, { halfWidth, 0.0f } };
	b2Segment leftSeg = { { -halfWidth, 0.0f }, { -halfWidth, 40.0f } };
	b2Segment rightSeg = { { halfWidth, 0.0f }, { halfWidth, 40.0f } };
	b2CreateSegmentShape( ground, &gd, &floorSeg );
	b2CreateSegmentShape( ground, &gd, &leftSeg );
	b2CreateSegmentShape( ground, &gd, &rightSeg );
	for ( int k = 0; k < bodyCount; ++k )
	{
		float x = b2sRandomFloatRange( rng, -halfWidth + 1.0f, halfWidth - 1.0f );
		float y = b2sRandomFloatRange( rng, 1.0f, 20.0f );
		b2BodyId body = b2sBody( s, b2_dynamicBody, x, y );
		b2ShapeDef sd = b2DefaultShapeDef();
		sd.material.friction = b2sRandomFloatRange( rng, 0.2f, 0.9f );
		sd.material.restitution = b2sRandomFloatRange( rng, 0.0f, 0.3f );
		int kind = b2sRandomIntRange( rng, 0, 2 );
		if ( kind == 0 )
		{
			float h = b2sRandomFloatRange( rng, 0.2f, 0.8f );
			b2Polygon box = b2MakeBox( h, h );
			b2CreatePolygonShape( body, &sd, &box );
		}
		else if ( kind == 1 )
		{
			b2Circle c = { { 0.0f, 0.0f }, b2sRandomFloatRange( rng, 0.1f, 0.5f ) };
			b2CreateCircleShape( body, &sd, &c );
		}
		else
		{
			float hl = b2sRandomFloatRange( rng, 0.1f, 0.5f );
			b2Capsule cap = { { -hl, 0.0f }, { hl, 0.0f }, b2sRandomFloatRange( rng, 0.1f, 0.3f ) };
			b2CreateCapsuleShape( body, &sd, &cap );
		}
		b2Vec2 v;
		v.x = b2sRandomNormal( rng, 1.0f );
		v.y = b2sRandomNormal( rng, 1.0f );
		b2Body_SetLinearVelocity( body, v );
	}
}

/* One world of the differentiable batch: columns x rows boxes of 0.5 m side stacked on a
   static ramp inclined U(10, 30) degrees; initial velocities N(0, 0.5), friction
   U(0.3, 0.8). The target point is drawn from the same stream. */
static void b2sRampWorld( b2sScene* s, int columns, int rows, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	float angle = b2sRandomFloatRange( rng, 10.0f, 30.0f ) * 3.14159265359f / 180.0f;
	b2BodyDef gdef = b2DefaultBodyDef();
	gdef.rotation = b2MakeRot( -angle );
	b2BodyId ground = b2CreateBody( s->worldId, &gdef );
	b2sAddBody( s, ground, 0 );
	b2ShapeDef gd = b2DefaultShapeDef();
	b2Polygon ramp = b2MakeBox( 30.0f, 0.5f );
	if ( s->flags & 64 )
	{
		/* the ramp's top face as a segment: segment-polygon contacts */
		b2Segment top = { { -30.0f, 0.5f }, { 30.0f, 0.5f } };
		b2CreateSegmentShape( ground, &gd, &top );
	}
	else
	{
		b2CreatePolygonShape( ground, &gd, &ramp );
	}
	b2Rot q = b2MakeRot( -angle );
	float h = 0.25f;
	for ( int c = 0; c < columns; ++c )
	{
		for ( int r = 0; r < rows; ++r )
		{
			float lx = -4.0f + 1.0f * c;
			float ly = 0.5f + h + 2.0f * h * r + 0.01f * r;
			b2BodyDef bd = b2DefaultBodyDef();
			bd.type = b2_dynamicBody;
			bd.position.x = q.c * lx - q.s * ly;
			bd.position.y = q.s * lx + q.c * ly;
			bd.rotation = q;
			bd.linearVelocity.x = b2sRandomNormal( rng, 0.5f );
			bd.linearVelocity.y = b2sRandomNormal( rng, 0.5f );
			bd.angularVelocity = b2sRandomNormal( rng, 0.5f );
			bd.enableContactRecycling = ( s->flags & 4 ) == 0;
			b2BodyId body = b2CreateBody( s->worldId, &bd );
			b2sAddBody( s, body, 1 );
			b2ShapeDef sd = b2DefaultShapeDef();
			sd.material.friction = b2sRandomFloatRange( rng, 0.3f, 0.8f );
			b2Polygon box = b2MakeBox( h, h );
			if ( s->flags & 8 )
			{
				/* rounded boxes with rolling resistance (contact.c:553-560 gives their contacts
				   max(rolling resistance) times the larger radius) */
				box = b2MakeRoundedBox( h - 0.05f, h - 0.05f, 0.05f );
				sd.material.rollingResistance = 0.3f;
			}
			if ( ( s->flags & 16 ) && ( c + r ) % 2 == 1 )
			{
				/* every other body a ball: polygon-circle and circle-circle contacts */
				b2Circle ball = { { 0.0f, 0.0f }, h };
				b2CreateCircleShape( body, &sd, &ball );
			}
			else if ( ( s->flags & 32 ) && ( c == 1 || c == columns - 2 ) && r == 0 )
			{
				/* two capsules at the far ends of the bottom row among the boxes:
				   polygon-capsule contacts */
				b2Capsule capsule = { { -0.5f * h, 0.0f }, { 0.5f * h, 0.0f }, 0.5f * h };
				b2CreateCapsuleShape( body, &sd, &capsule );
			}
			else
			{
				b2CreatePolygonShape( body, &sd, &box );
			}
		}
	}
	s->targetX = b2sRandomFloatRange( rng, -10.0f, 10.0f );
	s->targetY = b2sRandomFloatRange( rng, -5.0f, 5.0f );
}

/* A single box dropped on a ground box (test_world.c:19-99, HelloWorld) */
static void b2sHelloWorld( b2sScene* s )
{
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, -10.0f );
	b2Polygon groundBox = b2MakeBox( 50.0f, 10.0f );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2CreatePolygonShape( ground, &gsd, &groundBox );
	b2BodyId body = b2sBody( s, b2_dynamicBody, 0.0f, 4.0f );
	b2Polygon box = b2MakeBox( 1.0f, 1.0f );
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.material.friction = 0.3f;
	b2CreatePolygonShape( body, &sd, &box );
}

/* A mixed bag of every shape pair on a box ground: circles, capsules, boxes and rounded
   polygons falling onto each other and onto segments; used by the manifold parity tests. */
static void b2sShapeZoo( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	b2ShapeDef gd = b2DefaultShapeDef();
	b2Polygon gbox = b2MakeOffsetBox( 20.0f, 0.5f, ( b2Vec2 ){ 0.0f, -0.5f }, b2MakeRot( 0.0f ) );
	b2CreatePolygonShape( ground, &gd, &gbox );
	b2Segment s1 = { { -20.0f, 0.0f }, { -20.0f, 20.0f } };
	b2Segment s2 = { { 20.0f, 0.0f }, { 20.0f, 20.0f } };
	b2CreateSegmentShape( ground, &gd, &s1 );
	b2CreateSegmentShape( ground, &gd, &s2 );
	for ( int k = 0; k < count; ++k )
	{
		float x = b2sRandomFloatRange( rng, -18.0f, 18.0f );
		float y = b2sRandomFloatRange( rng, 1.0f, 15.0f );
		b2BodyDef bd = b2DefaultBodyDef();
		bd.type = b2_dynamicBody;
		bd.position.x = x;
		bd.position.y = y;
		bd.rotation = b2MakeRot( b2sRandomFloatRange( rng, -3.0f, 3.0f ) );
		b2BodyId body = b2CreateBody( s->worldId, &bd );
		b2sAddBody( s, body, 1 );
		b2ShapeDef sd = b2DefaultShapeDef();
		sd.material.friction = b2sRandomFloatRange( rng, 0.1f, 0.9f );
		sd.material.restitution = b2sRandomFloatRange( rng, 0.0f, 0.4f );
		sd.enableContactEvents = ( k & 1 ) == 0; /* begin/end touch events for half the shapes */
		int kind = b2sRandomIntRange( rng, 0, 3 );
		if ( kind == 0 )
		{
			b2Circle c = { { 0.0f, 0.0f }, b2sRandomFloatRange( rng, 0.2f, 0.6f ) };
			b2CreateCircleShape( body, &sd, &c );
		}
		else if ( kind == 1 )
		{
			float hl = b2sRandomFloatRange( rng, 0.2f, 0.7f );
			b2Capsule cap = { { -hl, 0.0f }, { hl, 0.0f }, b2sRandomFloatRange( rng, 0.1f, 0.4f ) };
			b2CreateCapsuleShape( body, &sd, &cap );
		}
		else if ( kind == 2 )
		{
			float hx = b2sRandomFloatRange( rng, 0.2f, 0.8f );
			float hy = b2sRandomFloatRange( rng, 0.2f, 0.8f );
			b2Polygon box = b2MakeBox( hx, hy );
			b2CreatePolygonShape( body, &sd, &box );
		}
		else
		{
			int count = b2sRandomIntRange( rng, 3, 8 );
			float radius = b2sRandomFloatRange( rng, 0.3f, 0.7f );
			b2Vec2 pts[8];
			for ( int v = 0; v < count; ++v )
			{
				float angle = 2.0f * 3.14159265359f * v / count + b2sRandomFloatRange( rng, -0.2f, 0.2f );
				b2CosSin cs = b2ComputeCosSin( angle );
				pts[v].x = radius * cs.cosine;
				pts[v].y = radius * cs.sine;
			}
			b2Hull hull = b2ComputeHull( pts, count );
			b2Polygon poly = hull.count >= 3 ? b2MakePolygon( &hull, b2sRandomFloatRange( rng, 0.0f, 0.1f ) ) : b2MakeBox( 0.4f, 0.4f );
			b2CreatePolygonShape( body, &sd, &poly );
		}
	}
}

/* Joint zoo: `count` copies, 14 m apart, of five mechanisms on one static ground segment --
   a prismatic slider (limits, and a motor or a spring), a welded chain (rigid or soft), a
   two-wheeled cart on wheel joints (spring, limits, motor), a chain of circles on distance
   joints (rigid, spring with limits, motor) and a revolute pendulum (limits, motor, spring)
   -- plus a few boxes dropped onto them. */
static b2JointDef b2sJointBase( b2BodyId a, b2BodyId b, float ax, float ay, float bx, float by )
{
	b2JointDef j;
	memset( &j, 0, sizeof( j ) );
	j.bodyIdA = a;
	j.bodyIdB = b;
	j.localFrameA.p.x = ax;
	j.localFrameA.p.y = ay;
	j.localFrameA.q.c = 1.0f;
	j.localFrameB.p.x = bx;
	j.localFrameB.p.y = by;
	j.localFrameB.q.c = 1.0f;
	j.forceThreshold = FLT_MAX;
	j.torqueThreshold = FLT_MAX;
	j.drawScale = 1.0f;
	return j;
}

/* Motor, pogo, mover and filter joints (motor_joint.c, pogo_joint.c, mover_joint.c,
   joint.c:436-459): per cell a box driven by a motor joint to the ground (velocity control
   in even cells, spring control in odd ones) with a circle dropped on it, a pair of boxes
   with a motor joint as top-down friction, a box held up by a pogo joint, a box walked by
   a mover joint, and two overlapping boxes whose filter joint keeps them from colliding. */
static void b2sJointMix( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	{
		b2ShapeDef sd = b2DefaultShapeDef();
		b2Segment seg = { { -10.0f, 0.0f }, { 12.0f * count + 10.0f, 0.0f } };
		b2CreateSegmentShape( ground, &sd, &seg );
	}
	b2ShapeDef sd = b2DefaultShapeDef();
	for ( int k = 0; k < count; ++k )
	{
		float x0 = 12.0f * k;
		int variant = k % 2;
		{
			float bx = x0 + b2sRandomFloatRange( rng, -0.5f, 0.5f ), by = 3.0f;
			b2BodyId box = b2sBody( s, b2_dynamicBody, bx, by );
			b2Polygon p = b2MakeBox( 0.6f, 0.3f );
			b2CreatePolygonShape( box, &sd, &p );
			b2MotorJointDef jd = b2DefaultMotorJointDef();
			jd.base = b2sJointBase( ground, box, x0, 2.0f, 0.0f, 0.0f );
			if ( variant == 0 )
			{
				jd.linearVelocity.x = b2sRandomFloatRange( rng, -1.0f, 1.0f );
				jd.linearVelocity.y = 0.5f;
				jd.maxVelocityForce = 40.0f;
				jd.angularVelocity = b2sRandomFloatRange( rng, -1.0f, 1.0f );
				jd.maxVelocityTorque = 10.0f;
			}
			else
			{
				jd.linearHertz = 3.0f;
				jd.linearDampingRatio = 0.7f;
				jd.maxSpringForce = 200.0f;
				jd.angularHertz = 2.0f;
				jd.angularDampingRatio = 0.5f;
				jd.maxSpringTorque = 50.0f;
				jd.maxVelocityForce = 2.0f;
			}
			b2CreateMotorJoint( s->worldId, &jd );
			b2BodyId ball = b2sBody( s, b2_dynamicBody, bx + 0.2f, by + 1.5f );
			b2Circle c = { { 0.0f, 0.0f }, 0.25f };
			b2CreateCircleShape( ball, &sd, &c );
		}
		{
			b2BodyId a = b2sBody( s, b2_dynamicBody, x0 + 3.0f, 0.5f );
			b2BodyId b = b2sBody( s, b2_dynamicBody, x0 + 4.5f, 0.5f );
			b2Polygon p = b2MakeBox( 0.5f, 0.5f );
			b2CreatePolygonShape( a, &sd, &p );
			b2CreatePolygonShape( b, &sd, &p );
			b2MotorJointDef jd = b2DefaultMotorJointDef();
			jd.base = b2sJointBase( a, b, 0.0f, 0.0f, 0.0f, 0.0f );
			jd.base.collideConnected = true;
			jd.maxVelocityForce = 5.0f;
			jd.maxVelocityTorque = 2.0f;
			b2CreateMotorJoint( s->worldId, &jd );
			b2Body_SetLinearVelocity( a, ( b2Vec2 ){ 2.0f, 0.0f } );
		}
		{
			b2BodyId mover = b2sBody( s, b2_dynamicBody, x0 + 7.0f, 1.6f );
			b2Polygon p = b2MakeBox( 0.3f, 0.5f );
			b2CreatePolygonShape( mover, &sd, &p );
			b2PogoJointDef jd = b2DefaultPogoJointDef();
			jd.base = b2sJointBase( ground, mover, x0 + 7.0f, 0.0f, 0.0f, -0.5f );
			jd.normal.x = 0.0f;
			jd.normal.y = 1.0f;
			jd.hertz = variant == 0 ? 5.0f : 2.0f;
			jd.dampingRatio = 0.7f;
			jd.restLength = 0.8f;
			jd.maxTensionForce = 20.0f;
			jd.maxCompressionForce = 400.0f;
			b2CreatePogoJoint( s->worldId, &jd );
		}
		{
			b2BodyId walker = b2sBody( s, b2_dynamicBody, x0 + 5.5f, 2.0f );
			b2Polygon p = b2MakeBox( 0.3f, 0.3f );
			b2CreatePolygonShape( walker, &sd, &p );
			b2MoverJointDef jd = b2DefaultMoverJointDef();
			jd.base = b2sJointBase( ground, walker, x0 + 5.5f, 2.0f, 0.0f, 0.0f );
			jd.linearVelocity.x = variant == 0 ? 1.5f : -1.0f;
			jd.linearVelocity.y = 0.0f;
			jd.maxVelocityForce.x = 30.0f;
			jd.maxVelocityForce.y = variant == 0 ? 0.0f : 5.0f;
			b2CreateMoverJoint( s->worldId, &jd );
		}
		{
			b2BodyId a = b2sBody( s, b2_dynamicBody, x0 + 9.5f, 0.5f );
			b2BodyId b = b2sBody( s, b2_dynamicBody, x0 + 9.8f, 0.9f );
			b2Polygon p = b2MakeBox( 0.5f, 0.5f );
			b2CreatePolygonShape( a, &sd, &p );
			b2CreatePolygonShape( b, &sd, &p );
			b2FilterJointDef jd = b2DefaultFilterJointDef();
			jd.base = b2sJointBase( a, b, 0.0f, 0.0f, 0.0f, 0.0f );
			b2CreateFilterJoint( s->worldId, &jd );
		}
	}
}

static void b2sJointZoo( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	{
		b2ShapeDef sd = b2DefaultShapeDef();
		b2Segment seg = { { -10.0f, 0.0f }, { 14.0f * count + 10.0f, 0.0f } };
		b2CreateSegmentShape( ground, &sd, &seg );
	}
	b2ShapeDef sd = b2DefaultShapeDef();
	for ( int k = 0; k < count; ++k )
	{
		float x0 = 14.0f * k;
		int variant = k % 2;
		/* prismatic slider on a tilted axis */
		{
			b2BodyId box = b2sBody( s, b2_dynamicBody, x0, 4.0f );
			b2Polygon p = b2MakeBox( 0.5f, 0.25f );
			b2CreatePolygonShape( box, &sd, &p );
			b2PrismaticJointDef jd = b2DefaultPrismaticJointDef();
			b2JointDef base = b2sJointBase( ground, box, x0, 4.0f, 0.0f, 0.0f );
			float angle = b2sRandomFloatRange( rng, -0.8f, 0.8f );
			base.localFrameA.q = b2MakeRot( angle );
			base.localFrameB.q = b2MakeRot( angle );
			jd.base = base;
			jd.base.constraintHertz = 60.0f;
			jd.base.constraintDampingRatio = 2.0f;
			jd.enableLimit = true;
			jd.lowerTranslation = -2.0f;
			jd.upperTranslation = 2.0f;
			if ( variant == 0 )
			{
				jd.enableMotor = true;
				jd.maxMotorForce = 50.0f;
				jd.motorSpeed = b2sRandomFloatRange( rng, -2.0f, 2.0f );
			}
			else
			{
				jd.enableSpring = true;
				jd.hertz = 2.0f;
				jd.dampingRatio = 0.5f;
				jd.targetTranslation = 0.5f;
			}
			b2CreatePrismaticJoint( s->worldId, &jd );
		}
		/* welded chain hanging from a static anchor */
		{
			b2BodyId prev = ground;
			float px = x0 + 3.0f, py = 6.0f;
			for ( int i = 0; i < 4; ++i )
			{
				b2BodyId link = b2sBody( s, b2_dynamicBody, px + 0.8f * i + 0.4f, py );
				b2Polygon p = b2MakeBox( 0.4f, 0.1f );
				b2CreatePolygonShape( link, &sd, &p );
				b2WeldJointDef jd = b2DefaultWeldJointDef();
				float ax = i == 0 ? px : 0.4f;
				jd.base = b2sJointBase( prev, link, ax, i == 0 ? py : 0.0f, -0.4f, 0.0f );
				jd.base.constraintHertz = 60.0f;
				jd.base.constraintDampingRatio = 2.0f;
				if ( variant == 1 )
				{
					jd.linearHertz = 5.0f;
					jd.angularHertz = 3.0f;
					jd.linearDampingRatio = 0.7f;
					jd.angularDampingRatio = 0.5f;
				}
				b2CreateWeldJoint( s->worldId, &jd );
				prev = link;
			}
		}
		/* cart on two wheel joints */
		{
			float cx = x0 + 8.0f, cy = 1.2f;
			b2BodyId chassis = b2sBody( s, b2_dynamicBody, cx, cy );
			b2Polygon p = b2MakeBox( 1.0f, 0.25f );
			b2CreatePolygonShape( chassis, &sd, &p );
			for ( int wi = 0; wi < 2; ++wi )
			{
				float wx = wi == 0 ? -0.7f : 0.7f;
				b2BodyId wheel = b2sBody( s, b2_dynamicBody, cx + wx, cy - 0.55f );
				b2Circle c = { { 0.0f, 0.0f }, 0.3f };
				b2CreateCircleShape( wheel, &sd, &c );
				b2WheelJointDef jd = b2DefaultWheelJointDef();
				jd.base = b2sJointBase( chassis, wheel, wx, -0.55f, 0.0f, 0.0f );
				jd.base.localFrameA.q = b2MakeRot( 0.5f * B2_PI );
				jd.base.constraintHertz = 60.0f;
				jd.base.constraintDampingRatio = 2.0f;
				jd.enableSpring = true;
				jd.hertz = 4.0f;
				jd.dampingRatio = 0.7f;
				jd.enableLimit = true;
				jd.lowerTranslation = -0.25f;
				jd.upperTranslation = 0.25f;
				jd.enableMotor = wi == 0;
				jd.maxMotorTorque = 10.0f;
				jd.motorSpeed = variant == 0 ? -5.0f : 3.0f;
				b2CreateWheelJoint( s->worldId, &jd );
			}
		}
		/* chain of circles on distance joints */
		{
			b2BodyId prev = ground;
			float px = x0 + 11.0f, py = 8.0f;
			for ( int i = 0; i < 5; ++i )
			{
				b2BodyId bead = b2sBody( s, b2_dynamicBody, px + 0.5f * ( i + 1 ), py );
				b2Circle c = { { 0.0f, 0.0f }, 0.15f };
				b2CreateCircleShape( bead, &sd, &c );
				b2DistanceJointDef jd = b2DefaultDistanceJointDef();
				jd.base = b2sJointBase( prev, bead, i == 0 ? px : 0.0f, i == 0 ? py : 0.0f, 0.0f, 0.0f );
				jd.base.constraintHertz = 60.0f;
				jd.base.constraintDampingRatio = 2.0f;
				jd.length = 0.5f;
				int mode = ( i + k ) % 3;
				if ( mode == 1 )
				{
					jd.enableSpring = true;
					jd.hertz = 3.0f;
					jd.dampingRatio = 0.3f;
					jd.enableLimit = true;
					jd.minLength = 0.3f;
					jd.maxLength = 0.8f;
				}
				else if ( mode == 2 )
				{
					jd.enableSpring = true;
					jd.hertz = 0.0f;
					jd.enableMotor = true;
					jd.maxMotorForce = 5.0f;
					jd.motorSpeed = 0.5f;
					jd.enableLimit = true;
					jd.minLength = 0.2f;
					jd.maxLength = 1.0f;
				}
				b2CreateDistanceJoint( s->worldId, &jd );
				prev = bead;
			}
		}
		/* revolute pendulum */
		{
			b2BodyId arm = b2sBody( s, b2_dynamicBody, x0 + 1.0f, 10.0f );
			b2Polygon p = b2MakeBox( 1.0f, 0.1f );
			b2CreatePolygonShape( arm, &sd, &p );
			b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
			jd.base = b2sJointBase( ground, arm, x0, 10.0f, -1.0f, 0.0f );
			jd.base.constraintHertz = 60.0f;
			jd.base.constraintDampingRatio = 2.0f;
			jd.enableLimit = true;
			jd.lowerAngle = -0.5f * B2_PI;
			jd.upperAngle = 0.25f * B2_PI;
			jd.enableMotor = variant == 0;
			jd.maxMotorTorque = 20.0f;
			jd.motorSpeed = 1.0f;
			jd.enableSpring = variant == 1;
			jd.hertz = 1.0f;
			jd.dampingRatio = 0.2f;
			b2CreateRevoluteJoint( s->worldId, &jd );
		}
		/* boxes dropped onto the mechanisms */
		for ( int i = 0; i < 3; ++i )
		{
			float bx = x0 + b2sRandomFloatRange( rng, 0.0f, 12.0f );
			float by = b2sRandomFloatRange( rng, 12.0f, 16.0f );
			b2BodyId box = b2sBody( s, b2_dynamicBody, bx, by );
			b2Polygon p = b2MakeSquare( 0.3f );
			b2CreatePolygonShape( box, &sd, &p );
		}
	}
}

/* Falling hinges: the scene of the reference's determinism test (shared/determinism.c:11-108,
   test/test_determinism.c): a 40 x 1 ground box, four columns of twenty 0.25 m squares tilted
   by +-0.1 rad, each pair joined by a revolute joint with limit, spring and motor. Sleeping
   stays on: the test runs until every island is asleep. */
static void b2sFallingHinges( b2sScene* s )
{
	{
		b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, -1.0f );
		b2Polygon box = b2MakeBox( 40.0f, 1.0f );
		b2ShapeDef sd = b2DefaultShapeDef();
		b2CreatePolygonShape( ground, &sd, &box );
	}
	const int columnCount = 4, rowCount = 20;
	const float h = 0.25f;
	b2Polygon square = b2MakeSquare( h );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
	jd.enableLimit = true;
	jd.lowerAngle = -0.1f * B2_PI;
	jd.upperAngle = 0.2f * B2_PI;
	jd.enableSpring = true;
	jd.hertz = 1.0f;
	jd.dampingRatio = 1.0f;
	jd.enableMotor = true;
	jd.maxMotorTorque = 0.25f;
	jd.base.localFrameA.p.x = -h;
	jd.base.localFrameA.p.y = h;
	jd.base.localFrameB.p.x = -h;
	jd.base.localFrameB.p.y = -h;
	jd.base.constraintHertz = 60.0f;
	jd.base.constraintDampingRatio = 0.0f;
	jd.base.drawScale = 0.5f;
	float offset = 0.4f * h;
	float dx = 10.0f * h;
	float xBase = -0.5f * dx * ( columnCount - 1.0f );
	for ( int j = 0; j < columnCount; ++j )
	{
		float x = xBase + j * dx;
		b2BodyId prev = { 0 };
		for ( int i = 0; i < rowCount; ++i )
		{
			b2BodyDef bd = b2DefaultBodyDef();
			bd.type = b2_dynamicBody;
			bd.position.x = x + offset * i;
			bd.position.y = h + 2.0f * h * i;
			float angle = ( i & 1 ) == 0 ? -0.1f : 0.1f;
			bd.rotation = b2MakeRot( angle );
			b2BodyId body = b2CreateBody( s->worldId, &bd );
			b2sAddBody( s, body, 1 );
			if ( ( i & 1 ) == 0 )
			{
				prev = body;
			}
			else
			{
				jd.base.bodyIdA = prev;
				jd.base.bodyIdB = body;
				b2CreateRevoluteJoint( s->worldId, &jd );
				prev = ( b2BodyId ){ 0 };
			}
			b2CreatePolygonShape( body, &sd, &square );
		}
	}
}

/* Sleeping pyramids: `a` pyramids of `b` rows (0.5 m boxes on one ground box, sleeping on)
   and one box dropped from height `c` onto the first pyramid after the stacks have gone to
   sleep, which wakes them through a contact that starts touching. */
static void b2sSleepPyramids( b2sScene* s, int pyramidCount, int rows, int dropHeight )
{
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	b2Polygon groundBox = b2MakeOffsetBox( 40.0f, 1.0f, ( b2Vec2 ){ 0.0f, -1.0f }, b2MakeRot( 0.0f ) );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2CreatePolygonShape( ground, &sd, &groundBox );
	b2Polygon box = b2MakeSquare( 0.5f );
	for ( int p = 0; p < pyramidCount; ++p )
	{
		float x0 = -30.0f + 12.0f * p;
		for ( int i = 0; i < rows; ++i )
		{
			for ( int k = 0; k < rows - i; ++k )
			{
				b2BodyId body = b2sBody( s, b2_dynamicBody, x0 + 0.5f * i + 1.0f * k, 0.5f + 1.0f * i );
				b2CreatePolygonShape( body, &sd, &box );
			}
		}
	}
	b2BodyId drop = b2sBody( s, b2_dynamicBody, -30.0f + 0.5f * ( rows - 1 ) + 0.3f, (float)dropHeight );
	b2CreatePolygonShape( drop, &sd, &box );
}

/* Overflow scene: bodies with more constraints than the graph has colors, so the solver's
   overflow path (constraints past the colors, solved one by one before the colors in each
   stage; contact_solver.c:24-545, joint.c:1542-1591) runs. Per cell: a 24 m plank resting
   on the ground under 40 small boxes (40 dynamic-vs-dynamic contacts on one body: the
   first 20 get the 20 dynamic colors, the rest overflow; every other box has restitution),
   and a hub falling with 28 satellites held by distance joints (28 joints on one body). */
static void b2sOverflowScene( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, -1.0f );
	{
		b2ShapeDef sd = b2DefaultShapeDef();
		b2Polygon box = b2MakeOffsetBox( 40.0f * count + 20.0f, 1.0f, ( b2Vec2 ){ 20.0f * count, 0.0f }, b2MakeRot( 0.0f ) );
		b2CreatePolygonShape( ground, &sd, &box );
	}
	for ( int k = 0; k < count; ++k )
	{
		float x0 = 40.0f * k;
		b2ShapeDef sd = b2DefaultShapeDef();
		b2BodyId plank = b2sBody( s, b2_dynamicBody, x0, 0.25f );
		b2Polygon p = b2MakeBox( 12.0f, 0.25f );
		b2CreatePolygonShape( plank, &sd, &p );
		b2Polygon small = b2MakeBox( 0.25f, 0.25f );
		for ( int i = 0; i < 40; ++i )
		{
			float jitter = b2sRandomFloatRange( rng, -0.02f, 0.02f );
			b2BodyId b = b2sBody( s, b2_dynamicBody, x0 - 10.75f + 0.55f * i + jitter, 0.76f );
			b2ShapeDef bs = b2DefaultShapeDef();
			bs.material.restitution = ( i & 1 ) ? 0.3f : 0.0f;
			bs.enableContactEvents = true;
			b2CreatePolygonShape( b, &bs, &small );
		}
		float hx = x0 + b2sRandomFloatRange( rng, -1.0f, 1.0f ), hy = 9.0f;
		b2BodyId hub = b2sBody( s, b2_dynamicBody, hx, hy );
		b2Circle hc = { { 0.0f, 0.0f }, 0.5f };
		b2CreateCircleShape( hub, &sd, &hc );
		for ( int i = 0; i < 28; ++i )
		{
			float angle = 6.2831853f * (float)i / 28.0f + b2sRandomFloatRange( rng, -0.05f, 0.05f );
			b2CosSin cs = b2ComputeCosSin( angle );
			b2BodyId sat = b2sBody( s, b2_dynamicBody, hx + 2.5f * cs.cosine, hy + 2.5f * cs.sine );
			b2Circle c = { { 0.0f, 0.0f }, 0.15f };
			b2CreateCircleShape( sat, &sd, &c );
			b2DistanceJointDef jd = b2DefaultDistanceJointDef();
			jd.base = b2sJointBase( hub, sat, 0.0f, 0.0f, 0.0f, 0.0f );
			jd.length = 2.5f;
			jd.enableSpring = ( i % 3 ) == 0;
			jd.hertz = 4.0f;
			jd.dampingRatio = 0.5f;
			b2CreateDistanceJoint( s->worldId, &jd );
		}
	}
}

/* Sensor scene (sensor.c, shape.c:180-205): static sensor boxes on the floor, a thin static
   sensor gate at 6 m and a static sensor circle in the air, a kinematic body carrying a sensor capsule across the scene, a
   dynamic body whose sensor circle rides on its own solid box (a sensor never sees shapes
   of its own body), a static sensor whose sensor events are off, and `count` falling
   shapes of which two in three report to sensors and every fifth is in a category the
   sensors' mask excludes. Sleeping is off. */
static void b2sSensorZoo( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	b2ShapeDef gd = b2DefaultShapeDef();
	b2Polygon gbox = b2MakeOffsetBox( 20.0f, 0.5f, ( b2Vec2 ){ 0.0f, -0.5f }, b2MakeRot( 0.0f ) );
	b2CreatePolygonShape( ground, &gd, &gbox );
	b2Segment w1 = { { -20.0f, 0.0f }, { -20.0f, 20.0f } };
	b2Segment w2 = { { 20.0f, 0.0f }, { 20.0f, 20.0f } };
	b2CreateSegmentShape( ground, &gd, &w1 );
	b2CreateSegmentShape( ground, &gd, &w2 );
	b2ShapeDef sensorDef = b2DefaultShapeDef();
	sensorDef.isSensor = true;
	sensorDef.enableSensorEvents = true;
	sensorDef.filter.maskBits = ~(uint64_t)4;
	for ( int i = 0; i < 3; ++i )
	{
		b2Polygon zone = b2MakeOffsetBox( 2.0f, 1.0f, ( b2Vec2 ){ -12.0f + 12.0f * i, 1.0f }, b2MakeRot( 0.0f ) );
		b2CreatePolygonShape( ground, &sensorDef, &zone );
	}
	{
		/* a thin gate the falling shapes cross within one step: seen by continuous sweeps */
		b2Polygon gate = b2MakeOffsetBox( 18.0f, 0.02f, ( b2Vec2 ){ 0.0f, 6.0f }, b2MakeRot( 0.0f ) );
		b2CreatePolygonShape( ground, &sensorDef, &gate );
	}
	{
		b2Circle zone = { { 5.0f, 4.0f }, 1.5f };
		b2CreateCircleShape( ground, &sensorDef, &zone );
		b2ShapeDef quiet = sensorDef;
		quiet.enableSensorEvents = false;
		b2Circle silent = { { -5.0f, 4.0f }, 1.5f };
		b2CreateCircleShape( ground, &quiet, &silent );
	}
	{
		b2BodyDef bd = b2DefaultBodyDef();
		bd.type = b2_kinematicBody;
		bd.position.x = -18.0f;
		bd.position.y = 6.0f;
		bd.linearVelocity.x = 1.5f;
		b2BodyId mover = b2CreateBody( s->worldId, &bd );
		b2sAddBody( s, mover, 0 );
		b2Capsule cap = { { -1.0f, 0.0f }, { 1.0f, 0.0f }, 0.5f };
		b2CreateCapsuleShape( mover, &sensorDef, &cap );
	}
	{
		b2BodyId carrier = b2sBody( s, b2_dynamicBody, 0.0f, 9.0f );
		b2ShapeDef solid = b2DefaultShapeDef();
		solid.enableSensorEvents = true;
		b2Polygon box = b2MakeBox( 0.5f, 0.5f );
		b2CreatePolygonShape( carrier, &solid, &box );
		b2Circle ring = { { 0.0f, 0.0f }, 1.2f };
		b2CreateCircleShape( carrier, &sensorDef, &ring );
	}
	for ( int k = 0; k < count; ++k )
	{
		float x = b2sRandomFloatRange( rng, -18.0f, 18.0f );
		float y = b2sRandomFloatRange( rng, 2.0f, 14.0f );
		b2BodyId body = b2sBody( s, b2_dynamicBody, x, y );
		b2ShapeDef sd = b2DefaultShapeDef();
		sd.enableSensorEvents = ( k % 3 ) != 0;
		if ( k % 5 == 4 ) sd.filter.categoryBits = 4;
		int kind = b2sRandomIntRange( rng, 0, 2 );
		if ( kind == 0 )
		{
			b2Circle c = { { 0.0f, 0.0f }, b2sRandomFloatRange( rng, 0.2f, 0.5f ) };
			b2CreateCircleShape( body, &sd, &c );
		}
		else if ( kind == 1 )
		{
			float hx = b2sRandomFloatRange( rng, 0.2f, 0.5f );
			float hy = b2sRandomFloatRange( rng, 0.2f, 0.5f );
			b2Polygon p = b2MakeBox( hx, hy );
			b2CreatePolygonShape( body, &sd, &p );
		}
		else
		{
			float r = b2sRandomFloatRange( rng, 0.15f, 0.3f );
			b2Capsule c = { { -0.3f, 0.0f }, { 0.3f, 0.0f }, r };
			b2CreateCapsuleShape( body, &sd, &c );
		}
	}
}

#ifndef B2S_NO_CHAINS
/* Chain scene (shape.c:439-640, manifold.c:1042-1641): a closed chain forming a container
   with a wavy floor (clockwise, so every segment's one-sided normal points inward), an open
   chain ramp inside it, a loose chain segment shape, and `count` circles, capsules, boxes and
   rounded convex polygons dropped from up to 18 m. Per-segment materials on the floor. */
static void b2sChainZoo( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	{
		enum { floorCount = 31 };
		b2Vec2 pts[floorCount + 3];
		b2SurfaceMaterial mats[floorCount + 3];
		int n = 0;
		for ( int i = 0; i < floorCount; ++i )
		{
			float x = 15.0f - 1.0f * (float)i;
			b2CosSin cs = b2ComputeCosSin( 0.6f * x );
			pts[n].x = x;
			pts[n].y = 0.8f * cs.sine + 1.0f;
			n += 1;
		}
		pts[n].x = -15.0f;
		pts[n].y = 22.0f;
		n += 1;
		pts[n].x = 15.0f;
		pts[n].y = 22.0f;
		n += 1;
		for ( int i = 0; i < n; ++i )
		{
			memset( mats + i, 0, sizeof( b2SurfaceMaterial ) );
			mats[i].friction = ( i % 3 ) == 0 ? 0.2f : 0.7f;
			mats[i].restitution = ( i % 4 ) == 0 ? 0.3f : 0.0f;
		}
		b2ChainDef cd = b2DefaultChainDef();
		cd.points = pts;
		cd.count = n;
		cd.materials = mats;
		cd.materialCount = n;
		cd.isLoop = true;
		b2CreateChain( ground, &cd );
	}
	{
		b2Vec2 ramp[6] = { { 9.0f, 9.0f }, { 7.0f, 8.0f }, { 4.0f, 7.0f }, { 1.0f, 6.5f }, { -2.0f, 6.8f }, { -4.0f, 7.8f } };
		b2ChainDef cd = b2DefaultChainDef();
		cd.points = ramp;
		cd.count = 6;
		b2CreateChain( ground, &cd );
	}
	{
		b2ShapeDef sd = b2DefaultShapeDef();
		b2ChainSegment seg = { { -6.0f, 12.0f }, { { -8.0f, 12.0f }, { -12.0f, 11.0f } }, { -14.0f, 11.0f }, -1 };
		b2CreateChainSegmentShape( ground, &sd, &seg );
	}
	for ( int k = 0; k < count; ++k )
	{
		float x = b2sRandomFloatRange( rng, -13.0f, 13.0f );
		float y = b2sRandomFloatRange( rng, 4.0f, 18.0f );
		b2BodyDef bd = b2DefaultBodyDef();
		bd.type = b2_dynamicBody;
		bd.position.x = x;
		bd.position.y = y;
		bd.rotation = b2MakeRot( b2sRandomFloatRange( rng, -3.0f, 3.0f ) );
		b2BodyId body = b2CreateBody( s->worldId, &bd );
		b2sAddBody( s, body, 1 );
		b2ShapeDef sd = b2DefaultShapeDef();
		sd.material.friction = b2sRandomFloatRange( rng, 0.2f, 0.9f );
		int kind = b2sRandomIntRange( rng, 0, 3 );
		if ( kind == 0 )
		{
			b2Circle c = { { 0.0f, 0.0f }, b2sRandomFloatRange( rng, 0.2f, 0.5f ) };
			b2CreateCircleShape( body, &sd, &c );
		}
		else if ( kind == 1 )
		{
			float half = b2sRandomFloatRange( rng, 0.2f, 0.6f );
			b2Capsule c = { { -half, 0.0f }, { half, 0.0f }, b2sRandomFloatRange( rng, 0.1f, 0.3f ) };
			b2CreateCapsuleShape( body, &sd, &c );
		}
		else if ( kind == 2 )
		{
			float hx = b2sRandomFloatRange( rng, 0.2f, 0.6f );
			float hy = b2sRandomFloatRange( rng, 0.2f, 0.6f );
			b2Polygon p = b2MakeBox( hx, hy );
			b2CreatePolygonShape( body, &sd, &p );
		}
		else
		{
			int nv = b2sRandomIntRange( rng, 3, 7 );
			b2Vec2 pts[8];
			float radius = b2sRandomFloatRange( rng, 0.3f, 0.6f );
			for ( int i = 0; i < nv; ++i )
			{
				float a = 6.2831853f * (float)i / (float)nv;
				b2CosSin cs = b2ComputeCosSin( a );
				pts[i].x = radius * cs.cosine;
				pts[i].y = radius * cs.sine;
			}
			b2Hull hull = b2ComputeHull( pts, nv );
			b2Polygon p = b2MakePolygon( &hull, b2sRandomFloatRange( rng, 0.0f, 0.05f ) );
			b2CreatePolygonShape( body, &sd, &p );
		}
	}
}
#endif

/* Bullet scene (solver.c:1917-1989): a wall of boxes and a stack of thin planks on the
   ground, hit by `count` bullet bodies (small circles and boxes flagged isBullet) fired at
   80-250 m/s from both sides at staggered heights, so that they are swept against dynamic
   bodies as well as static ones. */
static void b2sBulletZoo( b2sScene* s, int count, b2sRng* rng )
{
	b2World_EnableSleeping( s->worldId, false );
	b2BodyId ground = b2sBody( s, b2_staticBody, 0.0f, 0.0f );
	b2ShapeDef gd = b2DefaultShapeDef();
	b2Polygon gbox = b2MakeOffsetBox( 60.0f, 0.5f, ( b2Vec2 ){ 0.0f, -0.5f }, b2MakeRot( 0.0f ) );
	b2CreatePolygonShape( ground, &gd, &gbox );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon brick = b2MakeBox( 0.25f, 0.25f );
	for ( int i = 0; i < 12; ++i )
		for ( int j = 0; j < 4; ++j )
		{
			b2BodyId b = b2sBody( s, b2_dynamicBody, -1.0f + 0.5f * j, 0.25f + 0.5f * i );
			b2CreatePolygonShape( b, &sd, &brick );
		}
	b2Polygon plank = b2MakeBox( 0.05f, 1.0f );
	for ( int k = 0; k < 6; ++k )
	{
		b2BodyId b = b2sBody( s, b2_dynamicBody, 8.0f + 0.4f * k, 1.0f );
		b2CreatePolygonShape( b, &sd, &plank );
	}
	for ( int k = 0; k < count; ++k )
	{
		float side = ( k & 1 ) ? 1.0f : -1.0f;
		b2BodyDef bd = b2DefaultBodyDef();
		bd.type = b2_dynamicBody;
		bd.isBullet = true;
		bd.position.x = side * b2sRandomFloatRange( rng, 20.0f, 40.0f );
		bd.position.y = b2sRandomFloatRange( rng, 0.3f, 5.5f );
		bd.linearVelocity.x = -side * b2sRandomFloatRange( rng, 80.0f, 250.0f );
		bd.linearVelocity.y = b2sRandomFloatRange( rng, -2.0f, 2.0f );
		b2BodyId b = b2CreateBody( s->worldId, &bd );
		b2sAddBody( s, b, 1 );
		b2ShapeDef bs = b2DefaultShapeDef();
		bs.density = 4.0f;
		if ( k % 3 == 0 )
		{
			b2Polygon p = b2MakeBox( 0.08f, 0.08f );
			b2CreatePolygonShape( b, &bs, &p );
		}
		else
		{
			b2Circle c = { { 0.0f, 0.0f }, b2sRandomFloatRange( rng, 0.05f, 0.12f ) };
			b2CreateCircleShape( b, &bs, &c );
		}
	}
}

enum
{
	B2S_LARGE_PYRAMID = 0,
	B2S_MANY_PYRAMIDS_RAIN = 1,
	B2S_JOINT_GRID_MIXED = 2,
	B2S_BATCH_WORLD = 3,
	B2S_RAMP_WORLD = 4,
	B2S_MANY_PYRAMIDS_REF = 5,
	B2S_JOINT_GRID_REF = 6,
	B2S_HELLO_WORLD = 7,
	B2S_SHAPE_ZOO = 8,
	B2S_JOINT_ZOO = 9,
	B2S_FALLING_HINGES = 10,
	B2S_SLEEP_PYRAMIDS = 11,
	B2S_JOINT_MIX = 12,
	B2S_OVERFLOW = 13,
	B2S_SENSOR_ZOO = 14,
	B2S_CHAIN_ZOO = 15,
	B2S_BULLET_ZOO = 16,
};

/* Worker threads requested in the world definition of scenes created from now on (0 keeps
   the default). A library with a built-in task system (the reference: workerCount > 1
   starts its scheduler, physics_world.c:307-314) uses them; the GB300 library ignores it. */
static int b2s_workerCount = 0;

B2S_EXPORT void b2s_set_workers( int count )
{
	b2s_workerCount = count > 0 ? count : 0;
}

/* Create a scene. kind selects the builder; a, b, c are its size parameters; seed feeds
   the random stream (0 means 12345). flags bit 0 disables continuous collision.
   Returns a handle >= 0, or -1 when the scene table is full or the world was refused. */
B2S_EXPORT int b2s_create( int kind, int a, int b, int c, uint32_t seed, int flags )
{
	int h = -1;
	for ( int i = 0; i < B2S_MAX_SCENES; ++i )
	{
		if ( b2s_scenes[i].inUse == 0 )
		{
			h = i;
			break;
		}
	}
	if ( h < 0 ) return -1;
	b2sScene* s = b2s_scenes + h;
	memset( s, 0, sizeof( *s ) );
	b2WorldDef wd = b2DefaultWorldDef();
	if ( b2s_workerCount > 0 ) wd.workerCount = b2s_workerCount;
	if ( flags & 1 ) wd.enableContinuous = false;
	s->worldId = b2CreateWorld( &wd );
	if ( s->worldId.index1 == 0 ) return -1;
	s->inUse = 1;
	s->flags = flags;
	if ( flags & 2 ) b2World_EnableWarmStarting( s->worldId, false );
	b2sRng rng = { seed ? seed : 12345u };
	switch ( kind )
	{
		case B2S_LARGE_PYRAMID: b2sLargePyramid( s, a, b ); break;
		case B2S_MANY_PYRAMIDS_RAIN: b2sManyPyramidsRain( s, a, b, c, &rng ); break;
		case B2S_JOINT_GRID_MIXED: b2sJointGrid( s, a, 1, b, &rng ); break;
		case B2S_BATCH_WORLD: b2sBatchWorld( s, a, &rng ); break;
		case B2S_RAMP_WORLD: b2sRampWorld( s, a, b, &rng ); break;
		case B2S_MANY_PYRAMIDS_REF: b2sManyPyramidsReference( s, a, b ); break;
		case B2S_JOINT_GRID_REF: b2sJointGrid( s, a, 0, 0, &rng ); break;
		case B2S_HELLO_WORLD: b2sHelloWorld( s ); break;
		case B2S_SHAPE_ZOO: b2sShapeZoo( s, a, &rng ); break;
		case B2S_JOINT_ZOO: b2sJointZoo( s, a, &rng ); break;
		case B2S_FALLING_HINGES: b2sFallingHinges( s ); break;
		case B2S_SLEEP_PYRAMIDS: b2sSleepPyramids( s, a, b, c ); break;
		case B2S_JOINT_MIX: b2sJointMix( s, a, &rng ); break;
		case B2S_OVERFLOW: b2sOverflowScene( s, a, &rng ); break;
		case B2S_SENSOR_ZOO: b2sSensorZoo( s, a, &rng ); break;
#ifndef B2S_NO_CHAINS
		case B2S_CHAIN_ZOO: b2sChainZoo( s, a, &rng ); break;
#endif
		case B2S_BULLET_ZOO: b2sBulletZoo( s, a, &rng ); break;
		default: break;
	}
	return h;
}

/* step `count` scenes `steps` times each with one batched call per step where the library
   has one (b2World_StepBatch), else one world after the other */
B2S_EXPORT void b2s_step_batch( const int* handles, int count, float timeStep, int subStepCount, int steps, int threads )
{
	b2WorldId* ids = malloc( (size_t)( count > 0 ? count : 1 ) * sizeof( b2WorldId ) );
	for ( int i = 0; i < count; ++i ) ids[i] = b2s_scenes[handles[i]].worldId;
	for ( int k = 0; k < steps; ++k )
	{
#ifdef B2S_BATCH_API
		b2World_StepBatch( ids, count, timeStep, subStepCount, threads );
#else
		(void)threads;
		for ( int i = 0; i < count; ++i ) b2World_Step( ids[i], timeStep, subStepCount );
#endif
	}
	free( ids );
}

B2S_EXPORT void b2s_destroy( int h )
{
	b2sScene* s = b2s_scenes + h;
	if ( s->inUse == 0 ) return;
	b2DestroyWorld( s->worldId );
	free( s->bodies );
	free( s->image );
	free( s->imageBodies );
	memset( s, 0, sizeof( *s ) );
}

B2S_EXPORT void b2s_step( int h, float dt, int subSteps, int count )
{
	for ( int i = 0; i < count; ++i ) b2World_Step( b2s_scenes[h].worldId, dt, subSteps );
}

/* The determinism test's loop (test/test_determinism.c:28-50, shared/determinism.c:110-134):
   step until a step reports no body move events (every island asleep), then hash the
   transforms of the scene's dynamic bodies in creation order with b2Hash. Returns the step
   count at that moment (the test's sleepStep) and the hash, or -1 within `stepLimit`. */
B2S_EXPORT int b2s_run_until_asleep( int h, int stepLimit, uint32_t* hashOut )
{
	b2sScene* s = b2s_scenes + h;
	*hashOut = 0;
	for ( int stepCount = 0; stepCount < stepLimit; ++stepCount )
	{
		b2World_Step( s->worldId, 1.0f / 60.0f, 4 );
		b2BodyEvents events = b2World_GetBodyEvents( s->worldId );
		if ( events.moveCount == 0 )
		{
			uint32_t hash = 5381; /* B2_HASH_INIT */
			for ( int i = 0; i < s->bodyCount; ++i )
			{
				if ( b2Body_GetType( s->bodies[i] ) == b2_staticBody ) continue;
				b2WorldTransform xf = b2Body_GetTransform( s->bodies[i] );
				hash = b2Hash( hash, (const uint8_t*)&xf, (int)sizeof( b2WorldTransform ) );
			}
			*hashOut = hash;
			return stepCount;
		}
	}
	return -1;
}

/* scripted changes between steps (sleeping scenes): a body's velocity, which wakes it when
   nonzero; putting a body's island to sleep or waking it; switching sleeping off */
B2S_EXPORT void b2s_set_body_velocity( int h, int bodyIndex, float vx, float vy, float w )
{
	b2BodyId id = b2s_scenes[h].bodies[bodyIndex];
	b2Body_SetLinearVelocity( id, ( b2Vec2 ){ vx, vy } );
	b2Body_SetAngularVelocity( id, w );
}

#ifndef B2S_NO_SNAPSHOT
/* b2World_Snapshot of the scene's world into an image the scene keeps, with a copy of its
   body list; returns the image size */
B2S_EXPORT int b2s_snapshot( int h )
{
	b2sScene* s = b2s_scenes + h;
	int size = b2World_Snapshot( s->worldId, NULL, 0 );
	if ( size <= 0 ) return size;
	free( s->image );
	s->image = malloc( (size_t)size );
	s->imageSize = b2World_Snapshot( s->worldId, s->image, size );
	free( s->imageBodies );
	s->imageBodies = malloc( (size_t)( s->bodyCount > 0 ? s->bodyCount : 1 ) * sizeof( b2BodyId ) );
	memcpy( s->imageBodies, s->bodies, (size_t)s->bodyCount * sizeof( b2BodyId ) );
	s->imageBodyCount = s->bodyCount;
	return s->imageSize;
}

/* b2World_Restore of the scene's world from its kept image, and the body list of that
   instant; returns 1 when the restore succeeded */
B2S_EXPORT int b2s_restore( int h )
{
	b2sScene* s = b2s_scenes + h;
	if ( s->image == NULL ) return 0;
	if ( b2World_Restore( s->worldId, s->image, s->imageSize ) == false ) return 0;
	memcpy( s->bodies, s->imageBodies, (size_t)s->imageBodyCount * sizeof( b2BodyId ) );
	s->bodyCount = s->imageBodyCount;
	return 1;
}

/* a new scene whose world is b2CreateWorldFromSnapshot of the scene's kept image, with the
   body list of that instant pointed at the new world; returns its handle, or -1 */
B2S_EXPORT int b2s_from_snapshot( int h )
{
	b2sScene* s = b2s_scenes + h;
	if ( s->image == NULL ) return -1;
	int n = -1;
	for ( int i = 0; i < B2S_MAX_SCENES; ++i )
	{
		if ( b2s_scenes[i].inUse == 0 )
		{
			n = i;
			break;
		}
	}
	if ( n < 0 ) return -1;
	b2WorldId id = b2CreateWorldFromSnapshot( s->image, s->imageSize, b2s_workerCount );
	if ( b2World_IsValid( id ) == false ) return -1;
	b2sScene* t = b2s_scenes + n;
	memset( t, 0, sizeof( *t ) );
	t->inUse = 1;
	t->worldId = id;
	t->flags = s->flags;
	t->dynamicCount = s->dynamicCount;
	t->targetX = s->targetX;
	t->targetY = s->targetY;
	t->bodyCapacity = s->imageBodyCount > 0 ? s->imageBodyCount : 1;
	t->bodies = malloc( (size_t)t->bodyCapacity * sizeof( b2BodyId ) );
	t->bodyCount = s->imageBodyCount;
	for ( int i = 0; i < t->bodyCount; ++i )
	{
		t->bodies[i] = s->imageBodies[i];
		if ( B2_IS_NON_NULL( t->bodies[i] ) ) t->bodies[i].world0 = (uint16_t)( id.index1 - 1 );
	}
	return n;
}

/* a dynamic 0.5 m box at (x, y) added to the scene; returns its index in the body list */
B2S_EXPORT int b2s_add_box( int h, float x, float y )
{
	b2sScene* s = b2s_scenes + h;
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.position = ( b2Vec2 ){ x, y };
	b2BodyId id = b2CreateBody( s->worldId, &bd );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon box = b2MakeBox( 0.5f, 0.5f );
	b2CreatePolygonShape( id, &sd, &box );
	b2sAddBody( s, id, 1 );
	return s->bodyCount - 1;
}

B2S_EXPORT int b2s_body_valid( int h, int bodyIndex )
{
	return b2Body_IsValid( b2s_scenes[h].bodies[bodyIndex] ) ? 1 : 0;
}
#endif

#ifndef B2S_NO_ISLANDS
B2S_EXPORT void b2s_set_awake( int h, int bodyIndex, int awake )
{
	b2Body_SetAwake( b2s_scenes[h].bodies[bodyIndex], awake != 0 );
}
#endif

/* One scripted change to a scene body between steps, through the public body API:
   kind 0 b2Body_ApplyForce (force (a, b) at the center of mass + (c, d)), 1 ApplyForceToCenter,
   2 ApplyTorque (a), 3 ApplyLinearImpulse (impulse (a, b) at the center + (c, d)),
   4 ApplyLinearImpulseToCenter, 5 ApplyAngularImpulse (a), 6 SetTransform (position (a, b),
   angle c), 7 SetTargetTransform (position (a, b), angle c, time step d), 8 b2DestroyBody
   (the scene then reports the body as zeros), 9 b2DestroyShape of its first shape with a
   mass update. Forces and impulses wake the body. */
B2S_EXPORT void b2s_body_action( int h, int kind, int bodyIndex, float a, float b, float c, float d )
{
	b2BodyId id = b2s_scenes[h].bodies[bodyIndex];
	b2Vec2 v = { a, b };
	b2Vec2 center = b2Body_GetWorldCenter( id );
	b2Vec2 point = { center.x + c, center.y + d };
	switch ( kind )
	{
		case 0: b2Body_ApplyForce( id, v, point, true ); break;
		case 1: b2Body_ApplyForceToCenter( id, v, true ); break;
		case 2: b2Body_ApplyTorque( id, a, true ); break;
		case 3: b2Body_ApplyLinearImpulse( id, v, point, true ); break;
		case 4: b2Body_ApplyLinearImpulseToCenter( id, v, true ); break;
		case 5: b2Body_ApplyAngularImpulse( id, a, true ); break;
		case 6: b2Body_SetTransform( id, v, b2MakeRot( c ) ); break;
		case 7:
		{
			b2Transform target = { v, b2MakeRot( c ) };
			b2Body_SetTargetTransform( id, target, d, true );
			break;
		}
#ifndef B2S_NO_DESTROY
		case 8:
			b2DestroyBody( id );
			b2s_scenes[h].bodies[bodyIndex] = b2_nullBodyId;
			break;
		case 9:
		{
			b2ShapeId shapes[16];
			int n = b2Body_GetShapes( id, shapes, 16 );
			if ( n > 0 ) b2DestroyShape( shapes[0], true );
			break;
		}
#endif
		default: break;
	}
}

B2S_EXPORT void b2s_enable_sleep( int h, int flag ) { b2World_EnableSleeping( b2s_scenes[h].worldId, flag != 0 ); }

/* awake body count and the per-body awake flags (creation order) */
B2S_EXPORT int b2s_awake( int h, int* out )
{
	b2sScene* s = b2s_scenes + h;
	for ( int i = 0; i < s->bodyCount; ++i ) out[i] = B2_IS_NON_NULL( s->bodies[i] ) && b2Body_IsAwake( s->bodies[i] ) ? 1 : 0;
	return b2World_GetAwakeBodyCount( s->worldId );
}

B2S_EXPORT int b2s_body_count( int h ) { return b2s_scenes[h].bodyCount; }

B2S_EXPORT int b2s_dynamic_count( int h ) { return b2s_scenes[h].dynamicCount; }

B2S_EXPORT uint32_t b2s_world_id( int h )
{
	b2WorldId id = b2s_scenes[h].worldId;
	return ( (uint32_t)id.index1 << 16 ) | id.generation;
}

/* 7 floats per body in creation order: p.x, p.y, q.c, q.s, v.x, v.y, w */
/* the last step's body move events (b2World_GetBodyEvents): 4 floats per event
   (p.x, p.y, q.c, q.s) up to capacity; returns the event count */
B2S_EXPORT int b2s_move_events( int handle, float* out, int capacity )
{
	b2BodyEvents ev = b2World_GetBodyEvents( b2s_scenes[handle].worldId );
	int n = ev.moveCount < capacity ? ev.moveCount : capacity;
	for ( int i = 0; i < n; ++i )
	{
		b2Transform xf = ev.moveEvents[i].transform;
		out[4 * i] = xf.p.x;
		out[4 * i + 1] = xf.p.y;
		out[4 * i + 2] = xf.q.c;
		out[4 * i + 3] = xf.q.s;
	}
	return ev.moveCount;
}

/* the move events of `count` scenes after a batched step, one world after the other
   through b2World_GetBodyEvents, as a C program stepping a batch reads them; 4 floats per
   event up to `capacity` events in all; returns the event count */
B2S_EXPORT int b2s_move_events_many( const int* handles, int count, float* out, int capacity )
{
	int total = 0;
	for ( int k = 0; k < count; ++k )
	{
		b2BodyEvents ev = b2World_GetBodyEvents( b2s_scenes[handles[k]].worldId );
		for ( int i = 0; i < ev.moveCount && total < capacity; ++i, ++total )
		{
			b2Transform xf = ev.moveEvents[i].transform;
			out[4 * total] = xf.p.x;
			out[4 * total + 1] = xf.p.y;
			out[4 * total + 2] = xf.q.c;
			out[4 * total + 3] = xf.q.s;
		}
	}
	return total;
}

B2S_EXPORT void b2s_get_state( int h, float* out )
{
	b2sScene* s = b2s_scenes + h;
	for ( int i = 0; i < s->bodyCount; ++i )
	{
		float* o = out + 7 * i;
		if ( B2_IS_NULL( s->bodies[i] ) )
		{
			/* a body destroyed by a scripted change */
			memset( o, 0, 7 * sizeof( float ) );
			continue;
		}
		b2Transform xf = b2Body_GetTransform( s->bodies[i] );
		b2Vec2 v = b2Body_GetLinearVelocity( s->bodies[i] );
		float w = b2Body_GetAngularVelocity( s->bodies[i] );
		o[0] = (float)xf.p.x;
		o[1] = (float)xf.p.y;
		o[2] = xf.q.c;
		o[3] = xf.q.s;
		o[4] = v.x;
		o[5] = v.y;
		o[6] = w;
	}
}

/* The last step's contact begin/end touch events (b2World_GetContactEvents), 5 ints per
   event in the library's order, begin events first: kind (0 begin, 1 end), shape A id,
   shape B id (index1 - 1), contact id index1 - 1 and its generation, up to capacity.
   Returns the event count. */
B2S_EXPORT int b2s_contact_events( int h, int* out, int capacity )
{
	b2ContactEvents e = b2World_GetContactEvents( b2s_scenes[h].worldId );
	int n = 0;
	for ( int i = 0; i < e.beginCount; ++i, ++n )
	{
		if ( n >= capacity ) continue;
		int* o = out + 5 * n;
		o[0] = 0;
		o[1] = e.beginEvents[i].shapeIdA.index1 - 1;
		o[2] = e.beginEvents[i].shapeIdB.index1 - 1;
		o[3] = e.beginEvents[i].contactId.index1 - 1;
		o[4] = (int)e.beginEvents[i].contactId.generation;
	}
	for ( int i = 0; i < e.endCount; ++i, ++n )
	{
		if ( n >= capacity ) continue;
		int* o = out + 5 * n;
		o[0] = 1;
		o[1] = e.endEvents[i].shapeIdA.index1 - 1;
		o[2] = e.endEvents[i].shapeIdB.index1 - 1;
		o[3] = e.endEvents[i].contactId.index1 - 1;
		o[4] = (int)e.endEvents[i].contactId.generation;
	}
	return n;
}

#ifndef B2S_NO_SENSORS
/* The last step's sensor begin/end touch events (b2World_GetSensorEvents), 5 ints per event,
   begin events first: kind (0 begin, 1 end), sensor shape id, visitor shape id (index1 - 1),
   sensor shape generation, visitor shape generation. Returns the event count. */
B2S_EXPORT int b2s_sensor_events( int h, int* out, int capacity )
{
	b2SensorEvents e = b2World_GetSensorEvents( b2s_scenes[h].worldId );
	int n = 0;
	for ( int i = 0; i < e.beginCount + e.endCount; ++i, ++n )
	{
		if ( n >= capacity ) continue;
		int end = i >= e.beginCount;
		b2ShapeId sensor = end ? e.endEvents[i - e.beginCount].sensorShapeId : e.beginEvents[i].sensorShapeId;
		b2ShapeId visitor = end ? e.endEvents[i - e.beginCount].visitorShapeId : e.beginEvents[i].visitorShapeId;
		int* o = out + 5 * n;
		o[0] = end;
		o[1] = sensor.index1 - 1;
		o[2] = visitor.index1 - 1;
		o[3] = sensor.generation;
		o[4] = visitor.generation;
	}
	return n;
}
#endif

#ifndef B2S_NO_ISLANDS
/* the library's own b2World_GetStateHash of the scene's world */
B2S_EXPORT uint64_t b2s_world_state_hash( int h )
{
	return b2World_GetStateHash( b2s_scenes[h].worldId );
}
#endif

/* FNV-1a 64 over the bit patterns of b2s_get_state */
B2S_EXPORT uint64_t b2s_state_hash( int h )
{
	b2sScene* s = b2s_scenes + h;
	uint64_t hash = 14695981039346656037ull;
	float buf[7];
	for ( int i = 0; i < s->bodyCount; ++i )
	{
		if ( B2_IS_NULL( s->bodies[i] ) )
		{
			memset( buf, 0, sizeof( buf ) );
			for ( int k = 0; k < 7; ++k ) hash = hash * 1099511628211ull;
			continue;
		}
		b2Transform xf = b2Body_GetTransform( s->bodies[i] );
		b2Vec2 v = b2Body_GetLinearVelocity( s->bodies[i] );
		buf[0] = (float)xf.p.x;
		buf[1] = (float)xf.p.y;
		buf[2] = xf.q.c;
		buf[3] = xf.q.s;
		buf[4] = v.x;
		buf[5] = v.y;
		buf[6] = b2Body_GetAngularVelocity( s->bodies[i] );
		for ( int k = 0; k < 7; ++k )
		{
			uint32_t bits;
			memcpy( &bits, buf + k, 4 );
			hash = ( hash ^ bits ) * 1099511628211ull;
		}
	}
	return hash;
}

/* Apply a per-body linear and angular velocity (3 floats per body, creation order;
   static bodies are skipped by the library). */
B2S_EXPORT void b2s_set_velocities( int h, const float* in )
{
	b2sScene* s = b2s_scenes + h;
	for ( int i = 0; i < s->bodyCount; ++i )
	{
		b2Vec2 v = { in[3 * i], in[3 * i + 1] };
		b2Body_SetLinearVelocity( s->bodies[i], v );
		b2Body_SetAngularVelocity( s->bodies[i], in[3 * i + 2] );
	}
}

/* friction of every shape on the scene's bodies, indexed by shape id (count entries) */
B2S_EXPORT void b2s_set_friction( int h, const float* byShape, int count )
{
	b2sScene* s = b2s_scenes + h;
	b2ShapeId ids[16];
	for ( int i = 0; i < s->bodyCount; ++i )
	{
		int n = b2Body_GetShapes( s->bodies[i], ids, 16 );
		for ( int k = 0; k < n; ++k )
			if ( ids[k].index1 - 1 < count ) b2Shape_SetFriction( ids[k], byShape[ids[k].index1 - 1] );
	}
}

B2S_EXPORT void b2s_get_friction( int h, float* byShape, int count )
{
	b2sScene* s = b2s_scenes + h;
	b2ShapeId ids[16];
	for ( int i = 0; i < s->bodyCount; ++i )
	{
		int n = b2Body_GetShapes( s->bodies[i], ids, 16 );
		for ( int k = 0; k < n; ++k )
			if ( ids[k].index1 - 1 < count ) byShape[ids[k].index1 - 1] = b2Shape_GetFriction( ids[k] );
	}
}

/* world center of mass of each scene body (2 floats), in the order of b2s_get_state */
B2S_EXPORT void b2s_get_centers( int h, float* out )
{
	b2sScene* s = b2s_scenes + h;
	for ( int i = 0; i < s->bodyCount; ++i )
	{
		b2Pos c = b2Body_GetWorldCenter( s->bodies[i] );
		out[2 * i] = (float)c.x;
		out[2 * i + 1] = (float)c.y;
	}
}

/* body id of each scene body, in the order of b2s_get_state */
B2S_EXPORT void b2s_body_ids( int h, int* out )
{
	b2sScene* s = b2s_scenes + h;
	for ( int i = 0; i < s->bodyCount; ++i ) out[i] = s->bodies[i].index1 - 1;
}

B2S_EXPORT void b2s_target( int h, float* out )
{
	out[0] = b2s_scenes[h].targetX;
	out[1] = b2s_scenes[h].targetY;
}

B2S_EXPORT void b2s_counters( int h, int* out )
{
	b2Counters c = b2World_GetCounters( b2s_scenes[h].worldId );
	out[0] = c.bodyCount;
	out[1] = c.shapeCount;
	out[2] = c.contactCount;
	out[3] = c.jointCount;
	for ( int i = 0; i < 24; ++i ) out[4 + i] = c.colorCounts[i];
	out[28] = c.awakeContactCount;
	out[29] = c.recycledContactCount;
}
