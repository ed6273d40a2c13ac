/*
 * Public API entry points of the GB300 step library (box2d.h subset) and the host's serial
 * bookkeeping: worlds, bodies, shapes, contact records, graph coloring and the move buffer
 * (physics_world.c, body.c, shape.c, contact.c, constraint_graph.c, broad_phase.h in the
 * reference). Numeric body state lives on the device after the first step; getters read
 * it back lazily (one bulk copy per step), setters write through.
 */
#include "b2g_world.h"

#include <stdio.h>

static h_world h_worlds[H_MAX_WORLDS];

h_world* h_worldByIndex( int index ) { return h_worlds + index; }

h_world* h_worldFromId( b2WorldId id )
{
	if ( id.index1 < 1 || id.index1 > H_MAX_WORLDS ) return NULL;
	h_world* w = h_worlds + ( id.index1 - 1 );
	if ( w->inUse == 0 || w->generation != id.generation ) return NULL;
	return w;
}

void h_fail( h_world* w, const char* what, int code )
{
	fprintf( stderr, "box2d_gb300: %s failed: %s\n", what, b2gDev_ErrorString( code ) );
	if ( w ) w->lastStatus = code;
	abort();
}

/* ---------------- pair set ---------------- */
static uint64_t h_hashKey( uint64_t k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdull;
	k ^= k >> 33;
	return k;
}

static void h_pairSetGrow( h_pairSet* s )
{
	int oldCap = s->capacity;
	uint64_t* old = s->keys;
	s->capacity = oldCap == 0 ? 1024 : oldCap * 2;
	s->keys = malloc( (size_t)s->capacity * 8 );
	memset( s->keys, 0xff, (size_t)s->capacity * 8 );
	s->count = 0;
	for ( int i = 0; i < oldCap; ++i )
		if ( old[i] != UINT64_MAX ) h_pairSetAdd( s, old[i] );
	free( old );
}

void h_pairSetAdd( h_pairSet* s, uint64_t key )
{
	if ( 2 * ( s->count + 1 ) > s->capacity ) h_pairSetGrow( s );
	uint64_t mask = (uint64_t)s->capacity - 1;
	uint64_t i = h_hashKey( key ) & mask;
	while ( s->keys[i] != UINT64_MAX )
	{
		if ( s->keys[i] == key ) return;
		i = ( i + 1 ) & mask;
	}
	s->keys[i] = key;
	s->count += 1;
}

int h_pairSetContains( const h_pairSet* s, uint64_t key )
{
	if ( s->capacity == 0 ) return 0;
	uint64_t mask = (uint64_t)s->capacity - 1;
	uint64_t i = h_hashKey( key ) & mask;
	while ( s->keys[i] != UINT64_MAX )
	{
		if ( s->keys[i] == key ) return 1;
		i = ( i + 1 ) & mask;
	}
	return 0;
}

void h_pairSetPrefetch( const h_pairSet* s, uint64_t key )
{
	if ( s->capacity == 0 ) return;
	uint64_t mask = (uint64_t)s->capacity - 1;
	__builtin_prefetch( s->keys + ( h_hashKey( key ) & mask ), 0, 3 );
}

void h_pairSetRemove( h_pairSet* s, uint64_t key )
{
	if ( s->capacity == 0 ) return;
	uint64_t mask = (uint64_t)s->capacity - 1;
	uint64_t i = h_hashKey( key ) & mask;
	while ( s->keys[i] != UINT64_MAX )
	{
		if ( s->keys[i] == key ) break;
		i = ( i + 1 ) & mask;
	}
	if ( s->keys[i] == UINT64_MAX ) return;
	/* backward-shift deletion */
	uint64_t j = i;
	while ( 1 )
	{
		j = ( j + 1 ) & mask;
		if ( s->keys[j] == UINT64_MAX ) break;
		uint64_t h = h_hashKey( s->keys[j] ) & mask;
		int shouldMove = ( i <= j ) ? ( h <= i || h > j ) : ( h <= i && h > j );
		if ( shouldMove )
		{
			s->keys[i] = s->keys[j];
			i = j;
		}
	}
	s->keys[i] = UINT64_MAX;
	s->count -= 1;
}

void h_pairSetFree( h_pairSet* s )
{
	free( s->keys );
	memset( s, 0, sizeof( *s ) );
}

/* ---------------- defaults (types.c:8-89, joint.c:16-112) ---------------- */
b2WorldDef b2DefaultWorldDef( void )
{
	b2WorldDef def;
	memset( &def, 0, sizeof( def ) );
	def.gravity = h_v( 0.0f, -10.0f );
	def.hitEventThreshold = 1.0f;
	def.restitutionThreshold = 1.0f;
	def.contactSpeed = 3.0f;
	def.contactHertz = 30.0f;
	def.contactDampingRatio = 10.0f;
	def.maximumLinearSpeed = 400.0f;
	def.enableSleep = true;
	def.enableContinuous = true;
	def.internalValue = 1152023;
	return def;
}

b2BodyDef b2DefaultBodyDef( void )
{
	b2BodyDef def;
	memset( &def, 0, sizeof( def ) );
	def.type = b2_staticBody;
	def.rotation.c = 1.0f;
	def.safetyFactor = 0.5f;
	def.sleepThreshold = 0.05f;
	def.gravityScale = 1.0f;
	def.enableSleep = true;
	def.enableContactRecycling = true;
	def.isAwake = true;
	def.isEnabled = true;
	def.internalValue = 1152023;
	return def;
}

b2Filter b2DefaultFilter( void )
{
	b2Filter f = { B2_DEFAULT_CATEGORY_BITS, B2_DEFAULT_MASK_BITS, 0 };
	return f;
}

b2SurfaceMaterial b2DefaultSurfaceMaterial( void )
{
	b2SurfaceMaterial m;
	memset( &m, 0, sizeof( m ) );
	m.friction = 0.6f;
	return m;
}

b2ShapeDef b2DefaultShapeDef( void )
{
	b2ShapeDef def;
	memset( &def, 0, sizeof( def ) );
	def.material.friction = 0.6f;
	def.density = 1.0f;
	def.filter = b2DefaultFilter();
	def.updateBodyMass = true;
	def.invokeContactCreation = true;
	def.internalValue = 1152023;
	return def;
}

/* ---------------- world (physics_world.c:159-444) ---------------- */
b2WorldId b2CreateWorld( const b2WorldDef* def )
{
	int index = -1;
	for ( int i = 0; i < H_MAX_WORLDS; ++i )
	{
		if ( h_worlds[i].inUse == 0 )
		{
			index = i;
			break;
		}
	}
	b2WorldId nullId = { 0, 0 };
	if ( index < 0 ) return nullId;
	h_world* w = h_worlds + index;
	uint16_t generation = w->generation;
	memset( w, 0, sizeof( *w ) );
	w->worldId = (uint16_t)index;
	w->generation = generation;
	h_islandsInit( w );
	int rc = b2gDev_Create( &w->dev );
	if ( rc != 0 )
	{
		fprintf( stderr, "box2d_gb300: no usable CUDA device (%s); the GB300 step library has no CPU path\n",
				 b2gDev_ErrorString( rc ) );
		return nullId;
	}
	w->inUse = 1;
	for ( int i = 0; i < 3; ++i ) w->trees[i] = h_treeCreate( 16 );
	w->gravity = def->gravity;
	w->hitEventThreshold = def->hitEventThreshold;
	w->restitutionThreshold = def->restitutionThreshold;
	w->maxLinearSpeed = def->maximumLinearSpeed;
	w->contactSpeed = def->contactSpeed;
	w->contactHertz = def->contactHertz;
	w->contactDampingRatio = def->contactDampingRatio;
	w->enableSleep = def->enableSleep;
	w->enableWarmStarting = 1;
	w->enableContactSoftening = def->enableContactSoftening;
	w->enableContinuous = def->enableContinuous;
	w->hostStateValid = 1;
	w->jointsHostValid = 1;
	w->colorsDirty = 1;
	w->jointsDirty = 1;
	for ( int t = 0; t < 3; ++t ) w->uploadedTreeVersion[t] = -1;
	b2WorldId id = { (uint16_t)( index + 1 ), w->generation };
	return id;
}

/* frees every array of the world's simulation state (what a snapshot holds); the device
   world, the rebuild worker and the tape stay */
void h_freeWorldArrays( h_world* w )
{
	free( w->moveBoxes );
	free( w->moveShapes );
	free( w->specKeys );
	free( w->specBoxes );
	w->moveBoxes = w->specBoxes = NULL;
	w->moveShapes = w->specKeys = NULL;
	w->moveBufCap = w->specCap = 0;
	w->specIssued = 0;
	for ( int i = 0; i < 3; ++i )
	{
		h_treeDestroy( w->trees + i );
		free( w->movedProxies[i].bits );
	}
	h_free( w->bodyIdPool.freeArray );
	h_free( w->shapeIdPool.freeArray );
	h_free( w->chainIdPool.freeArray );
	h_free( w->contactIdPool.freeArray );
	h_free( w->jointIdPool.freeArray );
	h_free( w->bodies );
	h_free( w->shapes );
	h_free( w->contacts );
	h_free( w->joints );
	h_free( w->jointRecords );
	h_free( w->awakeBodyIds );
	h_free( w->awakeContactIds );
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
	{
		free( w->colors[i].bodySet.bits );
		h_free( w->colors[i].contactIds );
		h_free( w->colors[i].jointIds );
	}
	h_free( w->moveArray );
	h_pairSetFree( &w->pairSet );
	h_free( w->moveEvents );
	h_freeSensors( w );
	for ( int i = 0; i < w->chains.count; ++i ) free( w->chains.data[i].shapeIndices );
	h_free( w->chains );
	h_free( w->beginEvents );
	h_free( w->endEvents[0] );
	h_free( w->endEvents[1] );
	h_free( w->pendingInits );
	h_free( w->pendingKills );
	h_free( w->forcedBodies );
	h_free( w->staticBodyIds );
	h_free( w->staticJointIds );
	h_islandsFree( w );
}

void b2DestroyWorld( b2WorldId worldId )
{
	h_world* w = h_worldFromId( worldId );
	if ( w == NULL ) return;
	h_stopRebuildWorker( w );
	h_tapeDetach( w );
	b2gDev_Destroy( w->dev );
	h_freeWorldArrays( w );
	uint16_t generation = w->generation;
	memset( w, 0, sizeof( *w ) );
	w->generation = generation + 1;
}

bool b2World_IsValid( b2WorldId id ) { return h_worldFromId( id ) != NULL; }

/* physics_world.c:1704-1734: switching sleep off wakes every sleeping set */
void b2World_EnableSleeping( b2WorldId worldId, bool flag )
{
	h_world* w = h_worldFromId( worldId );
	if ( w && w->locked == 0 && flag == false && w->enableSleep )
	{
		for ( int i = H_FIRST_SLEEPING_SET; i < w->sets.count; ++i )
			if ( w->sets.data[i].setIndex != B2_NULL_INDEX && w->sets.data[i].bodyIds.count > 0 ) h_wakeSolverSet( w, i );
	}
	if ( w ) w->enableSleep = flag;
}

bool b2World_IsSleepingEnabled( b2WorldId worldId ) { return h_worldFromId( worldId )->enableSleep; }

void b2World_EnableContinuous( b2WorldId worldId, bool flag )
{
	h_world* w = h_worldFromId( worldId );
	if ( w ) w->enableContinuous = flag;
}

bool b2World_IsContinuousEnabled( b2WorldId worldId ) { return h_worldFromId( worldId )->enableContinuous; }

void b2World_EnableWarmStarting( b2WorldId worldId, bool flag )
{
	h_world* w = h_worldFromId( worldId );
	if ( w ) w->enableWarmStarting = flag;
}

void b2World_SetGravity( b2WorldId worldId, b2Vec2 gravity )
{
	h_world* w = h_worldFromId( worldId );
	if ( w ) w->gravity = gravity;
}

b2Vec2 b2World_GetGravity( b2WorldId worldId ) { return h_worldFromId( worldId )->gravity; }

int b2World_GetAwakeBodyCount( b2WorldId worldId ) { return h_worldFromId( worldId )->awakeBodyIds.count; }

/* ---- state hash (world_snapshot.c:1003-1187, b2World_GetStateHash) ----
   FNV-1a 64 over every live body's transform, its velocity when awake and its solver-set
   slot; every live contact's set, color and slot and its manifold impulses; every live
   joint's set, color, slot and accumulated impulses; the id pools and the solver-set count.
   Two worlds that simulate identically, with identical bookkeeping, give the same value. */
#define H_FNV_INIT 14695981039346656037ull
#define H_FNV_PRIME 1099511628211ull

/* the hash under construction; `words`, when set, also receives every value mixed in (a
   probe for locating where two worlds' bookkeeping differs) */
typedef struct h_fnv
{
	uint64_t hash;
	uint32_t* words;
	int count, capacity;
} h_fnv;

static void h_fnvWord( h_fnv* f, uint32_t bits )
{
	f->hash = ( f->hash ^ (uint64_t)bits ) * H_FNV_PRIME;
	if ( f->words != NULL && f->count < f->capacity ) f->words[f->count] = bits;
	f->count += 1;
}
static void h_fnvFloat( h_fnv* f, float v )
{
	uint32_t bits;
	memcpy( &bits, &v, 4 );
	h_fnvWord( f, bits );
}
static void h_fnvInt( h_fnv* f, int v ) { h_fnvWord( f, (uint32_t)v ); }
static void h_fnvBytes( h_fnv* f, const void* data, int n )
{
	const uint8_t* b = (const uint8_t*)data;
	for ( int i = 0; i < n; ++i ) h_fnvWord( f, b[i] );
}
static void h_fnvPool( h_fnv* f, const h_idPool* pool )
{
	h_fnvInt( f, pool->nextIndex );
	h_fnvInt( f, pool->nextIndex - pool->freeArray.count );
}

static void h_stateHash( h_world* w, h_fnv* f )
{
	h_syncFromDevice( w );
	h_syncJointsFromDevice( w );
	for ( int i = 0; i < w->bodies.count; ++i )
	{
		const h_body* b = w->bodies.data + i;
		if ( b->id != i ) continue;
		h_fnvFloat( f, b->transform.p.x );
		h_fnvFloat( f, b->transform.p.y );
		h_fnvFloat( f, b->transform.q.c );
		h_fnvFloat( f, b->transform.q.s );
		if ( b->setIndex == H_AWAKE_SET )
		{
			h_fnvFloat( f, b->linearVelocity.x );
			h_fnvFloat( f, b->linearVelocity.y );
			h_fnvFloat( f, b->angularVelocity );
		}
		h_fnvInt( f, b->setIndex );
		h_fnvInt( f, b->localIndex );
	}
	int nc = w->contacts.count;
	b2gContact* dc = NULL;
	if ( nc > 0 && w->dev != NULL )
	{
		dc = malloc( (size_t)nc * sizeof( b2gContact ) );
		int rc = b2gDev_DownloadContacts( w->dev, dc, nc );
		if ( rc != 0 ) h_fail( w, "contact download", rc );
	}
	for ( int i = 0; i < nc; ++i )
	{
		const h_contact* c = w->contacts.data + i;
		if ( c->contactId != i ) continue;
		h_fnvInt( f, c->setIndex );
		h_fnvInt( f, c->colorIndex );
		h_fnvInt( f, c->localIndex );
		const b2Manifold* m = dc != NULL ? &dc[i].manifold : NULL;
		int pointCount = m != NULL ? m->pointCount : 0;
		h_fnvInt( f, pointCount );
		for ( int k = 0; k < pointCount; ++k )
		{
			h_fnvFloat( f, m->points[k].normalImpulse );
			h_fnvFloat( f, m->points[k].tangentImpulse );
			h_fnvFloat( f, m->points[k].totalNormalImpulse );
		}
	}
	free( dc );
	for ( int i = 0; i < w->joints.count; ++i )
	{
		const h_joint* j = w->joints.data + i;
		if ( j->jointId != i ) continue;
		h_fnvInt( f, j->setIndex );
		h_fnvInt( f, j->colorIndex );
		h_fnvInt( f, j->localIndex );
		const float* s = w->jointRecords.data[i].s;
		/* the accumulated impulses of each type, in the slots host/joint.c lists */
		switch ( j->type )
		{
			case b2_distanceJoint:
			case b2_wheelJoint:
			case b2_revoluteJoint:
			case b2_prismaticJoint:
			{
				int first = 0, count = j->type == b2_distanceJoint ? 4 : ( j->type == b2_wheelJoint ? 5 : 6 );
				if ( j->type == b2_revoluteJoint || j->type == b2_prismaticJoint )
				{
					h_fnvBytes( f, s, 2 * (int)sizeof( float ) );
					first = 2;
				}
				for ( int k = first; k < count; ++k ) h_fnvFloat( f, s[k] );
				break;
			}
			case b2_weldJoint:
				h_fnvBytes( f, s, 2 * (int)sizeof( float ) );
				h_fnvFloat( f, s[2] );
				break;
			case b2_moverJoint:
			case b2_pogoJoint:
				h_fnvFloat( f, s[0] );
				h_fnvFloat( f, s[1] );
				break;
			case b2_motorJoint:
				for ( int k = 0; k < 6; ++k ) h_fnvFloat( f, s[k] );
				break;
			default:
				break;
		}
	}
	h_fnvPool( f, &w->bodyIdPool );
	h_fnvPool( f, &w->shapeIdPool );
	h_fnvPool( f, &w->chainIdPool );
	h_fnvPool( f, &w->contactIdPool );
	h_fnvPool( f, &w->jointIdPool );
	h_fnvPool( f, &w->islandIdPool );
	h_fnvPool( f, &w->setIdPool );
	h_fnvInt( f, w->sets.count );
}

uint64_t b2World_GetStateHash( b2WorldId worldId )
{
	h_world* w = h_worldFromId( worldId );
	if ( w == NULL ) return 0;
	h_fnv f = { H_FNV_INIT, NULL, 0, 0 };
	h_stateHash( w, &f );
	return f.hash;
}

/* the values b2World_GetStateHash mixes, in order (probe); returns their count */
int h_stateHashWords( h_world* w, uint32_t* words, int capacity )
{
	h_fnv f = { H_FNV_INIT, words, 0, capacity };
	h_stateHash( w, &f );
	return f.count;
}

b2Profile b2World_GetProfile( b2WorldId worldId ) { return h_worldFromId( worldId )->profile; }

b2Counters b2World_GetCounters( b2WorldId worldId )
{
	h_world* w = h_worldFromId( worldId );
	b2Counters c;
	memset( &c, 0, sizeof( c ) );
	c.bodyCount = w->bodyIdPool.nextIndex - w->bodyIdPool.freeArray.count;
	c.shapeCount = w->shapeIdPool.nextIndex - w->shapeIdPool.freeArray.count;
	c.contactCount = w->contactIdPool.nextIndex - w->contactIdPool.freeArray.count;
	c.jointCount = w->jointIdPool.nextIndex - w->jointIdPool.freeArray.count;
	c.staticTreeHeight = h_treeHeight( w->trees + b2_staticBody );
	c.treeHeight = h_treeHeight( w->trees + b2_dynamicBody );
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
		c.colorCounts[i] = w->colors[i].contactIds.count + w->colors[i].jointIds.count;
	c.awakeContactCount = w->awakeContactIds.count;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i ) c.awakeContactCount += w->colors[i].contactIds.count;
	c.islandCount = w->islandIdPool.nextIndex - w->islandIdPool.freeArray.count;
	c.recycledContactCount = w->recycledContactCount;
	return c;
}

b2BodyEvents b2World_GetBodyEvents( b2WorldId worldId )
{
	h_world* w = h_worldFromId( worldId );
	if ( w->moveEventsValid == 0 && w->stepIndex > 0 ) h_buildMoveEvents( w );
	b2BodyEvents e = { w->moveEvents.data, w->moveEvents.count };
	return e;
}

/* materialize the move events of the last step from the device state: one per body of
   the awake set as the finalize saw it (solver.c:608-622); the sleep pass builds them
   before it moves bodies out of the awake set */
static void h_fetchMirror( h_world* w )
{
	if ( w->mirrorValid ) return;
	int rc = b2gDev_DownloadState( w->dev, w->bodies.count, w->awakeBodyIds.count, &w->mirrorXf, &w->mirrorCenter,
								   &w->mirrorFlags, &w->mirrorV, &w->mirrorSleep );
	if ( rc != 0 ) h_fail( w, "device download", rc );
	w->mirrorValid = 1;
}

void h_buildMoveEvents( h_world* w )
{
	/* transforms straight from the downloaded state when the host bodies are stale */
	const float* xf = NULL;
	if ( w->hostStateValid == 0 && w->devReady )
	{
		h_fetchMirror( w );
		xf = w->mirrorXf;
	}
	int n = w->awakeBodyIds.count;
	h_reserve( w->moveEvents, n );
	w->moveEvents.count = n;
	for ( int i = 0; i < n; ++i )
	{
		h_body* b = w->bodies.data + w->awakeBodyIds.data[i];
		b2BodyMoveEvent* ev = w->moveEvents.data + i;
		if ( xf != NULL )
		{
			const float* x = xf + 4 * b->id;
			ev->transform.p = h_v( x[0], x[1] );
			ev->transform.q.c = x[2];
			ev->transform.q.s = x[3];
		}
		else
		{
			ev->transform = b->transform;
		}
		ev->bodyId.index1 = b->id + 1;
		ev->bodyId.world0 = w->worldId;
		ev->bodyId.generation = b->generation;
		ev->userData = b->userData;
		ev->fellAsleep = false;
		b->bodyMoveIndex = i;
	}
	w->moveEventsValid = 1;
}

b2ContactEvents b2World_GetContactEvents( b2WorldId worldId )
{
	h_world* w = h_worldFromId( worldId );
	/* the step flips the end-event buffers when it ends: the events of the last step (and of
	   changes made before it) are in the previous buffer (physics_world.c:1486-1487) */
	int endIndex = 1 - w->endEventArrayIndex;
	b2ContactEvents e;
	memset( &e, 0, sizeof( e ) );
	e.beginEvents = w->beginEvents.data;
	e.beginCount = w->beginEvents.count;
	e.endEvents = w->endEvents[endIndex].data;
	e.endCount = w->endEvents[endIndex].count;
	return e;
}

/* ---------------- device mirror ---------------- */

/* Pull transforms, centers and velocities (and joint impulses) back from the device. */
/* bring body transforms and velocities back from the device (what the getters and the
   move events read); joint impulses come back only before host-side changes */
void h_syncFromDevice( h_world* w )
{
	if ( w->hostStateValid || w->devReady == 0 ) return;
	int nb = w->bodies.count;
	int na = w->awakeBodyIds.count;
	h_fetchMirror( w );
	const float *xf = w->mirrorXf, *center = w->mirrorCenter, *sv = w->mirrorV, *sleepTime = w->mirrorSleep;
	const uint32_t* typeFlags = w->mirrorFlags;
	for ( int i = 0; i < nb; ++i )
	{
		h_body* b = w->bodies.data + i;
		if ( b->id != i ) continue;
		b->transform.p = h_v( xf[4 * i], xf[4 * i + 1] );
		b->transform.q.c = xf[4 * i + 2];
		b->transform.q.s = xf[4 * i + 3];
		b->center = h_v( center[2 * i], center[2 * i + 1] );
		b->flags = ( b->flags & ~(uint32_t)B2G_TRANSIENT ) | ( typeFlags[i] & B2G_TRANSIENT );
	}
	for ( int a = 0; a < na; ++a )
	{
		h_body* b = w->bodies.data + w->awakeBodyIds.data[a];
		b->linearVelocity = h_v( sv[4 * a], sv[4 * a + 1] );
		b->angularVelocity = sv[4 * a + 2];
		b->sleepTime = sleepTime[a];
	}
	w->hostStateValid = 1;
}

void h_syncJointsFromDevice( h_world* w )
{
	if ( w->jointsHostValid || w->devReady == 0 ) return;
	if ( w->joints.count > 0 )
	{
		int rc = b2gDev_DownloadJoints( w->dev, w->jointRecords.data, w->jointRecords.count );
		if ( rc != 0 ) h_fail( w, "joint download", rc );
	}
	w->jointsHostValid = 1;
}

void h_syncShapeBoxes( h_world* w )
{
	if ( w->shapeBoxesValid || w->devReady == 0 ) return;
	int ns = w->shapes.count;
	if ( ns > 0 )
	{
		float* boxes = malloc( (size_t)ns * 8 * sizeof( float ) );
		int rc = b2gDev_DownloadShapeBoxes( w->dev, ns, boxes, boxes + 4 * (size_t)ns );
		if ( rc != 0 ) h_fail( w, "shape box download", rc );
		for ( int i = 0; i < ns; ++i )
		{
			h_shape* s = w->shapes.data + i;
			if ( s->id != i ) continue;
			b2AABB box = { { boxes[4 * i], boxes[4 * i + 1] }, { boxes[4 * i + 2], boxes[4 * i + 3] } };
			s->aabb = box;
		}
		free( boxes );
	}
	w->shapeBoxesValid = 1;
}

void h_markHostChanged( h_world* w )
{
	/* the trees may still be in the rebuild worker's hands (the last step's enlargement) */
	h_joinRebuild( w );
	h_syncFromDevice( w );
	h_syncJointsFromDevice( w );
	/* the device boxes are sent again from the host's before the next step */
	h_syncShapeBoxes( w );
	w->devReady = 0;
}

/* Upload every body, shape, joint and tree (cold data) when the host world changed. */
void h_ensureDevice( h_world* w )
{
	if ( w->devReady ) return;
	int nb = w->bodies.count;
	int na = w->awakeBodyIds.count;
	int ns = w->shapes.count;
	size_t nbc = (size_t)( nb > 0 ? nb : 1 ), nac = (size_t)( na > 0 ? na : 1 ), nsc = (size_t)( ns > 0 ? ns : 1 );
	float* xf = calloc( nbc * 4, sizeof( float ) );
	float* center = calloc( nbc * 2, sizeof( float ) );
	float* localCenter = calloc( nbc * 2, sizeof( float ) );
	float* invMass = calloc( nbc, sizeof( float ) );
	float* invI = calloc( nbc, sizeof( float ) );
	float* minExtent = calloc( nbc, sizeof( float ) );
	float* maxExtent = calloc( nbc, sizeof( float ) );
	float* sleepThreshold = calloc( nbc, sizeof( float ) );
	float* safetyFactor = calloc( nbc, sizeof( float ) );
	int* awakeIndex = calloc( nbc, sizeof( int ) );
	uint32_t* typeFlags = calloc( nbc, sizeof( uint32_t ) );
	int* shapeStart = calloc( nbc, sizeof( int ) );
	int* shapeCount = calloc( nbc, sizeof( int ) );
	int* shapeList = calloc( nsc, sizeof( int ) );
	int listCount = 0;
	for ( int i = 0; i < nb; ++i )
	{
		h_body* b = w->bodies.data + i;
		awakeIndex[i] = -1;
		if ( b->id != i ) continue;
		xf[4 * i] = b->transform.p.x;
		xf[4 * i + 1] = b->transform.p.y;
		xf[4 * i + 2] = b->transform.q.c;
		xf[4 * i + 3] = b->transform.q.s;
		center[2 * i] = b->center.x;
		center[2 * i + 1] = b->center.y;
		localCenter[2 * i] = b->localCenter.x;
		localCenter[2 * i + 1] = b->localCenter.y;
		invMass[i] = b->invMass;
		invI[i] = b->invInertia;
		minExtent[i] = b->minExtent;
		maxExtent[i] = b->maxExtent;
		sleepThreshold[i] = b->sleepThreshold;
		safetyFactor[i] = b->safetyFactor;
		awakeIndex[i] = b->setIndex == H_AWAKE_SET ? b->localIndex : -1;
		typeFlags[i] = (uint32_t)b->type | ( b->flags << 2 );
		shapeStart[i] = listCount;
		int sid = b->headShapeId;
		while ( sid != B2_NULL_INDEX )
		{
			shapeList[listCount++] = sid;
			sid = w->shapes.data[sid].nextShapeId;
		}
		shapeCount[i] = listCount - shapeStart[i];
	}
	int* awakeBodyId = w->awakeBodyIds.data;
	float* sv = calloc( nac * 4, sizeof( float ) );
	float* sd = calloc( nac * 4, sizeof( float ) );
	float* params = calloc( nac * 8, sizeof( float ) );
	float* c0 = calloc( nac * 4, sizeof( float ) );
	float* sleepTimes = calloc( nac, sizeof( float ) );
	for ( int a = 0; a < na; ++a )
	{
		h_body* b = w->bodies.data + awakeBodyId[a];
		sleepTimes[a] = b->sleepTime;
		uint32_t fl = b->simFlags;
		float flBits;
		memcpy( &flBits, &fl, 4 );
		sv[4 * a] = b->linearVelocity.x;
		sv[4 * a + 1] = b->linearVelocity.y;
		sv[4 * a + 2] = b->angularVelocity;
		sv[4 * a + 3] = flBits;
		sd[4 * a + 2] = 1.0f;
		params[8 * a + 0] = b->force.x;
		params[8 * a + 1] = b->force.y;
		params[8 * a + 2] = b->torque;
		params[8 * a + 3] = b->linearDamping;
		params[8 * a + 4] = b->angularDamping;
		params[8 * a + 5] = b->gravityScale;
		params[8 * a + 6] = b->invMass;
		params[8 * a + 7] = b->invInertia;
		c0[4 * a] = b->center.x;
		c0[4 * a + 1] = b->center.y;
		c0[4 * a + 2] = b->transform.q.c;
		c0[4 * a + 3] = b->transform.q.s;
	}
	b2gShape* shapes = calloc( nsc, sizeof( b2gShape ) );
	float* aabbs = calloc( nsc * 4, sizeof( float ) );
	float* fats = calloc( nsc * 4, sizeof( float ) );
	for ( int i = 0; i < ns; ++i )
	{
		h_shape* s = w->shapes.data + i;
		b2gShape* d = shapes + i;
		if ( s->id != i )
		{
			d->type = -1;
			d->proxyKey = -1;
			continue;
		}
		d->type = s->type;
		d->bodyId = s->bodyId;
		d->enableHitEvents = s->enableHitEvents;
		switch ( s->type )
		{
			case b2_circleShape:
				d->v[0] = s->circle.center;
				d->radius = s->circle.radius;
				d->count = 1;
				break;
			case b2_capsuleShape:
				d->v[0] = s->capsule.center1;
				d->v[1] = s->capsule.center2;
				d->radius = s->capsule.radius;
				d->count = 2;
				break;
			case b2_segmentShape:
				d->v[0] = s->segment.point1;
				d->v[1] = s->segment.point2;
				d->count = 2;
				break;
			case b2_chainSegmentShape:
				/* the segment in v[0], v[1]; its ghost vertices in v[2] (before) and v[3] (after) */
				d->v[0] = s->chainSegment.segment.point1;
				d->v[1] = s->chainSegment.segment.point2;
				d->v[2] = s->chainSegment.ghost1;
				d->v[3] = s->chainSegment.ghost2;
				d->count = 2;
				break;
			case b2_polygonShape:
				memcpy( d->v, s->polygon.vertices, sizeof( d->v ) );
				memcpy( d->n, s->polygon.normals, sizeof( d->n ) );
				d->centroid = s->polygon.centroid;
				d->radius = s->polygon.radius;
				d->count = s->polygon.count;
				break;
			default:
				break;
		}
		d->aabbMargin = s->aabbMargin;
		d->friction = s->material.friction;
		d->restitution = s->material.restitution;
		d->rollingResistance = s->material.rollingResistance;
		d->tangentSpeed = s->material.tangentSpeed;
		d->categoryBits = s->filter.categoryBits;
		d->maskBits = s->filter.maskBits;
		d->groupIndex = s->filter.groupIndex;
		d->isSensor = s->isSensor;
		d->enableSensorEvents = s->enableSensorEvents;
		d->proxyKey = s->proxyKey;
		{
			b2Vec2 centroid = h_getShapeCentroid( s );
			float minExtent, maxExtent;
			h_computeShapeExtent( s, centroid, &minExtent, &maxExtent );
			d->ccdCentroid = centroid;
			d->ccdCoreRadius = 0.25f * minExtent;
		}
		aabbs[4 * i] = s->aabb.lowerBound.x;
		aabbs[4 * i + 1] = s->aabb.lowerBound.y;
		aabbs[4 * i + 2] = s->aabb.upperBound.x;
		aabbs[4 * i + 3] = s->aabb.upperBound.y;
		fats[4 * i] = s->fatAABB.lowerBound.x;
		fats[4 * i + 1] = s->fatAABB.lowerBound.y;
		fats[4 * i + 2] = s->fatAABB.upperBound.x;
		fats[4 * i + 3] = s->fatAABB.upperBound.y;
	}
	int rc = b2gDev_UploadBodies( w->dev, nb, xf, center, localCenter, invMass, invI, minExtent, maxExtent, sleepThreshold, safetyFactor,
								  awakeIndex, typeFlags,
								  shapeStart, shapeCount, shapeList, listCount );
	if ( rc == 0 ) rc = b2gDev_UploadAwake( w->dev, na, awakeBodyId, sv, sd, params, c0, sleepTimes );
	if ( rc == 0 ) rc = b2gDev_UploadShapes( w->dev, shapes, aabbs, fats, ns );
	if ( rc != 0 ) h_fail( w, "device upload", rc );
	free( xf );
	free( center );
	free( localCenter );
	free( invMass );
	free( invI );
	free( minExtent );
	free( maxExtent );
	free( sleepThreshold );
	free( safetyFactor );
	free( awakeIndex );
	free( typeFlags );
	free( shapeStart );
	free( shapeCount );
	free( shapeList );
	free( sv );
	free( sd );
	free( params );
	free( c0 );
	free( sleepTimes );
	free( shapes );
	free( aabbs );
	free( fats );
	w->jointsDirty = 1;

	w->colorsDirty = 1;
	w->islandsDirty = 1;
	w->devReady = 1;
}

/* ---------------- bodies (body.c:174-330, :524-650) ---------------- */
static h_body* h_getBody( b2BodyId id ) { return h_worlds[id.world0].bodies.data + ( id.index1 - 1 ); }

b2BodyId b2CreateBody( b2WorldId worldId, const b2BodyDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2BodyId nullId = { 0, 0, 0 };
	if ( w == NULL || w->locked ) return nullId;
	h_markHostChanged( w );
	int bodyId = h_allocId( &w->bodyIdPool );
	if ( bodyId == w->bodies.count )
	{
		h_body z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->bodies, z );
	}
	h_body* b = w->bodies.data + bodyId;
	uint16_t generation = b->generation;
	memset( b, 0, sizeof( *b ) );
	uint32_t flags = 0;
	flags |= def->motionLocks.linearX ? B2G_LOCK_X : 0;
	flags |= def->motionLocks.linearY ? B2G_LOCK_Y : 0;
	flags |= def->motionLocks.angularZ ? B2G_LOCK_Z : 0;
	flags |= def->isBullet ? B2G_IS_BULLET : 0;
	flags |= def->allowFastRotation ? B2G_ALLOW_FAST_ROTATION : 0;
	flags |= def->type == b2_dynamicBody ? B2G_DYNAMIC_FLAG : 0;
	flags |= def->enableSleep ? B2G_ENABLE_SLEEP : 0;
	flags |= def->enableContactRecycling ? B2G_ENABLE_RECYCLING : 0;
	b->transform.p = def->position;
	b->transform.q = def->rotation;
	b->center = def->position;
	b->minExtent = H_HUGE;
	b->maxExtent = 0.0f;
	b->linearDamping = def->linearDamping;
	b->angularDamping = def->angularDamping;
	b->gravityScale = def->gravityScale;
	b->simFlags = flags;
	b->linearVelocity = def->linearVelocity;
	b->angularVelocity = def->angularVelocity;
	b->userData = def->userData;
	/* body.c:194-226: a body created asleep gets a sleeping set of its own and no state */
	int isAwake = def->isAwake || def->enableSleep == false;
	if ( def->type == b2_staticBody )
	{
		b->setIndex = H_STATIC_SET;
		b->localIndex = w->staticCount++;
		h_push( w->staticBodyIds, bodyId );
	}
	else if ( isAwake )
	{
		b->setIndex = H_AWAKE_SET;
		b->localIndex = w->awakeBodyIds.count;
		h_push( w->awakeBodyIds, bodyId );
	}
	else
	{
		int setId = h_allocSleepingSet( w );
		h_sleepSet* set = w->sets.data + setId;
		b->setIndex = setId;
		b->localIndex = set->bodyIds.count;
		h_push( set->bodyIds, bodyId );
		b->linearVelocity = h_v( 0.0f, 0.0f );
		b->angularVelocity = 0.0f;
	}
	b->islandId = B2_NULL_INDEX;
	b->islandIndex = B2_NULL_INDEX;
	b->bodyMoveIndex = B2_NULL_INDEX;
	b->generation = generation + 1;
	b->headShapeId = B2_NULL_INDEX;
	b->headContactKey = B2_NULL_INDEX;
	b->headJointKey = B2_NULL_INDEX;
	b->headChainId = B2_NULL_INDEX;
	b->id = bodyId;
	b->sleepThreshold = def->sleepThreshold;
	b->safetyFactor = def->safetyFactor;
	b->type = def->type;
	b->flags = flags;
	/* dynamic and kinematic bodies get an island (body.c:319-323) */
	if ( b->setIndex >= H_AWAKE_SET ) h_createIslandForBody( w, b->setIndex, b );
	b2BodyId id = { bodyId + 1, w->worldId, w->bodies.data[bodyId].generation };
	return id;
}

bool b2Body_IsValid( b2BodyId id )
{
	if ( id.world0 >= H_MAX_WORLDS ) return false;
	h_world* w = h_worlds + id.world0;
	if ( w->inUse == 0 || id.index1 < 1 || id.index1 > w->bodies.count ) return false;
	h_body* b = w->bodies.data + id.index1 - 1;
	return b->id == id.index1 - 1 && b->generation == id.generation;
}

/* shape.c b2Shape_IsValid, joint.c b2Joint_IsValid: the slot is live and of the same generation */
bool b2Shape_IsValid( b2ShapeId id )
{
	if ( id.world0 >= H_MAX_WORLDS ) return false;
	h_world* w = h_worlds + id.world0;
	if ( w->inUse == 0 || id.index1 < 1 || id.index1 > w->shapes.count ) return false;
	const h_shape* s = w->shapes.data + id.index1 - 1;
	return s->id == id.index1 - 1 && s->generation == id.generation;
}

bool b2Joint_IsValid( b2JointId id )
{
	if ( id.world0 >= H_MAX_WORLDS ) return false;
	h_world* w = h_worlds + id.world0;
	if ( w->inUse == 0 || id.index1 < 1 || id.index1 > w->joints.count ) return false;
	const h_joint* j = w->joints.data + id.index1 - 1;
	return j->jointId == id.index1 - 1 && j->generation == id.generation;
}

/* shape.c b2Shape_GetAABB: the shape's box as the last step's finalize computed it */
b2AABB b2Shape_GetAABB( b2ShapeId id )
{
	b2AABB empty = { { 0.0f, 0.0f }, { 0.0f, 0.0f } };
	if ( b2Shape_IsValid( id ) == false ) return empty;
	h_world* w = h_worlds + id.world0;
	h_syncShapeBoxes( w );
	return w->shapes.data[id.index1 - 1].aabb;
}

b2BodyType b2Body_GetType( b2BodyId bodyId ) { return h_getBody( bodyId )->type; }

b2WorldTransform b2Body_GetTransform( b2BodyId bodyId )
{
	h_syncFromDevice( h_worlds + bodyId.world0 );
	return h_getBody( bodyId )->transform;
}

b2Pos b2Body_GetPosition( b2BodyId bodyId ) { return b2Body_GetTransform( bodyId ).p; }

b2Rot b2Body_GetRotation( b2BodyId bodyId ) { return b2Body_GetTransform( bodyId ).q; }

b2Vec2 b2Body_GetLocalPoint( b2BodyId bodyId, b2Pos worldPoint )
{
	return h_invTransformPoint( b2Body_GetTransform( bodyId ), worldPoint );
}

b2Pos b2Body_GetWorldPoint( b2BodyId bodyId, b2Vec2 localPoint )
{
	return h_transformWorldPoint( b2Body_GetTransform( bodyId ), localPoint );
}

b2Vec2 b2Body_GetLinearVelocity( b2BodyId bodyId )
{
	h_syncFromDevice( h_worlds + bodyId.world0 );
	h_body* b = h_getBody( bodyId );
	return b->setIndex == H_AWAKE_SET ? b->linearVelocity : h_v( 0.0f, 0.0f );
}

float b2Body_GetAngularVelocity( b2BodyId bodyId )
{
	h_syncFromDevice( h_worlds + bodyId.world0 );
	h_body* b = h_getBody( bodyId );
	return b->setIndex == H_AWAKE_SET ? b->angularVelocity : 0.0f;
}

/* body.c:790-840: a nonzero velocity wakes a sleeping body; the new velocity of an awake
   body goes to the host record and straight to the device */
void b2Body_SetLinearVelocity( b2BodyId bodyId, b2Vec2 v )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( b->type == b2_staticBody ) return;
	if ( v.x * v.x + v.y * v.y > 0.0f ) h_wakeBody( w, b );
	if ( b->setIndex != H_AWAKE_SET ) return;
	b->linearVelocity = v;
	if ( w->devReady )
	{
		int rc = b2gDev_SetBodyVelocity( w->dev, b->localIndex, v.x, v.y, 0.0f, 1 );
		if ( rc != 0 ) h_fail( w, "set velocity", rc );
	}
}

void b2Body_SetAngularVelocity( b2BodyId bodyId, float av )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( b->type == b2_staticBody || ( b->flags & B2G_LOCK_Z ) ) return;
	if ( av != 0.0f ) h_wakeBody( w, b );
	if ( b->setIndex != H_AWAKE_SET ) return;
	b->angularVelocity = av;
	if ( w->devReady )
	{
		int rc = b2gDev_SetBodyVelocity( w->dev, b->localIndex, 0.0f, 0.0f, av, 2 );
		if ( rc != 0 ) h_fail( w, "set velocity", rc );
	}
}

/* body.c:713-768: teleport; shapes get new boxes and move in the broadphase when they
   leave their fat box */
void b2Body_SetTransform( b2BodyId bodyId, b2Pos position, b2Rot rotation )
{
	h_world* w = h_worlds + bodyId.world0;
	if ( w->locked ) return;
	h_markHostChanged( w );
	h_body* b = h_getBody( bodyId );
	b->transform.p = position;
	b->transform.q = rotation;
	b->center = h_transformWorldPoint( b->transform, b->localCenter );
	for ( int sid = b->headShapeId; sid != B2_NULL_INDEX; sid = w->shapes.data[sid].nextShapeId )
	{
		h_shape* s = w->shapes.data + sid;
		b2AABB aabb = h_computeFatShapeAABB( s, b->transform, H_SPECULATIVE_DISTANCE );
		s->aabb = aabb;
		if ( h_aabbContains( s->fatAABB, aabb ) ) continue;
		float margin = s->aabbMargin;
		b2AABB fat = { { aabb.lowerBound.x - margin, aabb.lowerBound.y - margin },
					   { aabb.upperBound.x + margin, aabb.upperBound.y + margin } };
		s->fatAABB = fat;
		if ( s->proxyKey != B2_NULL_INDEX )
		{
			h_treeMoveProxy( w->trees + H_PROXY_TYPE( s->proxyKey ), H_PROXY_ID( s->proxyKey ), fat );
			h_bufferMove( w, s->proxyKey );
		}
	}
}

/* ---- destruction (body.c:346-430, shape.c:322-437, joint.c:721-840, shape.c:582-640) ---- */

static void h_updateBodyMassData( h_world* w, h_body* body );

/* broad_phase.c:80-126: the proxy leaves the move buffer (swap-removal, as the reference
   does) and its tree */
static void h_destroyProxy( h_world* w, h_shape* s )
{
	if ( s->proxyKey == B2_NULL_INDEX ) return;
	int type = H_PROXY_TYPE( s->proxyKey ), id = H_PROXY_ID( s->proxyKey );
	if ( h_bitGet( w->movedProxies + type, id ) )
	{
		h_bitClear( w->movedProxies + type, id );
		for ( int i = 0; i < w->moveArray.count; ++i )
			if ( w->moveArray.data[i] == s->proxyKey )
			{
				h_removeSwap( w->moveArray, i );
				break;
			}
	}
	h_treeDestroyProxy( w->trees + type, id );
	s->proxyKey = B2_NULL_INDEX;
}

/* sensor.c:388-420: a destroyed sensor ends its overlaps; the last sensor takes its slot */
static void h_destroySensor( h_world* w, h_shape* s )
{
	h_sensor* sensor = w->sensors.data + s->sensorIndex;
	for ( int i = 0; i < sensor->overlaps2.count; ++i )
	{
		b2SensorEndTouchEvent ev = { { s->id + 1, w->worldId, s->generation },
									 { sensor->overlaps2.data[i].shapeId + 1, w->worldId, sensor->overlaps2.data[i].generation } };
		h_push( w->sensorEndEvents[w->endEventArrayIndex], ev );
	}
	h_free( sensor->overlaps1 );
	h_free( sensor->overlaps2 );
	h_free( sensor->hits );
	int slot = s->sensorIndex;
	int moved = h_removeSwap( w->sensors, slot );
	if ( moved != B2_NULL_INDEX ) w->shapes.data[w->sensors.data[slot].shapeId].sensorIndex = slot;
	s->sensorIndex = B2_NULL_INDEX;
}

/* shape.c:322-410 */
static void h_destroyShapeInternal( h_world* w, h_shape* s, h_body* body )
{
	int shapeId = s->id;
	if ( s->prevShapeId != B2_NULL_INDEX ) w->shapes.data[s->prevShapeId].nextShapeId = s->nextShapeId;
	if ( s->nextShapeId != B2_NULL_INDEX ) w->shapes.data[s->nextShapeId].prevShapeId = s->prevShapeId;
	if ( shapeId == body->headShapeId ) body->headShapeId = s->nextShapeId;
	body->shapeCount -= 1;
	h_destroyProxy( w, s );
	int key = body->headContactKey;
	while ( key != B2_NULL_INDEX )
	{
		h_contact* c = w->contacts.data + ( key >> 1 );
		key = c->edges[key & 1].nextKey;
		if ( c->shapeIdA == shapeId || c->shapeIdB == shapeId ) h_destroyContact( w, c );
	}
	if ( s->sensorIndex != B2_NULL_INDEX ) h_destroySensor( w, s );
	h_freeId( &w->shapeIdPool, shapeId );
	s->id = B2_NULL_INDEX;
}

void b2DestroyShape( b2ShapeId shapeId, bool updateBodyMass )
{
	h_world* w = h_worlds + shapeId.world0;
	if ( w->locked ) return;
	h_shape* s = w->shapes.data + ( shapeId.index1 - 1 );
	/* a segment of a chain goes with its chain (shape.c:421-426) */
	if ( s->type == b2_chainSegmentShape && s->chainSegment.chainId != B2_NULL_INDEX ) return;
	h_markHostChanged( w );
	h_body* body = w->bodies.data + s->bodyId;
	h_destroyShapeInternal( w, s, body );
	if ( updateBodyMass ) h_updateBodyMassData( w, body );
}

void b2DestroyChain( b2ChainId chainId )
{
	h_world* w = h_worlds + chainId.world0;
	if ( w->locked ) return;
	h_markHostChanged( w );
	h_chain* chain = w->chains.data + ( chainId.index1 - 1 );
	h_body* body = w->bodies.data + chain->bodyId;
	int* link = &body->headChainId;
	while ( *link != B2_NULL_INDEX && *link != chain->id ) link = &w->chains.data[*link].nextChainId;
	if ( *link == B2_NULL_INDEX ) return;
	*link = chain->nextChainId;
	for ( int i = 0; i < chain->count; ++i ) h_destroyShapeInternal( w, w->shapes.data + chain->shapeIndices[i], body );
	free( chain->shapeIndices );
	chain->shapeIndices = NULL;
	h_freeId( &w->chainIdPool, chain->id );
	chain->id = B2_NULL_INDEX;
}

/* joint.c:721-821 */
static void h_destroyJointInternal( h_world* w, h_joint* j )
{
	int jointId = j->jointId;
	h_body* bodies[2];
	for ( int e = 0; e < 2; ++e )
	{
		h_jointEdge* edge = j->edges + e;
		h_body* body = w->bodies.data + edge->bodyId;
		bodies[e] = body;
		if ( edge->prevKey != B2_NULL_INDEX ) w->joints.data[edge->prevKey >> 1].edges[edge->prevKey & 1].nextKey = edge->nextKey;
		if ( edge->nextKey != B2_NULL_INDEX ) w->joints.data[edge->nextKey >> 1].edges[edge->nextKey & 1].prevKey = edge->prevKey;
		if ( body->headJointKey == ( ( jointId << 1 ) | e ) ) body->headJointKey = edge->nextKey;
		body->jointCount -= 1;
	}
	if ( j->islandId != B2_NULL_INDEX ) h_unlinkJoint( w, j );
	if ( j->setIndex == H_AWAKE_SET )
	{
		h_removeJointFromGraph( w, j->edges[0].bodyId, j->edges[1].bodyId, j->colorIndex, j->localIndex );
	}
	else
	{
		h_intArray* list = j->setIndex == H_STATIC_SET ? &w->staticJointIds : &w->sets.data[j->setIndex].jointIds;
		int localIndex = j->localIndex;
		int moved = h_removeSwap( *list, localIndex );
		if ( moved != B2_NULL_INDEX ) w->joints.data[list->data[localIndex]].localIndex = localIndex;
		if ( j->setIndex == H_STATIC_SET ) w->staticJointCount -= 1;
	}
	j->setIndex = B2_NULL_INDEX;
	j->localIndex = B2_NULL_INDEX;
	j->colorIndex = B2_NULL_INDEX;
	j->jointId = B2_NULL_INDEX;
	h_freeId( &w->jointIdPool, jointId );
	w->jointsDirty = 1;
	h_wakeBody( w, bodies[0] );
	h_wakeBody( w, bodies[1] );
}

void b2DestroyJoint( b2JointId jointId )
{
	h_world* w = h_worlds + jointId.world0;
	if ( w->locked ) return;
	h_markHostChanged( w );
	h_destroyJointInternal( w, w->joints.data + ( jointId.index1 - 1 ) );
}

/* body.c:346-430 */
void b2DestroyBody( b2BodyId bodyId )
{
	h_world* w = h_worlds + bodyId.world0;
	if ( w->locked ) return;
	h_markHostChanged( w );
	h_body* body = h_getBody( bodyId );
	int key = body->headJointKey;
	while ( key != B2_NULL_INDEX )
	{
		h_joint* j = w->joints.data + ( key >> 1 );
		key = j->edges[key & 1].nextKey;
		h_destroyJointInternal( w, j );
	}
	key = body->headContactKey;
	while ( key != B2_NULL_INDEX )
	{
		h_contact* c = w->contacts.data + ( key >> 1 );
		key = c->edges[key & 1].nextKey;
		h_destroyContact( w, c );
	}
	for ( int sid = body->headShapeId; sid != B2_NULL_INDEX; )
	{
		h_shape* s = w->shapes.data + sid;
		if ( s->sensorIndex != B2_NULL_INDEX ) h_destroySensor( w, s );
		h_destroyProxy( w, s );
		h_freeId( &w->shapeIdPool, sid );
		s->id = B2_NULL_INDEX;
		sid = s->nextShapeId;
	}
	for ( int cid = body->headChainId; cid != B2_NULL_INDEX; )
	{
		h_chain* chain = w->chains.data + cid;
		free( chain->shapeIndices );
		chain->shapeIndices = NULL;
		h_freeId( &w->chainIdPool, cid );
		chain->id = B2_NULL_INDEX;
		cid = chain->nextChainId;
	}
	h_removeBodyFromIsland( w, body );
	int localIndex = body->localIndex;
	if ( body->setIndex == H_AWAKE_SET || body->setIndex == H_STATIC_SET || body->setIndex >= H_FIRST_SLEEPING_SET )
	{
		h_intArray* list = body->setIndex == H_AWAKE_SET	 ? &w->awakeBodyIds
						   : body->setIndex == H_STATIC_SET ? &w->staticBodyIds
															 : &w->sets.data[body->setIndex].bodyIds;
		int moved = h_removeSwap( *list, localIndex );
		if ( moved != B2_NULL_INDEX ) w->bodies.data[list->data[localIndex]].localIndex = localIndex;
		if ( body->setIndex == H_STATIC_SET ) w->staticCount -= 1;
		if ( body->setIndex >= H_FIRST_SLEEPING_SET && list->count == 0 ) h_freeSleepingSet( w, body->setIndex );
	}
	h_freeId( &w->bodyIdPool, body->id );
	body->setIndex = B2_NULL_INDEX;
	body->localIndex = B2_NULL_INDEX;
	body->id = B2_NULL_INDEX;
}

/* ---- forces and impulses (body.c:935-1090) ---- */

/* a force, torque or impulse reaches a dynamic body that is awake (after waking it when
   asked); returns whether it applies */
static int h_applyTarget( h_world* w, h_body* b, bool wake )
{
	if ( b->type != b2_dynamicBody || b->setIndex == H_DISABLED_SET ) return 0;
	if ( wake && b->setIndex >= H_FIRST_SLEEPING_SET ) h_wakeBody( w, b );
	return b->setIndex == H_AWAKE_SET;
}

static void h_pushForce( h_world* w, h_body* b )
{
	h_push( w->forcedBodies, b->id );
	if ( w->devReady )
	{
		int rc = b2gDev_SetBodyForce( w->dev, b->localIndex, b->force.x, b->force.y, b->torque );
		if ( rc != 0 ) h_fail( w, "set force", rc );
	}
}

void b2Body_ApplyForce( b2BodyId bodyId, b2Vec2 force, b2Pos point, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( h_applyTarget( w, b, wake ) == 0 ) return;
	h_syncFromDevice( w );
	b->force = h_add( b->force, force );
	b->torque += h_cross( h_sub( point, b->center ), force );
	h_pushForce( w, b );
}

void b2Body_ApplyForceToCenter( b2BodyId bodyId, b2Vec2 force, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( h_applyTarget( w, b, wake ) == 0 ) return;
	b->force = h_add( b->force, force );
	h_pushForce( w, b );
}

void b2Body_ApplyTorque( b2BodyId bodyId, float torque, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( h_applyTarget( w, b, wake ) == 0 ) return;
	b->torque += torque;
	h_pushForce( w, b );
}

void b2Body_ClearForces( b2BodyId bodyId )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	b->force = h_v( 0.0f, 0.0f );
	b->torque = 0.0f;
	if ( b->setIndex == H_AWAKE_SET ) h_pushForce( w, b );
}

/* new velocities of an awake body: host record and device state */
static void h_setVelocities( h_world* w, h_body* b, b2Vec2 v, float av )
{
	b->linearVelocity = v;
	b->angularVelocity = av;
	if ( w->devReady )
	{
		int rc = b2gDev_SetBodyVelocity( w->dev, b->localIndex, v.x, v.y, 0.0f, 1 );
		if ( rc == 0 ) rc = b2gDev_SetBodyVelocity( w->dev, b->localIndex, 0.0f, 0.0f, av, 2 );
		if ( rc != 0 ) h_fail( w, "set velocity", rc );
	}
}

/* body.h b2LimitVelocity: clamp the linear speed to the world's maximum */
static b2Vec2 h_limitVelocity( b2Vec2 v, float maxLinearSpeed )
{
	float v2 = h_lengthSq( v );
	if ( v2 > maxLinearSpeed * maxLinearSpeed ) v = h_mulSV( maxLinearSpeed / sqrtf( v2 ), v );
	return v;
}

void b2Body_ApplyLinearImpulse( b2BodyId bodyId, b2Vec2 impulse, b2Pos point, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( h_applyTarget( w, b, wake ) == 0 ) return;
	h_syncFromDevice( w );
	b2Vec2 v = h_mulAdd( b->linearVelocity, b->invMass, impulse );
	float av = b->angularVelocity + b->invInertia * h_cross( h_sub( point, b->center ), impulse );
	h_setVelocities( w, b, h_limitVelocity( v, w->maxLinearSpeed ), av );
}

void b2Body_ApplyLinearImpulseToCenter( b2BodyId bodyId, b2Vec2 impulse, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( h_applyTarget( w, b, wake ) == 0 ) return;
	h_syncFromDevice( w );
	b2Vec2 v = h_mulAdd( b->linearVelocity, b->invMass, impulse );
	h_setVelocities( w, b, h_limitVelocity( v, w->maxLinearSpeed ), b->angularVelocity );
}

void b2Body_ApplyAngularImpulse( b2BodyId bodyId, float impulse, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( h_applyTarget( w, b, wake ) == 0 ) return;
	h_syncFromDevice( w );
	h_setVelocities( w, b, b->linearVelocity, b->angularVelocity + b->invInertia * impulse );
}

/* body.c:842-920: velocities that carry the body to the target transform over timeStep */
void b2Body_SetTargetTransform( b2BodyId bodyId, b2WorldTransform target, float timeStep, bool wake )
{
	h_world* w = h_worlds + bodyId.world0;
	h_body* b = h_getBody( bodyId );
	if ( b->setIndex == H_DISABLED_SET || b->type == b2_staticBody || timeStep <= 0.0f ) return;
	if ( b->setIndex != H_AWAKE_SET && wake == false ) return;
	h_syncFromDevice( w );
	b2Vec2 targetCenter = h_transformWorldPoint( target, b->localCenter );
	b2Vec2 delta = h_sub( targetCenter, b->center );
	float invTimeStep = 1.0f / timeStep;
	b2Vec2 v = h_mulSV( invTimeStep, delta );
	b2Rot q1 = b->transform.q, q2 = target.q;
	float s = q1.c * q2.s - q1.s * q2.c;
	float c = q1.c * q2.c + q1.s * q2.s;
	float av = invTimeStep * b2Atan2( s, c );
	if ( b->setIndex != H_AWAKE_SET )
	{
		float maxVelocity = h_length( v ) + h_abs( av ) * b->maxExtent;
		if ( maxVelocity < b->sleepThreshold ) return;
		h_wakeBody( w, b );
	}
	h_setVelocities( w, b, v, av );
}

float b2Body_GetMass( b2BodyId bodyId ) { return h_getBody( bodyId )->mass; }

float b2Body_GetRotationalInertia( b2BodyId bodyId ) { return h_getBody( bodyId )->inertia; }

b2Vec2 b2Body_GetLocalCenter( b2BodyId bodyId ) { return h_getBody( bodyId )->localCenter; }

b2Pos b2Body_GetWorldCenter( b2BodyId bodyId )
{
	h_syncFromDevice( h_worlds + bodyId.world0 );
	return h_getBody( bodyId )->center;
}

bool b2Body_IsAwake( b2BodyId bodyId ) { return h_getBody( bodyId )->setIndex == H_AWAKE_SET; }

/* body.c:1550-1575: wake the body's set, or put its island to sleep (split first when
   constraints were removed from it) */
void b2Body_SetAwake( b2BodyId bodyId, bool awake )
{
	h_world* w = h_worlds + bodyId.world0;
	if ( w->inUse == 0 || w->locked ) return;
	h_body* b = h_getBody( bodyId );
	if ( awake && b->setIndex >= H_FIRST_SLEEPING_SET )
	{
		h_wakeBody( w, b );
	}
	else if ( awake == false && b->setIndex == H_AWAKE_SET )
	{
		h_markHostChanged( w );
		if ( w->islands.data[b->islandId].constraintRemoveCount > 0 ) h_splitIsland( w, b->islandId );
		h_trySleepIsland( w, b->islandId );
	}
}

/* body.c b2Body_GetSleepThreshold / b2Body_SetSleepThreshold */
float b2Body_GetSleepThreshold( b2BodyId bodyId ) { return h_getBody( bodyId )->sleepThreshold; }

/* body.c b2Body_GetShapeCount / b2Body_GetShapes: the body's shape list, head first */
int b2Body_GetShapeCount( b2BodyId bodyId ) { return h_getBody( bodyId )->shapeCount; }

int b2Body_GetShapes( b2BodyId bodyId, b2ShapeId* shapeArray, int capacity )
{
	h_world* w = h_worlds + bodyId.world0;
	int n = 0;
	for ( int id = h_getBody( bodyId )->headShapeId; id != B2_NULL_INDEX && n < capacity; id = w->shapes.data[id].nextShapeId )
	{
		b2ShapeId sid = { id + 1, bodyId.world0, w->shapes.data[id].generation };
		shapeArray[n++] = sid;
	}
	return n;
}

/* body.c:524-650 */
static void h_updateBodyMassData( h_world* w, h_body* body )
{
	body->flags &= ~B2G_DIRTY_MASS;
	body->mass = 0.0f;
	body->inertia = 0.0f;
	body->invMass = 0.0f;
	body->invInertia = 0.0f;
	body->localCenter = h_v( 0.0f, 0.0f );
	body->minExtent = H_HUGE;
	body->maxExtent = 0.0f;
	if ( body->type != b2_dynamicBody )
	{
		body->center = body->transform.p;
		if ( body->type == b2_kinematicBody )
		{
			int sid = body->headShapeId;
			while ( sid != B2_NULL_INDEX )
			{
				const h_shape* s = w->shapes.data + sid;
				float mn, mx;
				h_computeShapeExtent( s, h_v( 0.0f, 0.0f ), &mn, &mx );
				body->minExtent = h_min( body->minExtent, mn );
				body->maxExtent = h_max( body->maxExtent, mx );
				sid = s->nextShapeId;
			}
		}
		return;
	}
	int shapeCount = body->shapeCount;
	b2MassData* masses = calloc( (size_t)( shapeCount > 0 ? shapeCount : 1 ), sizeof( b2MassData ) );
	b2Vec2 localCenter = h_v( 0.0f, 0.0f );
	int sid = body->headShapeId;
	int si = 0;
	while ( sid != B2_NULL_INDEX )
	{
		const h_shape* s = w->shapes.data + sid;
		sid = s->nextShapeId;
		if ( s->density == 0.0f )
		{
			si += 1;
			continue;
		}
		b2MassData md = h_computeShapeMass( s );
		body->mass += md.mass;
		localCenter = h_mulAdd( localCenter, md.mass, md.center );
		masses[si++] = md;
	}
	if ( body->mass > 0.0f )
	{
		body->invMass = 1.0f / body->mass;
		localCenter = h_mulSV( body->invMass, localCenter );
	}
	for ( si = 0; si < shapeCount; ++si )
	{
		b2MassData md = masses[si];
		if ( md.mass == 0.0f ) continue;
		b2Vec2 offset = h_sub( localCenter, md.center );
		float inertia = md.rotationalInertia + md.mass * h_dot( offset, offset );
		body->inertia += inertia;
	}
	free( masses );
	if ( body->inertia > 0.0f && ( body->flags & B2G_LOCK_Z ) == 0 )
	{
		body->invInertia = 1.0f / body->inertia;
	}
	else
	{
		body->inertia = 0.0f;
		body->invInertia = 0.0f;
	}
	b2Vec2 oldCenter = body->center;
	body->localCenter = localCenter;
	body->center = h_transformWorldPoint( body->transform, body->localCenter );
	if ( body->setIndex == H_AWAKE_SET )
	{
		b2Vec2 dl = h_crossSV( body->angularVelocity, h_sub( body->center, oldCenter ) );
		body->linearVelocity = h_add( body->linearVelocity, dl );
	}
	sid = body->headShapeId;
	while ( sid != B2_NULL_INDEX )
	{
		const h_shape* s = w->shapes.data + sid;
		float mn, mx;
		h_computeShapeExtent( s, localCenter, &mn, &mx );
		body->minExtent = h_min( body->minExtent, mn );
		body->maxExtent = h_max( body->maxExtent, mx );
		sid = s->nextShapeId;
	}
}

/* ---------------- move buffer (broad_phase.h:70-80) ---------------- */
void h_bufferMove( h_world* w, int proxyKey )
{
	int type = H_PROXY_TYPE( proxyKey );
	int id = H_PROXY_ID( proxyKey );
	if ( h_bitGet( w->movedProxies + type, id ) == 0 )
	{
		h_bitSet1( w->movedProxies + type, id );
		h_push( w->moveArray, proxyKey );
	}
}

/* ---------------- shapes (shape.c:85-270, :1034-1044) ---------------- */
/* shape.c:115-205 b2CreateShapeInternal, plus the mass update or dirty-mass mark of
   b2CreateShape (shape.c:207-240) unless `internal` (a chain's segments) */
static b2ShapeId h_createShapeImpl( b2BodyId bodyId, const b2ShapeDef* def, const void* geometry, b2ShapeType type,
									int internal )
{
	h_world* w = h_worlds + bodyId.world0;
	h_markHostChanged( w );
	h_body* body = h_getBody( bodyId );
	b2Transform transform = body->transform;
	int shapeId = h_allocId( &w->shapeIdPool );
	if ( shapeId == w->shapes.count )
	{
		h_shape z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->shapes, z );
	}
	h_shape* s = w->shapes.data + shapeId;
	uint16_t generation = s->generation;
	memset( s, 0, sizeof( *s ) );
	switch ( type )
	{
		case b2_capsuleShape: s->capsule = *(const b2Capsule*)geometry; break;
		case b2_circleShape: s->circle = *(const b2Circle*)geometry; break;
		case b2_polygonShape: s->polygon = *(const b2Polygon*)geometry; break;
		case b2_segmentShape: s->segment = *(const b2Segment*)geometry; break;
		case b2_chainSegmentShape: s->chainSegment = *(const b2ChainSegment*)geometry; break;
		default: break;
	}
	s->id = shapeId;
	s->bodyId = body->id;
	s->type = type;
	s->density = def->density;
	s->material = def->material;
	s->filter = def->filter;
	s->userData = def->userData;
	s->enableContactEvents = def->enableContactEvents;
	s->enableHitEvents = def->enableHitEvents;
	s->isSensor = def->isSensor;
	s->enableSensorEvents = def->enableSensorEvents;
	s->sensorIndex = B2_NULL_INDEX;
	s->proxyKey = B2_NULL_INDEX;
	s->localCentroid = h_getShapeCentroid( s );
	s->aabbMargin = h_computeShapeMargin( s );
	s->generation = generation + 1;
	{
		b2BodyType proxyType = body->type;
		b2AABB aabb = h_computeFatShapeAABB( s, transform, H_SPECULATIVE_DISTANCE );
		s->aabb = aabb;
		float margin = proxyType == b2_staticBody ? H_SPECULATIVE_DISTANCE : s->aabbMargin;
		b2AABB fat = { { aabb.lowerBound.x - margin, aabb.lowerBound.y - margin },
					   { aabb.upperBound.x + margin, aabb.upperBound.y + margin } };
		s->fatAABB = fat;
		int proxyId = h_treeCreateProxy( w->trees + proxyType, s->fatAABB, s->filter.categoryBits, (uint64_t)shapeId );
		s->proxyKey = H_PROXY_KEY( proxyId, proxyType );
		if ( proxyType != b2_staticBody || def->invokeContactCreation || def->isSensor ) h_bufferMove( w, s->proxyKey );
	
	}
	if ( body->headShapeId != B2_NULL_INDEX ) w->shapes.data[body->headShapeId].prevShapeId = shapeId;
	s->prevShapeId = B2_NULL_INDEX;
	s->nextShapeId = body->headShapeId;
	body->headShapeId = shapeId;
	body->shapeCount += 1;
	if ( def->isSensor ) h_createSensor( w, s );
	if ( internal == 0 )
	{
		if ( def->updateBodyMass ) h_updateBodyMassData( w, body );
		else body->flags |= B2G_DIRTY_MASS;
	}
	b2ShapeId id = { s->id + 1, bodyId.world0, s->generation };
	return id;
}

static b2ShapeId h_createShape( b2BodyId bodyId, const b2ShapeDef* def, const void* geometry, b2ShapeType type )
{
	return h_createShapeImpl( bodyId, def, geometry, type, 0 );
}

b2ShapeId b2CreateCircleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Circle* circle )
{
	return h_createShape( bodyId, def, circle, b2_circleShape );
}

b2ShapeId b2CreateCapsuleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Capsule* capsule )
{
	if ( h_distanceSq( capsule->center1, capsule->center2 ) <= H_LINEAR_SLOP * H_LINEAR_SLOP )
	{
		b2ShapeId nullId = { 0, 0, 0 };
		return nullId;
	}
	return h_createShape( bodyId, def, capsule, b2_capsuleShape );
}

b2ShapeId b2CreatePolygonShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Polygon* polygon )
{
	return h_createShape( bodyId, def, polygon, b2_polygonShape );
}

b2ShapeId b2CreateSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Segment* segment )
{
	if ( h_distanceSq( segment->point1, segment->point2 ) <= H_LINEAR_SLOP * H_LINEAR_SLOP )
	{
		b2ShapeId nullId = { 0, 0, 0 };
		return nullId;
	}
	return h_createShape( bodyId, def, segment, b2_segmentShape );
}

/* ---- chains (shape.c:300-315, 439-640) ---- */

b2ChainDef b2DefaultChainDef( void )
{
	static const b2SurfaceMaterial defaultMaterial = { 0.6f, 0.0f, 0.0f, 0.0f, 0, 0 };
	b2ChainDef def;
	memset( &def, 0, sizeof( def ) );
	def.materials = &defaultMaterial;
	def.materialCount = 1;
	def.filter = b2DefaultFilter();
	def.internalValue = 1152023;
	return def;
}

b2ShapeId b2CreateChainSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2ChainSegment* chainSegment )
{
	if ( h_distanceSq( chainSegment->segment.point1, chainSegment->segment.point2 ) <= H_LINEAR_SLOP * H_LINEAR_SLOP )
	{
		b2ShapeId nullId = { 0, 0, 0 };
		return nullId;
	}
	b2ChainSegment local = *chainSegment;
	local.chainId = B2_NULL_INDEX;
	return h_createShape( bodyId, def, &local, b2_chainSegmentShape );
}

/* one segment of a chain: the chain's filter and sensor flag, the segment's material, no
   contact or hit events, the body's mass left as it is */
static int h_chainSegmentShape( b2BodyId bodyId, const b2ChainDef* def, int materialIndex, b2Vec2 g1, b2Vec2 p1, b2Vec2 p2,
								b2Vec2 g2, int chainId )
{
	b2ShapeDef shapeDef = b2DefaultShapeDef();
	shapeDef.userData = def->userData;
	shapeDef.filter = def->filter;
	shapeDef.enableSensorEvents = def->enableSensorEvents;
	shapeDef.enableContactEvents = false;
	shapeDef.enableHitEvents = false;
	shapeDef.updateBodyMass = false;
	shapeDef.material = def->materials[materialIndex];
	b2ChainSegment seg = { g1, { p1, p2 }, g2, chainId };
	b2ShapeId id = h_createShapeImpl( bodyId, &shapeDef, &seg, b2_chainSegmentShape, 1 );
	return id.index1 - 1;
}

b2ChainId b2CreateChain( b2BodyId bodyId, const b2ChainDef* def )
{
	b2ChainId nullId = { 0, 0, 0 };
	h_world* w = h_worlds + bodyId.world0;
	if ( w->locked || def->count < 4 ) return nullId;
	h_markHostChanged( w );
	h_body* body = h_getBody( bodyId );
	int chainId = h_allocId( &w->chainIdPool );
	if ( chainId == w->chains.count )
	{
		h_chain z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->chains, z );
	}
	h_chain* chain = w->chains.data + chainId;
	chain->id = chainId;
	chain->bodyId = body->id;
	chain->nextChainId = body->headChainId;
	chain->generation += 1;
	body->headChainId = chainId;
	const b2Vec2* pts = def->points;
	int n = def->count;
	int one = def->materialCount == 1;
	if ( def->isLoop )
	{
		chain->count = n;
		chain->shapeIndices = malloc( (size_t)n * sizeof( int ) );
		int prev = n - 1;
		for ( int i = 0; i < n - 2; ++i )
		{
			chain->shapeIndices[i] =
				h_chainSegmentShape( bodyId, def, one ? 0 : i, pts[prev], pts[i], pts[i + 1], pts[i + 2], chainId );
			prev = i;
		}
		chain->shapeIndices[n - 2] =
			h_chainSegmentShape( bodyId, def, one ? 0 : n - 2, pts[n - 3], pts[n - 2], pts[n - 1], pts[0], chainId );
		chain->shapeIndices[n - 1] =
			h_chainSegmentShape( bodyId, def, one ? 0 : n - 1, pts[n - 2], pts[n - 1], pts[0], pts[1], chainId );
	}
	else
	{
		/* the first and last points only shape the ends (ghost vertices); the material of a
		   segment is that of its leading point */
		chain->count = n - 3;
		chain->shapeIndices = malloc( (size_t)( n - 3 ) * sizeof( int ) );
		for ( int i = 0; i < n - 3; ++i )
			chain->shapeIndices[i] =
				h_chainSegmentShape( bodyId, def, one ? 0 : i + 1, pts[i], pts[i + 1], pts[i + 2], pts[i + 3], chainId );
	}
	b2ChainId id = { chainId + 1, w->worldId, chain->generation };
	return id;
}

bool b2Chain_IsValid( b2ChainId id )
{
	if ( id.world0 >= H_MAX_WORLDS ) return false;
	h_world* w = h_worlds + id.world0;
	if ( w->inUse == 0 || id.index1 < 1 || id.index1 > w->chains.count ) return false;
	const h_chain* chain = w->chains.data + ( id.index1 - 1 );
	return chain->id == id.index1 - 1 && chain->generation == id.generation;
}

int b2Chain_GetSegmentCount( b2ChainId chainId ) { return h_worlds[chainId.world0].chains.data[chainId.index1 - 1].count; }

int b2Chain_GetSegments( b2ChainId chainId, b2ShapeId* segmentArray, int capacity )
{
	h_world* w = h_worlds + chainId.world0;
	const h_chain* chain = w->chains.data + ( chainId.index1 - 1 );
	int count = chain->count < capacity ? chain->count : capacity;
	for ( int i = 0; i < count; ++i )
	{
		const h_shape* s = w->shapes.data + chain->shapeIndices[i];
		b2ShapeId id = { s->id + 1, chainId.world0, s->generation };
		segmentArray[i] = id;
	}
	return count;
}

b2ShapeType b2Shape_GetType( b2ShapeId shapeId ) { return h_worlds[shapeId.world0].shapes.data[shapeId.index1 - 1].type; }

b2ChainSegment b2Shape_GetChainSegment( b2ShapeId shapeId )
{
	return h_worlds[shapeId.world0].shapes.data[shapeId.index1 - 1].chainSegment;
}

b2ChainId b2Shape_GetParentChain( b2ShapeId shapeId )
{
	h_world* w = h_worlds + shapeId.world0;
	const h_shape* s = w->shapes.data + ( shapeId.index1 - 1 );
	b2ChainId nullId = { 0, 0, 0 };
	if ( s->type != b2_chainSegmentShape || s->chainSegment.chainId == B2_NULL_INDEX ) return nullId;
	int chainId = s->chainSegment.chainId;
	b2ChainId id = { chainId + 1, shapeId.world0, w->chains.data[chainId].generation };
	return id;
}

void b2Shape_SetFriction( b2ShapeId shapeId, float friction )
{
	h_world* w = h_worlds + shapeId.world0;
	h_markHostChanged( w );
	w->shapes.data[shapeId.index1 - 1].material.friction = friction;
}

float b2Shape_GetFriction( b2ShapeId shapeId )
{
	return h_worlds[shapeId.world0].shapes.data[shapeId.index1 - 1].material.friction;
}

/* ---------------- contact register table (contact.c:188-206) ---------------- */
/* shape types: circle 0, capsule 1, segment 2, polygon 3, chain segment 4. Segments and
   chain segments collide with circles, capsules and polygons only, as shape A. */
int h_canCollide( b2ShapeType a, b2ShapeType b )
{
	if ( (int)a > 4 || (int)b > 4 ) return 0;
	int lineA = a == b2_segmentShape || a == b2_chainSegmentShape;
	int lineB = b == b2_segmentShape || b == b2_chainSegmentShape;
	return !( lineA && lineB );
}

int h_isPrimary( b2ShapeType a, b2ShapeType b )
{
	static const int prim[5][5] = {
		{ 1, 0, 0, 0, 0 },
		{ 1, 1, 0, 0, 0 },
		{ 1, 1, 0, 1, 0 },
		{ 1, 1, 0, 1, 0 },
		{ 1, 1, 0, 1, 0 },
	};
	if ( (int)a > 4 || (int)b > 4 ) return 0;
	return prim[a][b];
}

/* ---------------- contacts (contact.c:214-501) ---------------- */
void h_createContact( h_world* w, h_shape* shapeA, h_shape* shapeB )
{
	if ( h_canCollide( shapeA->type, shapeB->type ) == 0 ) return;
	if ( h_isPrimary( shapeA->type, shapeB->type ) == 0 )
	{
		h_createContact( w, shapeB, shapeA );
		return;
	}
	h_body* bodyA = w->bodies.data + shapeA->bodyId;
	h_body* bodyB = w->bodies.data + shapeB->bodyId;
	int contactId = h_allocId( &w->contactIdPool );
	if ( contactId == w->contacts.count )
	{
		h_contact z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->contacts, z );
	}
	h_contact* c = w->contacts.data + contactId;
	c->contactId = contactId;
	c->generation += 1;
	/* contact.c:241-252: in the awake set when a body is awake, else in the disabled set */
	int awake = bodyA->setIndex == H_AWAKE_SET || bodyB->setIndex == H_AWAKE_SET;
	c->setIndex = awake ? H_AWAKE_SET : H_DISABLED_SET;
	c->colorIndex = B2_NULL_INDEX;
	c->localIndex = awake ? w->awakeContactIds.count : w->disabledContactIds.count;
	c->islandId = B2_NULL_INDEX;
	c->islandIndex = B2_NULL_INDEX;
	c->shapeIdA = shapeA->id;
	c->shapeIdB = shapeB->id;
	c->flags = 0;
	if ( ( bodyA->flags & B2G_ENABLE_RECYCLING ) && ( bodyB->flags & B2G_ENABLE_RECYCLING ) ) c->flags |= B2G_C_RECYCLE;
	if ( shapeA->enableContactEvents || shapeB->enableContactEvents ) c->flags |= B2G_C_ENABLE_EVENTS;
	{
		c->edges[0].bodyId = shapeA->bodyId;
		c->edges[0].prevKey = B2_NULL_INDEX;
		c->edges[0].nextKey = bodyA->headContactKey;
		int keyA = ( contactId << 1 ) | 0;
		int head = bodyA->headContactKey;
		if ( head != B2_NULL_INDEX ) w->contacts.data[head >> 1].edges[head & 1].prevKey = keyA;
		bodyA->headContactKey = keyA;
		bodyA->contactCount += 1;
	}
	{
		c->edges[1].bodyId = shapeB->bodyId;
		c->edges[1].prevKey = B2_NULL_INDEX;
		c->edges[1].nextKey = bodyB->headContactKey;
		int keyB = ( contactId << 1 ) | 1;
		int head = bodyB->headContactKey;
		if ( head != B2_NULL_INDEX ) w->contacts.data[head >> 1].edges[head & 1].prevKey = keyB;
		bodyB->headContactKey = keyB;
		bodyB->contactCount += 1;
	}
	h_pairSetAdd( &w->pairSet, H_SHAPE_PAIR_KEY( shapeA->id, shapeB->id ) );
	if ( awake ) h_push( w->awakeContactIds, contactId );
	else h_push( w->disabledContactIds, contactId );
	b2gContactInit init;
	init.contactId = contactId;
	init.shapeIdA = shapeA->id;
	init.shapeIdB = shapeB->id;
	init.simFlags = c->flags | ( awake ? 0u : (uint32_t)B2G_S_ASLEEP );
	init.friction = sqrtf( shapeA->material.friction * shapeB->material.friction );
	init.restitution = h_max( shapeA->material.restitution, shapeB->material.restitution );
	h_push( w->pendingInits, init );
}

static void h_removeNonTouchingContact( h_world* w, int localIndex )
{
	int moved = h_removeSwap( w->awakeContactIds, localIndex );
	if ( moved != B2_NULL_INDEX ) w->contacts.data[w->awakeContactIds.data[localIndex]].localIndex = localIndex;
}

void h_destroyContact( h_world* w, h_contact* c )
{
	h_pairSetRemove( &w->pairSet, H_SHAPE_PAIR_KEY( c->shapeIdA, c->shapeIdB ) );
	h_contactEdge* eA = c->edges + 0;
	h_contactEdge* eB = c->edges + 1;
	int bodyIdA = eA->bodyId, bodyIdB = eB->bodyId;
	h_body* bodyA = w->bodies.data + bodyIdA;
	h_body* bodyB = w->bodies.data + bodyIdB;
	uint32_t flags = c->flags;
	if ( ( flags & B2G_C_TOUCHING ) && ( flags & B2G_C_ENABLE_EVENTS ) )
	{
		const h_shape* sA = w->shapes.data + c->shapeIdA;
		const h_shape* sB = w->shapes.data + c->shapeIdB;
		b2ContactEndTouchEvent ev;
		memset( &ev, 0, sizeof( ev ) );
		ev.shapeIdA.index1 = sA->id + 1;
		ev.shapeIdA.world0 = w->worldId;
		ev.shapeIdA.generation = sA->generation;
		ev.shapeIdB.index1 = sB->id + 1;
		ev.shapeIdB.world0 = w->worldId;
		ev.shapeIdB.generation = sB->generation;
		ev.contactId.index1 = c->contactId + 1;
		ev.contactId.world0 = w->worldId;
		ev.contactId.generation = c->generation;
		h_push( w->endEvents[w->endEventArrayIndex], ev );
	}
	if ( eA->prevKey != B2_NULL_INDEX ) w->contacts.data[eA->prevKey >> 1].edges[eA->prevKey & 1].nextKey = eA->nextKey;
	if ( eA->nextKey != B2_NULL_INDEX ) w->contacts.data[eA->nextKey >> 1].edges[eA->nextKey & 1].prevKey = eA->prevKey;
	int contactId = c->contactId;
	if ( bodyA->headContactKey == ( ( contactId << 1 ) | 0 ) ) bodyA->headContactKey = eA->nextKey;
	bodyA->contactCount -= 1;
	if ( eB->prevKey != B2_NULL_INDEX ) w->contacts.data[eB->prevKey >> 1].edges[eB->prevKey & 1].nextKey = eB->nextKey;
	if ( eB->nextKey != B2_NULL_INDEX ) w->contacts.data[eB->nextKey >> 1].edges[eB->nextKey & 1].prevKey = eB->prevKey;
	if ( bodyB->headContactKey == ( ( contactId << 1 ) | 1 ) ) bodyB->headContactKey = eB->nextKey;
	bodyB->contactCount -= 1;
	/* contact.c:462-500: leave the island, then the array that holds the contact */
	if ( c->islandId != B2_NULL_INDEX ) h_unlinkContact( w, c );
	if ( c->colorIndex != B2_NULL_INDEX ) h_removeContactFromGraph( w, bodyIdA, bodyIdB, c->colorIndex, c->localIndex );
	else if ( c->setIndex == H_AWAKE_SET ) h_removeNonTouchingContact( w, c->localIndex );
	else
	{
		h_intArray* list = c->setIndex == H_DISABLED_SET ? &w->disabledContactIds : &w->sets.data[c->setIndex].contactIds;
		int localIndex = c->localIndex;
		int moved = h_removeSwap( *list, localIndex );
		if ( moved != B2_NULL_INDEX ) w->contacts.data[list->data[localIndex]].localIndex = localIndex;
	}
	c->contactId = B2_NULL_INDEX;
	c->setIndex = B2_NULL_INDEX;
	c->colorIndex = B2_NULL_INDEX;
	c->localIndex = B2_NULL_INDEX;
	h_freeId( &w->contactIdPool, contactId );
	h_push( w->pendingKills, contactId );
	/* a touching contact that goes away wakes its bodies */
	if ( flags & B2G_C_TOUCHING )
	{
		h_wakeBody( w, w->bodies.data + bodyIdA );
		h_wakeBody( w, w->bodies.data + bodyIdB );
	}
}

/* ---------------- graph coloring (constraint_graph.c:66-291) ---------------- */
void h_addContactToGraph( h_world* w, h_contact* contact )
{
	int colorIndex = B2G_OVERFLOW_INDEX;
	int bodyIdA = contact->edges[0].bodyId, bodyIdB = contact->edges[1].bodyId;
	b2BodyType typeA = w->bodies.data[bodyIdA].type, typeB = w->bodies.data[bodyIdB].type;
	if ( typeA == b2_dynamicBody && typeB == b2_dynamicBody )
	{
		for ( int i = 0; i < B2_GRAPH_COLOR_COUNT - 4; ++i )
		{
			h_color* color = w->colors + i;
			if ( h_bitGet( &color->bodySet, bodyIdA ) || h_bitGet( &color->bodySet, bodyIdB ) ) continue;
			h_bitSet1( &color->bodySet, bodyIdA );
			h_bitSet1( &color->bodySet, bodyIdB );
			colorIndex = i;
			break;
		}
	}
	else if ( typeA == b2_dynamicBody )
	{
		for ( int i = B2G_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			h_color* color = w->colors + i;
			if ( h_bitGet( &color->bodySet, bodyIdA ) ) continue;
			h_bitSet1( &color->bodySet, bodyIdA );
			colorIndex = i;
			break;
		}
	}
	else if ( typeB == b2_dynamicBody )
	{
		for ( int i = B2G_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			h_color* color = w->colors + i;
			if ( h_bitGet( &color->bodySet, bodyIdB ) ) continue;
			h_bitSet1( &color->bodySet, bodyIdB );
			colorIndex = i;
			break;
		}
	}
	h_color* color = w->colors + colorIndex;
	contact->colorIndex = colorIndex;
	contact->localIndex = color->contactIds.count;
	h_push( color->contactIds, contact->contactId );
	w->colorsDirty = 1;
}

void h_removeContactFromGraph( h_world* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex )
{
	h_color* color = w->colors + colorIndex;
	if ( colorIndex != B2G_OVERFLOW_INDEX )
	{
		h_bitClear( &color->bodySet, bodyIdA );
		h_bitClear( &color->bodySet, bodyIdB );
	}
	int moved = h_removeSwap( color->contactIds, localIndex );
	if ( moved != B2_NULL_INDEX ) w->contacts.data[color->contactIds.data[localIndex]].localIndex = localIndex;
	w->colorsDirty = 1;
}

int h_assignJointColor( h_world* w, int bodyIdA, int bodyIdB, b2BodyType typeA, b2BodyType typeB )
{
	if ( typeA == b2_dynamicBody && typeB == b2_dynamicBody )
	{
		for ( int i = 0; i < B2_GRAPH_COLOR_COUNT - 4; ++i )
		{
			h_color* color = w->colors + i;
			if ( h_bitGet( &color->bodySet, bodyIdA ) || h_bitGet( &color->bodySet, bodyIdB ) ) continue;
			h_bitSet1( &color->bodySet, bodyIdA );
			h_bitSet1( &color->bodySet, bodyIdB );
			return i;
		}
	}
	else if ( typeA == b2_dynamicBody )
	{
		for ( int i = B2G_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			h_color* color = w->colors + i;
			if ( h_bitGet( &color->bodySet, bodyIdA ) ) continue;
			h_bitSet1( &color->bodySet, bodyIdA );
			return i;
		}
	}
	else if ( typeB == b2_dynamicBody )
	{
		for ( int i = B2G_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			h_color* color = w->colors + i;
			if ( h_bitGet( &color->bodySet, bodyIdB ) ) continue;
			h_bitSet1( &color->bodySet, bodyIdB );
			return i;
		}
	}
	return B2G_OVERFLOW_INDEX;
}

/* body.c:2076-2110 */
int h_shouldBodiesCollide( h_world* w, h_body* bodyA, h_body* bodyB )
{
	if ( bodyA->type != b2_dynamicBody && bodyB->type != b2_dynamicBody ) return 0;
	int jointKey, otherBodyId;
	if ( bodyA->jointCount < bodyB->jointCount )
	{
		jointKey = bodyA->headJointKey;
		otherBodyId = bodyB->id;
	}
	else
	{
		jointKey = bodyB->headJointKey;
		otherBodyId = bodyA->id;
	}
	while ( jointKey != B2_NULL_INDEX )
	{
		int jointId = jointKey >> 1;
		int edgeIndex = jointKey & 1;
		h_joint* j = w->joints.data + jointId;
		if ( j->collideConnected == 0 && j->edges[edgeIndex ^ 1].bodyId == otherBodyId ) return 0;
		jointKey = j->edges[edgeIndex].nextKey;
	}
	return 1;
}

/* tree node storage: page-locked above 4096 nodes so the per-step upload is a plain DMA */
void* h_nodeAlloc( size_t bytes, int* pinned )
{
	*pinned = 0;
	if ( bytes >= 4096 * sizeof( h_treeNode ) )
	{
		void* p = b2gDev_HostAlloc( bytes );
		if ( p != NULL )
		{
			*pinned = 1;
			return p;
		}
	}
	void* p = malloc( bytes );
	if ( p == NULL )
	{
		fprintf( stderr, "box2d_gb300: out of host memory (%zu bytes)\n", bytes );
		abort();
	}
	return p;
}

void h_nodeFree( void* p, int pinned )
{
	if ( p == NULL ) return;
	if ( pinned ) b2gDev_HostFree( p );
	else free( p );
}
