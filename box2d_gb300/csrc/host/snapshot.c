/*
 * World snapshots (world_snapshot.c in the reference: b2World_Snapshot, b2World_Restore,
 * b2CreateWorldFromSnapshot; box2d.h:286-338).
 *
 * An image holds a world's simulation state at a step boundary: the host bookkeeping in
 * the reference's array orders (id pools, bodies, shapes, contacts, joints, islands,
 * solver sets, graph colors, broadphase trees, move buffer, pair set, sensors, chains, the
 * contact and sleep operations waiting for the next step) and the device-resident state
 * brought back for it (body transforms, velocities and sleep times, joint records with
 * their impulses, every contact slot's manifold, impulses, flags and simplex cache, the
 * shapes' tight boxes). A restore rebuilds the host world from the image, writes the
 * contact slots back to the device and marks every other device array stale, so the next
 * step sends them again: the world then continues bit for bit as the original did from
 * that instant.
 *
 * Layout: a header (magic, version, the sizes of the records, the payload length and an
 * FNV-1a 64 checksum of the payload), then the world record and each array as (count,
 * elements). An image is checked and parsed into a separate world record before the world
 * being restored is touched, so a rejected image leaves it unchanged. Records are written
 * as they lie in memory: images are for this library on the same machine type. Object user
 * data is not stored and reads back as NULL, as in the reference; event arrays start empty.
 */
#include "b2g_world.h"

#include <limits.h>
#include <stdio.h>

#define H_SNAP_MAGIC 0x53324742u /* "BG2S" */
#define H_SNAP_VERSION 1u
#define H_SNAP_LAYOUT_COUNT 14

typedef struct h_snapHeader
{
	uint32_t magic, version;
	uint32_t layout[H_SNAP_LAYOUT_COUNT];
	uint64_t payloadBytes;
	uint64_t checksum;
} h_snapHeader;

static void h_snapLayout( uint32_t* l )
{
	l[0] = sizeof( h_world );
	l[1] = sizeof( h_body );
	l[2] = sizeof( h_shape );
	l[3] = sizeof( h_contact );
	l[4] = sizeof( h_joint );
	l[5] = sizeof( b2gJoint );
	l[6] = sizeof( b2gContact );
	l[7] = sizeof( h_treeNode );
	l[8] = sizeof( h_island );
	l[9] = sizeof( h_sleepSet );
	l[10] = sizeof( h_chain );
	l[11] = sizeof( h_sensor );
	l[12] = sizeof( b2gContactInit );
	l[13] = sizeof( void* );
}

static uint64_t h_fnv64( const uint8_t* p, size_t n )
{
	uint64_t h = 14695981039346656037ull;
	for ( size_t i = 0; i < n; ++i )
	{
		h ^= p[i];
		h *= 1099511628211ull;
	}
	return h;
}

/* ---- writer: counts the bytes, and copies them when it has an output ---- */

typedef struct h_snapWriter
{
	uint8_t* out;
	size_t size;
} h_snapWriter;

static void h_put( h_snapWriter* s, const void* p, size_t n )
{
	if ( s->out != NULL && n > 0 ) memcpy( s->out + s->size, p, n );
	s->size += n;
}

static void h_putInt( h_snapWriter* s, int v ) { h_put( s, &v, sizeof( v ) ); }

#define H_PUT_ARRAY( s, a )                                                                                                    \
	do                                                                                                                           \
	{                                                                                                                            \
		h_putInt( s, ( a ).count );                                                                                              \
		h_put( s, ( a ).data, (size_t)( a ).count * sizeof( *( a ).data ) );                                                    \
	} while ( 0 )

static void h_putBits( h_snapWriter* s, const h_bitSet* b )
{
	h_putInt( s, b->blockCount );
	h_put( s, b->bits, (size_t)b->blockCount * sizeof( uint64_t ) );
}

/* the world record, then every array in a fixed order, then the device contact slots */
static void h_snapWorld( const h_world* w, h_snapWriter* s, const b2gContact* contacts, int contactSlots )
{
	h_put( s, w, sizeof( *w ) );
	const h_idPool* pools[] = { &w->bodyIdPool, &w->shapeIdPool,  &w->contactIdPool, &w->jointIdPool,
								&w->chainIdPool, &w->islandIdPool, &w->setIdPool };
	for ( int i = 0; i < 7; ++i ) H_PUT_ARRAY( s, pools[i]->freeArray );
	H_PUT_ARRAY( s, w->bodies );
	H_PUT_ARRAY( s, w->shapes );
	H_PUT_ARRAY( s, w->contacts );
	H_PUT_ARRAY( s, w->joints );
	H_PUT_ARRAY( s, w->jointRecords );
	H_PUT_ARRAY( s, w->awakeBodyIds );
	H_PUT_ARRAY( s, w->staticBodyIds );
	H_PUT_ARRAY( s, w->staticJointIds );
	H_PUT_ARRAY( s, w->awakeContactIds );
	H_PUT_ARRAY( s, w->disabledContactIds );
	H_PUT_ARRAY( s, w->islands );
	for ( int i = 0; i < w->islands.count; ++i )
	{
		H_PUT_ARRAY( s, w->islands.data[i].bodies );
		H_PUT_ARRAY( s, w->islands.data[i].contacts );
		H_PUT_ARRAY( s, w->islands.data[i].joints );
	}
	H_PUT_ARRAY( s, w->awakeIslandIds );
	H_PUT_ARRAY( s, w->sets );
	for ( int i = 0; i < w->sets.count; ++i )
	{
		H_PUT_ARRAY( s, w->sets.data[i].bodyIds );
		H_PUT_ARRAY( s, w->sets.data[i].contactIds );
		H_PUT_ARRAY( s, w->sets.data[i].jointIds );
		H_PUT_ARRAY( s, w->sets.data[i].islandIds );
	}
	H_PUT_ARRAY( s, w->pendingContacts );
	for ( int c = 0; c < B2_GRAPH_COLOR_COUNT; ++c )
	{
		h_putBits( s, &w->colors[c].bodySet );
		H_PUT_ARRAY( s, w->colors[c].contactIds );
		H_PUT_ARRAY( s, w->colors[c].jointIds );
	}
	for ( int t = 0; t < 3; ++t )
	{
		h_put( s, w->trees[t].nodes, (size_t)w->trees[t].nodeCapacity * sizeof( h_treeNode ) );
		h_putBits( s, &w->movedProxies[t] );
	}
	H_PUT_ARRAY( s, w->moveArray );
	h_put( s, w->pairSet.keys, (size_t)w->pairSet.capacity * sizeof( uint64_t ) );
	H_PUT_ARRAY( s, w->chains );
	for ( int i = 0; i < w->chains.count; ++i )
		h_put( s, w->chains.data[i].shapeIndices, (size_t)w->chains.data[i].count * sizeof( int ) );
	H_PUT_ARRAY( s, w->sensors );
	for ( int i = 0; i < w->sensors.count; ++i )
	{
		H_PUT_ARRAY( s, w->sensors.data[i].overlaps1 );
		H_PUT_ARRAY( s, w->sensors.data[i].overlaps2 );
		H_PUT_ARRAY( s, w->sensors.data[i].hits );
	}
	H_PUT_ARRAY( s, w->pendingInits );
	H_PUT_ARRAY( s, w->pendingKills );
	H_PUT_ARRAY( s, w->forcedBodies );
	h_putInt( s, contactSlots );
	h_put( s, contacts, (size_t)contactSlots * sizeof( b2gContact ) );
}

/* ---- reader: bounds-checked; after a failure every read yields zeros ---- */

typedef struct h_snapReader
{
	const uint8_t* p;
	size_t size, pos;
	int ok;
} h_snapReader;

static void h_get( h_snapReader* r, void* dst, size_t n )
{
	if ( r->ok == 0 || n > r->size - r->pos )
	{
		r->ok = 0;
		if ( dst != NULL && n > 0 ) memset( dst, 0, n );
		return;
	}
	if ( n > 0 ) memcpy( dst, r->p + r->pos, n );
	r->pos += n;
}

/* an element count that the rest of the image can hold */
static int h_getCount( h_snapReader* r, size_t elem )
{
	int n = 0;
	h_get( r, &n, sizeof( n ) );
	if ( n < 0 || (size_t)n > ( r->size - r->pos ) / ( elem > 0 ? elem : 1 ) )
	{
		r->ok = 0;
		return 0;
	}
	return n;
}

#define H_GET_ARRAY( r, a )                                                                                                    \
	do                                                                                                                           \
	{                                                                                                                            \
		( a ).data = NULL;                                                                                                       \
		( a ).count = ( a ).capacity = 0;                                                                                        \
		int n_ = h_getCount( r, sizeof( *( a ).data ) );                                                                         \
		if ( n_ > 0 )                                                                                                            \
		{                                                                                                                        \
			h_reserve( a, n_ );                                                                                                  \
			h_get( r, ( a ).data, (size_t)n_ * sizeof( *( a ).data ) );                                                          \
			( a ).count = n_;                                                                                                    \
		}                                                                                                                        \
	} while ( 0 )

static void h_getBits( h_snapReader* r, h_bitSet* b )
{
	b->bits = NULL;
	b->blockCount = 0;
	int n = h_getCount( r, sizeof( uint64_t ) );
	if ( n > 0 )
	{
		b->bits = calloc( (size_t)n, sizeof( uint64_t ) );
		h_get( r, b->bits, (size_t)n * sizeof( uint64_t ) );
		b->blockCount = n;
	}
}

/* every owned pointer of a world record read from an image cleared before its arrays are
   read, so that a record whose parse stops part way can still be freed */
static void h_snapClearPointers( h_world* t )
{
	h_idPool* pools[] = { &t->bodyIdPool, &t->shapeIdPool,	&t->contactIdPool, &t->jointIdPool,
						  &t->chainIdPool, &t->islandIdPool, &t->setIdPool };
	for ( int i = 0; i < 7; ++i ) memset( &pools[i]->freeArray, 0, sizeof( pools[i]->freeArray ) );
	memset( &t->bodies, 0, sizeof( t->bodies ) );
	memset( &t->shapes, 0, sizeof( t->shapes ) );
	memset( &t->contacts, 0, sizeof( t->contacts ) );
	memset( &t->joints, 0, sizeof( t->joints ) );
	memset( &t->jointRecords, 0, sizeof( t->jointRecords ) );
	memset( &t->awakeBodyIds, 0, sizeof( t->awakeBodyIds ) );
	memset( &t->staticBodyIds, 0, sizeof( t->staticBodyIds ) );
	memset( &t->staticJointIds, 0, sizeof( t->staticJointIds ) );
	memset( &t->awakeContactIds, 0, sizeof( t->awakeContactIds ) );
	memset( &t->disabledContactIds, 0, sizeof( t->disabledContactIds ) );
	memset( &t->islands, 0, sizeof( t->islands ) );
	memset( &t->awakeIslandIds, 0, sizeof( t->awakeIslandIds ) );
	memset( &t->sets, 0, sizeof( t->sets ) );
	t->sleepPerm = NULL;
	memset( &t->pendingWake, 0, sizeof( t->pendingWake ) );
	memset( &t->pendingContacts, 0, sizeof( t->pendingContacts ) );
	memset( &t->sleptBodies, 0, sizeof( t->sleptBodies ) );
	memset( t->colors, 0, sizeof( t->colors ) );
	for ( int i = 0; i < 3; ++i )
	{
		t->trees[i].nodes = NULL;
		t->trees[i].pinned = 0;
		t->trees[i].leafIndices = NULL;
		t->trees[i].leafCenters = NULL;
		t->trees[i].rebuildCapacity = 0;
		memset( &t->movedProxies[i], 0, sizeof( t->movedProxies[i] ) );
	}
	memset( &t->moveArray, 0, sizeof( t->moveArray ) );
	t->moveBoxes = NULL;
	t->moveShapes = NULL;
	t->moveBufCap = 0;
	t->specKeys = NULL;
	t->specBoxes = NULL;
	t->specCap = 0;
	t->specIssued = 0;
	t->pairSet.keys = NULL;
	memset( &t->chains, 0, sizeof( t->chains ) );
	memset( &t->sensors, 0, sizeof( t->sensors ) );
	memset( &t->sensorBeginEvents, 0, sizeof( t->sensorBeginEvents ) );
	memset( t->sensorEndEvents, 0, sizeof( t->sensorEndEvents ) );
	memset( &t->moveEvents, 0, sizeof( t->moveEvents ) );
	memset( &t->beginEvents, 0, sizeof( t->beginEvents ) );
	memset( t->endEvents, 0, sizeof( t->endEvents ) );
	memset( &t->pendingInits, 0, sizeof( t->pendingInits ) );
	memset( &t->pendingKills, 0, sizeof( t->pendingKills ) );
	memset( &t->forcedBodies, 0, sizeof( t->forcedBodies ) );
	t->dev = NULL;
	t->tape = NULL;
	t->rebuildWorker = NULL;
	t->mirrorXf = t->mirrorCenter = t->mirrorV = t->mirrorSleep = NULL;
	t->mirrorFlags = NULL;
	memset( (void*)t->uploadedTreeNodes, 0, sizeof( t->uploadedTreeNodes ) );
}

/* checks the header and parses the image into *t (a world record with its own arrays) and
   the contact slots; returns 0, leaving nothing allocated, for a rejected image */
static int h_snapParse( const uint8_t* image, int size, h_world* t, b2gContact** contacts, int* contactSlots )
{
	*contacts = NULL;
	*contactSlots = 0;
	if ( image == NULL || size < (int)sizeof( h_snapHeader ) ) return 0;
	h_snapHeader hdr;
	memcpy( &hdr, image, sizeof( hdr ) );
	uint32_t layout[H_SNAP_LAYOUT_COUNT];
	h_snapLayout( layout );
	if ( hdr.magic != H_SNAP_MAGIC || hdr.version != H_SNAP_VERSION ) return 0;
	if ( memcmp( hdr.layout, layout, sizeof( layout ) ) != 0 ) return 0;
	if ( hdr.payloadBytes != (uint64_t)( size - (int)sizeof( h_snapHeader ) ) ) return 0;
	const uint8_t* payload = image + sizeof( h_snapHeader );
	if ( h_fnv64( payload, (size_t)hdr.payloadBytes ) != hdr.checksum ) return 0;

	h_snapReader rd = { payload, (size_t)hdr.payloadBytes, 0, 1 };
	h_snapReader* r = &rd;
	h_get( r, t, sizeof( *t ) );
	h_snapClearPointers( t );
	if ( r->ok == 0 ) return 0;
	h_idPool* pools[] = { &t->bodyIdPool, &t->shapeIdPool,	&t->contactIdPool, &t->jointIdPool,
						  &t->chainIdPool, &t->islandIdPool, &t->setIdPool };
	for ( int i = 0; i < 7; ++i ) H_GET_ARRAY( r, pools[i]->freeArray );
	H_GET_ARRAY( r, t->bodies );
	H_GET_ARRAY( r, t->shapes );
	H_GET_ARRAY( r, t->contacts );
	H_GET_ARRAY( r, t->joints );
	H_GET_ARRAY( r, t->jointRecords );
	H_GET_ARRAY( r, t->awakeBodyIds );
	H_GET_ARRAY( r, t->staticBodyIds );
	H_GET_ARRAY( r, t->staticJointIds );
	H_GET_ARRAY( r, t->awakeContactIds );
	H_GET_ARRAY( r, t->disabledContactIds );
	H_GET_ARRAY( r, t->islands );
	for ( int i = 0; i < t->islands.count; ++i )
	{
		h_island* island = t->islands.data + i;
		memset( &island->bodies, 0, sizeof( island->bodies ) );
		memset( &island->contacts, 0, sizeof( island->contacts ) );
		memset( &island->joints, 0, sizeof( island->joints ) );
	}
	for ( int i = 0; i < t->islands.count; ++i )
	{
		H_GET_ARRAY( r, t->islands.data[i].bodies );
		H_GET_ARRAY( r, t->islands.data[i].contacts );
		H_GET_ARRAY( r, t->islands.data[i].joints );
	}
	H_GET_ARRAY( r, t->awakeIslandIds );
	H_GET_ARRAY( r, t->sets );
	for ( int i = 0; i < t->sets.count; ++i )
	{
		h_sleepSet* set = t->sets.data + i;
		memset( &set->bodyIds, 0, sizeof( set->bodyIds ) );
		memset( &set->contactIds, 0, sizeof( set->contactIds ) );
		memset( &set->jointIds, 0, sizeof( set->jointIds ) );
		memset( &set->islandIds, 0, sizeof( set->islandIds ) );
	}
	for ( int i = 0; i < t->sets.count; ++i )
	{
		H_GET_ARRAY( r, t->sets.data[i].bodyIds );
		H_GET_ARRAY( r, t->sets.data[i].contactIds );
		H_GET_ARRAY( r, t->sets.data[i].jointIds );
		H_GET_ARRAY( r, t->sets.data[i].islandIds );
	}
	H_GET_ARRAY( r, t->pendingContacts );
	for ( int c = 0; c < B2_GRAPH_COLOR_COUNT; ++c )
	{
		h_getBits( r, &t->colors[c].bodySet );
		H_GET_ARRAY( r, t->colors[c].contactIds );
		H_GET_ARRAY( r, t->colors[c].jointIds );
	}
	for ( int k = 0; k < 3; ++k )
	{
		h_tree* tree = t->trees + k;
		int capacity = tree->nodeCapacity;
		if ( r->ok == 0 || capacity < 1 || (size_t)capacity > ( r->size - r->pos ) / sizeof( h_treeNode ) )
		{
			r->ok = 0;
			tree->nodeCapacity = 0;
		}
		else
		{
			tree->nodes = h_nodeAlloc( (size_t)capacity * sizeof( h_treeNode ), &tree->pinned );
			h_get( r, tree->nodes, (size_t)capacity * sizeof( h_treeNode ) );
		}
		h_getBits( r, &t->movedProxies[k] );
	}
	H_GET_ARRAY( r, t->moveArray );
	{
		int capacity = t->pairSet.capacity;
		if ( r->ok == 0 || capacity < 0 || (size_t)capacity > ( r->size - r->pos ) / sizeof( uint64_t ) )
		{
			r->ok = 0;
			t->pairSet.capacity = 0;
			t->pairSet.count = 0;
		}
		else if ( capacity > 0 )
		{
			t->pairSet.keys = malloc( (size_t)capacity * sizeof( uint64_t ) );
			h_get( r, t->pairSet.keys, (size_t)capacity * sizeof( uint64_t ) );
		}
	}
	H_GET_ARRAY( r, t->chains );
	for ( int i = 0; i < t->chains.count; ++i ) t->chains.data[i].shapeIndices = NULL;
	for ( int i = 0; i < t->chains.count; ++i )
	{
		h_chain* chain = t->chains.data + i;
		int n = chain->count;
		if ( r->ok == 0 || n < 0 || (size_t)n > ( r->size - r->pos ) / sizeof( int ) )
		{
			r->ok = 0;
			chain->count = 0;
			continue;
		}
		if ( n > 0 )
		{
			chain->shapeIndices = malloc( (size_t)n * sizeof( int ) );
			h_get( r, chain->shapeIndices, (size_t)n * sizeof( int ) );
		}
	}
	H_GET_ARRAY( r, t->sensors );
	for ( int i = 0; i < t->sensors.count; ++i )
	{
		h_sensor* sensor = t->sensors.data + i;
		memset( &sensor->overlaps1, 0, sizeof( sensor->overlaps1 ) );
		memset( &sensor->overlaps2, 0, sizeof( sensor->overlaps2 ) );
		memset( &sensor->hits, 0, sizeof( sensor->hits ) );
	}
	for ( int i = 0; i < t->sensors.count; ++i )
	{
		H_GET_ARRAY( r, t->sensors.data[i].overlaps1 );
		H_GET_ARRAY( r, t->sensors.data[i].overlaps2 );
		H_GET_ARRAY( r, t->sensors.data[i].hits );
	}
	H_GET_ARRAY( r, t->pendingInits );
	H_GET_ARRAY( r, t->pendingKills );
	H_GET_ARRAY( r, t->forcedBodies );
	int slots = h_getCount( r, sizeof( b2gContact ) );
	b2gContact* slotData = NULL;
	if ( r->ok && slots > 0 )
	{
		slotData = malloc( (size_t)slots * sizeof( b2gContact ) );
		h_get( r, slotData, (size_t)slots * sizeof( b2gContact ) );
	}
	if ( r->ok == 0 || r->pos != r->size )
	{
		free( slotData );
		h_freeWorldArrays( t );
		return 0;
	}
	/* object user data is host wiring, not simulation state */
	for ( int i = 0; i < t->bodies.count; ++i ) t->bodies.data[i].userData = NULL;
	for ( int i = 0; i < t->shapes.count; ++i ) t->shapes.data[i].userData = NULL;
	for ( int i = 0; i < t->joints.count; ++i ) t->joints.data[i].userData = NULL;
	*contacts = slotData;
	*contactSlots = slots;
	return 1;
}

/* ---- public API ---- */

int b2World_Snapshot( b2WorldId worldId, uint8_t* image, int capacity )
{
	h_world* w = h_worldFromId( worldId );
	if ( w == NULL || w->locked ) return 0;
	h_joinRebuild( w );
	int slots = w->contactIdPool.nextIndex;
	h_snapWriter counter = { NULL, 0 };
	h_snapWorld( w, &counter, NULL, slots );
	size_t total = sizeof( h_snapHeader ) + counter.size;
	if ( total > (size_t)INT_MAX ) return 0;
	if ( image == NULL || (int)total > capacity ) return (int)total;

	/* bring the device-resident state back (none of this changes a count) */
	h_syncFromDevice( w );
	h_syncJointsFromDevice( w );
	h_syncShapeBoxes( w );
	b2gContact* contacts = NULL;
	if ( slots > 0 )
	{
		contacts = malloc( (size_t)slots * sizeof( b2gContact ) );
		int rc = b2gDev_DownloadContacts( w->dev, contacts, slots );
		if ( rc != 0 ) h_fail( w, "snapshot contact download", rc );
	}
	h_snapWriter s = { image + sizeof( h_snapHeader ), 0 };
	h_snapWorld( w, &s, contacts, slots );
	free( contacts );

	h_snapHeader hdr;
	memset( &hdr, 0, sizeof( hdr ) );
	hdr.magic = H_SNAP_MAGIC;
	hdr.version = H_SNAP_VERSION;
	h_snapLayout( hdr.layout );
	hdr.payloadBytes = s.size;
	hdr.checksum = h_fnv64( image + sizeof( h_snapHeader ), s.size );
	memcpy( image, &hdr, sizeof( hdr ) );
	return (int)total;
}

bool b2World_Restore( b2WorldId worldId, const uint8_t* image, int size )
{
	h_world* w = h_worldFromId( worldId );
	if ( w == NULL || w->locked ) return false;
	h_world* t = calloc( 1, sizeof( h_world ) );
	b2gContact* contacts = NULL;
	int slots = 0;
	if ( t == NULL || h_snapParse( image, size, t, &contacts, &slots ) == 0 )
	{
		free( t );
		return false;
	}

	/* the world keeps its slot, generation, device world, rebuild worker and tape; a pair
	   query issued for the next step is dropped */
	h_joinRebuild( w );
	h_dropSpeculativePairs( w );
	h_freeWorldArrays( w );
	h_world live = *w;
	*w = *t;
	free( t );
	w->inUse = 1;
	w->worldId = live.worldId;
	w->generation = live.generation;
	w->dev = live.dev;
	w->rebuildWorker = live.rebuildWorker;
	w->tape = live.tape;
	memcpy( w->hostMs, live.hostMs, sizeof( w->hostMs ) );
	w->locked = 0;
	w->lastStatus = 0;
	/* the host records are authoritative; every device array is sent before the next step */
	w->devReady = 0;
	w->hostStateValid = 1;
	w->jointsHostValid = 1;
	w->shapeBoxesValid = 1;
	w->mirrorValid = 0;
	w->moveEventsValid = 0;
	w->colorsDirty = 1;
	w->jointsDirty = 1;
	w->islandsDirty = 1;
	for ( int k = 0; k < 3; ++k )
	{
		w->uploadedTreeVersion[k] = -1;
		w->uploadedTreeNodes[k] = NULL;
	}
	int rc = b2gDev_UploadContacts( w->dev, contacts, slots );
	free( contacts );
	if ( rc != 0 ) h_fail( w, "snapshot contact upload", rc );
	return true;
}

b2WorldId b2CreateWorldFromSnapshot( const uint8_t* image, int size, int workerCount )
{
	(void)workerCount; /* the step's parallel work runs on the device */
	b2WorldId nullId = { 0, 0 };
	if ( image == NULL || size < (int)sizeof( h_snapHeader ) ) return nullId;
	b2WorldDef def = b2DefaultWorldDef();
	b2WorldId id = b2CreateWorld( &def );
	if ( b2World_IsValid( id ) == false ) return nullId;
	if ( b2World_Restore( id, image, size ) == false )
	{
		b2DestroyWorld( id );
		return nullId;
	}
	return id;
}
