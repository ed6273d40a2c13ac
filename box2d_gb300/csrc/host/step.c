/*
 * b2World_Step for the GB300 step library (physics_world.c:845-1005 in the reference).
 *
 * The stage order is the reference's: pair update -> narrowphase -> contact-state pass ->
 * Soft Step solver -> finalize -> proxy enlargement. The data-parallel parts run on the
 * device; the host keeps only the serial, order-defining bookkeeping:
 *   - contact creation in move-array order from the device pair lists,
 *   - the contact-state pass in ascending contact id (begin/end events, graph colors),
 *   - proxy enlargement in ascending awake index, which builds the next move array.
 * Each of these reads one compact list back from the device.
 */
#include "b2g_world.h"

#include <pthread.h>
#include <stddef.h>
#include <stdio.h>

static float h_ms( uint64_t t0 ) { return b2GetMilliseconds( t0 ); }

/* add the time since *t to phase `phase` and restart *t */
static void h_lap( h_world* w, int phase, uint64_t* t )
{
	uint64_t now = b2GetTicks();
	w->hostMs[phase] += b2GetMilliseconds( *t );
	*t = now;
}

/* The partial tree rebuild after the pair query (b2UpdateTreesTask, broad_phase.c:401-410)
   touches only the trees, which nothing else uses until the proxies are enlarged at the
   end of the solve. The reference runs it as a task beside the narrowphase; here a
   per-world host thread runs it while the device does the narrowphase and the solver.
   The same thread applies the step's proxy enlargement to the host trees after the step
   (the device enlarges its own copies, so the next pair query does not wait for it); its
   jobs run in the order they were posted. */
typedef struct h_rebuildWorker
{
	pthread_t thread;
	pthread_mutex_t mu;
	pthread_cond_t cv;
	int rebuildPending, enlargePending, busy, quit;
	h_world* w;
	/* the enlargement to apply: proxy ids and fat boxes, [0] kinematic tree, [1] dynamic */
	h_intArray enlargeIds[2];
	H_ARRAY( b2AABB ) enlargeBoxes[2];
} h_rebuildWorker;

static void h_rebuildTrees( h_world* w )
{
	h_treeRebuild( w->trees + b2_dynamicBody, 0 );
	h_treeRebuild( w->trees + b2_kinematicBody, 0 );
}

static void* h_rebuildMain( void* arg )
{
	h_rebuildWorker* k = arg;
	pthread_mutex_lock( &k->mu );
	for ( ;; )
	{
		while ( k->rebuildPending == 0 && k->enlargePending == 0 && k->quit == 0 ) pthread_cond_wait( &k->cv, &k->mu );
		if ( k->quit ) break;
		if ( k->enlargePending )
		{
			k->enlargePending = 0;
			pthread_mutex_unlock( &k->mu );
			/* the device has copied the node arrays before they change */
			int rc = b2gDev_WaitTreeUploads( k->w->dev );
			if ( rc != 0 ) h_fail( k->w, "tree upload", rc );
			h_treeEnlargeProxies( k->w->trees + b2_kinematicBody, k->enlargeIds[0].data, k->enlargeBoxes[0].data,
								  k->enlargeIds[0].count );
			h_treeEnlargeProxies( k->w->trees + b2_dynamicBody, k->enlargeIds[1].data, k->enlargeBoxes[1].data,
								  k->enlargeIds[1].count );
			pthread_mutex_lock( &k->mu );
		}
		else
		{
			k->rebuildPending = 0;
			pthread_mutex_unlock( &k->mu );
			h_rebuildTrees( k->w );
			pthread_mutex_lock( &k->mu );
		}
		if ( k->rebuildPending == 0 && k->enlargePending == 0 )
		{
			k->busy = 0;
			pthread_cond_broadcast( &k->cv );
		}
	}
	pthread_mutex_unlock( &k->mu );
	return NULL;
}

/* the world's worker thread, started on first use; NULL if it cannot start */
static h_rebuildWorker* h_startWorker( h_world* w )
{
	h_rebuildWorker* k = w->rebuildWorker;
	if ( k != NULL ) return k;
	k = calloc( 1, sizeof( h_rebuildWorker ) );
	k->w = w;
	pthread_mutex_init( &k->mu, NULL );
	pthread_cond_init( &k->cv, NULL );
	if ( pthread_create( &k->thread, NULL, h_rebuildMain, k ) != 0 )
	{
		pthread_mutex_destroy( &k->mu );
		pthread_cond_destroy( &k->cv );
		free( k );
		return NULL;
	}
	w->rebuildWorker = k;
	/* the device tree enlargement comes with the worker: its setup happens here, not in the
	   first step that enlarges proxies */
	int rc = b2gDev_PrepareEnlarge( w->dev );
	if ( rc != 0 ) h_fail( w, "tree enlargement setup", rc );
	return k;
}

/* run the rebuild on the world's worker thread; small trees without a worker are rebuilt
   inline */
static void h_postRebuild( h_world* w )
{
	h_rebuildWorker* k = w->rebuildWorker;
	if ( k == NULL && w->trees[b2_dynamicBody].proxyCount >= 2048 ) k = h_startWorker( w );
	if ( k == NULL )
	{
		h_rebuildTrees( w );
		return;
	}
	pthread_mutex_lock( &k->mu );
	k->rebuildPending = 1;
	k->busy = 1;
	pthread_cond_broadcast( &k->cv );
	pthread_mutex_unlock( &k->mu );
}

/* wait for the posted jobs; the trees are the main thread's again afterwards */
void h_joinRebuild( h_world* w )
{
	h_rebuildWorker* k = w->rebuildWorker;
	if ( k == NULL ) return;
	pthread_mutex_lock( &k->mu );
	while ( k->busy ) pthread_cond_wait( &k->cv, &k->mu );
	pthread_mutex_unlock( &k->mu );
}

void h_stopRebuildWorker( h_world* w )
{
	h_rebuildWorker* k = w->rebuildWorker;
	if ( k == NULL ) return;
	pthread_mutex_lock( &k->mu );
	while ( k->busy ) pthread_cond_wait( &k->cv, &k->mu );
	k->quit = 1;
	pthread_cond_broadcast( &k->cv );
	pthread_mutex_unlock( &k->mu );
	pthread_join( k->thread, NULL );
	pthread_mutex_destroy( &k->mu );
	pthread_cond_destroy( &k->cv );
	for ( int i = 0; i < 2; ++i )
	{
		h_free( k->enlargeIds[i] );
		h_free( k->enlargeBoxes[i] );
	}
	free( k );
	w->rebuildWorker = NULL;
}

/* upload one broadphase tree when it changed since its last upload; the node array is
   sent as is (page-locked for large trees) and converted to query nodes on the device */
_Static_assert( sizeof( h_treeNode ) == sizeof( b2gHostTreeNode ), "host tree node layout" );
_Static_assert( offsetof( h_treeNode, userData ) == offsetof( b2gHostTreeNode, userData ), "host tree node layout" );
_Static_assert( offsetof( h_treeNode, flags ) == offsetof( b2gHostTreeNode, flags ), "host tree node layout" );
_Static_assert( H_NODE_LEAF == 0x4, "leaf flag" );

static void h_uploadTree( h_world* w, int type )
{
	h_tree* t = w->trees + type;
	if ( w->uploadedTreeVersion[type] == t->version && w->uploadedTreeNodes[type] == t->nodes ) return;
	int rc = b2gDev_UploadTree( w->dev, type, (const b2gHostTreeNode*)t->nodes, t->nodeCapacity,
								t->nodeCount == 0 ? -1 : t->root, t->pinned );
	if ( rc != 0 ) h_fail( w, "tree upload", rc );
	w->uploadedTreeVersion[type] = t->version;
	w->uploadedTreeNodes[type] = t->nodes;
}

static int h_shouldShapesCollide( b2Filter a, b2Filter b )
{
	if ( a.groupIndex == b.groupIndex && a.groupIndex != 0 ) return a.groupIndex > 0;
	return ( a.maskBits & b.categoryBits ) != 0 && ( a.categoryBits & b.maskBits ) != 0;
}

/* broad_phase.c:412-529. The device returns, per move, every overlapping proxy in the
   reference's query order (kinematic, static, dynamic trees; DFS child2 first) after the
   self and moved-pair dedupe, less the pairs that have a contact already; the host applies
   the remaining filters and creates contacts newest-first per move, as the reference's
   prepended pair lists do. */
static void h_flushContacts( h_world* w );

/* the moved proxies' fat boxes and shapes, in move order, into the world's buffers */
static void h_moveBoxes( h_world* w )
{
	int moveCount = w->moveArray.count;
	if ( moveCount > w->moveBufCap )
	{
		int cap = w->moveBufCap > 0 ? w->moveBufCap : 256;
		while ( cap < moveCount ) cap *= 2;
		free( w->moveBoxes );
		free( w->moveShapes );
		w->moveBoxes = malloc( (size_t)cap * 4 * sizeof( float ) );
		w->moveShapes = malloc( (size_t)cap * sizeof( int ) );
		w->moveBufCap = cap;
	}
	float* boxes = w->moveBoxes;
	int* shapeIds = w->moveShapes;
	for ( int i = 0; i < moveCount; ++i )
	{
		/* the moved proxies' nodes and shapes are scattered: a later move's node and a
		   nearer move's shape are requested ahead */
		if ( i + 16 < moveCount )
		{
			int k16 = w->moveArray.data[i + 16];
			__builtin_prefetch( w->trees[H_PROXY_TYPE( k16 )].nodes + H_PROXY_ID( k16 ), 0, 3 );
		}
		if ( i + 8 < moveCount )
		{
			int k8 = w->moveArray.data[i + 8];
			int s8 = (int)w->trees[H_PROXY_TYPE( k8 )].nodes[H_PROXY_ID( k8 )].userData;
			__builtin_prefetch( &w->shapes.data[s8].fatAABB, 0, 3 );
		}
		/* a leaf's box is its shape's fat box; the shape's copy is read because the worker
		   may still be enlarging the host tree after the last step */
		int key = w->moveArray.data[i];
		const h_tree* tree = w->trees + H_PROXY_TYPE( key );
		int shapeId = (int)tree->nodes[H_PROXY_ID( key )].userData;
		const b2AABB fat = w->shapes.data[shapeId].fatAABB;
		boxes[4 * i] = fat.lowerBound.x;
		boxes[4 * i + 1] = fat.lowerBound.y;
		boxes[4 * i + 2] = fat.upperBound.x;
		boxes[4 * i + 3] = fat.upperBound.y;
		shapeIds[i] = shapeId;
	}
}

void h_dropSpeculativePairs( h_world* w )
{
	if ( w->specIssued == 0 ) return;
	w->specIssued = 0;
	int rc = b2gDev_FindPairsDiscard( w->dev );
	if ( rc != 0 ) h_fail( w, "pair query", rc );
}

/* the query issued at the last step's end answers this step's when it read what this one
   would: the same move keys, the same boxes (the shapes' fat boxes now), the same tree
   versions, no contact created or destroyed since, and no world change that re-sends the
   device state */
static int h_speculationHolds( h_world* w )
{
	int n = w->moveArray.count;
	if ( w->specStale || n != w->specCount || w->pendingKills.count != 0 || w->pendingInits.count != 0 ) return 0;
	for ( int t = 0; t < 3; ++t )
		if ( w->trees[t].version != w->specTreeVersion[t] ) return 0;
	if ( memcmp( w->moveArray.data, w->specKeys, (size_t)n * sizeof( int ) ) != 0 ) return 0;
	h_moveBoxes( w );
	return memcmp( w->moveBoxes, w->specBoxes, (size_t)n * 4 * sizeof( float ) ) == 0;
}

/* issue the pair query of the moved proxies (or keep the one issued at the last step's
   end); returns whether one is pending */
static int h_pairsIssue( h_world* w )
{
	int moveCount = w->moveArray.count;
	if ( w->specIssued )
	{
		if ( moveCount > 0 && b2gDev_IsRecording( w->dev ) == 0 && h_speculationHolds( w ) )
		{
			w->specIssued = 0;
			return 1;
		}
		h_dropSpeculativePairs( w );
	}
	if ( moveCount == 0 ) return 0;
	/* the device drops pairs whose contact exists: contacts destroyed since the last step
	   (shape filters, destroyed joints) must leave its pair set before the query */
	h_flushContacts( w );
	uint64_t lap = b2GetTicks();
	for ( int t = 0; t < 3; ++t ) h_uploadTree( w, t );
	h_lap( w, H_PHASE_TREE_UPLOAD, &lap );
	h_moveBoxes( w );
	int rc = b2gDev_FindPairsIssue( w->dev, w->moveArray.data, w->moveBoxes, w->moveShapes, moveCount );
	if ( rc != 0 ) h_fail( w, "pair query", rc );
	return 1;
}

/* Issue the next step's pair query at this step's end, behind the state download: it runs
   while the host finishes the step and the caller works between steps, and the next step
   waits for its results instead of issuing it (B2G_SPECULATE=0: never). */
static void h_pairsSpeculate( h_world* w )
{
	static int s_on = -1;
	if ( s_on < 0 )
	{
		const char* e = getenv( "B2G_SPECULATE" );
		s_on = e == NULL || atoi( e ) != 0;
	}
	if ( s_on == 0 || w->moveArray.count == 0 || b2gDev_IsRecording( w->dev ) || w->devReady == 0 ) return;
	/* the query, its contact flush and tree uploads change no body state: the state
	   download issued before it stays the step's */
	int prefetched = b2gDev_PrefetchIsValid( w->dev );
	int issued = h_pairsIssue( w );
	b2gDev_PrefetchKeep( w->dev, prefetched );
	if ( issued == 0 ) return;
	int n = w->moveArray.count;
	if ( n > w->specCap )
	{
		int cap = w->specCap > 0 ? w->specCap : 256;
		while ( cap < n ) cap *= 2;
		free( w->specKeys );
		free( w->specBoxes );
		w->specKeys = malloc( (size_t)cap * sizeof( int ) );
		w->specBoxes = malloc( (size_t)cap * 4 * sizeof( float ) );
		w->specCap = cap;
	}
	memcpy( w->specKeys, w->moveArray.data, (size_t)n * sizeof( int ) );
	memcpy( w->specBoxes, w->moveBoxes, (size_t)n * 4 * sizeof( float ) );
	for ( int t = 0; t < 3; ++t ) w->specTreeVersion[t] = w->trees[t].version;
	w->specCount = n;
	w->specStale = 0;
	w->specIssued = 1;
}

/* after the wait: filter the pairs and create contacts newest-first per move */
static void h_pairsFinish( h_world* w )
{
	int moveCount = w->moveArray.count;
	uint64_t lap = b2GetTicks();
	int* pairs = NULL;
	int* counts = NULL;
	int total = 0;
	int rc = b2gDev_FindPairsCollect( w->dev, &pairs, &counts, &total );
	if ( rc != 0 ) h_fail( w, "pair query", rc );
	h_lap( w, H_PHASE_PAIR_QUERY, &lap );
	/* most pairs exist already: their set lookups miss the cache one after another unless
	   the probed slots are requested first, all of them, so that the misses overlap */
	for ( int p = 0; p < total; ++p ) h_pairSetPrefetch( &w->pairSet, H_SHAPE_PAIR_KEY( pairs[2 * p], pairs[2 * p + 1] ) );
	int offset = 0;
	for ( int i = 0; i < moveCount; ++i )
	{
		int n = counts[i];
		for ( int k = n - 1; k >= 0; --k )
		{
			int shapeIdA = pairs[2 * ( offset + k )];
			int shapeIdB = pairs[2 * ( offset + k ) + 1];
			if ( h_pairSetContains( &w->pairSet, H_SHAPE_PAIR_KEY( shapeIdA, shapeIdB ) ) ) continue;
			h_shape* sA = w->shapes.data + shapeIdA;
			h_shape* sB = w->shapes.data + shapeIdB;
			if ( sA->bodyId == sB->bodyId ) continue;
			if ( sA->isSensor || sB->isSensor ) continue;
			if ( h_shouldShapesCollide( sA->filter, sB->filter ) == 0 ) continue;
			if ( h_canCollide( sA->type, sB->type ) == 0 ) continue;
			if ( h_shouldBodiesCollide( w, w->bodies.data + sA->bodyId, w->bodies.data + sB->bodyId ) == 0 ) continue;
			h_createContact( w, sA, sB );
		}
		offset += n;
	}
	h_lap( w, H_PHASE_CONTACT_CREATE, &lap );
	/* b2UpdateTreesTask (broad_phase.c:401-410), overlapped with the narrowphase and solver */
	h_postRebuild( w );
	h_lap( w, H_PHASE_TREE_REBUILD, &lap );
	for ( int i = 0; i < w->moveArray.count; ++i )
	{
		int key = w->moveArray.data[i];
		h_bitClear( w->movedProxies + H_PROXY_TYPE( key ), H_PROXY_ID( key ) );
	}
	w->moveArray.count = 0;
}

static void h_flushContacts( h_world* w )
{
	int rc = b2gDev_ReserveContacts( w->dev, w->contactIdPool.nextIndex );
	if ( rc == 0 && w->pendingKills.count > 0 ) rc = b2gDev_KillContacts( w->dev, w->pendingKills.data, w->pendingKills.count );
	if ( rc == 0 && w->pendingInits.count > 0 ) rc = b2gDev_InitContacts( w->dev, w->pendingInits.data, w->pendingInits.count );
	if ( rc != 0 ) h_fail( w, "contact upload", rc );
	w->pendingKills.count = 0;
	w->pendingInits.count = 0;
}

static void h_uploadColors( h_world* w )
{
	if ( w->colorsDirty == 0 ) return;
	int offsets[B2_GRAPH_COLOR_COUNT + 1];
	int total = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
	{
		offsets[i] = total;
		total += w->colors[i].contactIds.count;
	}
	offsets[B2_GRAPH_COLOR_COUNT] = total;
	const int* lists[B2_GRAPH_COLOR_COUNT];
	int counts[B2_GRAPH_COLOR_COUNT];
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
	{
		lists[i] = w->colors[i].contactIds.data;
		counts[i] = w->colors[i].contactIds.count;
	}
	int rc = b2gDev_UploadColorLists( w->dev, lists, counts, B2_GRAPH_COLOR_COUNT, offsets, total );
	if ( rc != 0 ) h_fail( w, "color upload", rc );
	w->colorsDirty = 0;
}

/* per body, the bodies joined to it by a joint that does not collide its bodies: the
   continuous sweep skips those pairs as b2ShouldBodiesCollide (body.c:2076-2112) does */
static void h_uploadJointPartners( h_world* w )
{
	int bodyCount = w->bodies.count;
	int* offsets = malloc( (size_t)( bodyCount + 1 ) * sizeof( int ) );
	int total = 0;
	for ( int i = 0; i < bodyCount; ++i )
	{
		offsets[i] = total;
		for ( int key = w->bodies.data[i].headJointKey; key != B2_NULL_INDEX; )
		{
			const h_joint* j = w->joints.data + ( key >> 1 );
			if ( j->collideConnected == 0 ) total += 1;
			key = j->edges[key & 1].nextKey;
		}
	}
	offsets[bodyCount] = total;
	int* list = malloc( (size_t)( total > 0 ? total : 1 ) * sizeof( int ) );
	for ( int i = 0, n = 0; i < bodyCount; ++i )
	{
		for ( int key = w->bodies.data[i].headJointKey; key != B2_NULL_INDEX; )
		{
			const h_joint* j = w->joints.data + ( key >> 1 );
			if ( j->collideConnected == 0 ) list[n++] = j->edges[( key & 1 ) ^ 1].bodyId;
			key = j->edges[key & 1].nextKey;
		}
	}
	int rc = b2gDev_UploadJointPartners( w->dev, offsets, bodyCount, list, total );
	free( offsets );
	free( list );
	if ( rc != 0 ) h_fail( w, "joint partner upload", rc );
}

static void h_uploadJoints( h_world* w )
{
	if ( w->jointsDirty == 0 ) return;
	h_uploadJointPartners( w );
	/* the host records must carry the device's accumulated impulses before the re-upload */
	h_syncJointsFromDevice( w );
	int offsets[B2_GRAPH_COLOR_COUNT + 1];
	int total = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
	{
		offsets[i] = total;
		total += w->colors[i].jointIds.count;
	}
	offsets[B2_GRAPH_COLOR_COUNT] = total;
	/* joints go to the device in color order; the device keeps the joint id in each record */
	b2gJoint* ordered = malloc( (size_t)( total > 0 ? total : 1 ) * sizeof( b2gJoint ) );
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
	{
		for ( int k = 0; k < w->colors[i].jointIds.count; ++k )
		{
			int jointId = w->colors[i].jointIds.data[k];
			ordered[offsets[i] + k] = w->jointRecords.data[jointId];
			ordered[offsets[i] + k].jointId = jointId;
		}
	}
	int rc = b2gDev_UploadJoints( w->dev, ordered, total, offsets );
	free( ordered );
	if ( rc != 0 ) h_fail( w, "joint upload", rc );
	w->jointsDirty = 0;
}

static int h_cmpInt( const void* a, const void* b )
{
	int x = *(const int*)a, y = *(const int*)b;
	return ( x > y ) - ( x < y );
}

/* physics_world.c:711-836: serial state pass in ascending contact id */
static void h_contactStatePass( h_world* w, const int* changes, int count )
{
	int endEventArrayIndex = w->endEventArrayIndex;
	/* the changed contacts are scattered over the contact array: their records are
	   requested first, and each iteration requests the shapes and bodies of a later one, so
	   that the cache misses overlap instead of following one another */
	for ( int i = 0; i < count; ++i ) __builtin_prefetch( w->contacts.data + changes[2 * i], 1, 3 );
	const int ahead = 8;
	for ( int i = 0; i < count; ++i )
	{
		if ( i + ahead < count )
		{
			const h_contact* next = w->contacts.data + changes[2 * ( i + ahead )];
			if ( next->shapeIdA >= 0 && next->shapeIdB >= 0 && next->edges[0].bodyId >= 0 && next->edges[1].bodyId >= 0 )
			{
				__builtin_prefetch( w->shapes.data + next->shapeIdA, 0, 3 );
				__builtin_prefetch( w->shapes.data + next->shapeIdB, 0, 3 );
				__builtin_prefetch( w->bodies.data + next->edges[0].bodyId, 1, 3 );
				__builtin_prefetch( w->bodies.data + next->edges[1].bodyId, 1, 3 );
			}
		}
		int contactId = changes[2 * i];
		uint32_t simFlags = (uint32_t)changes[2 * i + 1];
		h_contact* contact = w->contacts.data + contactId;
		int colorIndex = contact->colorIndex;
		int localIndex = contact->localIndex;
		const h_shape* shapeA = w->shapes.data + contact->shapeIdA;
		const h_shape* shapeB = w->shapes.data + contact->shapeIdB;
		b2ShapeId shapeIdA = { shapeA->id + 1, w->worldId, shapeA->generation };
		b2ShapeId shapeIdB = { shapeB->id + 1, w->worldId, shapeB->generation };
		b2ContactId fullId;
		fullId.index1 = contactId + 1;
		fullId.world0 = w->worldId;
		fullId.padding = 0;
		fullId.generation = contact->generation;
		uint32_t flags = contact->flags;
		if ( simFlags & B2G_S_DISJOINT )
		{
			h_destroyContact( w, contact );
		}
		else if ( simFlags & B2G_S_STARTED )
		{
			if ( flags & B2G_C_ENABLE_EVENTS )
			{
				b2ContactBeginTouchEvent ev = { shapeIdA, shapeIdB, fullId };
				h_push( w->beginEvents, ev );
			}
			/* link first: this wakes a sleeping partner (island.c:172-230), which appends to
			   the awake arrays and leaves this contact's slot in place */
			contact->flags |= B2G_C_TOUCHING;
			h_linkContact( w, contact );
			h_addContactToGraph( w, contact );
			int moved = h_removeSwap( w->awakeContactIds, localIndex );
			if ( moved != B2_NULL_INDEX ) w->contacts.data[w->awakeContactIds.data[localIndex]].localIndex = localIndex;
		}
		else if ( simFlags & B2G_S_STOPPED )
		{
			contact->flags &= ~B2G_C_TOUCHING;
			if ( contact->flags & B2G_C_ENABLE_EVENTS )
			{
				b2ContactEndTouchEvent ev = { shapeIdA, shapeIdB, fullId };
				h_push( w->endEvents[endEventArrayIndex], ev );
			}
			h_unlinkContact( w, contact );
			int bodyIdA = contact->edges[0].bodyId, bodyIdB = contact->edges[1].bodyId;
			contact->colorIndex = B2_NULL_INDEX;
			contact->localIndex = w->awakeContactIds.count;
			h_push( w->awakeContactIds, contactId );
			h_removeContactFromGraph( w, bodyIdA, bodyIdB, colorIndex, localIndex );
		}
	}
}

/* solver.c:1837-1909: enlarge proxies in ascending awake index; this builds the next move
   array. Each record is (awakeIndex, shapeId, enlargedFlag, bodyFast) + fat box. */
typedef struct h_enlargeJob
{
	h_world* w;
	const int* recs;
	const float* boxes;
	int count;
} h_enlargeJob;

#define H_ENLARGE_CHUNK 512

/* one chunk of records: the shapes' fat boxes and the tree enlargements (every shape is
   in one record at most, so only tree ancestors are shared between chunks) */
static void h_enlargeChunk( void* ctx, int chunk )
{
	const h_enlargeJob* job = ctx;
	int end = ( chunk + 1 ) * H_ENLARGE_CHUNK < job->count ? ( chunk + 1 ) * H_ENLARGE_CHUNK : job->count;
	for ( int i = chunk * H_ENLARGE_CHUNK; i < end; ++i )
	{
		const int* r = job->recs + 4 * i;
		if ( r[3] != 0 || r[2] == 0 ) continue;
		h_shape* s = job->w->shapes.data + r[1];
		const float* f = job->boxes + 4 * i;
		b2AABB fat = { { f[0], f[1] }, { f[2], f[3] } };
		s->fatAABB = fat;
		h_treeEnlargeProxyShared( job->w->trees + H_PROXY_TYPE( s->proxyKey ), H_PROXY_ID( s->proxyKey ), fat );
	}
}

/* The enlargement split between the device and the worker: the trees as the rebuild left
   them go to the device, which enlarges its copies at once (order-independent, so equal to
   the host's serial enlargement); the move buffer is built here in record order; the host
   trees are enlarged by the worker while the next step's pair query runs. Returns 0 when
   the world has no worker or its device work is being recorded (a batched step). */
static int h_enlargeOnDevice( h_world* w, const int* recs, const float* boxes, int count )
{
	h_rebuildWorker* k = w->rebuildWorker;
	if ( k == NULL || b2gDev_IsRecording( w->dev ) ) return 0;
	h_uploadTree( w, b2_kinematicBody );
	h_uploadTree( w, b2_dynamicBody );
	int rc = b2gDev_EnlargeTrees( w->dev, count );
	if ( rc != 0 ) h_fail( w, "tree enlargement", rc );
	for ( int t = 0; t < 2; ++t )
	{
		k->enlargeIds[t].count = 0;
		k->enlargeBoxes[t].count = 0;
	}
	for ( int i = 0; i < count; ++i )
	{
		/* the records' shapes are scattered: request a later record's shape ahead */
		if ( i + 8 < count ) __builtin_prefetch( &w->shapes.data[recs[4 * ( i + 8 ) + 1]].fatAABB, 1, 3 );
		int shapeId = recs[4 * i + 1];
		int enlarged = recs[4 * i + 2];
		int fastBullet = recs[4 * i + 3];
		h_shape* s = w->shapes.data + shapeId;
		if ( fastBullet == 0 && enlarged )
		{
			b2AABB fat = { { boxes[4 * i], boxes[4 * i + 1] }, { boxes[4 * i + 2], boxes[4 * i + 3] } };
			s->fatAABB = fat;
			int t = H_PROXY_TYPE( s->proxyKey ) == b2_dynamicBody ? 1 : 0;
			h_push( k->enlargeIds[t], H_PROXY_ID( s->proxyKey ) );
			h_push( k->enlargeBoxes[t], fat );
		}
		if ( fastBullet || enlarged ) h_bufferMove( w, s->proxyKey );
	}
	/* the device copies already hold the enlarged trees: the next upload is due only when
	   the host trees change again */
	const int types[2] = { b2_kinematicBody, b2_dynamicBody };
	for ( int t = 0; t < 2; ++t )
	{
		if ( k->enlargeIds[t].count == 0 ) continue;
		w->trees[types[t]].version += 1;
		w->uploadedTreeVersion[types[t]] = w->trees[types[t]].version;
	}
	if ( k->enlargeIds[0].count + k->enlargeIds[1].count > 0 )
	{
		pthread_mutex_lock( &k->mu );
		k->enlargePending = 1;
		k->busy = 1;
		pthread_cond_broadcast( &k->cv );
		pthread_mutex_unlock( &k->mu );
	}
	return 1;
}

static void h_enlargeProxies( h_world* w, const int* recs, const float* boxes, int count )
{
	if ( h_enlargeOnDevice( w, recs, boxes, count ) ) return;
	/* many records: the tree enlargements on the host pool, then the move buffer in order */
	if ( count >= 4 * H_ENLARGE_CHUNK )
	{
		h_enlargeJob job = { w, recs, boxes, count };
		int chunks = ( count + H_ENLARGE_CHUNK - 1 ) / H_ENLARGE_CHUNK;
		if ( h_parallelFor( h_hostThreads(), h_enlargeChunk, &job, chunks ) )
		{
			w->trees[b2_dynamicBody].version += 1;
			w->trees[b2_kinematicBody].version += 1;
			for ( int i = 0; i < count; ++i )
				if ( recs[4 * i + 3] != 0 || recs[4 * i + 2] != 0 ) h_bufferMove( w, w->shapes.data[recs[4 * i + 1]].proxyKey );
			return;
		}
	}
	for ( int i = 0; i < count; ++i )
	{
		int shapeId = recs[4 * i + 1];
		int enlarged = recs[4 * i + 2];
		int fastBullet = recs[4 * i + 3];
		h_shape* s = w->shapes.data + shapeId;
		if ( fastBullet )
		{
			h_bufferMove( w, s->proxyKey );
			continue;
		}
		if ( enlarged )
		{
			b2AABB fat = { { boxes[4 * i], boxes[4 * i + 1] }, { boxes[4 * i + 2], boxes[4 * i + 3] } };
			s->fatAABB = fat;
			h_treeEnlargeProxy( w->trees + H_PROXY_TYPE( s->proxyKey ), H_PROXY_ID( s->proxyKey ), fat );
			h_bufferMove( w, s->proxyKey );
		}
	}
}

/* solver.c:1917-1989: fast bullet bodies are swept after the broadphase enlargement,
   against the static, kinematic and dynamic trees as it left them; their shapes' grown
   boxes then enlarge the dynamic tree (their moves were buffered by the enlargement) */
static void h_solveBullets( h_world* w, const int* recs, int count )
{
	int* sims = NULL;
	int n = 0, last = -1;
	for ( int i = 0; i < count; ++i )
	{
		if ( recs[4 * i + 3] == 0 || recs[4 * i] == last ) continue;
		last = recs[4 * i];
		if ( sims == NULL ) sims = malloc( (size_t)count * sizeof( int ) );
		sims[n++] = last;
	}
	if ( n == 0 ) return;
	/* the host trees are swept as the enlargement left them */
	h_joinRebuild( w );
	/* a batched step records device work for its flushes; the bullet pass waits for its
	   results, so it runs on the world's own stream (the world's earlier work has been
	   flushed by now and nothing of this phase is recorded yet) */
	int recording = b2gDev_IsRecording( w->dev );
	if ( recording )
	{
		if ( b2gDev_RecordedCount( w->dev ) != 0 ) h_fail( w, "bullets inside a batched flush", -1 );
		b2gDev_BatchRecord( w->dev, 0 );
	}
	h_uploadTree( w, b2_kinematicBody );
	h_uploadTree( w, b2_dynamicBody );
	const int* brecs = NULL;
	const float* bboxes = NULL;
	int bcount = 0;
	int rc = b2gDev_SolveBullets( w->dev, &w->stepParams, w->awakeBodyIds.count, sims, n, &brecs, &bboxes, &bcount );
	free( sims );
	if ( recording ) b2gDev_BatchRecord( w->dev, 1 );
	if ( rc != 0 ) h_fail( w, "bullets", rc );
	h_tree* dynamicTree = w->trees + b2_dynamicBody;
	for ( int i = 0; i < bcount; ++i )
	{
		if ( brecs[2 * i + 1] == 0 ) continue;
		h_shape* s = w->shapes.data + brecs[2 * i];
		b2AABB fat = { { bboxes[4 * i], bboxes[4 * i + 1] }, { bboxes[4 * i + 2], bboxes[4 * i + 3] } };
		s->fatAABB = fat;
		h_treeEnlargeProxy( dynamicTree, H_PROXY_ID( s->proxyKey ), fat );
	}
}

/* ---- the step in four phases, split at its three waits/* ---- the step in four phases, split at its three waits (pair query, narrowphase,
   solver); b2World_Step runs them back to back, b2World_StepBatch runs each phase over
   many worlds and replaces the waits by one batched flush ---- */

/* phase 1: bookkeeping, device state, the pair query; returns whether work was issued */
int h_stepBegin( h_world* w, float timeStep, int subStepCount )
{
	w->moveEvents.count = 0;
	w->moveEventsValid = 0;
	w->shapeBoxesValid = 0;
	w->beginEvents.count = 0;
	w->sensorBeginEvents.count = 0;
	memset( &w->profile, 0, sizeof( w->profile ) );
	w->locked = 1;
	w->stepTicks = b2GetTicks();
	w->stepTimeStep = timeStep;

	/* a world change since the last step re-sends the device state: a query issued at the
	   last step's end does not hold */
	if ( w->devReady == 0 ) w->specStale = 1;
	h_ensureDevice( w );
	/* contacts whose solver set the API changed since the last step */
	w->wokeInStep = 0;
	h_flushSleepOps( w );
	/* from here on the device state moves on: host copies read before the step are stale */
	w->hostStateValid = 0;
	w->mirrorValid = 0;

	b2gStepParams* p = &w->stepParams;
	memset( p, 0, sizeof( *p ) );
	p->dt = timeStep;
	p->subStepCount = h_maxi( 1, subStepCount );
	if ( timeStep > 0.0f )
	{
		p->inv_dt = 1.0f / timeStep;
		p->h = timeStep / p->subStepCount;
		p->inv_h = p->subStepCount * p->inv_dt;
	}
	float contactHertz = h_min( w->contactHertz, 0.125f * p->inv_h );
	h_softness cs = h_makeSoft( contactHertz, w->contactDampingRatio, p->h );
	h_softness ss = h_makeSoft( 2.0f * contactHertz, w->contactDampingRatio, p->h );
	p->contactBiasRate = cs.biasRate;
	p->contactMassScale = cs.massScale;
	p->contactImpulseScale = cs.impulseScale;
	p->staticBiasRate = ss.biasRate;
	p->staticMassScale = ss.massScale;
	p->staticImpulseScale = ss.impulseScale;
	p->restitutionThreshold = w->restitutionThreshold;
	p->maxLinearVelocity = w->maxLinearSpeed;
	p->contactSpeed = w->contactSpeed;
	p->contactHertz = w->contactHertz;
	p->contactDampingRatio = w->contactDampingRatio;
	p->gravityX = w->gravity.x;
	p->gravityY = w->gravity.y;
	p->enableWarmStarting = w->enableWarmStarting;
	p->enableContinuous = w->enableContinuous;
	p->enableSleep = w->enableSleep;
	p->enableContactSoftening = w->enableContactSoftening;
	p->contactRecycleDistance = 10.0f * H_LINEAR_SLOP;

	w->stepT0 = b2GetTicks();
	w->stepPairsIssued = h_pairsIssue( w );
	return w->stepPairsIssued;
}

/* phase 2: contacts from the pairs, then the narrowphase is issued */
void h_stepPairs( h_world* w )
{
	if ( w->stepPairsIssued ) h_pairsFinish( w );
	w->profile.pairs = h_ms( w->stepT0 );
	w->stepT0 = b2GetTicks();
	uint64_t lap = w->stepT0;
	h_flushContacts( w );
	h_uploadColors( w );
	h_lap( w, H_PHASE_UPLOADS, &lap );
	int rc = b2gDev_CollideIssue( w->dev, &w->stepParams, w->contactIdPool.nextIndex );
	if ( rc != 0 ) h_fail( w, "narrowphase", rc );
}

/* phase 3: the contact-state pass and graph coloring, then the solver is issued unless
   `oneBlockOnly` is set and the world's solve is not a one-CTA solve (it is then issued in
   phase 4); returns whether the solver was issued */
int h_stepCollide( h_world* w, int oneBlockOnly )
{
	uint64_t lap = b2GetTicks();
	const int* changes = NULL;
	int changeCount = 0, recycled = 0;
	int rc = b2gDev_CollideCollect( w->dev, &changes, &changeCount, &recycled );
	if ( rc != 0 ) h_fail( w, "narrowphase", rc );
	/* contacts began or ended touching: the solve's component analysis starts on the device
	   now, beside the state pass */
	if ( changeCount > 0 && w->stepTimeStep > 0.0f && b2gDev_IsRecording( w->dev ) == 0 )
	{
		rc = b2gDev_ComponentsEarly( w->dev, w->awakeBodyIds.count );
		if ( rc != 0 ) h_fail( w, "component analysis", rc );
	}
	h_lap( w, H_PHASE_COLLIDE, &lap );
	w->recycledContactCount = recycled;
	h_contactStatePass( w, changes, changeCount );
	h_lap( w, H_PHASE_STATE_PASS, &lap );
	h_flushContacts( w );
	/* sets woken by contacts that started touching join the device awake set */
	h_flushSleepOps( w );
	h_lap( w, H_PHASE_UPLOADS, &lap );
	w->profile.collide = h_ms( w->stepT0 );
	w->stepSolveIssued = 0;
	w->stepSolveLate = 0;
	if ( w->stepTimeStep <= 0.0f ) return 0;
	w->stepT0 = b2GetTicks();
	lap = w->stepT0;
	w->stepIndex += 1;
	h_uploadColors( w );
	h_uploadJoints( w );
	if ( w->wokeInStep )
	{
		/* contacts that re-entered the colors take their bodies' new awake indices */
		int rc = b2gDev_RefreshContactBodies( w->dev );
		if ( rc != 0 ) h_fail( w, "contact refresh", rc );
		w->wokeInStep = 0;
	}
	h_lap( w, H_PHASE_UPLOADS, &lap );
	/* fast bodies sweep against the static tree in the finalize stage */
	if ( w->enableContinuous ) h_uploadTree( w, b2_staticBody );
	h_lap( w, H_PHASE_TREE_UPLOAD, &lap );
	if ( w->awakeBodyIds.count == 0 ) return 0;
	h_stepIslands( w );
	if ( oneBlockOnly && b2gDev_SolveFitsOneBlock( w->dev, w->awakeBodyIds.count ) == 0 )
	{
		w->stepSolveLate = 1;
		return 0;
	}
	return h_stepSolveIssue( w );
}

int h_stepSolveIssue( h_world* w )
{
	int activeColors[B2_GRAPH_COLOR_COUNT];
	int activeCount = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT - 1; ++i )
		if ( w->colors[i].contactIds.count + w->colors[i].jointIds.count > 0 ) activeColors[activeCount++] = i;
	uint64_t lap = b2GetTicks();
	if ( w->tape != NULL ) h_tapeCapture( w, &w->stepParams );
	h_lap( w, H_PHASE_TAPE, &lap );
	int rc = b2gDev_SolveIssue( w->dev, &w->stepParams, activeColors, activeCount, w->awakeBodyIds.count );
	if ( rc != 0 ) h_fail( w, "solver", rc );
	h_lap( w, H_PHASE_SOLVE, &lap );
	w->stepSolveIssued = 1;
	return 1;
}

/* phase 4: enlarged proxies into the broadphase, events, and the step's end */
void h_stepFinish( h_world* w )
{
	uint64_t lap = b2GetTicks();
	if ( w->stepSolveIssued )
	{
		const int* recs = NULL;
		const float* boxes = NULL;
		int enlargedCount = 0, status = 0;
		int rc = b2gDev_SolveCollect( w->dev, &recs, &enlargedCount, &boxes, &status );
		if ( rc != 0 ) h_fail( w, "solver", rc );
		h_lap( w, H_PHASE_SOLVE, &lap );
		h_joinRebuild( w );
		h_lap( w, H_PHASE_TREE_REBUILD, &lap );
		w->lastStatus |= status; /* sticky: every step's failures since the world was created */
		{
			b2gStepCounters sc;
			b2gDev_LastCounters( w->dev, &sc );
			w->continuousSweeps += sc.continuousSweeps;
			w->continuousHits += sc.continuousHits;
		}
		if ( status & B2G_STATUS_NAN ) fprintf( stderr, "box2d_gb300: unstable body state (NaN or infinite velocity)\n" );
		if ( status & B2G_STATUS_CAPACITY )
			fprintf( stderr, "box2d_gb300: a device query ran out of traversal stack; this step missed some pairs or sweeps\n" );
		/* the finalize kernel cleared the force and torque of every awake body (solver.c:710-712) */
		for ( int i = 0; i < w->forcedBodies.count; ++i )
		{
			h_body* fb = w->bodies.data + w->forcedBodies.data[i];
			fb->force = h_v( 0.0f, 0.0f );
			fb->torque = 0.0f;
		}
		w->forcedBodies.count = 0;
		h_enlargeProxies( w, recs, boxes, enlargedCount );
		h_solveBullets( w, recs, enlargedCount );
		h_lap( w, H_PHASE_ENLARGE, &lap );
		{
			/* island sleeping comes last (solver.c:2024-2080) */
			const uint32_t* bits = NULL;
			int islandCount = 0;
			unsigned long long splitKey = 0;
			b2gDev_IslandResults( w->dev, &bits, &islandCount, &splitKey );
			h_sleepPass( w, bits, splitKey );
		}
	}
	if ( w->stepTimeStep > 0.0f ) w->profile.solve = h_ms( w->stepT0 );
	/* a step that issued no solve still waits for its rebuild here; after a solve the worker
	   may go on enlarging the host trees past the step's end */
	if ( w->stepSolveIssued == 0 ) h_joinRebuild( w );
	/* sensor overlaps come last (physics_world.c:961-966); a batched step runs them after
	   its last flush, when the device state is final */
	if ( w->sensors.count > 0 && b2gDev_IsRecording( w->dev ) == 0 )
	{
		uint64_t sensorTicks = b2GetTicks();
		h_overlapSensors( w, w->endEventArrayIndex );
		w->profile.sensors = h_ms( sensorTicks );
	}
	w->hostStateValid = 0;
	w->mirrorValid = 0;
	w->jointsHostValid = 0;
	/* the step's body state follows its work down, so move events and body getters wait
	   for it instead of asking for it (physics_world.c:863-867 makes move events part of
	   the step's output) */
	if ( w->devReady )
	{
		int rc = b2gDev_PrefetchState( w->dev, w->bodies.count, w->awakeBodyIds.count );
		if ( rc != 0 ) h_fail( w, "state prefetch", rc );
	}
	if ( w->stepSolveIssued ) h_pairsSpeculate( w );
	w->profile.step = h_ms( w->stepTicks );
	w->endEventArrayIndex = 1 - w->endEventArrayIndex;
	w->endEvents[w->endEventArrayIndex].count = 0;
	w->sensorEndEvents[w->endEventArrayIndex].count = 0;
	w->locked = 0;
	(void)h_cmpInt;
}

void b2World_Step( b2WorldId worldId, float timeStep, int subStepCount )
{
	h_world* w = h_worldFromId( worldId );
	if ( w == NULL || w->locked ) return;
	if ( h_stepBegin( w, timeStep, subStepCount ) ) b2gDev_Synchronize( w->dev );
	h_stepPairs( w );
	b2gDev_Synchronize( w->dev );
	if ( h_stepCollide( w, 0 ) ) b2gDev_Synchronize( w->dev );
	h_stepFinish( w );
}
