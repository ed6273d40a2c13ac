/*
 * Islands, solver sets and island sleeping for the GB300 step library. Restates
 * island.c:14-640 (persistent islands: link, unlink, merge, union-find split),
 * solver_set.c:17-480 (wake, sleep and merge of solver sets) and the island parts of
 * solver.c:637-695 and :2024-2080 (sleep timers, split candidate, sleep pass) of the
 * reference, on the host records of b2g_world.h.
 *
 * The host keeps every order-defining array in the reference's order: island bodies,
 * contacts and joints, the awake set's island list, sleeping sets, the awake body list and
 * the graph colors. The device follows through a few bulk operations:
 *   - the finalize kernel updates the sleep timers and sets one bit per island that stays
 *     awake, and returns the split candidate (b2gDev_UploadIslands / b2gDev_IslandResults);
 *   - bodies woken inside a step are appended to the device awake set (b2gDev_WakeBodies),
 *     bodies put to sleep leave it by the same swap-removals as on the host
 *     (b2gDev_SleepBodies);
 *   - contacts moving in or out of the collided sets toggle a flag the narrowphase reads
 *     (b2gDev_SetContactsAsleep).
 * Changes made between steps by the API refill the device from the host instead.
 */
#include "b2g_world.h"

#include <stdio.h>

/* ---------------- setup ---------------- */

void h_islandsInit( h_world* w )
{
	w->splitIslandId = B2_NULL_INDEX;
	/* solver set ids 0, 1 and 2 are the static, disabled and awake sets
	   (physics_world.c:209-227); sleeping sets take the ids after them */
	for ( int i = 0; i < H_FIRST_SLEEPING_SET; ++i )
	{
		h_sleepSet z;
		memset( &z, 0, sizeof( z ) );
		z.setIndex = h_allocId( &w->setIdPool );
		h_push( w->sets, z );
	}
}

static void h_sleepSetClear( h_sleepSet* s )
{
	h_free( s->bodyIds );
	h_free( s->contactIds );
	h_free( s->jointIds );
	h_free( s->islandIds );
}

void h_islandsFree( h_world* w )
{
	for ( int i = 0; i < w->islands.count; ++i )
	{
		h_free( w->islands.data[i].bodies );
		h_free( w->islands.data[i].contacts );
		h_free( w->islands.data[i].joints );
	}
	h_free( w->islands );
	h_free( w->islandIdPool.freeArray );
	h_free( w->awakeIslandIds );
	for ( int i = 0; i < w->sets.count; ++i ) h_sleepSetClear( w->sets.data + i );
	h_free( w->sets );
	h_free( w->setIdPool.freeArray );
	h_free( w->disabledContactIds );
	h_free( w->pendingWake );
	h_free( w->pendingContacts );
	h_free( w->sleptBodies );
	free( w->sleepPerm );
	w->sleepPerm = NULL;
}

/* the island list of a set: the awake set's or a sleeping set's */
static h_intArray* h_setIslands( h_world* w, int setIndex )
{
	return setIndex == H_AWAKE_SET ? &w->awakeIslandIds : &w->sets.data[setIndex].islandIds;
}

/* ---------------- islands (island.c) ---------------- */

/* island.c:14-47 */
static h_island* h_createIsland( h_world* w, int setIndex )
{
	int islandId = h_allocId( &w->islandIdPool );
	if ( islandId == w->islands.count )
	{
		h_island z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->islands, z );
	}
	h_intArray* list = h_setIslands( w, setIndex );
	h_island* island = w->islands.data + islandId;
	island->setIndex = setIndex;
	island->localIndex = list->count;
	island->islandId = islandId;
	island->bodies.count = 0;
	island->contacts.count = 0;
	island->joints.count = 0;
	island->constraintRemoveCount = 0;
	h_push( *list, islandId );
	w->islandsDirty = 1;
	return island;
}

/* island.c:49-80: swap-remove from the set's island list, free the id */
static void h_destroySleepingSet( h_world* w, int setIndex );

static void h_destroyIsland( h_world* w, int islandId )
{
	if ( w->splitIslandId == islandId ) w->splitIslandId = B2_NULL_INDEX;
	h_island* island = w->islands.data + islandId;
	h_intArray* list = h_setIslands( w, island->setIndex );
	int localIndex = island->localIndex;
	int lastIndex = list->count - 1;
	int movedId = list->data[lastIndex];
	list->data[localIndex] = movedId;
	w->islands.data[movedId].localIndex = localIndex;
	list->count -= 1;
	h_free( island->bodies );
	h_free( island->contacts );
	h_free( island->joints );
	island->constraintRemoveCount = 0;
	island->localIndex = B2_NULL_INDEX;
	island->islandId = B2_NULL_INDEX;
	island->setIndex = B2_NULL_INDEX;
	h_freeId( &w->islandIdPool, islandId );
	w->islandsDirty = 1;
}

/* island.c:82-170: the bigger island (by body count, ties to A) takes the smaller one's
   bodies, contacts and joints in order */
static int h_mergeIslands( h_world* w, int islandIdA, int islandIdB )
{
	if ( islandIdA == islandIdB ) return islandIdA;
	if ( islandIdA == B2_NULL_INDEX ) return islandIdB;
	if ( islandIdB == B2_NULL_INDEX ) return islandIdA;
	h_island* islandA = w->islands.data + islandIdA;
	h_island* islandB = w->islands.data + islandIdB;
	h_island* big = islandA->bodies.count >= islandB->bodies.count ? islandA : islandB;
	h_island* small = big == islandA ? islandB : islandA;
	int bigId = big->islandId;
	for ( int i = 0; i < small->bodies.count; ++i )
	{
		int bodyId = small->bodies.data[i];
		h_body* body = w->bodies.data + bodyId;
		body->islandId = bigId;
		body->islandIndex = big->bodies.count;
		h_push( big->bodies, bodyId );
	}
	for ( int i = 0; i < small->contacts.count; ++i )
	{
		h_link link = small->contacts.data[i];
		h_contact* contact = w->contacts.data + link.id;
		contact->islandId = bigId;
		contact->islandIndex = big->contacts.count;
		h_push( big->contacts, link );
	}
	for ( int i = 0; i < small->joints.count; ++i )
	{
		h_link link = small->joints.data[i];
		h_joint* joint = w->joints.data + link.id;
		joint->islandId = bigId;
		joint->islandIndex = big->joints.count;
		h_push( big->joints, link );
	}
	big->constraintRemoveCount += small->constraintRemoveCount;
	h_destroyIsland( w, small->islandId );
	return bigId;
}

/* body.c:107-118 */
void h_createIslandForBody( h_world* w, int setIndex, h_body* body )
{
	int bodyId = body->id;
	h_island* island = h_createIsland( w, setIndex );
	h_push( island->bodies, bodyId );
	body = w->bodies.data + bodyId;
	body->islandId = island->islandId;
	body->islandIndex = 0;
}

/* island.c:172-230: a contact that starts touching wakes a sleeping partner of an awake
   body, then joins (and merges) the islands of its bodies */
void h_linkContact( h_world* w, h_contact* contact )
{
	int bodyIdA = contact->edges[0].bodyId, bodyIdB = contact->edges[1].bodyId;
	h_body* bodyA = w->bodies.data + bodyIdA;
	h_body* bodyB = w->bodies.data + bodyIdB;
	if ( bodyA->setIndex == H_AWAKE_SET && bodyB->setIndex >= H_FIRST_SLEEPING_SET ) h_wakeSolverSet( w, bodyB->setIndex );
	if ( bodyB->setIndex == H_AWAKE_SET && bodyA->setIndex >= H_FIRST_SLEEPING_SET ) h_wakeSolverSet( w, bodyA->setIndex );
	int islandId = h_mergeIslands( w, bodyA->islandId, bodyB->islandId );
	h_island* island = w->islands.data + islandId;
	contact->islandId = islandId;
	contact->islandIndex = island->contacts.count;
	h_link link = { contact->contactId, bodyIdA, bodyIdB };
	h_push( island->contacts, link );
	w->islandsDirty = 1;
}

/* island.c:232-259: the island keeps its bodies and counts the removal (a split candidate) */
void h_unlinkContact( h_world* w, h_contact* contact )
{
	h_island* island = w->islands.data + contact->islandId;
	int removeIndex = contact->islandIndex;
	int moved = h_removeSwap( island->contacts, removeIndex );
	if ( moved != B2_NULL_INDEX ) w->contacts.data[island->contacts.data[removeIndex].id].islandIndex = removeIndex;
	contact->islandId = B2_NULL_INDEX;
	contact->islandIndex = B2_NULL_INDEX;
	island->constraintRemoveCount += 1;
	w->islandsDirty = 1;
}

/* island.c:311-340 */
void h_unlinkJoint( h_world* w, h_joint* joint )
{
	if ( joint->islandId == B2_NULL_INDEX ) return;
	h_island* island = w->islands.data + joint->islandId;
	int removeIndex = joint->islandIndex;
	int moved = h_removeSwap( island->joints, removeIndex );
	if ( moved != B2_NULL_INDEX ) w->joints.data[island->joints.data[removeIndex].id].islandIndex = removeIndex;
	joint->islandId = B2_NULL_INDEX;
	joint->islandIndex = B2_NULL_INDEX;
	island->constraintRemoveCount += 1;
	w->islandsDirty = 1;
}

/* body.c:120-155: the body leaves its island (the last body takes its slot); an island
   left without bodies is destroyed */
void h_removeBodyFromIsland( h_world* w, h_body* body )
{
	if ( body->islandId == B2_NULL_INDEX ) return;
	int islandId = body->islandId;
	h_island* island = w->islands.data + islandId;
	int localIndex = body->islandIndex;
	int movedBodyId = island->bodies.data[island->bodies.count - 1];
	island->bodies.data[localIndex] = movedBodyId;
	w->bodies.data[movedBodyId].islandIndex = localIndex;
	island->bodies.count -= 1;
	if ( island->bodies.count == 0 ) h_destroyIsland( w, islandId );
	w->islandsDirty = 1;
	body->islandId = B2_NULL_INDEX;
	body->islandIndex = B2_NULL_INDEX;
}

/* solver_set.c:16-27 for a sleeping set left empty */
void h_freeSleepingSet( h_world* w, int setIndex ) { h_destroySleepingSet( w, setIndex ); }

/* island.c:280-307 */
void h_linkJoint( h_world* w, h_joint* joint )
{
	int bodyIdA = joint->edges[0].bodyId, bodyIdB = joint->edges[1].bodyId;
	h_body* bodyA = w->bodies.data + bodyIdA;
	h_body* bodyB = w->bodies.data + bodyIdB;
	if ( bodyA->setIndex == H_AWAKE_SET && bodyB->setIndex >= H_FIRST_SLEEPING_SET ) h_wakeSolverSet( w, bodyB->setIndex );
	else if ( bodyB->setIndex == H_AWAKE_SET && bodyA->setIndex >= H_FIRST_SLEEPING_SET ) h_wakeSolverSet( w, bodyA->setIndex );
	int islandId = h_mergeIslands( w, bodyA->islandId, bodyB->islandId );
	h_island* island = w->islands.data + islandId;
	joint->islandId = islandId;
	joint->islandIndex = island->joints.count;
	h_link link = { joint->jointId, bodyIdA, bodyIdB };
	h_push( island->joints, link );
	w->islandsDirty = 1;
}

/* union-find with path halving (island.c:338-380); union by rank */
static int h_findRoot( int* parents, int node )
{
	while ( parents[node] != node )
	{
		int grandParent = parents[parents[node]];
		parents[node] = grandParent;
		node = grandParent;
	}
	return node;
}

static void h_union( int* parents, int* ranks, int a, int b )
{
	int rootA = h_findRoot( parents, a ), rootB = h_findRoot( parents, b );
	if ( rootA == rootB ) return;
	if ( ranks[rootA] < ranks[rootB] ) parents[rootA] = rootB;
	else if ( ranks[rootA] > ranks[rootB] ) parents[rootB] = rootA;
	else
	{
		parents[rootB] = rootA;
		ranks[rootA] += 1;
	}
}

/* island.c:382-612: split an awake island into its connected components. Components are
   numbered by their first body in the island's body order; bodies, contacts and joints keep
   their order inside the new islands; static bodies connect nothing. */
void h_splitIsland( h_world* w, int baseId )
{
	h_island* base = w->islands.data + baseId;
	int bodyCount = base->bodies.count;
	int* parents = malloc( (size_t)( bodyCount > 0 ? bodyCount : 1 ) * sizeof( int ) );
	int* ranks = calloc( (size_t)( bodyCount > 0 ? bodyCount : 1 ), sizeof( int ) );
	for ( int i = 0; i < bodyCount; ++i ) parents[i] = i;
	for ( int pass = 0; pass < 2; ++pass )
	{
		const h_linkArray* links = pass == 0 ? &base->contacts : &base->joints;
		for ( int i = 0; i < links->count; ++i )
		{
			int indexA = w->bodies.data[links->data[i].bodyIdA].islandIndex;
			int indexB = w->bodies.data[links->data[i].bodyIdB].islandIndex;
			if ( indexA != B2_NULL_INDEX && indexB != B2_NULL_INDEX ) h_union( parents, ranks, indexA, indexB );
		}
	}
	free( ranks );
	int componentCount = 0;
	for ( int i = 0; i < bodyCount; ++i )
	{
		parents[i] = h_findRoot( parents, i );
		if ( parents[i] == i ) componentCount += 1;
	}
	if ( componentCount <= 1 )
	{
		base->constraintRemoveCount = 0;
		free( parents );
		w->islandsDirty = 1;
		return;
	}
	/* detach the base island's arrays: the new islands are filled from them */
	h_intArray bodies = base->bodies;
	h_linkArray contacts = base->contacts;
	h_linkArray joints = base->joints;
	memset( &base->bodies, 0, sizeof( base->bodies ) );
	memset( &base->contacts, 0, sizeof( base->contacts ) );
	memset( &base->joints, 0, sizeof( base->joints ) );
	base = NULL;
	int* rootMap = malloc( (size_t)bodyCount * sizeof( int ) );
	for ( int i = 0; i < bodyCount; ++i ) rootMap[i] = B2_NULL_INDEX;
	int islandCount = 0;
	for ( int i = 0; i < bodyCount; ++i )
		if ( rootMap[parents[i]] == B2_NULL_INDEX ) rootMap[parents[i]] = islandCount++;
	int* islandIds = malloc( (size_t)islandCount * sizeof( int ) );
	for ( int i = 0; i < islandCount; ++i ) islandIds[i] = h_createIsland( w, H_AWAKE_SET )->islandId;
	for ( int i = 0; i < bodyCount; ++i )
	{
		int bodyId = bodies.data[i];
		int islandId = islandIds[rootMap[parents[i]]];
		h_island* island = w->islands.data + islandId;
		h_body* body = w->bodies.data + bodyId;
		body->islandId = islandId;
		body->islandIndex = island->bodies.count;
		h_push( island->bodies, bodyId );
	}
	for ( int pass = 0; pass < 2; ++pass )
	{
		const h_linkArray* links = pass == 0 ? &contacts : &joints;
		for ( int i = 0; i < links->count; ++i )
		{
			h_link link = links->data[i];
			int islandIdA = w->bodies.data[link.bodyIdA].islandId;
			int islandId = islandIdA != B2_NULL_INDEX ? islandIdA : w->bodies.data[link.bodyIdB].islandId;
			h_island* island = w->islands.data + islandId;
			if ( pass == 0 )
			{
				h_contact* contact = w->contacts.data + link.id;
				contact->islandId = islandId;
				contact->islandIndex = island->contacts.count;
				h_push( island->contacts, link );
			}
			else
			{
				h_joint* joint = w->joints.data + link.id;
				joint->islandId = islandId;
				joint->islandIndex = island->joints.count;
				h_push( island->joints, link );
			}
		}
	}
	h_destroyIsland( w, baseId );
	free( bodies.data );
	free( contacts.data );
	free( joints.data );
	free( islandIds );
	free( rootMap );
	free( parents );
}

/* ---------------- solver sets (solver_set.c) ---------------- */

int h_allocSleepingSet( h_world* w )
{
	int setId = h_allocId( &w->setIdPool );
	if ( setId == w->sets.count )
	{
		h_sleepSet z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->sets, z );
	}
	h_sleepSet* set = w->sets.data + setId;
	h_sleepSetClear( set );
	set->setIndex = setId;
	return setId;
}

/* solver_set.c:17-27 */
static void h_destroySleepingSet( h_world* w, int setIndex )
{
	h_sleepSet* set = w->sets.data + setIndex;
	h_sleepSetClear( set );
	set->setIndex = B2_NULL_INDEX;
	h_freeId( &w->setIdPool, setIndex );
}

/* joints entering and leaving the graph colors (constraint_graph.c:216-330) */
void h_addJointToGraph( h_world* w, h_joint* joint )
{
	int bodyIdA = joint->edges[0].bodyId, bodyIdB = joint->edges[1].bodyId;
	int colorIndex = h_assignJointColor( w, bodyIdA, bodyIdB, w->bodies.data[bodyIdA].type, w->bodies.data[bodyIdB].type );
	h_color* color = w->colors + colorIndex;
	joint->colorIndex = colorIndex;
	joint->localIndex = color->jointIds.count;
	h_push( color->jointIds, joint->jointId );
	w->jointsDirty = 1;
}

void h_removeJointFromGraph( h_world* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex )
{
	h_color* color = w->colors + colorIndex;
	if ( colorIndex != B2G_OVERFLOW_INDEX )
	{
		h_bitClear( &color->bodySet, bodyIdA );
		h_bitClear( &color->bodySet, bodyIdB );
	}
	int moved = h_removeSwap( color->jointIds, localIndex );
	if ( moved != B2_NULL_INDEX ) w->joints.data[color->jointIds.data[localIndex]].localIndex = localIndex;
	w->jointsDirty = 1;
}

/* a set change made by the API between steps: the device is refilled from the host records
   before the next step (a change inside a step is sent by the step itself) */
static void h_setChangeOutsideStep( h_world* w )
{
	if ( w->locked == 0 ) h_markHostChanged( w );
}

/* solver_set.c:29-137: the set's bodies are appended to the awake set with zero velocity,
   its non-touching contacts in the disabled set come back to the awake set, its touching
   contacts and joints re-enter the graph colors, its islands join the awake set */
void h_wakeSolverSet( h_world* w, int setIndex )
{
	h_setChangeOutsideStep( w );
	h_sleepSet* set = w->sets.data + setIndex;
	for ( int i = 0; i < set->bodyIds.count; ++i )
	{
		int bodyId = set->bodyIds.data[i];
		h_body* body = w->bodies.data + bodyId;
		body->setIndex = H_AWAKE_SET;
		body->localIndex = w->awakeBodyIds.count;
		body->sleepTime = 0.0f;
		body->linearVelocity = h_v( 0.0f, 0.0f );
		body->angularVelocity = 0.0f;
		h_push( w->awakeBodyIds, bodyId );
		if ( w->locked )
		{
			float params[8] = { 0.0f, 0.0f, 0.0f, body->linearDamping, body->angularDamping, body->gravityScale, body->invMass,
								body->invInertia };
			int rec[10];
			rec[0] = bodyId;
			rec[1] = body->localIndex;
			memcpy( rec + 2, params, sizeof( params ) );
			for ( int k = 0; k < 10; ++k ) h_push( w->pendingWake, rec[k] );
			w->wokeInStep = 1;
		}
		for ( int key = body->headContactKey; key != B2_NULL_INDEX; )
		{
			h_contact* contact = w->contacts.data + ( key >> 1 );
			key = contact->edges[key & 1].nextKey;
			if ( contact->setIndex != H_DISABLED_SET ) continue;
			int localIndex = contact->localIndex;
			contact->setIndex = H_AWAKE_SET;
			contact->localIndex = w->awakeContactIds.count;
			h_push( w->awakeContactIds, contact->contactId );
			int moved = h_removeSwap( w->disabledContactIds, localIndex );
			if ( moved != B2_NULL_INDEX ) w->contacts.data[w->disabledContactIds.data[localIndex]].localIndex = localIndex;
			h_push( w->pendingContacts, contact->contactId );
		}
	}
	for ( int i = 0; i < set->contactIds.count; ++i )
	{
		h_contact* contact = w->contacts.data + set->contactIds.data[i];
		h_addContactToGraph( w, contact );
		contact->setIndex = H_AWAKE_SET;
		h_push( w->pendingContacts, contact->contactId );
	}
	for ( int i = 0; i < set->jointIds.count; ++i )
	{
		h_joint* joint = w->joints.data + set->jointIds.data[i];
		h_addJointToGraph( w, joint );
		joint->setIndex = H_AWAKE_SET;
	}
	for ( int i = 0; i < set->islandIds.count; ++i )
	{
		int islandId = set->islandIds.data[i];
		h_island* island = w->islands.data + islandId;
		island->setIndex = H_AWAKE_SET;
		island->localIndex = w->awakeIslandIds.count;
		h_push( w->awakeIslandIds, islandId );
	}
	h_destroySleepingSet( w, setIndex );
	w->islandsDirty = 1;
	w->setChangeCount += 1;
}

/* body.c:334-344 */
int h_wakeBody( h_world* w, h_body* body )
{
	if ( body->setIndex >= H_FIRST_SLEEPING_SET )
	{
		h_wakeSolverSet( w, body->setIndex );
		return 1;
	}
	return 0;
}

/* b2RemoveBodySim on the awake set (body.c:34-43); the sleep pass mirrors the move on the
   slot permutation it sends to the device */
static void h_removeAwakeBody( h_world* w, int localIndex )
{
	int moved = h_removeSwap( w->awakeBodyIds, localIndex );
	if ( moved != B2_NULL_INDEX )
	{
		w->bodies.data[w->awakeBodyIds.data[localIndex]].localIndex = localIndex;
		if ( w->sleepPerm != NULL ) w->sleepPerm[localIndex] = w->sleepPerm[moved];
	}
}

/* solver_set.c:139-397: an island whose bodies are all sleepy moves to a new sleeping set:
   its bodies leave the awake set (swap-removal), non-touching contacts between sleeping
   bodies go to the disabled set, touching contacts and joints leave the graph colors */
void h_trySleepIsland( h_world* w, int islandId )
{
	h_island* island = w->islands.data + islandId;
	if ( island->constraintRemoveCount > 0 && island->bodies.count > 1 ) return;
	h_setChangeOutsideStep( w );
	int sleepSetId = h_allocSleepingSet( w );
	h_sleepSet* sleepSet = w->sets.data + sleepSetId;
	for ( int i = 0; i < island->bodies.count; ++i )
	{
		int bodyId = island->bodies.data[i];
		h_body* body = w->bodies.data + bodyId;
		if ( body->bodyMoveIndex != B2_NULL_INDEX )
		{
			if ( w->moveEventsValid && body->bodyMoveIndex < w->moveEvents.count )
				w->moveEvents.data[body->bodyMoveIndex].fellAsleep = true;
			body->bodyMoveIndex = B2_NULL_INDEX;
		}
		int awakeIndex = body->localIndex;
		h_push( sleepSet->bodyIds, bodyId );
		h_removeAwakeBody( w, awakeIndex );
		if ( w->sleepPerm != NULL ) h_push( w->sleptBodies, bodyId );
		body->setIndex = sleepSetId;
		body->localIndex = sleepSet->bodyIds.count - 1;
		for ( int key = body->headContactKey; key != B2_NULL_INDEX; )
		{
			int contactId = key >> 1, edgeIndex = key & 1;
			h_contact* contact = w->contacts.data + contactId;
			key = contact->edges[edgeIndex].nextKey;
			if ( contact->setIndex == H_DISABLED_SET ) continue;
			if ( contact->colorIndex != B2_NULL_INDEX ) continue;
			int otherBodyId = contact->edges[edgeIndex ^ 1].bodyId;
			if ( w->bodies.data[otherBodyId].setIndex == H_AWAKE_SET ) continue;
			int localIndex = contact->localIndex;
			contact->setIndex = H_DISABLED_SET;
			contact->localIndex = w->disabledContactIds.count;
			h_push( w->disabledContactIds, contactId );
			int moved = h_removeSwap( w->awakeContactIds, localIndex );
			if ( moved != B2_NULL_INDEX ) w->contacts.data[w->awakeContactIds.data[localIndex]].localIndex = localIndex;
			h_push( w->pendingContacts, contactId );
		}
	}
	for ( int i = 0; i < island->contacts.count; ++i )
	{
		h_contact* contact = w->contacts.data + island->contacts.data[i].id;
		int colorIndex = contact->colorIndex;
		int localIndex = contact->localIndex;
		h_color* color = w->colors + colorIndex;
		if ( colorIndex != B2G_OVERFLOW_INDEX )
		{
			h_bitClear( &color->bodySet, contact->edges[0].bodyId );
			h_bitClear( &color->bodySet, contact->edges[1].bodyId );
		}
		h_push( sleepSet->contactIds, contact->contactId );
		int moved = h_removeSwap( color->contactIds, localIndex );
		if ( moved != B2_NULL_INDEX ) w->contacts.data[color->contactIds.data[localIndex]].localIndex = localIndex;
		contact->setIndex = sleepSetId;
		contact->colorIndex = B2_NULL_INDEX;
		contact->localIndex = sleepSet->contactIds.count - 1;
		h_push( w->pendingContacts, contact->contactId );
		w->colorsDirty = 1;
	}
	for ( int i = 0; i < island->joints.count; ++i )
	{
		h_joint* joint = w->joints.data + island->joints.data[i].id;
		h_push( sleepSet->jointIds, joint->jointId );
		h_removeJointFromGraph( w, joint->edges[0].bodyId, joint->edges[1].bodyId, joint->colorIndex, joint->localIndex );
		joint->setIndex = sleepSetId;
		joint->colorIndex = B2_NULL_INDEX;
		joint->localIndex = sleepSet->jointIds.count - 1;
	}
	{
		int islandIndex = island->localIndex;
		h_push( sleepSet->islandIds, islandId );
		int moved = h_removeSwap( w->awakeIslandIds, islandIndex );
		if ( moved != B2_NULL_INDEX ) w->islands.data[w->awakeIslandIds.data[islandIndex]].localIndex = islandIndex;
		island->setIndex = sleepSetId;
		island->localIndex = 0;
	}
	if ( w->splitIslandId == islandId ) w->splitIslandId = B2_NULL_INDEX;
	w->islandsDirty = 1;
	w->setChangeCount += 1;
}

/* solver_set.c:402-480: two sleeping sets joined by a new joint become one; the set with
   fewer bodies moves into the other */
void h_mergeSolverSets( h_world* w, int setId1, int setId2 )
{
	if ( w->sets.data[setId1].bodyIds.count < w->sets.data[setId2].bodyIds.count )
	{
		int t = setId1;
		setId1 = setId2;
		setId2 = t;
	}
	h_sleepSet* set1 = w->sets.data + setId1;
	h_sleepSet* set2 = w->sets.data + setId2;
	for ( int i = 0; i < set2->bodyIds.count; ++i )
	{
		h_body* body = w->bodies.data + set2->bodyIds.data[i];
		body->setIndex = setId1;
		body->localIndex = set1->bodyIds.count;
		h_push( set1->bodyIds, body->id );
	}
	for ( int i = 0; i < set2->contactIds.count; ++i )
	{
		h_contact* contact = w->contacts.data + set2->contactIds.data[i];
		contact->setIndex = setId1;
		contact->localIndex = set1->contactIds.count;
		h_push( set1->contactIds, contact->contactId );
	}
	for ( int i = 0; i < set2->jointIds.count; ++i )
	{
		h_joint* joint = w->joints.data + set2->jointIds.data[i];
		joint->setIndex = setId1;
		joint->localIndex = set1->jointIds.count;
		h_push( set1->jointIds, joint->jointId );
	}
	for ( int i = 0; i < set2->islandIds.count; ++i )
	{
		int islandId = set2->islandIds.data[i];
		h_island* island = w->islands.data + islandId;
		island->setIndex = setId1;
		island->localIndex = set1->islandIds.count;
		h_push( set1->islandIds, islandId );
	}
	h_destroySleepingSet( w, setId2 );
}

/* ---------------- the step's island work ---------------- */

/* device work of the set changes made since the last call: woken bodies (inside a step)
   and contacts that left or rejoined the collided sets */
void h_flushSleepOps( h_world* w )
{
	int rc = 0;
	if ( w->pendingWake.count > 0 )
	{
		if ( w->devReady ) rc = b2gDev_WakeBodies( w->dev, w->awakeBodyIds.count, w->pendingWake.data, w->pendingWake.count / 10 );
		w->pendingWake.count = 0;
	}
	if ( rc == 0 && w->pendingContacts.count > 0 )
	{
		/* the flag follows each contact's set as it is now; a destroyed contact is skipped */
		int n = w->pendingContacts.count;
		int* asleep = malloc( (size_t)n * sizeof( int ) );
		int* awake = malloc( (size_t)n * sizeof( int ) );
		int sleepCount = 0, awakeCount = 0;
		for ( int i = 0; i < n; ++i )
		{
			int contactId = w->pendingContacts.data[i];
			const h_contact* c = w->contacts.data + contactId;
			if ( c->contactId != contactId ) continue;
			if ( c->setIndex == H_AWAKE_SET ) awake[awakeCount++] = contactId;
			else asleep[sleepCount++] = contactId;
		}
		rc = b2gDev_SetContactsAsleep( w->dev, asleep, sleepCount, 1 );
		if ( rc == 0 ) rc = b2gDev_SetContactsAsleep( w->dev, awake, awakeCount, 0 );
		free( asleep );
		free( awake );
		w->pendingContacts.count = 0;
	}
	if ( rc != 0 ) h_fail( w, "island update", rc );
}

/* before the solve: split the island chosen by the last sleep pass (solver.c:1476-1494,
   done there beside the constraint solve, here before it), then send the finalize its
   island table when the islands changed */
void h_stepIslands( h_world* w )
{
	if ( w->splitIslandId != B2_NULL_INDEX ) h_splitIsland( w, w->splitIslandId );
	w->splitIslandId = B2_NULL_INDEX;
	if ( w->enableSleep == 0 )
	{
		int rc = b2gDev_UploadIslands( w->dev, NULL, 0, NULL, -1 );
		if ( rc != 0 ) h_fail( w, "island upload", rc );
		w->islandsDirty = 1;
		return;
	}
	if ( w->islandsDirty == 0 ) return;
	int n = w->awakeBodyIds.count, m = w->awakeIslandIds.count;
	int* local = malloc( (size_t)( n > 0 ? n : 1 ) * sizeof( int ) );
	int* info = malloc( (size_t)( m > 0 ? 2 * m : 1 ) * sizeof( int ) );
	for ( int i = 0; i < n; ++i )
	{
		const h_body* body = w->bodies.data + w->awakeBodyIds.data[i];
		local[i] = w->islands.data[body->islandId].localIndex;
	}
	for ( int k = 0; k < m; ++k )
	{
		const h_island* island = w->islands.data + w->awakeIslandIds.data[k];
		info[2 * k] = island->islandId;
		info[2 * k + 1] = island->constraintRemoveCount > 0 ? 1 : 0;
	}
	int rc = b2gDev_UploadIslands( w->dev, local, n, info, m );
	free( local );
	free( info );
	if ( rc != 0 ) h_fail( w, "island upload", rc );
	w->islandsDirty = 0;
}

/* solver.c:2024-2080, after the proxies are enlarged: keep the split candidate for the next
   step, then visit the awake islands in reverse and put to sleep each one whose bit the
   finalize left clear. The move events of the step are materialized first, so the bodies
   that fall asleep are reported as such. */
void h_sleepPass( h_world* w, const uint32_t* awakeIslandBits, uint64_t splitKey )
{
	if ( w->enableSleep == 0 || awakeIslandBits == NULL ) return;
	w->splitIslandId = splitKey != 0 ? (int)(uint32_t)( splitKey & 0xffffffffu ) : B2_NULL_INDEX;
	int count = w->awakeIslandIds.count;
	int any = 0;
	for ( int i = 0; i < count && any == 0; ++i )
	{
		if ( awakeIslandBits[i >> 5] & ( 1u << ( i & 31 ) ) ) continue;
		const h_island* island = w->islands.data + w->awakeIslandIds.data[i];
		any = !( island->constraintRemoveCount > 0 && island->bodies.count > 1 );
	}
	if ( any == 0 ) return;
	h_buildMoveEvents( w );
	int n = w->awakeBodyIds.count;
	w->sleepPerm = malloc( (size_t)( n > 0 ? n : 1 ) * sizeof( int ) );
	for ( int i = 0; i < n; ++i ) w->sleepPerm[i] = i;
	w->sleptBodies.count = 0;
	for ( int i = count - 1; i >= 0; --i )
	{
		if ( awakeIslandBits[i >> 5] & ( 1u << ( i & 31 ) ) ) continue;
		h_trySleepIsland( w, w->awakeIslandIds.data[i] );
	}
	/* the device follows: slept bodies leave, moved slots are gathered */
	int newCount = w->awakeBodyIds.count;
	int* pairs = malloc( (size_t)( newCount > 0 ? 2 * newCount : 1 ) * sizeof( int ) );
	int pairCount = 0;
	for ( int k = 0; k < newCount; ++k )
	{
		if ( w->sleepPerm[k] == k ) continue;
		pairs[2 * pairCount] = k;
		pairs[2 * pairCount + 1] = w->sleepPerm[k];
		pairCount += 1;
	}
	int rc = b2gDev_SleepBodies( w->dev, newCount, w->sleptBodies.data, w->sleptBodies.count, pairs, pairCount );
	free( pairs );
	free( w->sleepPerm );
	w->sleepPerm = NULL;
	w->sleptBodies.count = 0;
	if ( rc != 0 ) h_fail( w, "sleep", rc );
	h_flushSleepOps( w );
}
