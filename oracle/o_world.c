/*
 * Oracle (test checker only): world, bodies, shapes, broadphase pair update, contact
 * lifecycle, narrowphase and the serial contact-state pass. Restates physics_world.c,
 * body.c, shape.c, broad_phase.c, contact.c and constraint_graph.c (Box2D v3.2). Every
 * ordering rule that decides contact ids and graph colors is kept: move-array order,
 * per-proxy pair lists built by prepending (broad_phase.c:319-320), LIFO id pools and
 * swap-remove arrays.
 */
#include "o_core.h"

#include <stdio.h>

static o_world o_worlds[O_MAX_WORLDS];

o_world* o_getWorld( int index ) { return o_worlds + index; }

o_world* o_worldFromId( b2WorldId id )
{
	if ( id.index1 < 1 || id.index1 > O_MAX_WORLDS ) return NULL;
	o_world* w = o_worlds + ( id.index1 - 1 );
	if ( w->inUse == 0 || w->generation != id.generation ) return NULL;
	return w;
}

static o_world* o_worldByIndex( int world0 ) { return o_worlds + world0; }

/* ---------------- pair set ---------------- */
static uint64_t o_hashKey( uint64_t k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdull;
	k ^= k >> 33;
	return k;
}

static void o_pairSetGrow( o_pairSet* s )
{
	int oldCap = s->capacity;
	uint64_t* old = s->keys;
	s->capacity = oldCap == 0 ? 1024 : oldCap * 2;
	s->keys = malloc( (size_t)s->capacity * 8 );
	memset( s->keys, 0xff, (size_t)s->capacity * 8 );
	s->count = 0;
	for ( int i = 0; i < oldCap; ++i )
		if ( old[i] != UINT64_MAX ) o_pairSetAdd( s, old[i] );
	free( old );
}

void o_pairSetAdd( o_pairSet* s, uint64_t key )
{
	if ( 2 * ( s->count + 1 ) > s->capacity ) o_pairSetGrow( s );
	uint64_t mask = (uint64_t)s->capacity - 1;
	uint64_t i = o_hashKey( key ) & mask;
	while ( s->keys[i] != UINT64_MAX )
	{
		if ( s->keys[i] == key ) return;
		i = ( i + 1 ) & mask;
	}
	s->keys[i] = key;
	s->count += 1;
}

int o_pairSetContains( const o_pairSet* s, uint64_t key )
{
	if ( s->capacity == 0 ) return 0;
	uint64_t mask = (uint64_t)s->capacity - 1;
	uint64_t i = o_hashKey( key ) & mask;
	while ( s->keys[i] != UINT64_MAX )
	{
		if ( s->keys[i] == key ) return 1;
		i = ( i + 1 ) & mask;
	}
	return 0;
}

void o_pairSetRemove( o_pairSet* s, uint64_t key )
{
	if ( s->capacity == 0 ) return;
	uint64_t mask = (uint64_t)s->capacity - 1;
	uint64_t i = o_hashKey( key ) & mask;
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
		uint64_t h = o_hashKey( s->keys[j] ) & mask;
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

void o_pairSetFree( o_pairSet* s )
{
	free( s->keys );
	memset( s, 0, sizeof( *s ) );
}

/* ---------------- defaults (types.c:8-89, joint.c:16-112) ---------------- */
b2WorldDef b2DefaultWorldDef( void )
{
	b2WorldDef def;
	memset( &def, 0, sizeof( def ) );
	def.gravity = o_v( 0.0f, -10.0f );
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

/* ---------------- world ---------------- */
b2WorldId b2CreateWorld( const b2WorldDef* def )
{
	int index = -1;
	for ( int i = 0; i < O_MAX_WORLDS; ++i )
	{
		if ( o_worlds[i].inUse == 0 )
		{
			index = i;
			break;
		}
	}
	b2WorldId nullId = { 0, 0 };
	if ( index < 0 ) return nullId;
	o_world* w = o_worlds + index;
	uint16_t generation = w->generation;
	memset( w, 0, sizeof( *w ) );
	w->worldId = (uint16_t)index;
	w->generation = generation;
	w->inUse = 1;
	for ( int i = 0; i < 3; ++i ) w->trees[i] = o_treeCreate( 16 );
	w->gravity = def->gravity;
	w->hitEventThreshold = def->hitEventThreshold;
	w->restitutionThreshold = def->restitutionThreshold;
	w->maxLinearSpeed = def->maximumLinearSpeed;
	w->contactSpeed = def->contactSpeed;
	w->contactHertz = def->contactHertz;
	w->contactDampingRatio = def->contactDampingRatio;
	w->contactRecycleDistance = O_CONTACT_RECYCLE_DISTANCE;
	w->enableSleep = def->enableSleep;
	w->enableWarmStarting = 1;
	w->enableContactSoftening = def->enableContactSoftening;
	w->enableContinuous = def->enableContinuous;
	w->enableSpeculative = 1;
	b2WorldId id = { (uint16_t)( index + 1 ), w->generation };
	return id;
}

void b2DestroyWorld( b2WorldId worldId )
{
	o_world* w = o_worldFromId( worldId );
	if ( w == NULL ) return;
	for ( int i = 0; i < 3; ++i )
	{
		o_treeDestroy( w->trees + i );
		free( w->movedProxies[i].bits );
	}
	o_free( w->bodyIdPool.freeArray );
	o_free( w->shapeIdPool.freeArray );
	o_free( w->contactIdPool.freeArray );
	o_free( w->jointIdPool.freeArray );
	o_free( w->bodies );
	o_free( w->shapes );
	o_free( w->contacts );
	o_free( w->joints );
	o_free( w->awakeSims );
	o_free( w->awakeStates );
	o_free( w->awakeContactSims );
	o_free( w->staticSims );
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
	{
		free( w->colors[i].bodySet.bits );
		o_free( w->colors[i].contactSims );
		o_free( w->colors[i].jointSims );
	}
	o_free( w->moveArray );
	o_pairSetFree( &w->pairSet );
	o_free( w->moveEvents );
	o_free( w->beginEvents );
	o_free( w->endEvents[0] );
	o_free( w->endEvents[1] );
	free( w->contactStateBits.bits );
	free( w->enlargedSimBits.bits );
	uint16_t generation = w->generation;
	memset( w, 0, sizeof( *w ) );
	w->generation = generation + 1;
}

bool b2World_IsValid( b2WorldId id ) { return o_worldFromId( id ) != NULL; }

void b2World_EnableSleeping( b2WorldId worldId, bool flag )
{
	o_world* w = o_worldFromId( worldId );
	if ( w ) w->enableSleep = flag;
}

bool b2World_IsSleepingEnabled( b2WorldId worldId ) { return o_worldFromId( worldId )->enableSleep; }

void b2World_EnableContinuous( b2WorldId worldId, bool flag )
{
	o_world* w = o_worldFromId( worldId );
	if ( w ) w->enableContinuous = flag;
}

bool b2World_IsContinuousEnabled( b2WorldId worldId ) { return o_worldFromId( worldId )->enableContinuous; }

void b2World_EnableWarmStarting( b2WorldId worldId, bool flag )
{
	o_world* w = o_worldFromId( worldId );
	if ( w ) w->enableWarmStarting = flag;
}

void b2World_SetGravity( b2WorldId worldId, b2Vec2 gravity )
{
	o_world* w = o_worldFromId( worldId );
	if ( w ) w->gravity = gravity;
}

b2Vec2 b2World_GetGravity( b2WorldId worldId ) { return o_worldFromId( worldId )->gravity; }

int b2World_GetAwakeBodyCount( b2WorldId worldId ) { return o_worldFromId( worldId )->awakeSims.count; }

b2Profile b2World_GetProfile( b2WorldId worldId ) { return o_worldFromId( worldId )->profile; }

b2Counters b2World_GetCounters( b2WorldId worldId )
{
	o_world* w = o_worldFromId( worldId );
	b2Counters c;
	memset( &c, 0, sizeof( c ) );
	c.bodyCount = w->bodyIdPool.nextIndex - w->bodyIdPool.freeArray.count;
	c.shapeCount = w->shapeIdPool.nextIndex - w->shapeIdPool.freeArray.count;
	c.contactCount = w->contactIdPool.nextIndex - w->contactIdPool.freeArray.count;
	c.jointCount = w->jointIdPool.nextIndex - w->jointIdPool.freeArray.count;
	c.staticTreeHeight = o_treeHeight( w->trees + b2_staticBody );
	c.treeHeight = o_treeHeight( w->trees + b2_dynamicBody );
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i )
		c.colorCounts[i] = w->colors[i].contactSims.count + w->colors[i].jointSims.count;
	/* physics_world.c:1920-1927: colored contacts plus the awake set's non-touching ones */
	c.awakeContactCount = w->awakeContactSims.count;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i ) c.awakeContactCount += w->colors[i].contactSims.count;
	c.recycledContactCount = w->recycledContactCount;
	return c;
}

b2BodyEvents b2World_GetBodyEvents( b2WorldId worldId )
{
	o_world* w = o_worldFromId( worldId );
	b2BodyEvents e = { w->moveEvents.data, w->moveEvents.count };
	return e;
}

b2ContactEvents b2World_GetContactEvents( b2WorldId worldId )
{
	o_world* w = o_worldFromId( worldId );
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

/* ---------------- bodies ---------------- */
static o_body* o_getBody( b2BodyId id )
{
	o_world* w = o_worldByIndex( id.world0 );
	return w->bodies.data + ( id.index1 - 1 );
}

static o_bodySim* o_getBodySim( o_world* w, o_body* b )
{
	if ( b->setIndex == O_AWAKE_SET ) return w->awakeSims.data + b->localIndex;
	return w->staticSims.data + b->localIndex;
}

static o_bodyState* o_getBodyState( o_world* w, o_body* b )
{
	if ( b->setIndex == O_AWAKE_SET ) return w->awakeStates.data + b->localIndex;
	return NULL;
}

/* body.c:174-330 (islands are not kept: they only feed sleeping) */
b2BodyId b2CreateBody( b2WorldId worldId, const b2BodyDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2BodyId nullId = { 0, 0, 0 };
	if ( w == NULL || w->locked ) return nullId;
	int setId = def->type == b2_staticBody ? O_STATIC_SET : O_AWAKE_SET;
	int bodyId = o_allocId( &w->bodyIdPool );
	uint32_t lockFlags = 0;
	lockFlags |= def->motionLocks.linearX ? O_LOCK_X : 0;
	lockFlags |= def->motionLocks.linearY ? O_LOCK_Y : 0;
	lockFlags |= def->motionLocks.angularZ ? O_LOCK_Z : 0;
	o_bodySim sim;
	memset( &sim, 0, sizeof( sim ) );
	sim.transform.p = def->position;
	sim.transform.q = def->rotation;
	sim.center = def->position;
	sim.rotation0 = sim.transform.q;
	sim.center0 = sim.center;
	sim.minExtent = O_HUGE;
	sim.maxExtent = 0.0f;
	sim.linearDamping = def->linearDamping;
	sim.angularDamping = def->angularDamping;
	sim.gravityScale = def->gravityScale;
	sim.bodyId = bodyId;
	sim.flags = lockFlags;
	sim.flags |= def->isBullet ? O_IS_BULLET : 0;
	sim.flags |= def->allowFastRotation ? O_ALLOW_FAST_ROTATION : 0;
	sim.flags |= def->type == b2_dynamicBody ? O_DYNAMIC_FLAG : 0;
	sim.flags |= def->enableSleep ? O_ENABLE_SLEEP : 0;
	sim.flags |= def->enableContactRecycling ? O_ENABLE_RECYCLING : 0;
	int localIndex;
	if ( setId == O_AWAKE_SET )
	{
		o_push( w->awakeSims, sim );
		o_bodyState st;
		memset( &st, 0, sizeof( st ) );
		st.linearVelocity = def->linearVelocity;
		st.angularVelocity = def->angularVelocity;
		st.deltaRotation.c = 1.0f;
		st.flags = sim.flags;
		o_push( w->awakeStates, st );
		localIndex = w->awakeSims.count - 1;
	}
	else
	{
		o_push( w->staticSims, sim );
		localIndex = w->staticSims.count - 1;
	}
	if ( bodyId == w->bodies.count )
	{
		o_body z;
		memset( &z, 0, sizeof( z ) );
		o_push( w->bodies, z );
	}
	o_body* b = w->bodies.data + bodyId;
	b->userData = def->userData;
	b->setIndex = setId;
	b->localIndex = localIndex;
	b->generation += 1;
	b->headShapeId = B2_NULL_INDEX;
	b->shapeCount = 0;
	b->headContactKey = B2_NULL_INDEX;
	b->contactCount = 0;
	b->headJointKey = B2_NULL_INDEX;
	b->jointCount = 0;
	b->id = bodyId;
	b->mass = 0.0f;
	b->inertia = 0.0f;
	b->sleepThreshold = def->sleepThreshold;
	b->sleepTime = 0.0f;
	b->safetyFactor = def->safetyFactor;
	b->type = def->type;
	b->flags = sim.flags;
	b2BodyId id = { bodyId + 1, w->worldId, b->generation };
	return id;
}

bool b2Body_IsValid( b2BodyId id )
{
	if ( id.world0 >= O_MAX_WORLDS ) return false;
	o_world* w = o_worldByIndex( id.world0 );
	if ( w->inUse == 0 || id.index1 < 1 || id.index1 > w->bodies.count ) return false;
	o_body* b = w->bodies.data + id.index1 - 1;
	return b->id == id.index1 - 1 && b->generation == id.generation;
}

b2BodyType b2Body_GetType( b2BodyId bodyId ) { return o_getBody( bodyId )->type; }

b2WorldTransform b2Body_GetTransform( b2BodyId bodyId )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	return o_getBodySim( w, o_getBody( bodyId ) )->transform;
}

b2Pos b2Body_GetPosition( b2BodyId bodyId ) { return b2Body_GetTransform( bodyId ).p; }

b2Rot b2Body_GetRotation( b2BodyId bodyId ) { return b2Body_GetTransform( bodyId ).q; }

b2Vec2 b2Body_GetLocalPoint( b2BodyId bodyId, b2Pos worldPoint )
{
	return o_invTransformPoint( b2Body_GetTransform( bodyId ), worldPoint );
}

b2Pos b2Body_GetWorldPoint( b2BodyId bodyId, b2Vec2 localPoint )
{
	return o_transformWorldPoint( b2Body_GetTransform( bodyId ), localPoint );
}

b2Vec2 b2Body_GetLinearVelocity( b2BodyId bodyId )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_bodyState* s = o_getBodyState( w, o_getBody( bodyId ) );
	return s ? s->linearVelocity : o_v( 0.0f, 0.0f );
}

float b2Body_GetAngularVelocity( b2BodyId bodyId )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_bodyState* s = o_getBodyState( w, o_getBody( bodyId ) );
	return s ? s->angularVelocity : 0.0f;
}

void b2Body_SetLinearVelocity( b2BodyId bodyId, b2Vec2 v )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	if ( b->type == b2_staticBody ) return;
	o_bodyState* s = o_getBodyState( w, b );
	if ( s ) s->linearVelocity = v;
}

void b2Body_SetAngularVelocity( b2BodyId bodyId, float av )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	if ( b->type == b2_staticBody ) return;
	o_bodyState* s = o_getBodyState( w, b );
	if ( s ) s->angularVelocity = av;
}

/* body.c:713-768 */
void b2Body_SetTransform( b2BodyId bodyId, b2Pos position, b2Rot rotation )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	o_bodySim* sim = o_getBodySim( w, b );
	sim->transform.p = position;
	sim->transform.q = rotation;
	sim->center = o_transformWorldPoint( sim->transform, sim->localCenter );
	sim->rotation0 = sim->transform.q;
	sim->center0 = sim->center;
	for ( int sid = b->headShapeId; sid != B2_NULL_INDEX; sid = w->shapes.data[sid].nextShapeId )
	{
		o_shape* s = w->shapes.data + sid;
		b2AABB aabb = o_computeFatShapeAABB( s, sim->transform, O_SPECULATIVE_DISTANCE );
		s->aabb = aabb;
		if ( o_aabbContains( s->fatAABB, aabb ) ) continue;
		float margin = s->aabbMargin;
		b2AABB fat = { { aabb.lowerBound.x - margin, aabb.lowerBound.y - margin },
					   { aabb.upperBound.x + margin, aabb.upperBound.y + margin } };
		s->fatAABB = fat;
		if ( s->proxyKey != B2_NULL_INDEX )
		{
			o_treeMoveProxy( w->trees + O_PROXY_TYPE( s->proxyKey ), O_PROXY_ID( s->proxyKey ), fat );
			o_bufferMove( w, s->proxyKey );
		}
	}
}

/* body.c:935-1090; the oracle has no sleeping sets, so every dynamic body is awake */
static o_bodySim* o_forceTarget( o_world* w, o_body* b )
{
	if ( b->type != b2_dynamicBody ) return NULL;
	return o_getBodySim( w, b );
}

void b2Body_ApplyForce( b2BodyId bodyId, b2Vec2 force, b2Pos point, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_bodySim* sim = o_forceTarget( w, o_getBody( bodyId ) );
	if ( sim == NULL ) return;
	sim->force = o_add( sim->force, force );
	sim->torque += o_cross( o_sub( point, sim->center ), force );
}

void b2Body_ApplyForceToCenter( b2BodyId bodyId, b2Vec2 force, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_bodySim* sim = o_forceTarget( w, o_getBody( bodyId ) );
	if ( sim != NULL ) sim->force = o_add( sim->force, force );
}

void b2Body_ApplyTorque( b2BodyId bodyId, float torque, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_bodySim* sim = o_forceTarget( w, o_getBody( bodyId ) );
	if ( sim != NULL ) sim->torque += torque;
}

void b2Body_ClearForces( b2BodyId bodyId )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_bodySim* sim = o_getBodySim( w, o_getBody( bodyId ) );
	sim->force = o_v( 0.0f, 0.0f );
	sim->torque = 0.0f;
}

static b2Vec2 o_limitVelocity( b2Vec2 v, float maxLinearSpeed )
{
	float v2 = o_lengthSq( v );
	if ( v2 > maxLinearSpeed * maxLinearSpeed ) v = o_mulSV( maxLinearSpeed / sqrtf( v2 ), v );
	return v;
}

void b2Body_ApplyLinearImpulse( b2BodyId bodyId, b2Vec2 impulse, b2Pos point, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	o_bodySim* sim = o_forceTarget( w, b );
	if ( sim == NULL ) return;
	o_bodyState* st = o_getBodyState( w, b );
	st->linearVelocity = o_mulAdd( st->linearVelocity, sim->invMass, impulse );
	st->angularVelocity += sim->invInertia * o_cross( o_sub( point, sim->center ), impulse );
	st->linearVelocity = o_limitVelocity( st->linearVelocity, w->maxLinearSpeed );
}

void b2Body_ApplyLinearImpulseToCenter( b2BodyId bodyId, b2Vec2 impulse, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	o_bodySim* sim = o_forceTarget( w, b );
	if ( sim == NULL ) return;
	o_bodyState* st = o_getBodyState( w, b );
	st->linearVelocity = o_limitVelocity( o_mulAdd( st->linearVelocity, sim->invMass, impulse ), w->maxLinearSpeed );
}

void b2Body_ApplyAngularImpulse( b2BodyId bodyId, float impulse, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	o_bodySim* sim = o_forceTarget( w, b );
	if ( sim == NULL ) return;
	o_getBodyState( w, b )->angularVelocity += sim->invInertia * impulse;
}

/* body.c:842-920 */
void b2Body_SetTargetTransform( b2BodyId bodyId, b2WorldTransform target, float timeStep, bool wake )
{
	(void)wake;
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* b = o_getBody( bodyId );
	if ( b->type == b2_staticBody || timeStep <= 0.0f ) return;
	o_bodySim* sim = o_getBodySim( w, b );
	b2Vec2 delta = o_sub( o_transformWorldPoint( target, sim->localCenter ), sim->center );
	float invTimeStep = 1.0f / timeStep;
	b2Rot q1 = sim->transform.q, q2 = target.q;
	float s = q1.c * q2.s - q1.s * q2.c;
	float c = q1.c * q2.c + q1.s * q2.s;
	o_bodyState* st = o_getBodyState( w, b );
	st->linearVelocity = o_mulSV( invTimeStep, delta );
	st->angularVelocity = invTimeStep * b2Atan2( s, c );
}

float b2Body_GetMass( b2BodyId bodyId ) { return o_getBody( bodyId )->mass; }

float b2Body_GetRotationalInertia( b2BodyId bodyId ) { return o_getBody( bodyId )->inertia; }

b2Vec2 b2Body_GetLocalCenter( b2BodyId bodyId )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	return o_getBodySim( w, o_getBody( bodyId ) )->localCenter;
}

b2Pos b2Body_GetWorldCenter( b2BodyId bodyId )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	return o_getBodySim( w, o_getBody( bodyId ) )->center;
}

bool b2Body_IsAwake( b2BodyId bodyId ) { return o_getBody( bodyId )->setIndex == O_AWAKE_SET; }

/* body.c:524-650 */
static void o_updateBodyMassData( o_world* w, o_body* body )
{
	o_bodySim* sim = o_getBodySim( w, body );
	body->flags &= ~O_DIRTY_MASS;
	body->mass = 0.0f;
	body->inertia = 0.0f;
	sim->invMass = 0.0f;
	sim->invInertia = 0.0f;
	sim->localCenter = o_v( 0.0f, 0.0f );
	sim->minExtent = O_HUGE;
	sim->maxExtent = 0.0f;
	if ( body->type != b2_dynamicBody )
	{
		sim->center = sim->transform.p;
		sim->center0 = sim->center;
		if ( body->type == b2_kinematicBody )
		{
			int sid = body->headShapeId;
			while ( sid != B2_NULL_INDEX )
			{
				const o_shape* s = w->shapes.data + sid;
				float mn, mx;
				o_computeShapeExtent( s, o_v( 0.0f, 0.0f ), &mn, &mx );
				sim->minExtent = o_min( sim->minExtent, mn );
				sim->maxExtent = o_max( sim->maxExtent, mx );
				sid = s->nextShapeId;
			}
		}
		return;
	}
	int shapeCount = body->shapeCount;
	b2MassData* masses = calloc( (size_t)( shapeCount > 0 ? shapeCount : 1 ), sizeof( b2MassData ) );
	b2Vec2 localCenter = o_v( 0.0f, 0.0f );
	int sid = body->headShapeId;
	int si = 0;
	while ( sid != B2_NULL_INDEX )
	{
		const o_shape* s = w->shapes.data + sid;
		sid = s->nextShapeId;
		if ( s->density == 0.0f )
		{
			si += 1;
			continue;
		}
		b2MassData md = o_computeShapeMass( s );
		body->mass += md.mass;
		localCenter = o_mulAdd( localCenter, md.mass, md.center );
		masses[si++] = md;
	}
	if ( body->mass > 0.0f )
	{
		sim->invMass = 1.0f / body->mass;
		localCenter = o_mulSV( sim->invMass, localCenter );
	}
	for ( si = 0; si < shapeCount; ++si )
	{
		b2MassData md = masses[si];
		if ( md.mass == 0.0f ) continue;
		b2Vec2 offset = o_sub( localCenter, md.center );
		float inertia = md.rotationalInertia + md.mass * o_dot( offset, offset );
		body->inertia += inertia;
	}
	free( masses );
	if ( body->inertia > 0.0f && ( body->flags & O_LOCK_Z ) == 0 )
	{
		sim->invInertia = 1.0f / body->inertia;
	}
	else
	{
		body->inertia = 0.0f;
		sim->invInertia = 0.0f;
	}
	b2Vec2 oldCenter = sim->center;
	sim->localCenter = localCenter;
	sim->center = o_transformWorldPoint( sim->transform, sim->localCenter );
	sim->center0 = sim->center;
	o_bodyState* st = o_getBodyState( w, body );
	if ( st != NULL )
	{
		b2Vec2 dl = o_crossSV( st->angularVelocity, o_sub( sim->center, oldCenter ) );
		st->linearVelocity = o_add( st->linearVelocity, dl );
	}
	sid = body->headShapeId;
	while ( sid != B2_NULL_INDEX )
	{
		const o_shape* s = w->shapes.data + sid;
		float mn, mx;
		o_computeShapeExtent( s, localCenter, &mn, &mx );
		sim->minExtent = o_min( sim->minExtent, mn );
		sim->maxExtent = o_max( sim->maxExtent, mx );
		sid = s->nextShapeId;
	}
}

/* ---------------- broadphase move buffer (broad_phase.h:70-80) ---------------- */
void o_bufferMove( o_world* w, int proxyKey )
{
	int type = O_PROXY_TYPE( proxyKey );
	int id = O_PROXY_ID( proxyKey );
	if ( o_bitGet( w->movedProxies + type, id ) == 0 )
	{
		o_bitSet1( w->movedProxies + type, id );
		o_push( w->moveArray, proxyKey );
	}
}

/* ---------------- shapes (shape.c:85-270) ---------------- */
static b2ShapeId o_createShape( b2BodyId bodyId, const b2ShapeDef* def, const void* geometry, b2ShapeType type )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	o_body* body = o_getBody( bodyId );
	b2Transform transform = o_getBodySim( w, body )->transform;
	int shapeId = o_allocId( &w->shapeIdPool );
	if ( shapeId == w->shapes.count )
	{
		o_shape z;
		memset( &z, 0, sizeof( z ) );
		o_push( w->shapes, z );
	}
	o_shape* s = w->shapes.data + shapeId;
	switch ( type )
	{
		case b2_capsuleShape: s->capsule = *(const b2Capsule*)geometry; break;
		case b2_circleShape: s->circle = *(const b2Circle*)geometry; break;
		case b2_polygonShape: s->polygon = *(const b2Polygon*)geometry; break;
		case b2_segmentShape: s->segment = *(const b2Segment*)geometry; break;
		default: break;
	}
	s->id = shapeId;
	s->bodyId = body->id;
	s->type = type;
	s->density = def->density;
	s->material = def->material;
	s->filter = def->filter;
	s->userData = def->userData;
	s->enlargedAABB = 0;
	s->enableContactEvents = def->enableContactEvents;
	s->enableHitEvents = def->enableHitEvents;
	s->isSensor = def->isSensor;
	s->proxyKey = B2_NULL_INDEX;
	s->localCentroid = o_getShapeCentroid( s );
	s->aabbMargin = o_computeShapeMargin( s );
	s->generation += 1;
	/* b2CreateShapeProxy + b2UpdateShapeAABBs (shape.c:87-106, :1034-1044) */
	{
		b2BodyType proxyType = body->type;
		b2AABB aabb = o_computeFatShapeAABB( s, transform, O_SPECULATIVE_DISTANCE );
		s->aabb = aabb;
		float margin = proxyType == b2_staticBody ? O_SPECULATIVE_DISTANCE : s->aabbMargin;
		b2AABB fat = { { aabb.lowerBound.x - margin, aabb.lowerBound.y - margin },
					   { aabb.upperBound.x + margin, aabb.upperBound.y + margin } };
		s->fatAABB = fat;
		int proxyId = o_treeCreateProxy( w->trees + proxyType, s->fatAABB, s->filter.categoryBits, (uint64_t)shapeId );
		s->proxyKey = O_PROXY_KEY( proxyId, proxyType );
		if ( proxyType != b2_staticBody || def->invokeContactCreation || def->isSensor ) o_bufferMove( w, s->proxyKey );
	}
	if ( body->headShapeId != B2_NULL_INDEX ) w->shapes.data[body->headShapeId].prevShapeId = shapeId;
	s->prevShapeId = B2_NULL_INDEX;
	s->nextShapeId = body->headShapeId;
	body->headShapeId = shapeId;
	body->shapeCount += 1;
	if ( def->updateBodyMass ) o_updateBodyMassData( w, body );
	else body->flags |= O_DIRTY_MASS;
	b2ShapeId id = { s->id + 1, bodyId.world0, s->generation };
	return id;
}

b2ShapeId b2CreateCircleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Circle* circle )
{
	return o_createShape( bodyId, def, circle, b2_circleShape );
}

b2ShapeId b2CreateCapsuleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Capsule* capsule )
{
	float lengthSqr = o_distanceSq( capsule->center1, capsule->center2 );
	if ( lengthSqr <= O_LINEAR_SLOP * O_LINEAR_SLOP )
	{
		b2ShapeId nullId = { 0, 0, 0 };
		return nullId;
	}
	return o_createShape( bodyId, def, capsule, b2_capsuleShape );
}

b2ShapeId b2CreatePolygonShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Polygon* polygon )
{
	return o_createShape( bodyId, def, polygon, b2_polygonShape );
}

b2ShapeId b2CreateSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Segment* segment )
{
	float lengthSqr = o_distanceSq( segment->point1, segment->point2 );
	if ( lengthSqr <= O_LINEAR_SLOP * O_LINEAR_SLOP )
	{
		b2ShapeId nullId = { 0, 0, 0 };
		return nullId;
	}
	return o_createShape( bodyId, def, segment, b2_segmentShape );
}

void b2Shape_SetFriction( b2ShapeId shapeId, float friction )
{
	o_world* w = o_worldByIndex( shapeId.world0 );
	w->shapes.data[shapeId.index1 - 1].material.friction = friction;
}

float b2Shape_GetFriction( b2ShapeId shapeId )
{
	o_world* w = o_worldByIndex( shapeId.world0 );
	return w->shapes.data[shapeId.index1 - 1].material.friction;
}

/* body.c b2Body_GetShapeCount / b2Body_GetShapes: the body's shape list, head first */
int b2Body_GetShapeCount( b2BodyId bodyId ) { return o_getBody( bodyId )->shapeCount; }

int b2Body_GetShapes( b2BodyId bodyId, b2ShapeId* shapeArray, int capacity )
{
	o_world* w = o_worldByIndex( bodyId.world0 );
	int n = 0;
	for ( int id = o_getBody( bodyId )->headShapeId; id != B2_NULL_INDEX && n < capacity; id = w->shapes.data[id].nextShapeId )
	{
		b2ShapeId sid = { id + 1, bodyId.world0, w->shapes.data[id].generation };
		shapeArray[n++] = sid;
	}
	return n;
}

/* ---------------- contacts (contact.c:214-501) ---------------- */
void o_createContact( o_world* w, o_shape* shapeA, o_shape* shapeB )
{
	if ( o_canCollide( shapeA->type, shapeB->type ) == 0 ) return;
	if ( o_isPrimary( shapeA->type, shapeB->type ) == 0 )
	{
		o_createContact( w, shapeB, shapeA );
		return;
	}
	o_body* bodyA = w->bodies.data + shapeA->bodyId;
	o_body* bodyB = w->bodies.data + shapeB->bodyId;
	int contactId = o_allocId( &w->contactIdPool );
	if ( contactId == w->contacts.count )
	{
		o_contact z;
		memset( &z, 0, sizeof( z ) );
		o_push( w->contacts, z );
	}
	o_contact* c = w->contacts.data + contactId;
	c->contactId = contactId;
	c->generation += 1;
	c->setIndex = O_AWAKE_SET;
	c->colorIndex = B2_NULL_INDEX;
	c->localIndex = w->awakeContactSims.count;
	c->shapeIdA = shapeA->id;
	c->shapeIdB = shapeB->id;
	c->flags = 0;
	if ( ( bodyA->flags & O_ENABLE_RECYCLING ) && ( bodyB->flags & O_ENABLE_RECYCLING ) ) c->flags |= O_C_RECYCLE;
	if ( shapeA->enableContactEvents || shapeB->enableContactEvents ) c->flags |= O_C_ENABLE_EVENTS;
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
	o_pairSetAdd( &w->pairSet, O_SHAPE_PAIR_KEY( shapeA->id, shapeB->id ) );
	o_contactSim sim;
	memset( &sim, 0, sizeof( sim ) );
	sim.contactId = contactId;
	sim.bodySimIndexA = B2_NULL_INDEX;
	sim.bodySimIndexB = B2_NULL_INDEX;
	sim.shapeIdA = shapeA->id;
	sim.shapeIdB = shapeB->id;
	sim.friction = sqrtf( shapeA->material.friction * shapeB->material.friction );
	sim.restitution = o_max( shapeA->material.restitution, shapeB->material.restitution );
	sim.tangentSpeed = 0.0f;
	sim.simFlags = c->flags;
	o_push( w->awakeContactSims, sim );
}

static void o_removeNonTouchingContact( o_world* w, int localIndex )
{
	int moved = o_removeSwap( w->awakeContactSims, localIndex );
	if ( moved != B2_NULL_INDEX )
	{
		o_contactSim* ms = w->awakeContactSims.data + localIndex;
		w->contacts.data[ms->contactId].localIndex = localIndex;
	}
}

void o_destroyContact( o_world* w, o_contact* c )
{
	o_pairSetRemove( &w->pairSet, O_SHAPE_PAIR_KEY( c->shapeIdA, c->shapeIdB ) );
	o_contactEdge* eA = c->edges + 0;
	o_contactEdge* eB = c->edges + 1;
	int bodyIdA = eA->bodyId, bodyIdB = eB->bodyId;
	o_body* bodyA = w->bodies.data + bodyIdA;
	o_body* bodyB = w->bodies.data + bodyIdB;
	uint32_t flags = c->flags;
	int touching = ( flags & O_C_TOUCHING ) != 0;
	if ( touching && ( flags & O_C_ENABLE_EVENTS ) )
	{
		const o_shape* sA = w->shapes.data + c->shapeIdA;
		const o_shape* sB = w->shapes.data + c->shapeIdB;
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
		o_push( w->endEvents[w->endEventArrayIndex], ev );
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
	if ( c->colorIndex != B2_NULL_INDEX )
	{
		o_removeContactFromGraph( w, bodyIdA, bodyIdB, c->colorIndex, c->localIndex );
	}
	else
	{
		o_removeNonTouchingContact( w, c->localIndex );
	}
	c->contactId = B2_NULL_INDEX;
	c->setIndex = B2_NULL_INDEX;
	c->colorIndex = B2_NULL_INDEX;
	c->localIndex = B2_NULL_INDEX;
	o_freeId( &w->contactIdPool, contactId );
}

/* ---------------- graph coloring (constraint_graph.c:66-291) ---------------- */
void o_addContactToGraph( o_world* w, o_contactSim* contactSim, o_contact* contact )
{
	int colorIndex = O_OVERFLOW_INDEX;
	int bodyIdA = contact->edges[0].bodyId, bodyIdB = contact->edges[1].bodyId;
	o_body* bodyA = w->bodies.data + bodyIdA;
	o_body* bodyB = w->bodies.data + bodyIdB;
	b2BodyType typeA = bodyA->type, typeB = bodyB->type;
	if ( typeA == b2_dynamicBody && typeB == b2_dynamicBody )
	{
		for ( int i = 0; i < O_DYNAMIC_COLOR_COUNT; ++i )
		{
			o_graphColor* color = w->colors + i;
			if ( o_bitGet( &color->bodySet, bodyIdA ) || o_bitGet( &color->bodySet, bodyIdB ) ) continue;
			o_bitSet1( &color->bodySet, bodyIdA );
			o_bitSet1( &color->bodySet, bodyIdB );
			colorIndex = i;
			break;
		}
	}
	else if ( typeA == b2_dynamicBody )
	{
		for ( int i = O_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			o_graphColor* color = w->colors + i;
			if ( o_bitGet( &color->bodySet, bodyIdA ) ) continue;
			o_bitSet1( &color->bodySet, bodyIdA );
			colorIndex = i;
			break;
		}
	}
	else if ( typeB == b2_dynamicBody )
	{
		for ( int i = O_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			o_graphColor* color = w->colors + i;
			if ( o_bitGet( &color->bodySet, bodyIdB ) ) continue;
			o_bitSet1( &color->bodySet, bodyIdB );
			colorIndex = i;
			break;
		}
	}
	o_graphColor* color = w->colors + colorIndex;
	contact->colorIndex = colorIndex;
	contact->localIndex = color->contactSims.count;
	o_push( color->contactSims, *contactSim );
	o_contactSim* nc = color->contactSims.data + color->contactSims.count - 1;
	if ( typeA == b2_staticBody )
	{
		nc->bodySimIndexA = B2_NULL_INDEX;
		nc->invMassA = 0.0f;
		nc->invIA = 0.0f;
	}
	else
	{
		nc->bodySimIndexA = bodyA->localIndex;
		o_bodySim* sA = w->awakeSims.data + bodyA->localIndex;
		nc->invMassA = sA->invMass;
		nc->invIA = sA->invInertia;
	}
	if ( typeB == b2_staticBody )
	{
		nc->bodySimIndexB = B2_NULL_INDEX;
		nc->invMassB = 0.0f;
		nc->invIB = 0.0f;
	}
	else
	{
		nc->bodySimIndexB = bodyB->localIndex;
		o_bodySim* sB = w->awakeSims.data + bodyB->localIndex;
		nc->invMassB = sB->invMass;
		nc->invIB = sB->invInertia;
	}
}

void o_removeContactFromGraph( o_world* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex )
{
	o_graphColor* color = w->colors + colorIndex;
	if ( colorIndex != O_OVERFLOW_INDEX )
	{
		o_bitClear( &color->bodySet, bodyIdA );
		o_bitClear( &color->bodySet, bodyIdB );
	}
	int moved = o_removeSwap( color->contactSims, localIndex );
	if ( moved != B2_NULL_INDEX )
	{
		o_contactSim* ms = color->contactSims.data + localIndex;
		w->contacts.data[ms->contactId].localIndex = localIndex;
	}
}

int o_assignJointColor( o_world* w, int bodyIdA, int bodyIdB, b2BodyType typeA, b2BodyType typeB )
{
	if ( typeA == b2_dynamicBody && typeB == b2_dynamicBody )
	{
		for ( int i = 0; i < O_DYNAMIC_COLOR_COUNT; ++i )
		{
			o_graphColor* color = w->colors + i;
			if ( o_bitGet( &color->bodySet, bodyIdA ) || o_bitGet( &color->bodySet, bodyIdB ) ) continue;
			o_bitSet1( &color->bodySet, bodyIdA );
			o_bitSet1( &color->bodySet, bodyIdB );
			return i;
		}
	}
	else if ( typeA == b2_dynamicBody )
	{
		for ( int i = O_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			o_graphColor* color = w->colors + i;
			if ( o_bitGet( &color->bodySet, bodyIdA ) ) continue;
			o_bitSet1( &color->bodySet, bodyIdA );
			return i;
		}
	}
	else if ( typeB == b2_dynamicBody )
	{
		for ( int i = O_OVERFLOW_INDEX - 1; i >= 1; --i )
		{
			o_graphColor* color = w->colors + i;
			if ( o_bitGet( &color->bodySet, bodyIdB ) ) continue;
			o_bitSet1( &color->bodySet, bodyIdB );
			return i;
		}
	}
	return O_OVERFLOW_INDEX;
}

/* body.c:2076-2110 */
int o_shouldBodiesCollide( o_world* w, o_body* bodyA, o_body* bodyB )
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
		o_joint* j = w->joints.data + jointId;
		if ( j->collideConnected == 0 && j->edges[edgeIndex ^ 1].bodyId == otherBodyId ) return 0;
		jointKey = j->edges[edgeIndex].nextKey;
	}
	return 1;
}

static inline int o_shouldShapesCollide( b2Filter a, b2Filter b )
{
	if ( a.groupIndex == b.groupIndex && a.groupIndex != 0 ) return a.groupIndex > 0;
	return ( a.maskBits & b.categoryBits ) != 0 && ( a.categoryBits & b.maskBits ) != 0;
}

/* ---------------- pair finding (broad_phase.c:172-529) ---------------- */
typedef struct o_pair
{
	int shapeIdA, shapeIdB;
} o_pair;

typedef struct o_queryCtx
{
	o_world* w;
	O_ARRAY( o_pair ) * list;
	int queryTreeType, queryProxyKey, queryShapeIndex;
} o_queryCtx;

static int o_pairQueryCallback( int proxyId, uint64_t userData, void* context )
{
	int shapeId = (int)userData;
	o_queryCtx* q = context;
	o_world* w = q->w;
	int proxyKey = O_PROXY_KEY( proxyId, q->queryTreeType );
	int queryProxyKey = q->queryProxyKey;
	if ( proxyKey == queryProxyKey ) return 1;
	int treeType = q->queryTreeType;
	int queryProxyType = O_PROXY_TYPE( queryProxyKey );
	if ( queryProxyType == b2_dynamicBody )
	{
		if ( treeType == b2_dynamicBody && proxyKey < queryProxyKey )
		{
			if ( o_bitGet( w->movedProxies + treeType, proxyId ) ) return 1;
		}
	}
	else
	{
		if ( o_bitGet( w->movedProxies + treeType, proxyId ) ) return 1;
	}
	uint64_t pairKey = O_SHAPE_PAIR_KEY( shapeId, q->queryShapeIndex );
	if ( o_pairSetContains( &w->pairSet, pairKey ) ) return 1;
	int shapeIdA, shapeIdB;
	if ( proxyKey < queryProxyKey )
	{
		shapeIdA = shapeId;
		shapeIdB = q->queryShapeIndex;
	}
	else
	{
		shapeIdA = q->queryShapeIndex;
		shapeIdB = shapeId;
	}
	o_shape* sA = w->shapes.data + shapeIdA;
	o_shape* sB = w->shapes.data + shapeIdB;
	if ( sA->bodyId == sB->bodyId ) return 1;
	if ( sA->isSensor || sB->isSensor ) return 1;
	if ( o_shouldShapesCollide( sA->filter, sB->filter ) == 0 ) return 1;
	if ( o_canCollide( sA->type, sB->type ) == 0 ) return 1;
	if ( o_shouldBodiesCollide( w, w->bodies.data + sA->bodyId, w->bodies.data + sB->bodyId ) == 0 ) return 1;
	o_pair p = { shapeIdA, shapeIdB };
	o_push( *q->list, p );
	return 1;
}

void o_updateBroadPhasePairs( o_world* w )
{
	int moveCount = w->moveArray.count;
	if ( moveCount == 0 ) return;
	/* all queries run against the pair set as it was before this step's contacts exist
	   (b2FindPairsTask runs in parallel before the serial creation loop) */
	O_ARRAY( o_pair ) list;
	memset( &list, 0, sizeof( list ) );
	int* starts = malloc( (size_t)( moveCount + 1 ) * sizeof( int ) );
	for ( int i = 0; i < moveCount; ++i )
	{
		starts[i] = list.count;
		int proxyKey = w->moveArray.data[i];
		if ( proxyKey == B2_NULL_INDEX ) continue;
		int proxyType = O_PROXY_TYPE( proxyKey );
		int proxyId = O_PROXY_ID( proxyKey );
		const o_tree* baseTree = w->trees + proxyType;
		b2AABB fatAABB = baseTree->nodes[proxyId].aabb;
		o_queryCtx q;
		q.w = w;
		q.list = (void*)&list;
		q.queryProxyKey = proxyKey;
		q.queryShapeIndex = (int)baseTree->nodes[proxyId].userData;
		if ( proxyType == b2_dynamicBody )
		{
			q.queryTreeType = b2_kinematicBody;
			o_treeQuery( w->trees + b2_kinematicBody, fatAABB, B2_DEFAULT_MASK_BITS, o_pairQueryCallback, &q );
			q.queryTreeType = b2_staticBody;
			o_treeQuery( w->trees + b2_staticBody, fatAABB, B2_DEFAULT_MASK_BITS, o_pairQueryCallback, &q );
		}
		q.queryTreeType = b2_dynamicBody;
		o_treeQuery( w->trees + b2_dynamicBody, fatAABB, B2_DEFAULT_MASK_BITS, o_pairQueryCallback, &q );
	}
	starts[moveCount] = list.count;
	for ( int i = 0; i < moveCount; ++i )
	{
		/* the reference prepends each pair to the proxy's list, so creation runs newest first */
		for ( int k = starts[i + 1] - 1; k >= starts[i]; --k )
		{
			o_createContact( w, w->shapes.data + list.data[k].shapeIdA, w->shapes.data + list.data[k].shapeIdB );
		}
	}
	free( starts );
	o_free( list );
	/* b2UpdateTreesTask (broad_phase.c:401-410) runs after the queries */
	o_treeRebuild( w->trees + b2_dynamicBody, 0 );
	o_treeRebuild( w->trees + b2_kinematicBody, 0 );
	for ( int i = 0; i < w->moveArray.count; ++i )
	{
		int key = w->moveArray.data[i];
		o_bitClear( w->movedProxies + O_PROXY_TYPE( key ), O_PROXY_ID( key ) );
	}
	w->moveArray.count = 0;
}
