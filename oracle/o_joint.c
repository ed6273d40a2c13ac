/*
 * Oracle (test checker only): joint creation (joint.c:16-720), the per-type dispatch
 * (joint.c:1406-1540) and the joint solvers: revolute_joint.c:217-500,
 * prismatic_joint.c:295-667, weld_joint.c:148-454 (the non-block solver the reference
 * compiles, B2_WELD_BLOCK_SOLVE 0), wheel_joint.c:197-525, distance_joint.c:250-543.
 */
#include "o_core.h"

b2JointType b2Joint_GetType( b2JointId jointId )
{
	o_world* w = o_getWorld( jointId.world0 );
	return w->joints.data[jointId.index1 - 1].type;
}

static b2JointDef o_defaultJointDef( void )
{
	b2JointDef def;
	memset( &def, 0, sizeof( def ) );
	def.localFrameA.q.c = 1.0f;
	def.localFrameB.q.c = 1.0f;
	def.forceThreshold = FLT_MAX;
	def.torqueThreshold = FLT_MAX;
	def.constraintHertz = 60.0f;
	def.constraintDampingRatio = 2.0f;
	def.drawScale = 1.0f;
	return def;
}

b2DistanceJointDef b2DefaultDistanceJointDef( void )
{
	b2DistanceJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.lowerSpringForce = -FLT_MAX;
	def.upperSpringForce = FLT_MAX;
	def.length = 1.0f;
	def.maxLength = O_HUGE;
	def.internalValue = 1152023;
	return def;
}

b2PrismaticJointDef b2DefaultPrismaticJointDef( void )
{
	b2PrismaticJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2RevoluteJointDef b2DefaultRevoluteJointDef( void )
{
	b2RevoluteJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2WeldJointDef b2DefaultWeldJointDef( void )
{
	b2WeldJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2WheelJointDef b2DefaultWheelJointDef( void )
{
	b2WheelJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.enableSpring = true;
	def.hertz = 1.0f;
	def.dampingRatio = 0.7f;
	def.internalValue = 1152023;
	return def;
}

/* joint.c:161-196 */
static void o_destroyContactsBetweenBodies( o_world* w, o_body* bodyA, o_body* bodyB )
{
	int contactKey, otherBodyId;
	if ( bodyA->contactCount < bodyB->contactCount )
	{
		contactKey = bodyA->headContactKey;
		otherBodyId = bodyB->id;
	}
	else
	{
		contactKey = bodyB->headContactKey;
		otherBodyId = bodyA->id;
	}
	while ( contactKey != B2_NULL_INDEX )
	{
		int contactId = contactKey >> 1;
		int edgeIndex = contactKey & 1;
		o_contact* c = w->contacts.data + contactId;
		contactKey = c->edges[edgeIndex].nextKey;
		if ( c->edges[edgeIndex ^ 1].bodyId == otherBodyId ) o_destroyContact( w, c );
	}
}

/* joint.c:204-398. Only awake and static placements exist here (no sleeping sets). Joints
   between two non-dynamic bodies are kept off the graph and never solved. */
static o_jointSim* o_createJoint( o_world* w, const b2JointDef* def, b2JointType type, b2JointId* outId )
{
	o_body* bodyA = w->bodies.data + def->bodyIdA.index1 - 1;
	o_body* bodyB = w->bodies.data + def->bodyIdB.index1 - 1;
	if ( def->collideConnected == false ) o_destroyContactsBetweenBodies( w, bodyA, bodyB );
	int bodyIdA = bodyA->id, bodyIdB = bodyB->id;
	int jointId = o_allocId( &w->jointIdPool );
	if ( jointId == w->joints.count )
	{
		o_joint z;
		memset( &z, 0, sizeof( z ) );
		o_push( w->joints, z );
	}
	o_joint* j = w->joints.data + jointId;
	j->jointId = jointId;
	j->userData = def->userData;
	j->generation += 1;
	j->setIndex = B2_NULL_INDEX;
	j->colorIndex = B2_NULL_INDEX;
	j->localIndex = B2_NULL_INDEX;
	j->type = type;
	j->collideConnected = def->collideConnected;
	j->edges[0].bodyId = bodyIdA;
	j->edges[0].prevKey = B2_NULL_INDEX;
	j->edges[0].nextKey = bodyA->headJointKey;
	int keyA = ( jointId << 1 ) | 0;
	if ( bodyA->headJointKey != B2_NULL_INDEX )
		w->joints.data[bodyA->headJointKey >> 1].edges[bodyA->headJointKey & 1].prevKey = keyA;
	bodyA->headJointKey = keyA;
	bodyA->jointCount += 1;
	j->edges[1].bodyId = bodyIdB;
	j->edges[1].prevKey = B2_NULL_INDEX;
	j->edges[1].nextKey = bodyB->headJointKey;
	int keyB = ( jointId << 1 ) | 1;
	if ( bodyB->headJointKey != B2_NULL_INDEX )
		w->joints.data[bodyB->headJointKey >> 1].edges[bodyB->headJointKey & 1].prevKey = keyB;
	bodyB->headJointKey = keyB;
	bodyB->jointCount += 1;

	static o_jointSim scratch;
	o_jointSim* sim;
	if ( bodyA->type != b2_dynamicBody && bodyB->type != b2_dynamicBody )
	{
		j->setIndex = O_STATIC_SET;
		memset( &scratch, 0, sizeof( scratch ) );
		sim = &scratch;
	}
	else
	{
		j->setIndex = O_AWAKE_SET;
		int colorIndex = o_assignJointColor( w, bodyIdA, bodyIdB, bodyA->type, bodyB->type );
		o_jointSim z;
		memset( &z, 0, sizeof( z ) );
		o_push( w->colors[colorIndex].jointSims, z );
		j->colorIndex = colorIndex;
		j->localIndex = w->colors[colorIndex].jointSims.count - 1;
		sim = w->colors[colorIndex].jointSims.data + j->localIndex;
	}
	sim->jointId = jointId;
	sim->bodyIdA = bodyIdA;
	sim->bodyIdB = bodyIdB;
	sim->localFrameA = def->localFrameA;
	sim->localFrameB = def->localFrameB;
	sim->type = type;
	sim->constraintHertz = def->constraintHertz;
	sim->constraintDampingRatio = def->constraintDampingRatio;
	sim->constraintSoftness.biasRate = 0.0f;
	sim->constraintSoftness.massScale = 1.0f;
	sim->constraintSoftness.impulseScale = 0.0f;
	sim->forceThreshold = def->forceThreshold;
	sim->torqueThreshold = def->torqueThreshold;
	outId->index1 = jointId + 1;
	outId->world0 = w->worldId;
	outId->generation = j->generation;
	return sim;
}

b2JointId b2CreateDistanceJoint( b2WorldId worldId, const b2DistanceJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_distanceJoint, &id );
	memset( &j->distanceJoint, 0, sizeof( j->distanceJoint ) );
	o_distanceJoint* d = &j->distanceJoint;
	d->length = o_max( def->length, O_LINEAR_SLOP );
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->minLength = o_max( def->minLength, O_LINEAR_SLOP );
	d->maxLength = o_max( def->minLength, def->maxLength );
	d->maxMotorForce = def->maxMotorForce;
	d->motorSpeed = def->motorSpeed;
	d->enableSpring = def->enableSpring;
	d->lowerSpringForce = def->lowerSpringForce;
	d->upperSpringForce = def->upperSpringForce;
	d->enableLimit = def->enableLimit;
	d->enableMotor = def->enableMotor;
	return id;
}

b2JointId b2CreatePrismaticJoint( b2WorldId worldId, const b2PrismaticJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_prismaticJoint, &id );
	memset( &j->prismaticJoint, 0, sizeof( j->prismaticJoint ) );
	o_prismaticJoint* p = &j->prismaticJoint;
	p->hertz = def->hertz;
	p->dampingRatio = def->dampingRatio;
	p->targetTranslation = def->targetTranslation;
	p->lowerTranslation = def->lowerTranslation;
	p->upperTranslation = def->upperTranslation;
	p->maxMotorForce = def->maxMotorForce;
	p->motorSpeed = def->motorSpeed;
	p->enableSpring = def->enableSpring;
	p->enableLimit = def->enableLimit;
	p->enableMotor = def->enableMotor;
	return id;
}

b2JointId b2CreateRevoluteJoint( b2WorldId worldId, const b2RevoluteJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_revoluteJoint, &id );
	memset( &j->revoluteJoint, 0, sizeof( j->revoluteJoint ) );
	o_revoluteJoint* r = &j->revoluteJoint;
	r->targetAngle = o_clamp( def->targetAngle, -B2_PI, B2_PI );
	r->hertz = def->hertz;
	r->dampingRatio = def->dampingRatio;
	float lowerAngle = o_min( def->lowerAngle, def->upperAngle );
	float upperAngle = o_max( def->lowerAngle, def->upperAngle );
	r->lowerAngle = o_clamp( lowerAngle, -0.99f * B2_PI, 0.99f * B2_PI );
	r->upperAngle = o_clamp( upperAngle, -0.99f * B2_PI, 0.99f * B2_PI );
	r->maxMotorTorque = def->maxMotorTorque;
	r->motorSpeed = def->motorSpeed;
	r->enableSpring = def->enableSpring;
	r->enableLimit = def->enableLimit;
	r->enableMotor = def->enableMotor;
	return id;
}

b2JointId b2CreateWeldJoint( b2WorldId worldId, const b2WeldJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_weldJoint, &id );
	memset( &j->weldJoint, 0, sizeof( j->weldJoint ) );
	o_weldJoint* wj = &j->weldJoint;
	wj->linearHertz = def->linearHertz;
	wj->linearDampingRatio = def->linearDampingRatio;
	wj->angularHertz = def->angularHertz;
	wj->angularDampingRatio = def->angularDampingRatio;
	return id;
}

b2JointId b2CreateWheelJoint( b2WorldId worldId, const b2WheelJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_wheelJoint, &id );
	memset( &j->wheelJoint, 0, sizeof( j->wheelJoint ) );
	o_wheelJoint* wh = &j->wheelJoint;
	wh->lowerTranslation = def->lowerTranslation;
	wh->upperTranslation = def->upperTranslation;
	wh->maxMotorTorque = def->maxMotorTorque;
	wh->motorSpeed = def->motorSpeed;
	wh->hertz = def->hertz;
	wh->dampingRatio = def->dampingRatio;
	wh->enableSpring = def->enableSpring;
	wh->enableLimit = def->enableLimit;
	wh->enableMotor = def->enableMotor;
	return id;
}

/* joint.c:50-62, :72-78 */
b2FilterJointDef b2DefaultFilterJointDef( void )
{
	b2FilterJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2MotorJointDef b2DefaultMotorJointDef( void )
{
	b2MotorJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2PogoJointDef b2DefaultPogoJointDef( void )
{
	b2PogoJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2MoverJointDef b2DefaultMoverJointDef( void )
{
	b2MoverJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = o_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

/* joint.c b2CreateMoverJoint */
b2JointId b2CreateMoverJoint( b2WorldId worldId, const b2MoverJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_moverJoint, &id );
	memset( &j->moverJoint, 0, sizeof( j->moverJoint ) );
	j->moverJoint.linearVelocity = def->linearVelocity;
	j->moverJoint.maxVelocityForce = def->maxVelocityForce;
	return id;
}

/* joint.c:436-459: a graph edge and a colored constraint that does nothing */
b2JointId b2CreateFilterJoint( b2WorldId worldId, const b2FilterJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_createJoint( w, &def->base, b2_filterJoint, &id );
	return id;
}

/* joint.c:461-491 */
b2JointId b2CreateMotorJoint( b2WorldId worldId, const b2MotorJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_motorJoint, &id );
	memset( &j->motorJoint, 0, sizeof( j->motorJoint ) );
	o_motorJoint* m = &j->motorJoint;
	m->linearVelocity = def->linearVelocity;
	m->maxVelocityForce = def->maxVelocityForce;
	m->angularVelocity = def->angularVelocity;
	m->maxVelocityTorque = def->maxVelocityTorque;
	m->linearHertz = def->linearHertz;
	m->linearDampingRatio = def->linearDampingRatio;
	m->maxSpringForce = def->maxSpringForce;
	m->angularHertz = def->angularHertz;
	m->angularDampingRatio = def->angularDampingRatio;
	m->maxSpringTorque = def->maxSpringTorque;
	return id;
}

/* joint.c:521-560 */
b2JointId b2CreatePogoJoint( b2WorldId worldId, const b2PogoJointDef* def )
{
	o_world* w = o_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	o_jointSim* j = o_createJoint( w, &def->base, b2_pogoJoint, &id );
	memset( &j->pogoJoint, 0, sizeof( j->pogoJoint ) );
	o_pogoJoint* q = &j->pogoJoint;
	q->restLength = def->restLength;
	q->hertz = def->hertz;
	q->dampingRatio = def->dampingRatio;
	q->maxTensionForce = def->maxTensionForce;
	q->maxCompressionForce = def->maxCompressionForce;
	q->normal = def->normal;
	q->impulse = def->impulse;
	q->velocity = def->velocity;
	return id;
}

/* ---------------- shared helpers ---------------- */
static o_bodySim* o_jointBodySim( o_world* w, int bodyId, int* awakeIndex )
{
	o_body* b = w->bodies.data + bodyId;
	if ( b->setIndex == O_AWAKE_SET )
	{
		*awakeIndex = b->localIndex;
		return w->awakeSims.data + b->localIndex;
	}
	*awakeIndex = B2_NULL_INDEX;
	return w->staticSims.data + b->localIndex;
}

static float o_unwind( float radians )
{
	float x = o_clamp( radians, -1.0e6f, 1.0e6f );
	double twoPi = 2.0f * B2_PI;
	double roundToNearest = 6755399441055744.0;
	double a = x;
	double k = ( a / twoPi + roundToNearest ) - roundToNearest;
	return (float)( a - k * twoPi );
}

static b2Vec2 o_solve22( float a11, float a12, float a21, float a22, b2Vec2 b )
{
	float det = a11 * a22 - a12 * a21;
	if ( det != 0.0f ) det = 1.0f / det;
	b2Vec2 x = { det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) };
	return x;
}

/* ---------------- revolute (revolute_joint.c:217-500) ---------------- */
static void o_prepareRevolute( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float mA = simA->invMass, iA = simA->invInertia, mB = simB->invMass, iB = simB->invInertia;
	base->invMassA = mA;
	base->invMassB = mB;
	base->invIA = iA;
	base->invIB = iB;
	o_revoluteJoint* j = &base->revoluteJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->frameA.q = o_mulRot( simA->transform.q, base->localFrameA.q );
	j->frameA.p = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->frameB.q = o_mulRot( simB->transform.q, base->localFrameB.q );
	j->frameB.p = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	float k = iA + iB;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	j->springSoftness = o_makeSoft( j->hertz, j->dampingRatio, ctx->h );
	if ( ctx->enableWarmStarting == 0 )
	{
		j->linearImpulse = o_v( 0.0f, 0.0f );
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

static const o_bodyState o_dummyState = { { 0.0f, 0.0f }, 0.0f, 0, { 0.0f, 0.0f }, { 1.0f, 0.0f } };

static void o_warmStartRevolute( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_revoluteJoint* j = &base->revoluteJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	float axialImpulse = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, j->linearImpulse );
		sA->angularVelocity -= iA * ( o_cross( rA, j->linearImpulse ) + axialImpulse );
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, j->linearImpulse );
		sB->angularVelocity += iB * ( o_cross( rB, j->linearImpulse ) + axialImpulse );
	}
}

static void o_solveRevolute( o_world* w, o_stepContext* ctx, o_jointSim* base, int useBias )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_revoluteJoint* j = &base->revoluteJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	b2Rot qA = o_mulRot( sA->deltaRotation, j->frameA.q );
	b2Rot qB = o_mulRot( sB->deltaRotation, j->frameB.q );
	b2Rot relQ = o_invMulRot( qA, qB );
	int fixedRotation = ( iA + iB == 0.0f );
	if ( j->enableSpring && fixedRotation == 0 )
	{
		float jointAngle = b2Atan2( relQ.s, relQ.c );
		float C = o_unwind( jointAngle - j->targetAngle );
		float bias = j->springSoftness.biasRate * C;
		float massScale = j->springSoftness.massScale;
		float impulseScale = j->springSoftness.impulseScale;
		float Cdot = wB - wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableMotor && fixedRotation == 0 )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->axialMass * Cdot;
		float oldImpulse = j->motorImpulse;
		float maxImpulse = ctx->h * j->maxMotorTorque;
		j->motorImpulse = o_clamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableLimit && fixedRotation == 0 )
	{
		float jointAngle = b2Atan2( relQ.s, relQ.c );
		{
			float C = jointAngle - j->lowerAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * ctx->inv_h;
			else if ( useBias )
			{
				bias = base->constraintSoftness.biasRate * C;
				massScale = base->constraintSoftness.massScale;
				impulseScale = base->constraintSoftness.impulseScale;
			}
			float Cdot = wB - wA;
			float oldImpulse = j->lowerImpulse;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->lowerImpulse = o_max( oldImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - oldImpulse;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		{
			float C = j->upperAngle - jointAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * ctx->inv_h;
			else if ( useBias )
			{
				bias = base->constraintSoftness.biasRate * C;
				massScale = base->constraintSoftness.massScale;
				impulseScale = base->constraintSoftness.impulseScale;
			}
			float Cdot = wA - wB;
			float oldImpulse = j->upperImpulse;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->upperImpulse = o_max( oldImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - oldImpulse;
			wA += iA * impulse;
			wB -= iB * impulse;
		}
	}
	{
		b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
		b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
		b2Vec2 Cdot = o_sub( o_add( vB, o_crossSV( wB, rB ) ), o_add( vA, o_crossSV( wA, rA ) ) );
		b2Vec2 bias = { 0.0f, 0.0f };
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			b2Vec2 dcA = sA->deltaPosition, dcB = sB->deltaPosition;
			b2Vec2 separation = o_add( o_add( o_sub( dcB, dcA ), o_sub( rB, rA ) ), j->deltaCenter );
			bias = o_mulSV( base->constraintSoftness.biasRate, separation );
			massScale = base->constraintSoftness.massScale;
			impulseScale = base->constraintSoftness.impulseScale;
		}
		float k11 = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		float k12 = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		float k22 = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		b2Vec2 b = o_solve22( k11, k12, k12, k22, o_add( Cdot, bias ) );
		b2Vec2 impulse;
		impulse.x = -massScale * b.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * j->linearImpulse.y;
		j->linearImpulse.x += impulse.x;
		j->linearImpulse.y += impulse.y;
		vA = o_mulSub( vA, mA, impulse );
		wA -= iA * o_cross( rA, impulse );
		vB = o_mulAdd( vB, mB, impulse );
		wB += iB * o_cross( rB, impulse );
	}
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- prismatic (prismatic_joint.c:295-667) ---------------- */
static void o_preparePrismatic( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	base->invMassA = simA->invMass;
	base->invMassB = simB->invMass;
	base->invIA = simA->invInertia;
	base->invIB = simB->invInertia;
	o_prismaticJoint* j = &base->prismaticJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->frameA.q = o_mulRot( simA->transform.q, base->localFrameA.q );
	j->frameA.p = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->frameB.q = o_mulRot( simB->transform.q, base->localFrameB.q );
	j->frameB.p = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	j->springSoftness = o_makeSoft( j->hertz, j->dampingRatio, ctx->h );
	if ( ctx->enableWarmStarting == 0 )
	{
		j->impulse = o_v( 0.0f, 0.0f );
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

static void o_warmStartPrismatic( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_prismaticJoint* j = &base->prismaticJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	b2Vec2 d = o_add( o_add( o_sub( sB->deltaPosition, sA->deltaPosition ), j->deltaCenter ), o_sub( rB, rA ) );
	b2Vec2 axisA = o_rotate( j->frameA.q, o_v( 1.0f, 0.0f ) );
	axisA = o_rotate( sA->deltaRotation, axisA );
	float a1 = o_cross( o_add( rA, d ), axisA );
	float a2 = o_cross( rB, axisA );
	float axialImpulse = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
	b2Vec2 perpA = o_leftPerp( axisA );
	float s1 = o_cross( o_add( rA, d ), perpA );
	float s2 = o_cross( rB, perpA );
	float perpImpulse = j->impulse.x;
	float angleImpulse = j->impulse.y;
	b2Vec2 P = o_add( o_mulSV( axialImpulse, axisA ), o_mulSV( perpImpulse, perpA ) );
	float LA = axialImpulse * a1 + perpImpulse * s1 + angleImpulse;
	float LB = axialImpulse * a2 + perpImpulse * s2 + angleImpulse;
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, P );
		sA->angularVelocity -= iA * LA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, P );
		sB->angularVelocity += iB * LB;
	}
}

/* one axial row (spring, motor or limit) applied along axisA with lever arms a1, a2 */
static void o_applyAxial( b2Vec2* vA, float* wA, b2Vec2* vB, float* wB, float mA, float iA, float mB, float iB, b2Vec2 axisA,
						  float a1, float a2, float impulse )
{
	b2Vec2 P = o_mulSV( impulse, axisA );
	float LA = impulse * a1;
	float LB = impulse * a2;
	*vA = o_mulSub( *vA, mA, P );
	*wA -= iA * LA;
	*vB = o_mulAdd( *vB, mB, P );
	*wB += iB * LB;
}

static void o_solvePrismatic( o_world* w, o_stepContext* ctx, o_jointSim* base, int useBias )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_prismaticJoint* j = &base->prismaticJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	b2Rot qA = o_mulRot( sA->deltaRotation, j->frameA.q );
	b2Rot qB = o_mulRot( sB->deltaRotation, j->frameB.q );
	b2Rot relQ = o_invMulRot( qA, qB );
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	b2Vec2 d = o_add( o_add( o_sub( sB->deltaPosition, sA->deltaPosition ), j->deltaCenter ), o_sub( rB, rA ) );
	b2Vec2 axisA = o_rotate( j->frameA.q, o_v( 1.0f, 0.0f ) );
	axisA = o_rotate( sA->deltaRotation, axisA );
	float translation = o_dot( axisA, d );
	float a1 = o_cross( o_add( rA, d ), axisA );
	float a2 = o_cross( rB, axisA );
	float k = mA + mB + iA * a1 * a1 + iB * a2 * a2;
	float axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	o_softness softness = base->constraintSoftness;
	if ( j->enableSpring )
	{
		float C = translation - j->targetTranslation;
		float bias = j->springSoftness.biasRate * C;
		float massScale = j->springSoftness.massScale;
		float impulseScale = j->springSoftness.impulseScale;
		float Cdot = o_dot( axisA, o_sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float deltaImpulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += deltaImpulse;
		o_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, deltaImpulse );
	}
	if ( j->enableMotor )
	{
		float Cdot = o_dot( axisA, o_sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = axialMass * ( j->motorSpeed - Cdot );
		float oldImpulse = j->motorImpulse;
		float maxImpulse = ctx->h * j->maxMotorForce;
		j->motorImpulse = o_clamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		o_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, impulse );
	}
	if ( j->enableLimit )
	{
		float speculativeDistance = 0.25f * ( j->upperTranslation - j->lowerTranslation );
		{
			float C = translation - j->lowerTranslation;
			if ( C < speculativeDistance )
			{
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f ) bias = o_min( C, 1.0f ) * ctx->inv_h;
				else if ( useBias )
				{
					bias = softness.biasRate * C;
					massScale = softness.massScale;
					impulseScale = softness.impulseScale;
				}
				float oldImpulse = j->lowerImpulse;
				float Cdot = o_dot( axisA, o_sub( vB, vA ) ) + a2 * wB - a1 * wA;
				float deltaImpulse = -axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
				j->lowerImpulse = o_max( oldImpulse + deltaImpulse, 0.0f );
				deltaImpulse = j->lowerImpulse - oldImpulse;
				o_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, deltaImpulse );
			}
			else
			{
				j->lowerImpulse = 0.0f;
			}
		}
		{
			float C = j->upperTranslation - translation;
			if ( C < speculativeDistance )
			{
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f ) bias = o_min( C, 1.0f ) * ctx->inv_h;
				else if ( useBias )
				{
					bias = softness.biasRate * C;
					massScale = softness.massScale;
					impulseScale = softness.impulseScale;
				}
				float oldImpulse = j->upperImpulse;
				float Cdot = o_dot( axisA, o_sub( vA, vB ) ) + a1 * wA - a2 * wB;
				float deltaImpulse = -axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
				j->upperImpulse = o_max( oldImpulse + deltaImpulse, 0.0f );
				deltaImpulse = j->upperImpulse - oldImpulse;
				b2Vec2 P = o_mulSV( deltaImpulse, axisA );
				float LA = deltaImpulse * a1;
				float LB = deltaImpulse * a2;
				vA = o_mulAdd( vA, mA, P );
				wA += iA * LA;
				vB = o_mulSub( vB, mB, P );
				wB -= iB * LB;
			}
			else
			{
				j->upperImpulse = 0.0f;
			}
		}
	}
	{
		b2Vec2 perpA = o_leftPerp( axisA );
		float s1 = o_cross( o_add( d, rA ), perpA );
		float s2 = o_cross( rB, perpA );
		b2Vec2 Cdot;
		Cdot.x = o_dot( perpA, o_sub( vB, vA ) ) + s2 * wB - s1 * wA;
		Cdot.y = wB - wA;
		b2Vec2 bias = { 0.0f, 0.0f };
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			b2Vec2 C;
			C.x = o_dot( perpA, d );
			C.y = b2Atan2( relQ.s, relQ.c );
			bias = o_mulSV( softness.biasRate, C );
			massScale = softness.massScale;
			impulseScale = softness.impulseScale;
		}
		float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
		float k12 = iA * s1 + iB * s2;
		float k22 = iA + iB;
		if ( k22 == 0.0f ) k22 = 1.0f;
		b2Vec2 b = o_solve22( k11, k12, k12, k22, o_add( Cdot, bias ) );
		b2Vec2 deltaImpulse;
		deltaImpulse.x = -massScale * b.x - impulseScale * j->impulse.x;
		deltaImpulse.y = -massScale * b.y - impulseScale * j->impulse.y;
		j->impulse.x += deltaImpulse.x;
		j->impulse.y += deltaImpulse.y;
		b2Vec2 P = o_mulSV( deltaImpulse.x, perpA );
		float LA = deltaImpulse.x * s1 + deltaImpulse.y;
		float LB = deltaImpulse.x * s2 + deltaImpulse.y;
		vA = o_mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = o_mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- weld (weld_joint.c:148-454, the non-block solver) ---------------- */
static void o_prepareWeld( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float iA = simA->invInertia, iB = simB->invInertia;
	base->invMassA = simA->invMass;
	base->invMassB = simB->invMass;
	base->invIA = iA;
	base->invIB = iB;
	o_weldJoint* j = &base->weldJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->frameA.q = o_mulRot( simA->transform.q, base->localFrameA.q );
	j->frameA.p = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->frameB.q = o_mulRot( simB->transform.q, base->localFrameB.q );
	j->frameB.p = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	float ka = iA + iB;
	j->axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
	j->linearSpring = j->linearHertz == 0.0f ? base->constraintSoftness : o_makeSoft( j->linearHertz, j->linearDampingRatio, ctx->h );
	j->angularSpring =
		j->angularHertz == 0.0f ? base->constraintSoftness : o_makeSoft( j->angularHertz, j->angularDampingRatio, ctx->h );
	if ( ctx->enableWarmStarting == 0 )
	{
		j->linearImpulse = o_v( 0.0f, 0.0f );
		j->angularImpulse = 0.0f;
	}
}

static void o_warmStartWeld( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_weldJoint* j = &base->weldJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, j->linearImpulse );
		sA->angularVelocity -= iA * ( o_cross( rA, j->linearImpulse ) + j->angularImpulse );
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, j->linearImpulse );
		sB->angularVelocity += iB * ( o_cross( rB, j->linearImpulse ) + j->angularImpulse );
	}
}

static void o_solveWeld( o_world* w, o_jointSim* base, int useBias )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_weldJoint* j = &base->weldJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	{
		b2Rot qA = o_mulRot( sA->deltaRotation, j->frameA.q );
		b2Rot qB = o_mulRot( sB->deltaRotation, j->frameB.q );
		b2Rot relQ = o_invMulRot( qA, qB );
		float jointAngle = b2Atan2( relQ.s, relQ.c );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->angularHertz > 0.0f )
		{
			float C = jointAngle;
			bias = j->angularSpring.biasRate * C;
			massScale = j->angularSpring.massScale;
			impulseScale = j->angularSpring.impulseScale;
		}
		float Cdot = wB - wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->angularImpulse;
		j->angularImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
		b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
		b2Vec2 bias = { 0.0f, 0.0f };
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->linearHertz > 0.0f )
		{
			b2Vec2 dcA = sA->deltaPosition, dcB = sB->deltaPosition;
			b2Vec2 C = o_add( o_add( o_sub( dcB, dcA ), o_sub( rB, rA ) ), j->deltaCenter );
			bias = o_mulSV( j->linearSpring.biasRate, C );
			massScale = j->linearSpring.massScale;
			impulseScale = j->linearSpring.impulseScale;
		}
		b2Vec2 Cdot = o_sub( o_add( vB, o_crossSV( wB, rB ) ), o_add( vA, o_crossSV( wA, rA ) ) );
		float k11 = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		float k12 = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		float k22 = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		b2Vec2 b = o_solve22( k11, k12, k12, k22, o_add( Cdot, bias ) );
		b2Vec2 impulse = { -massScale * b.x - impulseScale * j->linearImpulse.x, -massScale * b.y - impulseScale * j->linearImpulse.y };
		j->linearImpulse = o_add( j->linearImpulse, impulse );
		vA = o_mulSub( vA, mA, impulse );
		wA -= iA * o_cross( rA, impulse );
		vB = o_mulAdd( vB, mB, impulse );
		wB += iB * o_cross( rB, impulse );
	}
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- wheel (wheel_joint.c:197-525) ---------------- */
static void o_prepareWheel( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float mA = simA->invMass, iA = simA->invInertia, mB = simB->invMass, iB = simB->invInertia;
	base->invMassA = mA;
	base->invMassB = mB;
	base->invIA = iA;
	base->invIB = iB;
	o_wheelJoint* j = &base->wheelJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->frameA.q = o_mulRot( simA->transform.q, base->localFrameA.q );
	j->frameA.p = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->frameB.q = o_mulRot( simB->transform.q, base->localFrameB.q );
	j->frameB.p = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	b2Vec2 rA = j->frameA.p, rB = j->frameB.p;
	b2Vec2 d = o_add( j->deltaCenter, o_sub( rB, rA ) );
	b2Vec2 axisA = o_rotate( j->frameA.q, o_v( 1.0f, 0.0f ) );
	b2Vec2 perpA = o_leftPerp( axisA );
	float s1 = o_cross( o_add( d, rA ), perpA );
	float s2 = o_cross( rB, perpA );
	float kp = mA + mB + iA * s1 * s1 + iB * s2 * s2;
	j->perpMass = kp > 0.0f ? 1.0f / kp : 0.0f;
	float a1 = o_cross( o_add( d, rA ), axisA );
	float a2 = o_cross( rB, axisA );
	float ka = mA + mB + iA * a1 * a1 + iB * a2 * a2;
	j->axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
	j->springSoftness = o_makeSoft( j->hertz, j->dampingRatio, ctx->h );
	float km = iA + iB;
	j->motorMass = km > 0.0f ? 1.0f / km : 0.0f;
	if ( ctx->enableWarmStarting == 0 )
	{
		j->perpImpulse = 0.0f;
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

static void o_warmStartWheel( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_wheelJoint* j = &base->wheelJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	b2Vec2 d = o_add( o_add( o_sub( sB->deltaPosition, sA->deltaPosition ), j->deltaCenter ), o_sub( rB, rA ) );
	b2Vec2 axisA = o_rotate( j->frameA.q, o_v( 1.0f, 0.0f ) );
	axisA = o_rotate( sA->deltaRotation, axisA );
	b2Vec2 perpA = o_leftPerp( axisA );
	float a1 = o_cross( o_add( d, rA ), axisA );
	float a2 = o_cross( rB, axisA );
	float s1 = o_cross( o_add( d, rA ), perpA );
	float s2 = o_cross( rB, perpA );
	float axialImpulse = j->springImpulse + j->lowerImpulse - j->upperImpulse;
	b2Vec2 P = o_add( o_mulSV( axialImpulse, axisA ), o_mulSV( j->perpImpulse, perpA ) );
	float LA = axialImpulse * a1 + j->perpImpulse * s1 + j->motorImpulse;
	float LB = axialImpulse * a2 + j->perpImpulse * s2 + j->motorImpulse;
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, P );
		sA->angularVelocity -= iA * LA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, P );
		sB->angularVelocity += iB * LB;
	}
}

static void o_solveWheel( o_world* w, o_stepContext* ctx, o_jointSim* base, int useBias )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_wheelJoint* j = &base->wheelJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	int fixedRotation = ( iA + iB == 0.0f );
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	b2Vec2 d = o_add( o_add( o_sub( sB->deltaPosition, sA->deltaPosition ), j->deltaCenter ), o_sub( rB, rA ) );
	b2Vec2 axisA = o_rotate( j->frameA.q, o_v( 1.0f, 0.0f ) );
	axisA = o_rotate( sA->deltaRotation, axisA );
	float translation = o_dot( axisA, d );
	float a1 = o_cross( o_add( d, rA ), axisA );
	float a2 = o_cross( rB, axisA );
	if ( j->enableMotor && fixedRotation == 0 )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->motorMass * Cdot;
		float oldImpulse = j->motorImpulse;
		float maxImpulse = ctx->h * j->maxMotorTorque;
		j->motorImpulse = o_clamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableSpring )
	{
		float C = translation;
		float bias = j->springSoftness.biasRate * C;
		float massScale = j->springSoftness.massScale;
		float impulseScale = j->springSoftness.impulseScale;
		float Cdot = o_dot( axisA, o_sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += impulse;
		o_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, impulse );
	}
	if ( j->enableLimit )
	{
		{
			float C = translation - j->lowerTranslation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * ctx->inv_h;
			else if ( useBias )
			{
				bias = base->constraintSoftness.biasRate * C;
				massScale = base->constraintSoftness.massScale;
				impulseScale = base->constraintSoftness.impulseScale;
			}
			float Cdot = o_dot( axisA, o_sub( vB, vA ) ) + a2 * wB - a1 * wA;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->lowerImpulse;
			float oldImpulse = j->lowerImpulse;
			j->lowerImpulse = o_max( oldImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - oldImpulse;
			o_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, impulse );
		}
		{
			float C = j->upperTranslation - translation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * ctx->inv_h;
			else if ( useBias )
			{
				bias = base->constraintSoftness.biasRate * C;
				massScale = base->constraintSoftness.massScale;
				impulseScale = base->constraintSoftness.impulseScale;
			}
			float Cdot = o_dot( axisA, o_sub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->upperImpulse;
			float oldImpulse = j->upperImpulse;
			j->upperImpulse = o_max( oldImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - oldImpulse;
			b2Vec2 P = o_mulSV( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = o_mulAdd( vA, mA, P );
			wA += iA * LA;
			vB = o_mulSub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		b2Vec2 perpA = o_leftPerp( axisA );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			float C = o_dot( perpA, d );
			bias = base->constraintSoftness.biasRate * C;
			massScale = base->constraintSoftness.massScale;
			impulseScale = base->constraintSoftness.impulseScale;
		}
		float s1 = o_cross( o_add( d, rA ), perpA );
		float s2 = o_cross( rB, perpA );
		float Cdot = o_dot( perpA, o_sub( vB, vA ) ) + s2 * wB - s1 * wA;
		float impulse = -massScale * j->perpMass * ( Cdot + bias ) - impulseScale * j->perpImpulse;
		j->perpImpulse += impulse;
		o_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, perpA, s1, s2, impulse );
	}
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- distance (distance_joint.c:250-543) ---------------- */
static void o_prepareDistance( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float mA = simA->invMass, iA = simA->invInertia, mB = simB->invMass, iB = simB->invInertia;
	base->invMassA = mA;
	base->invMassB = mB;
	base->invIA = iA;
	base->invIB = iB;
	o_distanceJoint* j = &base->distanceJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->anchorA = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->anchorB = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	b2Vec2 rA = j->anchorA, rB = j->anchorB;
	b2Vec2 separation = o_add( o_sub( rB, rA ), j->deltaCenter );
	b2Vec2 axis = o_normalize( separation );
	float crA = o_cross( rA, axis );
	float crB = o_cross( rB, axis );
	float k = mA + mB + iA * crA * crA + iB * crB * crB;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	j->distanceSoftness = o_makeSoft( j->hertz, j->dampingRatio, ctx->h );
	if ( ctx->enableWarmStarting == 0 )
	{
		j->impulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
		j->motorImpulse = 0.0f;
	}
}

static void o_warmStartDistance( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_distanceJoint* j = &base->distanceJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->anchorA );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->anchorB );
	b2Vec2 ds = o_add( o_sub( sB->deltaPosition, sA->deltaPosition ), o_sub( rB, rA ) );
	b2Vec2 separation = o_add( j->deltaCenter, ds );
	b2Vec2 axis = o_normalize( separation );
	float axialImpulse = j->impulse + j->lowerImpulse - j->upperImpulse + j->motorImpulse;
	b2Vec2 P = o_mulSV( axialImpulse, axis );
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, P );
		sA->angularVelocity -= iA * o_cross( rA, P );
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, P );
		sB->angularVelocity += iB * o_cross( rB, P );
	}
}

/* apply P = impulse * axis at anchors rA, rB */
static void o_applyLinear( b2Vec2* vA, float* wA, b2Vec2* vB, float* wB, float mA, float iA, float mB, float iB, b2Vec2 rA,
						   b2Vec2 rB, b2Vec2 P )
{
	*vA = o_mulSub( *vA, mA, P );
	*wA -= iA * o_cross( rA, P );
	*vB = o_mulAdd( *vB, mB, P );
	*wB += iB * o_cross( rB, P );
}

static void o_solveDistance( o_world* w, o_stepContext* ctx, o_jointSim* base, int useBias )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_distanceJoint* j = &base->distanceJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->anchorA );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->anchorB );
	b2Vec2 ds = o_add( o_sub( sB->deltaPosition, sA->deltaPosition ), o_sub( rB, rA ) );
	b2Vec2 separation = o_add( j->deltaCenter, ds );
	float length = o_length( separation );
	b2Vec2 axis = o_normalize( separation );
	if ( j->enableSpring && ( j->minLength < j->maxLength || j->enableLimit == 0 ) )
	{
		if ( j->hertz > 0.0f )
		{
			b2Vec2 vr = o_add( o_sub( vB, vA ), o_sub( o_crossSV( wB, rB ), o_crossSV( wA, rA ) ) );
			float cdot = o_dot( axis, vr );
			float c = length - j->length;
			float bias = j->distanceSoftness.biasRate * c;
			float m = j->distanceSoftness.massScale * j->axialMass;
			float oldImpulse = j->impulse;
			float impulse = -m * ( cdot + bias ) - j->distanceSoftness.impulseScale * oldImpulse;
			float h = ctx->h;
			j->impulse = o_clamp( j->impulse + impulse, j->lowerSpringForce * h, j->upperSpringForce * h );
			impulse = j->impulse - oldImpulse;
			o_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, o_mulSV( impulse, axis ) );
		}
		if ( j->enableMotor )
		{
			b2Vec2 vr = o_add( o_sub( vB, vA ), o_sub( o_crossSV( wB, rB ), o_crossSV( wA, rA ) ) );
			float Cdot = o_dot( axis, vr );
			float impulse = j->axialMass * ( j->motorSpeed - Cdot );
			float oldImpulse = j->motorImpulse;
			float maxImpulse = ctx->h * j->maxMotorForce;
			j->motorImpulse = o_clamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
			impulse = j->motorImpulse - oldImpulse;
			o_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, o_mulSV( impulse, axis ) );
		}
		if ( j->enableLimit )
		{
			{
				b2Vec2 vr = o_add( o_sub( vB, vA ), o_sub( o_crossSV( wB, rB ), o_crossSV( wA, rA ) ) );
				float cdot = o_dot( axis, vr );
				float c = length - j->minLength;
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( c > 0.0f ) bias = c * ctx->inv_h;
				else if ( useBias )
				{
					bias = base->constraintSoftness.biasRate * c;
					massScale = base->constraintSoftness.massScale;
					impulseScale = base->constraintSoftness.impulseScale;
				}
				float impulse = -massScale * j->axialMass * ( cdot + bias ) - impulseScale * j->lowerImpulse;
				float newImpulse = o_max( 0.0f, j->lowerImpulse + impulse );
				impulse = newImpulse - j->lowerImpulse;
				j->lowerImpulse = newImpulse;
				o_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, o_mulSV( impulse, axis ) );
			}
			{
				b2Vec2 vr = o_add( o_sub( vA, vB ), o_sub( o_crossSV( wA, rA ), o_crossSV( wB, rB ) ) );
				float Cdot = o_dot( axis, vr );
				float C = j->maxLength - length;
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f ) bias = C * ctx->inv_h;
				else if ( useBias )
				{
					bias = base->constraintSoftness.biasRate * C;
					massScale = base->constraintSoftness.massScale;
					impulseScale = base->constraintSoftness.impulseScale;
				}
				float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->upperImpulse;
				float newImpulse = o_max( 0.0f, j->upperImpulse + impulse );
				impulse = newImpulse - j->upperImpulse;
				j->upperImpulse = newImpulse;
				o_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, o_mulSV( -impulse, axis ) );
			}
		}
	}
	else
	{
		b2Vec2 vr = o_add( o_sub( vB, vA ), o_sub( o_crossSV( wB, rB ), o_crossSV( wA, rA ) ) );
		float Cdot = o_dot( axis, vr );
		float C = length - j->length;
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			bias = base->constraintSoftness.biasRate * C;
			massScale = base->constraintSoftness.massScale;
			impulseScale = base->constraintSoftness.impulseScale;
		}
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->impulse;
		j->impulse += impulse;
		o_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, o_mulSV( impulse, axis ) );
	}
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- motor (motor_joint.c:180-436) ---------------- */
/* math_functions.h b2GetInverse22 and b2MulMV, columns cx, cy */
static void o_inverse22( b2Vec2 cx, b2Vec2 cy, b2Vec2* ox, b2Vec2* oy )
{
	float a = cx.x, b = cy.x, c = cx.y, d = cy.y;
	float det = a * d - b * c;
	if ( det != 0.0f ) det = 1.0f / det;
	*ox = o_v( det * d, -det * c );
	*oy = o_v( -det * b, det * a );
}

static b2Vec2 o_mulMV( b2Vec2 cx, b2Vec2 cy, b2Vec2 v ) { return o_v( cx.x * v.x + cy.x * v.y, cx.y * v.x + cy.y * v.y ); }

static void o_motorLinearMass( o_motorJoint* j, float mA, float mB, float iA, float iB, b2Vec2 rA, b2Vec2 rB )
{
	b2Vec2 kx, ky;
	kx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
	kx.y = -rA.y * rA.x * iA - rB.y * rB.x * iB;
	ky.x = kx.y;
	ky.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
	o_inverse22( kx, ky, &j->linearMassCx, &j->linearMassCy );
}

static void o_prepareMotor( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float mA = simA->invMass, iA = simA->invInertia, mB = simB->invMass, iB = simB->invInertia;
	base->invMassA = mA;
	base->invMassB = mB;
	base->invIA = iA;
	base->invIB = iB;
	o_motorJoint* j = &base->motorJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->frameA.q = o_mulRot( simA->transform.q, base->localFrameA.q );
	j->frameA.p = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->frameB.q = o_mulRot( simB->transform.q, base->localFrameB.q );
	j->frameB.p = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	j->linearSpring = o_makeSoft( j->linearHertz, j->linearDampingRatio, ctx->h );
	j->angularSpring = o_makeSoft( j->angularHertz, j->angularDampingRatio, ctx->h );
	o_motorLinearMass( j, mA, mB, iA, iB, j->frameA.p, j->frameB.p );
	float ka = iA + iB;
	j->angularMass = ka > 0.0f ? 1.0f / ka : 0.0f;
	if ( ctx->enableWarmStarting == 0 )
	{
		j->linearVelocityImpulse = o_v( 0.0f, 0.0f );
		j->angularVelocityImpulse = 0.0f;
		j->linearSpringImpulse = o_v( 0.0f, 0.0f );
		j->angularSpringImpulse = 0.0f;
	}
}

static void o_warmStartMotor( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_motorJoint* j = &base->motorJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	b2Vec2 linearImpulse = o_add( j->linearVelocityImpulse, j->linearSpringImpulse );
	float angularImpulse = j->angularVelocityImpulse + j->angularSpringImpulse;
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, linearImpulse );
		sA->angularVelocity -= iA * ( o_cross( rA, linearImpulse ) + angularImpulse );
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, linearImpulse );
		sB->angularVelocity += iB * ( o_cross( rB, linearImpulse ) + angularImpulse );
	}
}

/* accumulate `impulse` into `*acc` and clamp the total's length to maxImpulse
   (motor_joint.c:383-392); returns the applied change */
static b2Vec2 o_clampedAccumulate( b2Vec2* acc, b2Vec2 impulse, float maxImpulse )
{
	b2Vec2 old = *acc;
	*acc = o_add( *acc, impulse );
	if ( o_lengthSq( *acc ) > maxImpulse * maxImpulse )
	{
		*acc = o_normalize( *acc );
		acc->x *= maxImpulse;
		acc->y *= maxImpulse;
	}
	return o_sub( *acc, old );
}

/* the motor joint ignores useBias: solve and relax are the same pass (joint.c:1506-1508) */
static void o_solveMotor( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_bodyState dummy = o_dummyState;
	o_motorJoint* j = &base->motorJoint;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	if ( j->maxSpringTorque > 0.0f && j->angularHertz > 0.0f )
	{
		b2Rot qA = o_mulRot( sA->deltaRotation, j->frameA.q );
		b2Rot qB = o_mulRot( sB->deltaRotation, j->frameB.q );
		b2Rot relQ = o_invMulRot( qA, qB );
		float c = b2Atan2( relQ.s, relQ.c );
		float bias = j->angularSpring.biasRate * c;
		float massScale = j->angularSpring.massScale;
		float impulseScale = j->angularSpring.impulseScale;
		float cdot = wB - wA;
		float maxImpulse = ctx->h * j->maxSpringTorque;
		float oldImpulse = j->angularSpringImpulse;
		float impulse = -massScale * j->angularMass * ( cdot + bias ) - impulseScale * oldImpulse;
		j->angularSpringImpulse = o_clamp( oldImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->angularSpringImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->maxVelocityTorque > 0.0f )
	{
		float cdot = wB - wA - j->angularVelocity;
		float impulse = -j->angularMass * cdot;
		float maxImpulse = ctx->h * j->maxVelocityTorque;
		float oldImpulse = j->angularVelocityImpulse;
		j->angularVelocityImpulse = o_clamp( oldImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->angularVelocityImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	if ( j->maxSpringForce > 0.0f && j->linearHertz > 0.0f )
	{
		b2Vec2 dcA = sA->deltaPosition, dcB = sB->deltaPosition;
		b2Vec2 c = o_add( o_add( o_sub( dcB, dcA ), o_sub( rB, rA ) ), j->deltaCenter );
		b2Vec2 bias = o_mulSV( j->linearSpring.biasRate, c );
		float massScale = j->linearSpring.massScale;
		float impulseScale = j->linearSpring.impulseScale;
		b2Vec2 cdot = o_sub( o_add( vB, o_crossSV( wB, rB ) ), o_add( vA, o_crossSV( wA, rA ) ) );
		cdot = o_add( cdot, bias );
		o_motorLinearMass( j, mA, mB, iA, iB, rA, rB );
		b2Vec2 b = o_mulMV( j->linearMassCx, j->linearMassCy, cdot );
		b2Vec2 old = j->linearSpringImpulse;
		b2Vec2 impulse = o_v( -massScale * b.x - impulseScale * old.x, -massScale * b.y - impulseScale * old.y );
		impulse = o_clampedAccumulate( &j->linearSpringImpulse, impulse, ctx->h * j->maxSpringForce );
		vA = o_mulSub( vA, mA, impulse );
		wA -= iA * o_cross( rA, impulse );
		vB = o_mulAdd( vB, mB, impulse );
		wB += iB * o_cross( rB, impulse );
	}
	if ( j->maxVelocityForce > 0.0f )
	{
		b2Vec2 cdot = o_sub( o_add( vB, o_crossSV( wB, rB ) ), o_add( vA, o_crossSV( wA, rA ) ) );
		cdot = o_sub( cdot, j->linearVelocity );
		b2Vec2 b = o_mulMV( j->linearMassCx, j->linearMassCy, cdot );
		b2Vec2 impulse = o_v( -b.x, -b.y );
		impulse = o_clampedAccumulate( &j->linearVelocityImpulse, impulse, ctx->h * j->maxVelocityForce );
		vA = o_mulSub( vA, mA, impulse );
		wA -= iA * o_cross( rA, impulse );
		vB = o_mulAdd( vB, mB, impulse );
		wB += iB * o_cross( rB, impulse );
	}
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- mover (mover_joint.c:43-170): linear only, rotation untouched ---------------- */
static void o_prepareMover( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float mA = simA->invMass, mB = simB->invMass;
	base->invMassA = mA;
	base->invMassB = mB;
	base->invIA = 0.0f;
	base->invIB = 0.0f;
	o_moverJoint* j = &base->moverJoint;
	j->indexA = ia;
	j->indexB = ib;
	float k = mA + mB;
	j->linearMass = k > 0.0f ? 1.0f / k : 0.0f;
	if ( ctx->enableWarmStarting == 0 ) j->linearVelocityImpulse = o_v( 0.0f, 0.0f );
}

static void o_warmStartMover( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB;
	o_moverJoint* j = &base->moverJoint;
	o_bodyState dummy = o_dummyState;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	if ( sA->flags & O_DYNAMIC_FLAG ) sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, j->linearVelocityImpulse );
	if ( sB->flags & O_DYNAMIC_FLAG ) sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, j->linearVelocityImpulse );
}

static void o_solveMover( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB;
	o_moverJoint* j = &base->moverJoint;
	o_bodyState dummy = o_dummyState;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	if ( j->maxVelocityForce.x > 0.0f || j->maxVelocityForce.y > 0.0f )
	{
		b2Vec2 cdot = o_sub( o_sub( vB, vA ), j->linearVelocity );
		b2Vec2 b = o_mulSV( j->linearMass, cdot );
		b2Vec2 impulse = o_v( -b.x, -b.y );
		b2Vec2 old = j->linearVelocityImpulse;
		j->linearVelocityImpulse = o_add( j->linearVelocityImpulse, impulse );
		b2Vec2 maxImpulse = o_mulSV( ctx->h, j->maxVelocityForce );
		/* x and y clamped separately (math_functions.h b2Clamp) */
		j->linearVelocityImpulse.x = o_clamp( j->linearVelocityImpulse.x, -maxImpulse.x, maxImpulse.x );
		j->linearVelocityImpulse.y = o_clamp( j->linearVelocityImpulse.y, -maxImpulse.y, maxImpulse.y );
		impulse = o_sub( j->linearVelocityImpulse, old );
		vA = o_mulSub( vA, mA, impulse );
		vB = o_mulAdd( vB, mB, impulse );
	}
	else
	{
		j->linearVelocityImpulse = o_v( 0.0f, 0.0f );
	}
	if ( sA->flags & O_DYNAMIC_FLAG ) sA->linearVelocity = vA;
	if ( sB->flags & O_DYNAMIC_FLAG ) sB->linearVelocity = vB;
}

/* ---------------- pogo (pogo_joint.c:98-281) ---------------- */
static void o_preparePogo( o_world* w, o_stepContext* ctx, o_jointSim* base )
{
	int ia, ib;
	o_bodySim* simA = o_jointBodySim( w, base->bodyIdA, &ia );
	o_bodySim* simB = o_jointBodySim( w, base->bodyIdB, &ib );
	float mA = simA->invMass, iA = simA->invInertia, mB = simB->invMass, iB = simB->invInertia;
	base->invMassA = mA;
	base->invMassB = mB;
	base->invIA = iA;
	base->invIB = iB;
	o_pogoJoint* j = &base->pogoJoint;
	j->indexA = ia;
	j->indexB = ib;
	j->frameA.q = o_mulRot( simA->transform.q, base->localFrameA.q );
	j->frameA.p = o_rotate( simA->transform.q, o_sub( base->localFrameA.p, simA->localCenter ) );
	j->frameB.q = o_mulRot( simB->transform.q, base->localFrameB.q );
	j->frameB.p = o_rotate( simB->transform.q, o_sub( base->localFrameB.p, simB->localCenter ) );
	j->deltaCenter = o_v( simB->center.x - simA->center.x, simB->center.y - simA->center.y );
	float crA = o_cross( j->frameA.p, j->normal );
	float crB = o_cross( j->frameB.p, j->normal );
	float k = mA + mB + iA * crA * crA + iB * crB * crB;
	j->linearMass = k > 0.0f ? 1.0f / k : 0.0f;
	if ( ctx->enableWarmStarting == 0 ) j->impulse = 0.0f;
}

static void o_warmStartPogo( o_world* w, o_jointSim* base )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_pogoJoint* j = &base->pogoJoint;
	if ( j->hertz == 0.0f )
	{
		j->impulse = 0.0f;
		return;
	}
	o_bodyState dummy = o_dummyState;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	b2Vec2 P = o_mulSV( j->impulse, j->normal );
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = o_mulSub( sA->linearVelocity, mA, P );
		sA->angularVelocity -= iA * o_cross( rA, P );
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = o_mulAdd( sB->linearVelocity, mB, P );
		sB->angularVelocity += iB * o_cross( rB, P );
	}
}

/* math_functions.h b2SpringDamper: implicit spring-damper velocity update */
static float o_springDamper( float hertz, float dampingRatio, float position, float velocity, float timeStep )
{
	float omega = 2.0f * B2_PI * hertz;
	float omegaH = omega * timeStep;
	return ( velocity - omega * omegaH * position ) / ( 1.0f + 2.0f * dampingRatio * omegaH + omegaH * omegaH );
}

static void o_solvePogo( o_world* w, o_stepContext* ctx, o_jointSim* base, int useBias )
{
	float mA = base->invMassA, mB = base->invMassB, iA = base->invIA, iB = base->invIB;
	o_pogoJoint* j = &base->pogoJoint;
	if ( j->hertz == 0.0f )
	{
		j->impulse = 0.0f;
		return;
	}
	o_bodyState dummy = o_dummyState;
	o_bodyState* sA = j->indexA == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexA;
	o_bodyState* sB = j->indexB == B2_NULL_INDEX ? &dummy : w->awakeStates.data + j->indexB;
	b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
	float wA = sA->angularVelocity, wB = sB->angularVelocity;
	b2Vec2 rA = o_rotate( sA->deltaRotation, j->frameA.p );
	b2Vec2 rB = o_rotate( sB->deltaRotation, j->frameB.p );
	float bias = 0.0f;
	if ( useBias )
	{
		b2Vec2 dcA = sA->deltaPosition, dcB = sB->deltaPosition;
		b2Vec2 d = o_add( o_add( o_sub( dcB, dcA ), o_sub( rB, rA ) ), j->deltaCenter );
		/* the pogo axis is frame B's y axis (pogo_joint.c:14) */
		b2Vec2 pogoAxis = o_rotate( j->frameB.q, o_v( 0.0f, 1.0f ) );
		float c = o_dot( pogoAxis, d ) - j->restLength;
		j->velocity = o_springDamper( j->hertz, j->dampingRatio, c, j->velocity, ctx->h );
		bias = -j->velocity;
	}
	b2Vec2 vr = o_sub( o_add( vB, o_crossSV( wB, rB ) ), o_add( vA, o_crossSV( wA, rA ) ) );
	float cdot = o_dot( j->normal, vr );
	float maxTensionImpulse = ctx->h * j->maxTensionForce;
	float maxCompressionImpulse = ctx->h * j->maxCompressionForce;
	float oldImpulse = j->impulse;
	float impulse = -j->linearMass * ( cdot + bias );
	j->impulse = o_clamp( j->impulse + impulse, -maxTensionImpulse, maxCompressionImpulse );
	impulse = j->impulse - oldImpulse;
	b2Vec2 P = o_mulSV( impulse, j->normal );
	vA = o_mulSub( vA, mA, P );
	wA -= iA * o_cross( rA, P );
	vB = o_mulAdd( vB, mB, P );
	wB += iB * o_cross( rB, P );
	if ( sA->flags & O_DYNAMIC_FLAG )
	{
		sA->linearVelocity = vA;
		sA->angularVelocity = wA;
	}
	if ( sB->flags & O_DYNAMIC_FLAG )
	{
		sB->linearVelocity = vB;
		sB->angularVelocity = wB;
	}
}

/* ---------------- dispatch (joint.c:1406-1540) ---------------- */
int o_unsupportedJoints = 0;

void o_prepareJoint( o_world* w, o_stepContext* ctx, o_jointSim* j )
{
	float hertz = o_min( j->constraintHertz, 0.25f * ctx->inv_h );
	j->constraintSoftness = o_makeSoft( hertz, j->constraintDampingRatio, ctx->h );
	switch ( j->type )
	{
		case b2_distanceJoint: o_prepareDistance( w, ctx, j ); break;
		case b2_prismaticJoint: o_preparePrismatic( w, ctx, j ); break;
		case b2_revoluteJoint: o_prepareRevolute( w, ctx, j ); break;
		case b2_weldJoint: o_prepareWeld( w, ctx, j ); break;
		case b2_wheelJoint: o_prepareWheel( w, ctx, j ); break;
		case b2_motorJoint: o_prepareMotor( w, ctx, j ); break;
		case b2_pogoJoint: o_preparePogo( w, ctx, j ); break;
		case b2_moverJoint: o_prepareMover( w, ctx, j ); break;
		case b2_filterJoint: break;
		default: o_unsupportedJoints += 1; break;
	}
}

void o_warmStartJoint( o_world* w, o_stepContext* ctx, o_jointSim* j )
{
	(void)ctx;
	switch ( j->type )
	{
		case b2_distanceJoint: o_warmStartDistance( w, j ); break;
		case b2_prismaticJoint: o_warmStartPrismatic( w, j ); break;
		case b2_revoluteJoint: o_warmStartRevolute( w, j ); break;
		case b2_weldJoint: o_warmStartWeld( w, j ); break;
		case b2_wheelJoint: o_warmStartWheel( w, j ); break;
		case b2_motorJoint: o_warmStartMotor( w, j ); break;
		case b2_pogoJoint: o_warmStartPogo( w, j ); break;
		case b2_moverJoint: o_warmStartMover( w, j ); break;
		default: break;
	}
}

void o_solveJoint( o_world* w, o_stepContext* ctx, o_jointSim* j, int useBias )
{
	switch ( j->type )
	{
		case b2_distanceJoint: o_solveDistance( w, ctx, j, useBias ); break;
		case b2_prismaticJoint: o_solvePrismatic( w, ctx, j, useBias ); break;
		case b2_revoluteJoint: o_solveRevolute( w, ctx, j, useBias ); break;
		case b2_weldJoint: o_solveWeld( w, j, useBias ); break;
		case b2_wheelJoint: o_solveWheel( w, ctx, j, useBias ); break;
		case b2_motorJoint: o_solveMotor( w, ctx, j ); break;
		case b2_pogoJoint: o_solvePogo( w, ctx, j, useBias ); break;
		case b2_moverJoint: o_solveMover( w, ctx, j ); break;
		default: break;
	}
}

float b2RevoluteJoint_GetAngle( b2JointId jointId )
{
	o_world* w = o_getWorld( jointId.world0 );
	o_joint* joint = w->joints.data + jointId.index1 - 1;
	if ( joint->colorIndex == B2_NULL_INDEX ) return 0.0f;
	o_jointSim* sim = w->colors[joint->colorIndex].jointSims.data + joint->localIndex;
	int ia, ib;
	o_bodySim* a = o_jointBodySim( w, sim->bodyIdA, &ia );
	o_bodySim* b = o_jointBodySim( w, sim->bodyIdB, &ib );
	b2Rot qA = o_mulRot( a->transform.q, sim->localFrameA.q );
	b2Rot qB = o_mulRot( b->transform.q, sim->localFrameB.q );
	b2Rot r = o_invMulRot( qA, qB );
	return b2Atan2( r.s, r.c );
}
