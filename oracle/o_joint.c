/*
 * Oracle (test checker only): joint creation (joint.c:16-720), the per-type dispatch
 * (joint.c:1406-1540) and the joint solvers. Revolute follows revolute_joint.c:217-500;
 * prismatic, weld, wheel and distance follow their *_joint.c files.
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

/* ---------------- dispatch (joint.c:1406-1540) ---------------- */
int o_unsupportedJoints = 0;

void o_prepareJoint( o_world* w, o_stepContext* ctx, o_jointSim* j )
{
	float hertz = o_min( j->constraintHertz, 0.25f * ctx->inv_h );
	j->constraintSoftness = o_makeSoft( hertz, j->constraintDampingRatio, ctx->h );
	switch ( j->type )
	{
		case b2_revoluteJoint: o_prepareRevolute( w, ctx, j ); break;
		default: o_unsupportedJoints += 1; break;
	}
}

void o_warmStartJoint( o_world* w, o_stepContext* ctx, o_jointSim* j )
{
	(void)ctx;
	switch ( j->type )
	{
		case b2_revoluteJoint: o_warmStartRevolute( w, j ); break;
		default: break;
	}
}

void o_solveJoint( o_world* w, o_stepContext* ctx, o_jointSim* j, int useBias )
{
	switch ( j->type )
	{
		case b2_revoluteJoint: o_solveRevolute( w, ctx, j, useBias ); break;
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
