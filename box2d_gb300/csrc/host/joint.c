/*
 * Joint creation for the GB300 step library (joint.c:16-720 in the reference). The host
 * keeps the joint graph edges and the color assignment (constraint_graph.c:216-291); the
 * solver record (b2gJoint) goes to the device, which owns the accumulated impulses.
 *
 * Per-type parameter slots in b2gJoint.p / .s:
 *   revolute : p = targetAngle, hertz, dampingRatio, lowerAngle, upperAngle, maxMotorTorque,
 *                  motorSpeed
 *              s = linearImpulse.x, linearImpulse.y, springImpulse, motorImpulse,
 *                  lowerImpulse, upperImpulse, axialMass, spring softness (3)
 *   prismatic: p = hertz, dampingRatio, targetTranslation, lowerTranslation,
 *                  upperTranslation, maxMotorForce, motorSpeed
 *              s = impulse.x, impulse.y, springImpulse, motorImpulse, lowerImpulse,
 *                  upperImpulse, spring softness (3)
 *   weld     : p = linearHertz, linearDampingRatio, angularHertz, angularDampingRatio
 *              s = linearImpulse.x, linearImpulse.y, angularImpulse, axialMass,
 *                  linear softness (3), angular softness (3)
 *   wheel    : p = lowerTranslation, upperTranslation, maxMotorTorque, motorSpeed, hertz,
 *                  dampingRatio
 *              s = perpImpulse, motorImpulse, springImpulse, lowerImpulse, upperImpulse,
 *                  perpMass, motorMass, axialMass, spring softness (3)
 *   distance : p = length, hertz, dampingRatio, lowerSpringForce, upperSpringForce,
 *                  minLength, maxLength, maxMotorForce, motorSpeed
 *              s = impulse, lowerImpulse, upperImpulse, motorImpulse, axialMass,
 *                  distance softness (3); the anchors are frameA.p and frameB.p
 *   motor    : p = linearVelocity (2), maxVelocityForce, angularVelocity,
 *                  maxVelocityTorque, linearHertz, linearDampingRatio, maxSpringForce,
 *                  angularHertz, angularDampingRatio, maxSpringTorque, angular spring
 *                  softness (3, written by the prepare stage)
 *              s = linearVelocityImpulse (2), angularVelocityImpulse, linearSpringImpulse
 *                  (2), angularSpringImpulse, linearMass (2x2, columns), angularMass,
 *                  linear spring softness (3)
 *   pogo     : p = normal (2), hertz, dampingRatio, restLength, maxTensionForce,
 *                  maxCompressionForce
 *              s = impulse, spring velocity, linearMass
 *   mover    : p = linearVelocity (2), maxVelocityForce (2)
 *              s = linearVelocityImpulse (2), linearMass
 *   filter   : no parameters; colored like any joint, no constraint
 */
#include "b2g_world.h"

static b2JointDef h_defaultJointDef( void )
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
	def.base = h_defaultJointDef();
	def.lowerSpringForce = -FLT_MAX;
	def.upperSpringForce = FLT_MAX;
	def.length = 1.0f;
	def.maxLength = H_HUGE;
	def.internalValue = 1152023;
	return def;
}

b2PrismaticJointDef b2DefaultPrismaticJointDef( void )
{
	b2PrismaticJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2RevoluteJointDef b2DefaultRevoluteJointDef( void )
{
	b2RevoluteJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2WeldJointDef b2DefaultWeldJointDef( void )
{
	b2WeldJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2WheelJointDef b2DefaultWheelJointDef( void )
{
	b2WheelJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.enableSpring = true;
	def.hertz = 1.0f;
	def.dampingRatio = 0.7f;
	def.internalValue = 1152023;
	return def;
}

/* joint.c:161-196 */
static void h_destroyContactsBetweenBodies( h_world* w, h_body* bodyA, h_body* bodyB )
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
		h_contact* c = w->contacts.data + contactId;
		contactKey = c->edges[edgeIndex].nextKey;
		if ( c->edges[edgeIndex ^ 1].bodyId == otherBodyId ) h_destroyContact( w, c );
	}
}

/* joint.c:204-398: the joint goes to the static set, the graph colors (waking a sleeping
   body), or the sleeping set of its bodies, then links their islands */
static b2gJoint* h_createJoint( h_world* w, const b2JointDef* def, b2JointType type, b2JointId* outId )
{
	h_syncFromDevice( w );
	h_syncJointsFromDevice( w );
	h_body* bodyA = w->bodies.data + def->bodyIdA.index1 - 1;
	h_body* bodyB = w->bodies.data + def->bodyIdB.index1 - 1;
	if ( def->collideConnected == false ) h_destroyContactsBetweenBodies( w, bodyA, bodyB );
	int bodyIdA = bodyA->id, bodyIdB = bodyB->id;
	int jointId = h_allocId( &w->jointIdPool );
	if ( jointId == w->joints.count )
	{
		h_joint z;
		memset( &z, 0, sizeof( z ) );
		h_push( w->joints, z );
		b2gJoint r;
		memset( &r, 0, sizeof( r ) );
		h_push( w->jointRecords, r );
	}
	h_joint* j = w->joints.data + jointId;
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
	j->islandId = B2_NULL_INDEX;
	j->islandIndex = B2_NULL_INDEX;
	int maxSetIndex = bodyA->setIndex > bodyB->setIndex ? bodyA->setIndex : bodyB->setIndex;
	if ( bodyA->type != b2_dynamicBody && bodyB->type != b2_dynamicBody )
	{
		/* joint.c:265-275: the static set holds it, at the end of its joint array */
		j->setIndex = H_STATIC_SET;
		j->colorIndex = B2_NULL_INDEX;
		j->localIndex = w->staticJointCount++;
		h_push( w->staticJointIds, jointId );
	}
	else if ( bodyA->setIndex == H_AWAKE_SET || bodyB->setIndex == H_AWAKE_SET )
	{
		/* a sleeping body of the pair wakes */
		if ( maxSetIndex >= H_FIRST_SLEEPING_SET ) h_wakeSolverSet( w, maxSetIndex );
		j->setIndex = H_AWAKE_SET;
		h_addJointToGraph( w, j );
	}
	else
	{
		/* between sleeping (and static) bodies: the joint sleeps with them; two sleeping
		   sets merge */
		j->setIndex = maxSetIndex;
		j->localIndex = w->sets.data[maxSetIndex].jointIds.count;
		h_push( w->sets.data[maxSetIndex].jointIds, jointId );
		if ( bodyA->setIndex != bodyB->setIndex && bodyA->setIndex >= H_FIRST_SLEEPING_SET &&
			 bodyB->setIndex >= H_FIRST_SLEEPING_SET )
			h_mergeSolverSets( w, bodyA->setIndex, bodyB->setIndex );
	}
	b2gJoint* r = w->jointRecords.data + jointId;
	memset( r, 0, sizeof( *r ) );
	r->type = type;
	r->bodyIdA = bodyIdA;
	r->bodyIdB = bodyIdB;
	r->localFrameA = def->localFrameA;
	r->localFrameB = def->localFrameB;
	r->constraintHertz = def->constraintHertz;
	r->constraintDampingRatio = def->constraintDampingRatio;
	r->softBias = 0.0f;
	r->softMass = 1.0f;
	r->softImpulse = 0.0f;
	r->jointId = jointId;
	w->jointsDirty = 1;
	if ( j->setIndex > H_DISABLED_SET ) h_linkJoint( w, j );
	outId->index1 = jointId + 1;
	outId->world0 = w->worldId;
	outId->generation = j->generation;
	return r;
}

b2JointId b2CreateRevoluteJoint( b2WorldId worldId, const b2RevoluteJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_revoluteJoint, &id );
	float lowerAngle = h_min( def->lowerAngle, def->upperAngle );
	float upperAngle = h_max( def->lowerAngle, def->upperAngle );
	r->p[0] = h_clamp( def->targetAngle, -B2_PI, B2_PI );
	r->p[1] = def->hertz;
	r->p[2] = def->dampingRatio;
	r->p[3] = h_clamp( lowerAngle, -0.99f * B2_PI, 0.99f * B2_PI );
	r->p[4] = h_clamp( upperAngle, -0.99f * B2_PI, 0.99f * B2_PI );
	r->p[5] = def->maxMotorTorque;
	r->p[6] = def->motorSpeed;
	r->enableSpring = def->enableSpring;
	r->enableLimit = def->enableLimit;
	r->enableMotor = def->enableMotor;
	return id;
}

b2JointId b2CreatePrismaticJoint( b2WorldId worldId, const b2PrismaticJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_prismaticJoint, &id );
	r->p[0] = def->hertz;
	r->p[1] = def->dampingRatio;
	r->p[2] = def->targetTranslation;
	r->p[3] = def->lowerTranslation;
	r->p[4] = def->upperTranslation;
	r->p[5] = def->maxMotorForce;
	r->p[6] = def->motorSpeed;
	r->enableSpring = def->enableSpring;
	r->enableLimit = def->enableLimit;
	r->enableMotor = def->enableMotor;
	return id;
}

b2JointId b2CreateWeldJoint( b2WorldId worldId, const b2WeldJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_weldJoint, &id );
	r->p[0] = def->linearHertz;
	r->p[1] = def->linearDampingRatio;
	r->p[2] = def->angularHertz;
	r->p[3] = def->angularDampingRatio;
	return id;
}

b2JointId b2CreateWheelJoint( b2WorldId worldId, const b2WheelJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_wheelJoint, &id );
	r->p[0] = def->lowerTranslation;
	r->p[1] = def->upperTranslation;
	r->p[2] = def->maxMotorTorque;
	r->p[3] = def->motorSpeed;
	r->p[4] = def->hertz;
	r->p[5] = def->dampingRatio;
	r->enableSpring = def->enableSpring;
	r->enableLimit = def->enableLimit;
	r->enableMotor = def->enableMotor;
	return id;
}

b2JointId b2CreateDistanceJoint( b2WorldId worldId, const b2DistanceJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_distanceJoint, &id );
	r->p[0] = h_max( def->length, H_LINEAR_SLOP );
	r->p[1] = def->hertz;
	r->p[2] = def->dampingRatio;
	r->p[3] = def->lowerSpringForce;
	r->p[4] = def->upperSpringForce;
	r->p[5] = h_max( def->minLength, H_LINEAR_SLOP );
	r->p[6] = h_max( def->minLength, def->maxLength );
	r->p[7] = def->maxMotorForce;
	r->p[8] = def->motorSpeed;
	r->enableSpring = def->enableSpring;
	r->enableLimit = def->enableLimit;
	r->enableMotor = def->enableMotor;
	return id;
}

/* joint.c:50-62, :72-78 */
b2FilterJointDef b2DefaultFilterJointDef( void )
{
	b2FilterJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2MotorJointDef b2DefaultMotorJointDef( void )
{
	b2MotorJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2PogoJointDef b2DefaultPogoJointDef( void )
{
	b2PogoJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

b2MoverJointDef b2DefaultMoverJointDef( void )
{
	b2MoverJointDef def;
	memset( &def, 0, sizeof( def ) );
	def.base = h_defaultJointDef();
	def.internalValue = 1152023;
	return def;
}

/* joint.c b2CreateMoverJoint */
b2JointId b2CreateMoverJoint( b2WorldId worldId, const b2MoverJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_moverJoint, &id );
	r->p[0] = def->linearVelocity.x;
	r->p[1] = def->linearVelocity.y;
	r->p[2] = def->maxVelocityForce.x;
	r->p[3] = def->maxVelocityForce.y;
	return id;
}

/* joint.c:436-459 */
b2JointId b2CreateFilterJoint( b2WorldId worldId, const b2FilterJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	h_createJoint( w, &def->base, b2_filterJoint, &id );
	return id;
}

/* joint.c:461-491 */
b2JointId b2CreateMotorJoint( b2WorldId worldId, const b2MotorJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_motorJoint, &id );
	r->p[0] = def->linearVelocity.x;
	r->p[1] = def->linearVelocity.y;
	r->p[2] = def->maxVelocityForce;
	r->p[3] = def->angularVelocity;
	r->p[4] = def->maxVelocityTorque;
	r->p[5] = def->linearHertz;
	r->p[6] = def->linearDampingRatio;
	r->p[7] = def->maxSpringForce;
	r->p[8] = def->angularHertz;
	r->p[9] = def->angularDampingRatio;
	r->p[10] = def->maxSpringTorque;
	return id;
}

/* joint.c:521-560 */
b2JointId b2CreatePogoJoint( b2WorldId worldId, const b2PogoJointDef* def )
{
	h_world* w = h_worldFromId( worldId );
	b2JointId id = { 0, 0, 0 };
	b2gJoint* r = h_createJoint( w, &def->base, b2_pogoJoint, &id );
	r->p[0] = def->normal.x;
	r->p[1] = def->normal.y;
	r->p[2] = def->hertz;
	r->p[3] = def->dampingRatio;
	r->p[4] = def->restLength;
	r->p[5] = def->maxTensionForce;
	r->p[6] = def->maxCompressionForce;
	r->s[0] = def->impulse;
	r->s[1] = def->velocity;
	return id;
}

b2JointType b2Joint_GetType( b2JointId jointId )
{
	return h_worldByIndex( jointId.world0 )->joints.data[jointId.index1 - 1].type;
}

/* revolute_joint.c b2RevoluteJoint_GetAngle: relative angle of the two joint frames */
float b2RevoluteJoint_GetAngle( b2JointId jointId )
{
	h_world* w = h_worldByIndex( jointId.world0 );
	h_syncFromDevice( w );
	const b2gJoint* r = w->jointRecords.data + jointId.index1 - 1;
	const h_body* a = w->bodies.data + r->bodyIdA;
	const h_body* b = w->bodies.data + r->bodyIdB;
	b2Rot qA = h_mulRot( a->transform.q, r->localFrameA.q );
	b2Rot qB = h_mulRot( b->transform.q, r->localFrameB.q );
	b2Rot q = h_invMulRot( qA, qB );
	return b2Atan2( q.s, q.c );
}
