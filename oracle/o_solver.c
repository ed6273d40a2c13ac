/*
 * Oracle (test checker only): narrowphase update and contact-state pass (b2Collide,
 * physics_world.c:451-836), the Soft Step solver (b2Solve, solver.c:1275-2081; contact
 * stages contact_solver.c:20-545 and :1573-2331) and b2World_Step (physics_world.c:845).
 *
 * The graph-color contact stages follow the SSE2 wide path lane by lane: one lane is one
 * contact, the second manifold point of a one-point manifold runs with the zeroed dummy
 * data of the reference (so signed zeros match), min/max use the SSE operand order
 * (a < b ? a : b, a > b ? a : b), and rolling resistance is applied to every lane of a
 * 4-wide group as soon as one lane of the group has it (contact_solver.c:2021).
 */
#include "o_core.h"

#include <stdio.h>

/* SSE min/max/clamp semantics (contact_solver.c:314-334) */
static inline float w_min( float a, float b ) { return a < b ? a : b; }
static inline float w_max( float a, float b ) { return a > b ? a : b; }
static inline float w_symClamp( float a, float b )
{
	float nb = -b;
	return w_max( nb, w_min( a, b ) );
}

/* one lane of b2ContactConstraintWide (contact_solver.c:1070-1100) */
typedef struct o_contactLane
{
	int indexA, indexB; /* 0 = null */
	float invMassA, invMassB, invIA, invIB;
	b2Vec2 normal;
	float friction, tangentSpeed, rollingResistance, rollingMass, rollingImpulse;
	float biasRate, massScale, impulseScale;
	b2Vec2 anchorA1, anchorB1;
	float normalMass1, tangentMass1, baseSeparation1, normalImpulse1, totalNormalImpulse1, tangentImpulse1;
	b2Vec2 anchorA2, anchorB2;
	float baseSeparation2, normalImpulse2, totalNormalImpulse2, tangentImpulse2, normalMass2, tangentMass2;
	float restitution, relativeVelocity1, relativeVelocity2;
	int groupHasRolling;
} o_contactLane;

/* contact_solver.h b2ContactConstraint (overflow, scalar path) */
typedef struct o_overflowPoint
{
	b2Vec2 anchorA, anchorB;
	float baseSeparation, relativeVelocity, normalImpulse, tangentImpulse, totalNormalImpulse, normalMass, tangentMass;
} o_overflowPoint;

typedef struct o_overflowConstraint
{
	int indexA, indexB;
	o_overflowPoint points[2];
	b2Vec2 normal;
	float invMassA, invMassB, invIA, invIB, friction, restitution, tangentSpeed, rollingResistance, rollingMass,
		rollingImpulse;
	o_softness softness;
	int pointCount;
} o_overflowConstraint;

static const o_bodyState o_identityState = { { 0.0f, 0.0f }, 0.0f, 0, { 0.0f, 0.0f }, { 1.0f, 0.0f } };

/* ---------------- prepare (contact_solver.c:1573-1809) ---------------- */
static void o_prepareLane( o_world* w, o_stepContext* ctx, const o_contactSim* cs, o_contactLane* c )
{
	const b2Manifold* m = &cs->manifold;
	float warmStartScale = w->enableWarmStarting ? 1.0f : 0.0f;
	int indexA = cs->bodySimIndexA, indexB = cs->bodySimIndexB;
	c->indexA = indexA + 1;
	c->indexB = indexB + 1;
	b2Vec2 vA = { 0.0f, 0.0f };
	float wA = 0.0f;
	float mA = cs->invMassA, iA = cs->invIA;
	if ( indexA != B2_NULL_INDEX )
	{
		vA = w->awakeStates.data[indexA].linearVelocity;
		wA = w->awakeStates.data[indexA].angularVelocity;
	}
	b2Vec2 vB = { 0.0f, 0.0f };
	float wB = 0.0f;
	float mB = cs->invMassB, iB = cs->invIB;
	if ( indexB != B2_NULL_INDEX )
	{
		vB = w->awakeStates.data[indexB].linearVelocity;
		wB = w->awakeStates.data[indexB].angularVelocity;
	}
	c->invMassA = mA;
	c->invMassB = mB;
	c->invIA = iA;
	c->invIB = iB;
	{
		float k = iA + iB;
		c->rollingMass = k > 0.0f ? 1.0f / k : 0.0f;
	}
	o_softness soft = ctx->contactSoftness;
	if ( indexA == B2_NULL_INDEX || indexB == B2_NULL_INDEX )
	{
		soft = ctx->staticSoftness;
	}
	else if ( w->enableContactSoftening )
	{
		float contactHertz = o_min( w->contactHertz, 0.125f * ctx->inv_h );
		float ratio = 1.0f;
		if ( mA < mB ) ratio = o_max( 0.5f, mA / mB );
		else if ( mB < mA ) ratio = o_max( 0.5f, mB / mA );
		soft = o_makeSoft( ratio * contactHertz, ratio * w->contactDampingRatio, ctx->h );
	}
	b2Vec2 normal = m->normal;
	c->normal = normal;
	c->friction = cs->friction;
	c->tangentSpeed = cs->tangentSpeed;
	c->restitution = cs->restitution;
	c->rollingResistance = cs->rollingResistance;
	c->rollingImpulse = warmStartScale * m->rollingImpulse;
	c->biasRate = soft.biasRate;
	c->massScale = soft.massScale;
	c->impulseScale = soft.impulseScale;
	b2Vec2 tangent = o_rightPerp( normal );
	{
		const b2ManifoldPoint* mp = m->points + 0;
		b2Vec2 rA = mp->anchorA, rB = mp->anchorB;
		c->anchorA1 = rA;
		c->anchorB1 = rB;
		c->baseSeparation1 = mp->separation - o_dot( o_sub( rB, rA ), normal );
		c->normalImpulse1 = warmStartScale * mp->normalImpulse;
		c->tangentImpulse1 = warmStartScale * mp->tangentImpulse;
		c->totalNormalImpulse1 = 0.0f;
		float rnA = o_cross( rA, normal ), rnB = o_cross( rB, normal );
		float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		c->normalMass1 = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
		float rtA = o_cross( rA, tangent ), rtB = o_cross( rB, tangent );
		float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		c->tangentMass1 = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
		b2Vec2 vrA = o_add( vA, o_crossSV( wA, rA ) );
		b2Vec2 vrB = o_add( vB, o_crossSV( wB, rB ) );
		c->relativeVelocity1 = o_dot( normal, o_sub( vrB, vrA ) );
	}
	if ( m->pointCount == 2 )
	{
		const b2ManifoldPoint* mp = m->points + 1;
		b2Vec2 rA = mp->anchorA, rB = mp->anchorB;
		c->anchorA2 = rA;
		c->anchorB2 = rB;
		c->baseSeparation2 = mp->separation - o_dot( o_sub( rB, rA ), normal );
		c->normalImpulse2 = warmStartScale * mp->normalImpulse;
		c->tangentImpulse2 = warmStartScale * mp->tangentImpulse;
		c->totalNormalImpulse2 = 0.0f;
		float rnA = o_cross( rA, normal ), rnB = o_cross( rB, normal );
		float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		c->normalMass2 = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
		float rtA = o_cross( rA, tangent ), rtB = o_cross( rB, tangent );
		float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		c->tangentMass2 = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
		b2Vec2 vrA = o_add( vA, o_crossSV( wA, rA ) );
		b2Vec2 vrB = o_add( vB, o_crossSV( wB, rB ) );
		c->relativeVelocity2 = o_dot( normal, o_sub( vrB, vrA ) );
	}
	else
	{
		c->baseSeparation2 = 0.0f;
		c->normalImpulse2 = 0.0f;
		c->tangentImpulse2 = 0.0f;
		c->totalNormalImpulse2 = 0.0f;
		c->anchorA2 = o_v( 0.0f, 0.0f );
		c->anchorB2 = o_v( 0.0f, 0.0f );
		c->normalMass2 = 0.0f;
		c->tangentMass2 = 0.0f;
		c->relativeVelocity2 = 0.0f;
	}
}

static inline o_bodyState o_gather( o_world* w, int index1 )
{
	return index1 == 0 ? o_identityState : w->awakeStates.data[index1 - 1];
}

static inline void o_scatter( o_world* w, int index1, const o_bodyState* b )
{
	if ( index1 == 0 ) return;
	o_bodyState* s = w->awakeStates.data + index1 - 1;
	if ( ( s->flags & O_DYNAMIC_FLAG ) == 0 ) return;
	s->linearVelocity = b->linearVelocity;
	s->angularVelocity = b->angularVelocity;
}

/* contact_solver.c:1811-1871 */
static void o_warmStartLane( o_world* w, o_contactLane* c )
{
	o_bodyState bA = o_gather( w, c->indexA ), bB = o_gather( w, c->indexB );
	float tangentX = c->normal.y;
	float tangentY = 0.0f - c->normal.x;
	{
		b2Vec2 rA = c->anchorA1, rB = c->anchorB1;
		float Px = c->normalImpulse1 * c->normal.x + c->tangentImpulse1 * tangentX;
		float Py = c->normalImpulse1 * c->normal.y + c->tangentImpulse1 * tangentY;
		bA.angularVelocity = bA.angularVelocity - c->invIA * ( rA.x * Py - rA.y * Px );
		bA.linearVelocity.x = bA.linearVelocity.x - c->invMassA * Px;
		bA.linearVelocity.y = bA.linearVelocity.y - c->invMassA * Py;
		bB.angularVelocity = bB.angularVelocity + c->invIB * ( rB.x * Py - rB.y * Px );
		bB.linearVelocity.x = bB.linearVelocity.x + c->invMassB * Px;
		bB.linearVelocity.y = bB.linearVelocity.y + c->invMassB * Py;
		c->totalNormalImpulse1 = c->totalNormalImpulse1 + c->normalImpulse1;
	}
	{
		b2Vec2 rA = c->anchorA2, rB = c->anchorB2;
		float Px = c->normalImpulse2 * c->normal.x + c->tangentImpulse2 * tangentX;
		float Py = c->normalImpulse2 * c->normal.y + c->tangentImpulse2 * tangentY;
		bA.angularVelocity = bA.angularVelocity - c->invIA * ( rA.x * Py - rA.y * Px );
		bA.linearVelocity.x = bA.linearVelocity.x - c->invMassA * Px;
		bA.linearVelocity.y = bA.linearVelocity.y - c->invMassA * Py;
		bB.angularVelocity = bB.angularVelocity + c->invIB * ( rB.x * Py - rB.y * Px );
		bB.linearVelocity.x = bB.linearVelocity.x + c->invMassB * Px;
		bB.linearVelocity.y = bB.linearVelocity.y + c->invMassB * Py;
		c->totalNormalImpulse2 = c->totalNormalImpulse2 + c->normalImpulse2;
	}
	bA.angularVelocity = bA.angularVelocity - c->invIA * c->rollingImpulse;
	bB.angularVelocity = bB.angularVelocity + c->invIB * c->rollingImpulse;
	o_scatter( w, c->indexA, &bA );
	o_scatter( w, c->indexB, &bB );
}

/* one non-penetration point (contact_solver.c:1913-1999) */
static inline void o_solveNormalPoint( o_contactLane* c, o_bodyState* bA, o_bodyState* bB, b2Vec2 dp, b2Vec2 rA, b2Vec2 rB,
									   float baseSeparation, float normalMass, float* normalImpulse, float* totalImpulse,
									   float biasRate, float massScale, float impulseScale, float inv_h,
									   float contactSpeed, float* totalNormalImpulse )
{
	/* moving anchors for current separation */
	float rsAx = bA->deltaRotation.c * rA.x - bA->deltaRotation.s * rA.y;
	float rsAy = bA->deltaRotation.s * rA.x + bA->deltaRotation.c * rA.y;
	float rsBx = bB->deltaRotation.c * rB.x - bB->deltaRotation.s * rB.y;
	float rsBy = bB->deltaRotation.s * rB.x + bB->deltaRotation.c * rB.y;
	float dsx = dp.x + ( rsBx - rsAx );
	float dsy = dp.y + ( rsBy - rsAy );
	float s = ( c->normal.x * dsx + c->normal.y * dsy ) + baseSeparation;
	int mask = s > 0.0f;
	float specBias = s * inv_h;
	float softBias = w_max( biasRate * s, contactSpeed );
	float bias = mask ? specBias : softBias;
	float pointMassScale = mask ? 1.0f : massScale;
	float pointImpulseScale = mask ? 0.0f : impulseScale;
	float dvx = ( bB->linearVelocity.x - bB->angularVelocity * rB.y ) - ( bA->linearVelocity.x - bA->angularVelocity * rA.y );
	float dvy = ( bB->linearVelocity.y + bB->angularVelocity * rB.x ) - ( bA->linearVelocity.y + bA->angularVelocity * rA.x );
	float vn = dvx * c->normal.x + dvy * c->normal.y;
	float negImpulse = normalMass * ( pointMassScale * vn + bias ) + pointImpulseScale * *normalImpulse;
	float newImpulse = w_max( *normalImpulse - negImpulse, 0.0f );
	float impulse = newImpulse - *normalImpulse;
	*normalImpulse = newImpulse;
	*totalImpulse = *totalImpulse + impulse;
	*totalNormalImpulse = *totalNormalImpulse + newImpulse;
	float Px = impulse * c->normal.x;
	float Py = impulse * c->normal.y;
	bA->linearVelocity.x = bA->linearVelocity.x - c->invMassA * Px;
	bA->linearVelocity.y = bA->linearVelocity.y - c->invMassA * Py;
	bA->angularVelocity = bA->angularVelocity - c->invIA * ( rA.x * Py - rA.y * Px );
	bB->linearVelocity.x = bB->linearVelocity.x + c->invMassB * Px;
	bB->linearVelocity.y = bB->linearVelocity.y + c->invMassB * Py;
	bB->angularVelocity = bB->angularVelocity + c->invIB * ( rB.x * Py - rB.y * Px );
}

static inline void o_solveFrictionPoint( o_contactLane* c, o_bodyState* bA, o_bodyState* bB, b2Vec2 rA, b2Vec2 rB,
										 float tangentMass, float normalImpulse, float* tangentImpulse )
{
	float tangentX = c->normal.y;
	float tangentY = 0.0f - c->normal.x;
	float dvx = ( bB->linearVelocity.x - bB->angularVelocity * rB.y ) - ( bA->linearVelocity.x - bA->angularVelocity * rA.y );
	float dvy = ( bB->linearVelocity.y + bB->angularVelocity * rB.x ) - ( bA->linearVelocity.y + bA->angularVelocity * rA.x );
	float vt = dvx * tangentX + dvy * tangentY;
	vt = vt - c->tangentSpeed;
	float negImpulse = tangentMass * vt;
	float maxFriction = c->friction * normalImpulse;
	float newImpulse = *tangentImpulse - negImpulse;
	newImpulse = w_max( 0.0f - maxFriction, w_min( newImpulse, maxFriction ) );
	float impulse = newImpulse - *tangentImpulse;
	*tangentImpulse = newImpulse;
	float Px = impulse * tangentX;
	float Py = impulse * tangentY;
	bA->linearVelocity.x = bA->linearVelocity.x - c->invMassA * Px;
	bA->linearVelocity.y = bA->linearVelocity.y - c->invMassA * Py;
	bA->angularVelocity = bA->angularVelocity - c->invIA * ( rA.x * Py - rA.y * Px );
	bB->linearVelocity.x = bB->linearVelocity.x + c->invMassB * Px;
	bB->linearVelocity.y = bB->linearVelocity.y + c->invMassB * Py;
	bB->angularVelocity = bB->angularVelocity + c->invIB * ( rB.x * Py - rB.y * Px );
}

/* contact_solver.c:1873-2116 */
static void o_solveLane( o_world* w, o_stepContext* ctx, o_contactLane* c, int useBias )
{
	o_bodyState bA = o_gather( w, c->indexA ), bB = o_gather( w, c->indexB );
	float biasRate, massScale, impulseScale;
	if ( useBias )
	{
		biasRate = c->massScale * c->biasRate;
		massScale = c->massScale;
		impulseScale = c->impulseScale;
	}
	else
	{
		biasRate = 0.0f;
		massScale = 1.0f;
		impulseScale = 0.0f;
	}
	float inv_h = ctx->inv_h;
	float contactSpeed = -w->contactSpeed;
	float totalNormalImpulse = 0.0f;
	b2Vec2 dp = { bB.deltaPosition.x - bA.deltaPosition.x, bB.deltaPosition.y - bA.deltaPosition.y };
	o_solveNormalPoint( c, &bA, &bB, dp, c->anchorA1, c->anchorB1, c->baseSeparation1, c->normalMass1, &c->normalImpulse1,
						&c->totalNormalImpulse1, biasRate, massScale, impulseScale, inv_h, contactSpeed, &totalNormalImpulse );
	o_solveNormalPoint( c, &bA, &bB, dp, c->anchorA2, c->anchorB2, c->baseSeparation2, c->normalMass2, &c->normalImpulse2,
						&c->totalNormalImpulse2, biasRate, massScale, impulseScale, inv_h, contactSpeed, &totalNormalImpulse );
	if ( useBias == 0 )
	{
		if ( c->groupHasRolling )
		{
			float deltaLambda = c->rollingMass * ( bA.angularVelocity - bB.angularVelocity );
			float lambda = c->rollingImpulse;
			float maxLambda = c->rollingResistance * totalNormalImpulse;
			c->rollingImpulse = w_symClamp( lambda + deltaLambda, maxLambda );
			deltaLambda = c->rollingImpulse - lambda;
			bA.angularVelocity = bA.angularVelocity - c->invIA * deltaLambda;
			bB.angularVelocity = bB.angularVelocity + c->invIB * deltaLambda;
		}
		o_solveFrictionPoint( c, &bA, &bB, c->anchorA1, c->anchorB1, c->tangentMass1, c->normalImpulse1, &c->tangentImpulse1 );
		o_solveFrictionPoint( c, &bA, &bB, c->anchorA2, c->anchorB2, c->tangentMass2, c->normalImpulse2, &c->tangentImpulse2 );
	}
	o_scatter( w, c->indexA, &bA );
	o_scatter( w, c->indexB, &bB );
}

static inline void o_restitutionPoint( o_contactLane* c, o_bodyState* bA, o_bodyState* bB, b2Vec2 rA, b2Vec2 rB,
									   float relativeVelocity, float totalImpulseIn, float normalMass, float threshold,
									   float* normalImpulse, float* totalImpulse )
{
	int mask = ( relativeVelocity + threshold > 0.0f ) || ( totalImpulseIn == 0.0f ) || ( c->restitution == 0.0f );
	float mass = mask ? 0.0f : normalMass;
	float dvx = ( bB->linearVelocity.x - bB->angularVelocity * rB.y ) - ( bA->linearVelocity.x - bA->angularVelocity * rA.y );
	float dvy = ( bB->linearVelocity.y + bB->angularVelocity * rB.x ) - ( bA->linearVelocity.y + bA->angularVelocity * rA.x );
	float vn = dvx * c->normal.x + dvy * c->normal.y;
	float negImpulse = mass * ( vn + c->restitution * relativeVelocity );
	float newImpulse = w_max( *normalImpulse - negImpulse, 0.0f );
	float deltaImpulse = newImpulse - *normalImpulse;
	*normalImpulse = newImpulse;
	*totalImpulse = *totalImpulse + deltaImpulse;
	float Px = deltaImpulse * c->normal.x;
	float Py = deltaImpulse * c->normal.y;
	bA->linearVelocity.x = bA->linearVelocity.x - c->invMassA * Px;
	bA->linearVelocity.y = bA->linearVelocity.y - c->invMassA * Py;
	bA->angularVelocity = bA->angularVelocity - c->invIA * ( rA.x * Py - rA.y * Px );
	bB->linearVelocity.x = bB->linearVelocity.x + c->invMassB * Px;
	bB->linearVelocity.y = bB->linearVelocity.y + c->invMassB * Py;
	bB->angularVelocity = bB->angularVelocity + c->invIB * ( rB.x * Py - rB.y * Px );
}

/* contact_solver.c:2118-2228; a group whose four lanes all have zero restitution is skipped */
static void o_restitutionLane( o_world* w, o_contactLane* c, int groupHasRestitution )
{
	if ( groupHasRestitution == 0 ) return;
	float threshold = w->restitutionThreshold;
	o_bodyState bA = o_gather( w, c->indexA ), bB = o_gather( w, c->indexB );
	o_restitutionPoint( c, &bA, &bB, c->anchorA1, c->anchorB1, c->relativeVelocity1, c->totalNormalImpulse1, c->normalMass1,
						threshold, &c->normalImpulse1, &c->totalNormalImpulse1 );
	o_restitutionPoint( c, &bA, &bB, c->anchorA2, c->anchorB2, c->relativeVelocity2, c->totalNormalImpulse2, c->normalMass2,
						threshold, &c->normalImpulse2, &c->totalNormalImpulse2 );
	o_scatter( w, c->indexA, &bA );
	o_scatter( w, c->indexB, &bB );
}

/* contact_solver.c:2238-2331 */
static void o_storeLane( o_contactSim* cs, const o_contactLane* c )
{
	b2Manifold* m = &cs->manifold;
	m->rollingImpulse = c->rollingImpulse;
	m->points[0].normalImpulse = c->normalImpulse1;
	m->points[0].tangentImpulse = c->tangentImpulse1;
	m->points[0].totalNormalImpulse = c->totalNormalImpulse1;
	m->points[0].normalVelocity = c->relativeVelocity1;
	m->points[1].normalImpulse = c->normalImpulse2;
	m->points[1].tangentImpulse = c->tangentImpulse2;
	m->points[1].totalNormalImpulse = c->totalNormalImpulse2;
	m->points[1].normalVelocity = c->relativeVelocity2;
}

/* ---------------- overflow contacts (contact_solver.c:20-545) ---------------- */
static void o_prepareOverflow( o_world* w, o_stepContext* ctx, o_overflowConstraint* cons )
{
	o_graphColor* color = w->colors + O_OVERFLOW_INDEX;
	float warmStartScale = w->enableWarmStarting ? 1.0f : 0.0f;
	for ( int i = 0; i < color->contactSims.count; ++i )
	{
		o_contactSim* cs = color->contactSims.data + i;
		const b2Manifold* m = &cs->manifold;
		int pointCount = m->pointCount;
		int indexA = cs->bodySimIndexA, indexB = cs->bodySimIndexB;
		o_overflowConstraint* c = cons + i;
		c->indexA = indexA + 1;
		c->indexB = indexB + 1;
		c->normal = m->normal;
		c->friction = cs->friction;
		c->restitution = cs->restitution;
		c->rollingResistance = cs->rollingResistance;
		c->rollingImpulse = warmStartScale * m->rollingImpulse;
		c->tangentSpeed = cs->tangentSpeed;
		c->pointCount = pointCount;
		b2Vec2 vA = { 0.0f, 0.0f };
		float wA = 0.0f, mA = cs->invMassA, iA = cs->invIA;
		if ( indexA != B2_NULL_INDEX )
		{
			vA = w->awakeStates.data[indexA].linearVelocity;
			wA = w->awakeStates.data[indexA].angularVelocity;
		}
		b2Vec2 vB = { 0.0f, 0.0f };
		float wB = 0.0f, mB = cs->invMassB, iB = cs->invIB;
		if ( indexB != B2_NULL_INDEX )
		{
			vB = w->awakeStates.data[indexB].linearVelocity;
			wB = w->awakeStates.data[indexB].angularVelocity;
		}
		c->softness = ( indexA == B2_NULL_INDEX || indexB == B2_NULL_INDEX ) ? ctx->staticSoftness : ctx->contactSoftness;
		c->invMassA = mA;
		c->invIA = iA;
		c->invMassB = mB;
		c->invIB = iB;
		{
			float k = iA + iB;
			c->rollingMass = k > 0.0f ? 1.0f / k : 0.0f;
		}
		b2Vec2 normal = c->normal;
		b2Vec2 tangent = o_rightPerp( c->normal );
		for ( int j = 0; j < pointCount; ++j )
		{
			const b2ManifoldPoint* mp = m->points + j;
			o_overflowPoint* cp = c->points + j;
			cp->normalImpulse = warmStartScale * mp->normalImpulse;
			cp->tangentImpulse = warmStartScale * mp->tangentImpulse;
			cp->totalNormalImpulse = 0.0f;
			b2Vec2 rA = mp->anchorA, rB = mp->anchorB;
			cp->anchorA = rA;
			cp->anchorB = rB;
			cp->baseSeparation = mp->separation - o_dot( o_sub( rB, rA ), normal );
			float rnA = o_cross( rA, normal ), rnB = o_cross( rB, normal );
			float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
			cp->normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
			float rtA = o_cross( rA, tangent ), rtB = o_cross( rB, tangent );
			float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
			cp->tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
			b2Vec2 vrA = o_add( vA, o_crossSV( wA, rA ) );
			b2Vec2 vrB = o_add( vB, o_crossSV( wB, rB ) );
			cp->relativeVelocity = o_dot( normal, o_sub( vrB, vrA ) );
		}
	}
}

static void o_warmStartOverflow( o_world* w, o_overflowConstraint* cons, int count )
{
	for ( int i = 0; i < count; ++i )
	{
		o_overflowConstraint* c = cons + i;
		o_bodyState dummy = o_identityState;
		o_bodyState* sA = c->indexA == 0 ? &dummy : w->awakeStates.data + c->indexA - 1;
		o_bodyState* sB = c->indexB == 0 ? &dummy : w->awakeStates.data + c->indexB - 1;
		b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
		float wA = sA->angularVelocity, wB = sB->angularVelocity;
		float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
		b2Vec2 normal = c->normal, tangent = o_rightPerp( c->normal );
		for ( int j = 0; j < c->pointCount; ++j )
		{
			o_overflowPoint* cp = c->points + j;
			b2Vec2 P = o_add( o_mulSV( cp->normalImpulse, normal ), o_mulSV( cp->tangentImpulse, tangent ) );
			cp->totalNormalImpulse += cp->normalImpulse;
			wA -= iA * o_cross( cp->anchorA, P );
			vA = o_mulAdd( vA, -mA, P );
			wB += iB * o_cross( cp->anchorB, P );
			vB = o_mulAdd( vB, mB, P );
		}
		wA -= iA * c->rollingImpulse;
		wB += iB * c->rollingImpulse;
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
}

static void o_solveOverflow( o_world* w, o_stepContext* ctx, o_overflowConstraint* cons, int count, int useBias )
{
	float inv_h = ctx->inv_h;
	float contactSpeed = w->contactSpeed;
	for ( int i = 0; i < count; ++i )
	{
		o_overflowConstraint* c = cons + i;
		float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
		o_bodyState dummy = o_identityState;
		o_bodyState* sA = c->indexA == 0 ? &dummy : w->awakeStates.data + c->indexA - 1;
		o_bodyState* sB = c->indexB == 0 ? &dummy : w->awakeStates.data + c->indexB - 1;
		b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
		float wA = sA->angularVelocity, wB = sB->angularVelocity;
		b2Rot dqA = sA->deltaRotation, dqB = sB->deltaRotation;
		b2Vec2 dp = o_sub( sB->deltaPosition, sA->deltaPosition );
		b2Vec2 normal = c->normal, tangent = o_rightPerp( normal );
		float friction = c->friction;
		o_softness softness = c->softness;
		float totalNormalImpulse = 0.0f;
		for ( int j = 0; j < c->pointCount; ++j )
		{
			o_overflowPoint* cp = c->points + j;
			b2Vec2 rA = cp->anchorA, rB = cp->anchorB;
			b2Vec2 ds = o_add( dp, o_sub( o_rotate( dqB, rB ), o_rotate( dqA, rA ) ) );
			float s = cp->baseSeparation + o_dot( ds, normal );
			float velocityBias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( s > 0.0f ) velocityBias = s * inv_h;
			else if ( useBias )
			{
				velocityBias = o_max( softness.massScale * softness.biasRate * s, -contactSpeed );
				massScale = softness.massScale;
				impulseScale = softness.impulseScale;
			}
			b2Vec2 vrA = o_add( vA, o_crossSV( wA, rA ) );
			b2Vec2 vrB = o_add( vB, o_crossSV( wB, rB ) );
			float vn = o_dot( o_sub( vrB, vrA ), normal );
			float impulse = -cp->normalMass * ( massScale * vn + velocityBias ) - impulseScale * cp->normalImpulse;
			float newImpulse = o_max( cp->normalImpulse + impulse, 0.0f );
			impulse = newImpulse - cp->normalImpulse;
			cp->normalImpulse = newImpulse;
			cp->totalNormalImpulse += impulse;
			totalNormalImpulse += newImpulse;
			b2Vec2 P = o_mulSV( impulse, normal );
			vA = o_mulSub( vA, mA, P );
			wA -= iA * o_cross( rA, P );
			vB = o_mulAdd( vB, mB, P );
			wB += iB * o_cross( rB, P );
		}
		if ( useBias == 0 )
		{
			for ( int j = 0; j < c->pointCount; ++j )
			{
				o_overflowPoint* cp = c->points + j;
				b2Vec2 rA = cp->anchorA, rB = cp->anchorB;
				b2Vec2 vrB = o_add( vB, o_crossSV( wB, rB ) );
				b2Vec2 vrA = o_add( vA, o_crossSV( wA, rA ) );
				float vt = o_dot( o_sub( vrB, vrA ), tangent ) - c->tangentSpeed;
				float impulse = cp->tangentMass * ( -vt );
				float maxFriction = friction * cp->normalImpulse;
				float newImpulse = o_clamp( cp->tangentImpulse + impulse, -maxFriction, maxFriction );
				impulse = newImpulse - cp->tangentImpulse;
				cp->tangentImpulse = newImpulse;
				b2Vec2 P = o_mulSV( impulse, tangent );
				vA = o_mulSub( vA, mA, P );
				wA -= iA * o_cross( rA, P );
				vB = o_mulAdd( vB, mB, P );
				wB += iB * o_cross( rB, P );
			}
			{
				float deltaLambda = -c->rollingMass * ( wB - wA );
				float lambda = c->rollingImpulse;
				float maxLambda = c->rollingResistance * totalNormalImpulse;
				c->rollingImpulse = o_clamp( lambda + deltaLambda, -maxLambda, maxLambda );
				deltaLambda = c->rollingImpulse - lambda;
				wA -= iA * deltaLambda;
				wB += iB * deltaLambda;
			}
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
}

static void o_restitutionOverflow( o_world* w, o_overflowConstraint* cons, int count )
{
	float threshold = w->restitutionThreshold;
	for ( int i = 0; i < count; ++i )
	{
		o_overflowConstraint* c = cons + i;
		float restitution = c->restitution;
		if ( restitution == 0.0f ) continue;
		float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
		o_bodyState dummy = o_identityState;
		o_bodyState* sA = c->indexA == 0 ? &dummy : w->awakeStates.data + c->indexA - 1;
		o_bodyState* sB = c->indexB == 0 ? &dummy : w->awakeStates.data + c->indexB - 1;
		b2Vec2 vA = sA->linearVelocity, vB = sB->linearVelocity;
		float wA = sA->angularVelocity, wB = sB->angularVelocity;
		b2Vec2 normal = c->normal;
		for ( int j = 0; j < c->pointCount; ++j )
		{
			o_overflowPoint* cp = c->points + j;
			if ( cp->relativeVelocity > -threshold || cp->totalNormalImpulse == 0.0f ) continue;
			b2Vec2 rA = cp->anchorA, rB = cp->anchorB;
			b2Vec2 vrB = o_add( vB, o_crossSV( wB, rB ) );
			b2Vec2 vrA = o_add( vA, o_crossSV( wA, rA ) );
			float vn = o_dot( o_sub( vrB, vrA ), normal );
			float impulse = -cp->normalMass * ( vn + restitution * cp->relativeVelocity );
			float newImpulse = o_max( cp->normalImpulse + impulse, 0.0f );
			impulse = newImpulse - cp->normalImpulse;
			cp->normalImpulse = newImpulse;
			cp->totalNormalImpulse += impulse;
			b2Vec2 P = o_mulSV( impulse, normal );
			vA = o_mulSub( vA, mA, P );
			wA -= iA * o_cross( rA, P );
			vB = o_mulAdd( vB, mB, P );
			wB += iB * o_cross( rB, P );
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
}

static void o_storeOverflow( o_world* w, o_overflowConstraint* cons )
{
	o_graphColor* color = w->colors + O_OVERFLOW_INDEX;
	for ( int i = 0; i < color->contactSims.count; ++i )
	{
		const o_overflowConstraint* c = cons + i;
		b2Manifold* m = &color->contactSims.data[i].manifold;
		for ( int j = 0; j < m->pointCount; ++j )
		{
			m->points[j].normalImpulse = c->points[j].normalImpulse;
			m->points[j].tangentImpulse = c->points[j].tangentImpulse;
			m->points[j].totalNormalImpulse = c->points[j].totalNormalImpulse;
			m->points[j].normalVelocity = c->points[j].relativeVelocity;
		}
		m->rollingImpulse = c->rollingImpulse;
	}
}

/* ---------------- body integration (solver.c:66-162) ---------------- */
typedef struct o_loopCtx
{
	o_world* w;
	o_stepContext* ctx;
	o_graphColor* color;
	o_contactLane* lanes;
	int* groupRestitution;
	int jointCount;
	int stage; /* 0 warm start, 1 solve, 2 relax */
	const int* prefix;
} o_loopCtx;

#define O_MIN_PARALLEL 256

static void o_integrateVelocitiesRange( void* p, int begin, int end )
{
	o_world* w = ( (o_loopCtx*)p )->w;
	o_stepContext* ctx = ( (o_loopCtx*)p )->ctx;
	b2Vec2 gravity = w->gravity;
	float h = ctx->h;
	for ( int i = begin; i < end; ++i )
	{
		o_bodySim* sim = w->awakeSims.data + i;
		o_bodyState* st = w->awakeStates.data + i;
		b2Vec2 v = st->linearVelocity;
		float av = st->angularVelocity;
		float linearDamping = 1.0f / ( 1.0f + h * sim->linearDamping );
		float angularDamping = 1.0f / ( 1.0f + h * sim->angularDamping );
		float gravityScale = sim->invMass > 0.0f ? sim->gravityScale : 0.0f;
		b2Vec2 lvd = o_add( o_mulSV( h * sim->invMass, sim->force ), o_mulSV( h * gravityScale, gravity ) );
		float avd = h * sim->invInertia * sim->torque;
		v = o_mulAdd( lvd, linearDamping, v );
		av = avd + angularDamping * av;
		st->linearVelocity = v;
		st->angularVelocity = av;
	}
}

static void o_integrateVelocities( o_world* w, o_stepContext* ctx )
{
	o_loopCtx c = { w, ctx, NULL, NULL, NULL, 0, 0, NULL };
	o_parallelFor( w->awakeSims.count, O_MIN_PARALLEL, o_integrateVelocitiesRange, &c );
}

static void o_integratePositionsRange( void* p, int begin, int end )
{
	o_world* w = ( (o_loopCtx*)p )->w;
	o_stepContext* ctx = ( (o_loopCtx*)p )->ctx;
	float h = ctx->h;
	float maxLinearSpeed = ctx->maxLinearVelocity;
	float maxAngularSpeed = O_MAX_ROTATION * ctx->inv_dt;
	float maxLinearSq = maxLinearSpeed * maxLinearSpeed;
	float maxAngularSq = maxAngularSpeed * maxAngularSpeed;
	for ( int i = begin; i < end; ++i )
	{
		o_bodyState* st = w->awakeStates.data + i;
		b2Vec2 v = st->linearVelocity;
		float av = st->angularVelocity;
		v.x = ( st->flags & O_LOCK_X ) ? 0.0f : v.x;
		v.y = ( st->flags & O_LOCK_Y ) ? 0.0f : v.y;
		av = ( st->flags & O_LOCK_Z ) ? 0.0f : av;
		if ( o_dot( v, v ) > maxLinearSq )
		{
			float ratio = maxLinearSpeed / o_length( v );
			v = o_mulSV( ratio, v );
			st->flags |= O_SPEED_CAPPED;
		}
		if ( av * av > maxAngularSq && ( st->flags & O_ALLOW_FAST_ROTATION ) == 0 )
		{
			float ratio = maxAngularSpeed / o_abs( av );
			av *= ratio;
			st->flags |= O_SPEED_CAPPED;
		}
		st->linearVelocity = v;
		st->angularVelocity = av;
		st->deltaPosition = o_mulAdd( st->deltaPosition, h, st->linearVelocity );
		st->deltaRotation = o_integrateRotation( st->deltaRotation, h * st->angularVelocity );
	}
}

static void o_integratePositions( o_world* w, o_stepContext* ctx )
{
	o_loopCtx c = { w, ctx, NULL, NULL, NULL, 0, 0, NULL };
	o_parallelFor( w->awakeStates.count, O_MIN_PARALLEL, o_integratePositionsRange, &c );
}

/* ---------------- finalize bodies (solver.c:553-743) ---------------- */
void o_solveContinuous( o_world* w, int simIndex );
extern int o_continuousSkipped;

static void o_finalizeRange( void* p, int begin, int end )
{
	o_world* w = ( (o_loopCtx*)p )->w;
	o_stepContext* ctx = ( (o_loopCtx*)p )->ctx;
	float timeStep = ctx->dt, invTimeStep = ctx->inv_dt;
	for ( int simIndex = begin; simIndex < end; ++simIndex )
	{
		o_bodyState* st = w->awakeStates.data + simIndex;
		o_bodySim* sim = w->awakeSims.data + simIndex;
		b2Vec2 v = st->linearVelocity;
		float av = st->angularVelocity;
		sim->center = o_add( sim->center, st->deltaPosition );
		sim->transform.q = o_normalizeRot( o_mulRot( st->deltaRotation, sim->transform.q ) );
		float maxVelocity = o_length( v ) + o_abs( av ) * sim->maxExtent;
		float maxDeltaPosition = o_length( st->deltaPosition ) + o_abs( st->deltaRotation.s ) * sim->maxExtent;
		float positionSleepFactor = 0.5f;
		float sleepVelocity = o_max( maxVelocity, positionSleepFactor * invTimeStep * maxDeltaPosition );
		st->deltaPosition = o_v( 0.0f, 0.0f );
		st->deltaRotation.c = 1.0f;
		st->deltaRotation.s = 0.0f;
		sim->transform.p = o_add( sim->center, o_neg( o_rotate( sim->transform.q, sim->localCenter ) ) );
		o_body* body = w->bodies.data + sim->bodyId;
		b2BodyMoveEvent* ev = w->moveEvents.data + simIndex;
		ev->transform = sim->transform;
		ev->bodyId.index1 = sim->bodyId + 1;
		ev->bodyId.world0 = w->worldId;
		ev->bodyId.generation = body->generation;
		ev->userData = body->userData;
		ev->fellAsleep = false;
		sim->force = o_v( 0.0f, 0.0f );
		sim->torque = 0.0f;
		body->flags &= ~O_TRANSIENT;
		body->flags |= ( sim->flags & ( O_SPEED_CAPPED | O_HAD_TOI ) );
		body->flags |= ( st->flags & ( O_SPEED_CAPPED | O_HAD_TOI ) );
		sim->flags &= ~O_TRANSIENT;
		st->flags &= ~O_TRANSIENT;
		if ( w->enableSleep == 0 || ( body->flags & O_ENABLE_SLEEP ) == 0 || sleepVelocity > body->sleepThreshold )
		{
			body->sleepTime = 0.0f;
			float maxMotion = o_max( maxDeltaPosition, maxVelocity * timeStep );
			if ( body->type == b2_dynamicBody && w->enableContinuous && maxMotion > body->safetyFactor * sim->minExtent )
			{
				body->flags |= O_IS_FAST;
				if ( sim->flags & O_IS_BULLET )
				{
					/* bullets are continuous against every body; not part of the GPU path */
					sim->center0 = sim->center;
					sim->rotation0 = sim->transform.q;
					__atomic_fetch_add( &o_continuousSkipped, 1, __ATOMIC_RELAXED );
				}
				else
				{
					o_solveContinuous( w, simIndex );
				}
			}
			else
			{
				sim->center0 = sim->center;
				sim->rotation0 = sim->transform.q;
			}
		}
		else
		{
			sim->center0 = sim->center;
			sim->rotation0 = sim->transform.q;
			body->sleepTime += timeStep;
		}
		b2Transform transform = sim->transform;
		int isFast = ( body->flags & O_IS_FAST ) != 0;
		int shapeId = body->headShapeId;
		while ( shapeId != B2_NULL_INDEX )
		{
			o_shape* shape = w->shapes.data + shapeId;
			if ( isFast )
			{
				o_bitSet1Atomic( &w->enlargedSimBits, simIndex );
			}
			else
			{
				b2AABB aabb = o_computeFatShapeAABB( shape, transform, O_SPECULATIVE_DISTANCE );
				shape->aabb = aabb;
				if ( o_aabbContains( shape->fatAABB, aabb ) == 0 )
				{
					float margin = shape->aabbMargin;
					b2AABB fat = { { aabb.lowerBound.x - margin, aabb.lowerBound.y - margin },
								   { aabb.upperBound.x + margin, aabb.upperBound.y + margin } };
					shape->fatAABB = fat;
					shape->enlargedAABB = 1;
					o_bitSet1Atomic( &w->enlargedSimBits, simIndex );
				}
			}
			shapeId = shape->nextShapeId;
		}
	}
}

static void o_finalizeBodies( o_world* w, o_stepContext* ctx )
{
	int n = w->awakeSims.count;
	o_bitReset( &w->enlargedSimBits, n );
	o_loopCtx c = { w, ctx, NULL, NULL, NULL, 0, 0, NULL };
	o_parallelFor( n, O_MIN_PARALLEL, o_finalizeRange, &c );
}

/* per-color loops of the solver stages (one item = one joint or one contact lane) */
static void o_prepareJointRange( void* p, int begin, int end )
{
	o_loopCtx* c = p;
	for ( int j = begin; j < end; ++j ) o_prepareJoint( c->w, c->ctx, c->color->jointSims.data + j );
}

static void o_prepareLaneRange( void* p, int begin, int end )
{
	o_loopCtx* c = p;
	for ( int k = begin; k < end; ++k ) o_prepareLane( c->w, c->ctx, c->color->contactSims.data + k, c->lanes + k );
}

static void o_colorStageRange( void* p, int begin, int end )
{
	o_loopCtx* c = p;
	for ( int i = begin; i < end; ++i )
	{
		if ( i < c->jointCount )
		{
			o_jointSim* j = c->color->jointSims.data + i;
			if ( c->stage == 0 ) o_warmStartJoint( c->w, c->ctx, j );
			else o_solveJoint( c->w, c->ctx, j, c->stage == 1 );
		}
		else
		{
			o_contactLane* lane = c->lanes + ( i - c->jointCount );
			if ( c->stage == 0 ) o_warmStartLane( c->w, lane );
			else o_solveLane( c->w, c->ctx, lane, c->stage == 1 );
		}
	}
}

static void o_restitutionRange( void* p, int begin, int end )
{
	o_loopCtx* c = p;
	for ( int k = begin; k < end; ++k ) o_restitutionLane( c->w, c->lanes + k, c->groupRestitution[k / O_SIMD_WIDTH] );
}

static void o_storeRange( void* p, int begin, int end )
{
	o_loopCtx* c = p;
	for ( int k = begin; k < end; ++k ) o_storeLane( c->color->contactSims.data + k, c->lanes + k );
}

/* ---------------- b2Solve (solver.c:1275-2081) ---------------- */
typedef O_ARRAY( o_contactLane ) o_laneArray;

void o_solve( o_world* w, o_stepContext* ctx )
{
	w->stepIndex += 1;
	int awakeBodyCount = w->awakeSims.count;
	if ( awakeBodyCount == 0 ) return;

	/* active colors */
	int activeColors[B2_GRAPH_COLOR_COUNT];
	int activeColorCount = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT - 1; ++i )
	{
		if ( w->colors[i].contactSims.count + w->colors[i].jointSims.count > 0 ) activeColors[activeColorCount++] = i;
	}
	o_reserve( w->moveEvents, awakeBodyCount );
	w->moveEvents.count = awakeBodyCount;

	/* per color lanes */
	o_contactLane* lanes[B2_GRAPH_COLOR_COUNT];
	int laneCounts[B2_GRAPH_COLOR_COUNT];
	int* groupRestitution[B2_GRAPH_COLOR_COUNT];
	for ( int a = 0; a < activeColorCount; ++a )
	{
		o_graphColor* color = w->colors + activeColors[a];
		int n = color->contactSims.count;
		laneCounts[a] = n;
		lanes[a] = calloc( (size_t)( n > 0 ? n : 1 ), sizeof( o_contactLane ) );
		int groups = ( n + O_SIMD_WIDTH - 1 ) / O_SIMD_WIDTH;
		groupRestitution[a] = calloc( (size_t)( groups > 0 ? groups : 1 ), sizeof( int ) );
	}

	/* prepare joints (joint.c:1593-1629) then contacts */
	for ( int a = 0; a < activeColorCount; ++a )
	{
		o_graphColor* color = w->colors + activeColors[a];
		o_loopCtx c = { w, ctx, color, lanes[a], groupRestitution[a], 0, 0, NULL };
		o_parallelFor( color->jointSims.count, O_MIN_PARALLEL, o_prepareJointRange, &c );
	}
	for ( int a = 0; a < activeColorCount; ++a )
	{
		o_graphColor* color = w->colors + activeColors[a];
		int n = laneCounts[a];
		o_loopCtx c = { w, ctx, color, lanes[a], groupRestitution[a], 0, 0, NULL };
		o_parallelFor( n, O_MIN_PARALLEL, o_prepareLaneRange, &c );
		for ( int g = 0; g * O_SIMD_WIDTH < n; ++g )
		{
			int anyRolling = 0, anyRestitution = 0;
			for ( int k = g * O_SIMD_WIDTH; k < n && k < ( g + 1 ) * O_SIMD_WIDTH; ++k )
			{
				anyRolling |= lanes[a][k].rollingResistance != 0.0f;
				anyRestitution |= lanes[a][k].restitution != 0.0f;
			}
			for ( int k = g * O_SIMD_WIDTH; k < n && k < ( g + 1 ) * O_SIMD_WIDTH; ++k ) lanes[a][k].groupHasRolling = anyRolling;
			groupRestitution[a][g] = anyRestitution;
		}
	}
	o_graphColor* overflow = w->colors + O_OVERFLOW_INDEX;
	int overflowCount = overflow->contactSims.count;
	o_overflowConstraint* ocons = calloc( (size_t)( overflowCount > 0 ? overflowCount : 1 ), sizeof( o_overflowConstraint ) );
	for ( int j = 0; j < overflow->jointSims.count; ++j ) o_prepareJoint( w, ctx, overflow->jointSims.data + j );
	o_prepareOverflow( w, ctx, ocons );

	for ( int sub = 0; sub < ctx->subStepCount; ++sub )
	{
		o_integrateVelocities( w, ctx );
		for ( int j = 0; j < overflow->jointSims.count; ++j ) o_warmStartJoint( w, ctx, overflow->jointSims.data + j );
		o_warmStartOverflow( w, ocons, overflowCount );
		for ( int a = 0; a < activeColorCount; ++a )
		{
			o_graphColor* color = w->colors + activeColors[a];
			o_loopCtx c = { w, ctx, color, lanes[a], groupRestitution[a], color->jointSims.count, 0, NULL };
			o_parallelFor( color->jointSims.count + laneCounts[a], O_MIN_PARALLEL, o_colorStageRange, &c );
		}
		for ( int j = 0; j < overflow->jointSims.count; ++j ) o_solveJoint( w, ctx, overflow->jointSims.data + j, 1 );
		o_solveOverflow( w, ctx, ocons, overflowCount, 1 );
		for ( int a = 0; a < activeColorCount; ++a )
		{
			o_graphColor* color = w->colors + activeColors[a];
			o_loopCtx c = { w, ctx, color, lanes[a], groupRestitution[a], color->jointSims.count, 1, NULL };
			o_parallelFor( color->jointSims.count + laneCounts[a], O_MIN_PARALLEL, o_colorStageRange, &c );
		}
		o_integratePositions( w, ctx );
		for ( int j = 0; j < overflow->jointSims.count; ++j ) o_solveJoint( w, ctx, overflow->jointSims.data + j, 0 );
		o_solveOverflow( w, ctx, ocons, overflowCount, 0 );
		for ( int a = 0; a < activeColorCount; ++a )
		{
			o_graphColor* color = w->colors + activeColors[a];
			o_loopCtx c = { w, ctx, color, lanes[a], groupRestitution[a], color->jointSims.count, 2, NULL };
			o_parallelFor( color->jointSims.count + laneCounts[a], O_MIN_PARALLEL, o_colorStageRange, &c );
		}
	}

	o_restitutionOverflow( w, ocons, overflowCount );
	for ( int a = 0; a < activeColorCount; ++a )
	{
		o_loopCtx c = { w, ctx, w->colors + activeColors[a], lanes[a], groupRestitution[a], 0, 0, NULL };
		o_parallelFor( laneCounts[a], O_MIN_PARALLEL, o_restitutionRange, &c );
	}
	o_storeOverflow( w, ocons );
	for ( int a = 0; a < activeColorCount; ++a )
	{
		o_graphColor* color = w->colors + activeColors[a];
		o_loopCtx c = { w, ctx, color, lanes[a], groupRestitution[a], 0, 0, NULL };
		o_parallelFor( laneCounts[a], O_MIN_PARALLEL, o_storeRange, &c );
		free( lanes[a] );
		free( groupRestitution[a] );
	}
	free( ocons );

	o_finalizeBodies( w, ctx );

	/* enlarge proxies and build the next move array (solver.c:1822-1915) */
	for ( int k = 0; k < w->enlargedSimBits.blockCount; ++k )
	{
		uint64_t word = w->enlargedSimBits.bits[k];
		while ( word != 0 )
		{
			int ctz = __builtin_ctzll( word );
			int simIndex = 64 * k + ctz;
			o_bodySim* sim = w->awakeSims.data + simIndex;
			o_body* body = w->bodies.data + sim->bodyId;
			int shapeId = body->headShapeId;
			if ( ( body->flags & ( O_IS_BULLET | O_IS_FAST ) ) == ( O_IS_BULLET | O_IS_FAST ) )
			{
				while ( shapeId != B2_NULL_INDEX )
				{
					o_shape* s = w->shapes.data + shapeId;
					o_bufferMove( w, s->proxyKey );
					shapeId = s->nextShapeId;
				}
			}
			else
			{
				while ( shapeId != B2_NULL_INDEX )
				{
					o_shape* s = w->shapes.data + shapeId;
					if ( s->enlargedAABB )
					{
						o_treeEnlargeProxy( w->trees + O_PROXY_TYPE( s->proxyKey ), O_PROXY_ID( s->proxyKey ), s->fatAABB );
						o_bufferMove( w, s->proxyKey );
						s->enlargedAABB = 0;
					}
					shapeId = s->nextShapeId;
				}
			}
			word = word & ( word - 1 );
		}
	}
}

/* ---------------- narrowphase (physics_world.c:451-836, contact.c:519-698) ---------------- */
static int o_updateContact( o_world* w, o_contactSim* cs, o_shape* shapeA, b2Transform xfA, b2Vec2 centerOffsetA,
							o_shape* shapeB, b2Transform xfB, b2Vec2 centerOffsetB )
{
	b2Manifold oldManifold = cs->manifold;
	b2Transform rel = o_invMulTransforms( xfA, xfB );
	b2LocalManifold local = o_collideShapes( shapeA, shapeB, rel );
	memset( &cs->manifold, 0, sizeof( cs->manifold ) );
	cs->manifold.normal = o_rotate( xfA.q, local.normal );
	cs->manifold.pointCount = local.pointCount;
	b2Vec2 originDelta = { xfA.p.x - xfB.p.x, xfA.p.y - xfB.p.y };
	for ( int i = 0; i < local.pointCount; ++i )
	{
		b2ManifoldPoint* mp = cs->manifold.points + i;
		mp->anchorA = o_rotate( xfA.q, local.points[i].point );
		mp->anchorB = o_add( mp->anchorA, originDelta );
		mp->separation = local.points[i].separation;
		mp->id = local.points[i].id;
	}
	cs->friction = sqrtf( shapeA->material.friction * shapeB->material.friction );
	cs->restitution = o_max( shapeA->material.restitution, shapeB->material.restitution );
	if ( shapeA->material.rollingResistance > 0.0f || shapeB->material.rollingResistance > 0.0f )
	{
		float maxRadius = o_max( o_shapeRadius( shapeA ), o_shapeRadius( shapeB ) );
		cs->rollingResistance = o_max( shapeA->material.rollingResistance, shapeB->material.rollingResistance ) * maxRadius;
	}
	else
	{
		cs->rollingResistance = 0.0f;
	}
	cs->tangentSpeed = shapeA->material.tangentSpeed + shapeB->material.tangentSpeed;
	int pointCount = cs->manifold.pointCount;
	int touching = pointCount > 0;
	if ( touching && ( shapeA->enableHitEvents || shapeB->enableHitEvents ) ) cs->simFlags |= O_S_HIT_EVENT;
	else cs->simFlags &= ~O_S_HIT_EVENT;
	if ( pointCount > 0 ) cs->manifold.rollingImpulse = oldManifold.rollingImpulse;
	for ( int i = 0; i < pointCount; ++i )
	{
		b2ManifoldPoint* mp2 = cs->manifold.points + i;
		mp2->anchorA = o_sub( mp2->anchorA, centerOffsetA );
		mp2->anchorB = o_sub( mp2->anchorB, centerOffsetB );
		mp2->normalImpulse = 0.0f;
		mp2->tangentImpulse = 0.0f;
		mp2->totalNormalImpulse = 0.0f;
		mp2->normalVelocity = 0.0f;
		mp2->persisted = false;
		uint16_t id2 = mp2->id;
		for ( int j = 0; j < oldManifold.pointCount; ++j )
		{
			b2ManifoldPoint* mp1 = oldManifold.points + j;
			if ( mp1->id == id2 )
			{
				mp2->normalImpulse = mp1->normalImpulse;
				mp2->tangentImpulse = mp1->tangentImpulse;
				mp2->persisted = true;
				mp1->normalImpulse = 0.0f;
				mp1->tangentImpulse = 0.0f;
				break;
			}
		}
	}
	if ( touching ) cs->simFlags |= O_S_TOUCHING;
	else cs->simFlags &= ~O_S_TOUCHING;
	return touching;
}

static o_bodySim* o_simOf( o_world* w, o_body* b )
{
	return b->setIndex == O_AWAKE_SET ? w->awakeSims.data + b->localIndex : w->staticSims.data + b->localIndex;
}

static void o_collideContact( o_world* w, o_contactSim* cs )
{
	float recycleDistance = w->contactRecycleDistance;
	float recycleNonTouching = o_min( recycleDistance, O_SPECULATIVE_DISTANCE );
	int contactId = cs->contactId;
	o_shape* shapeA = w->shapes.data + cs->shapeIdA;
	o_shape* shapeB = w->shapes.data + cs->shapeIdB;
	if ( o_aabbOverlaps( shapeA->fatAABB, shapeB->fatAABB ) == 0 )
	{
		cs->simFlags |= O_S_DISJOINT;
		cs->simFlags &= ~O_S_TOUCHING;
		o_bitSet1Atomic( &w->contactStateBits, contactId );
		return;
	}
	int wasTouching = ( cs->simFlags & O_S_TOUCHING ) != 0;
	o_body* bodyA = w->bodies.data + shapeA->bodyId;
	o_body* bodyB = w->bodies.data + shapeB->bodyId;
	o_bodySim* simA = o_simOf( w, bodyA );
	o_bodySim* simB = o_simOf( w, bodyB );
	b2Transform xfA = simA->transform, xfB = simB->transform;
	cs->bodySimIndexA = bodyA->setIndex == O_AWAKE_SET ? bodyA->localIndex : B2_NULL_INDEX;
	cs->invMassA = simA->invMass;
	cs->invIA = simA->invInertia;
	cs->bodySimIndexB = bodyB->setIndex == O_AWAKE_SET ? bodyB->localIndex : B2_NULL_INDEX;
	cs->invMassB = simB->invMass;
	cs->invIB = simB->invInertia;
	int isFast = ( bodyA->flags & O_IS_FAST ) || ( bodyB->flags & O_IS_FAST );
	if ( isFast == 0 && recycleDistance > 0.0f && ( cs->simFlags & O_S_RELATIVE_VALID ) && ( cs->simFlags & O_C_RECYCLE ) )
	{
		b2Rot cachedQA = cs->cachedRotationA, cachedQB = cs->cachedRotationB;
		b2Transform xfc = cs->cachedRelativePose;
		b2Transform xf = o_invMulTransforms( xfA, xfB );
		float cosA = o_relativeCos( xfA.q, cachedQA );
		float cosB = o_relativeCos( xfB.q, cachedQB );
		float minCos = o_min( cosA, cosB );
		float maxExtentA = bodyA->type == b2_staticBody ? 0.0f : simA->maxExtent;
		float maxExtentB = bodyB->type == b2_staticBody ? 0.0f : simB->maxExtent;
		float maxExtent = o_max( maxExtentA, maxExtentB );
		float distance = o_distance( xf.p, xfc.p );
		b2Rot qr = o_invMulRot( xf.q, xfc.q );
		float tolerance = wasTouching ? recycleDistance : recycleNonTouching;
		if ( minCos > O_CONTACT_RECYCLE_COS_ANGLE && distance + maxExtent * o_abs( qr.s ) < tolerance )
		{
			b2Rot dqA = o_mulRot( xfA.q, o_invertRot( cachedQA ) );
			b2Rot dqB = o_mulRot( xfB.q, o_invertRot( cachedQB ) );
			b2Vec2 normal = cs->manifold.normal;
			b2Vec2 dc = { simB->center.x - simA->center.x, simB->center.y - simA->center.y };
			for ( int i = 0; i < cs->manifold.pointCount; ++i )
			{
				b2ManifoldPoint* mp = cs->manifold.points + i;
				b2Vec2 rA = o_rotate( dqA, mp->anchorA );
				b2Vec2 rB = o_rotate( dqB, mp->anchorB );
				b2Vec2 dp = o_add( dc, o_sub( rB, rA ) );
				mp->separation = mp->baseSeparation + o_dot( dp, normal );
				mp->persisted = true;
			}
			__atomic_fetch_add( &w->recycledContactCount, 1, __ATOMIC_RELAXED );
			return;
		}
	}
	cs->cachedRotationA = xfA.q;
	cs->cachedRotationB = xfB.q;
	cs->cachedRelativePose = o_invMulTransforms( xfA, xfB );
	cs->simFlags |= O_S_RELATIVE_VALID;
	b2Vec2 centerOffsetA = o_rotate( xfA.q, simA->localCenter );
	b2Vec2 centerOffsetB = o_rotate( xfB.q, simB->localCenter );
	int touching = o_updateContact( w, cs, shapeA, xfA, centerOffsetA, shapeB, xfB, centerOffsetB );
	if ( touching && wasTouching == 0 )
	{
		cs->simFlags |= O_S_STARTED;
		o_bitSet1Atomic( &w->contactStateBits, contactId );
	}
	else if ( touching == 0 && wasTouching )
	{
		cs->simFlags |= O_S_STOPPED;
		o_bitSet1Atomic( &w->contactStateBits, contactId );
	}
	for ( int i = 0; i < cs->manifold.pointCount; ++i ) cs->manifold.points[i].baseSeparation = cs->manifold.points[i].separation;
}

static void o_collideRange( void* p, int begin, int end )
{
	o_loopCtx* c = p;
	o_world* w = c->w;
	int array = 0;
	for ( int i = begin; i < end; ++i )
	{
		while ( c->prefix[array + 1] <= i ) array += 1;
		int j = i - c->prefix[array];
		o_contactSim* cs = array < B2_GRAPH_COLOR_COUNT ? w->colors[array].contactSims.data + j : w->awakeContactSims.data + j;
		o_collideContact( w, cs );
	}
}

void o_collide( o_world* w, o_stepContext* ctx )
{
	(void)ctx;
	int contactCount = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i ) contactCount += w->colors[i].contactSims.count;
	contactCount += w->awakeContactSims.count;
	if ( contactCount == 0 ) return;
	o_bitReset( &w->contactStateBits, w->contactIdPool.nextIndex );
	w->recycledContactCount = 0;
	/* every color's contacts, then the non-touching ones, as one index space */
	int prefix[B2_GRAPH_COLOR_COUNT + 2];
	prefix[0] = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i ) prefix[i + 1] = prefix[i] + w->colors[i].contactSims.count;
	prefix[B2_GRAPH_COLOR_COUNT + 1] = prefix[B2_GRAPH_COLOR_COUNT] + w->awakeContactSims.count;
	o_loopCtx c = { w, ctx, NULL, NULL, NULL, 0, 0, prefix };
	o_parallelFor( prefix[B2_GRAPH_COLOR_COUNT + 1], O_MIN_PARALLEL, o_collideRange, &c );

	int endEventArrayIndex = w->endEventArrayIndex;
	for ( int k = 0; k < w->contactStateBits.blockCount; ++k )
	{
		uint64_t bits = w->contactStateBits.bits[k];
		while ( bits != 0 )
		{
			int ctz = __builtin_ctzll( bits );
			int contactId = 64 * k + ctz;
			o_contact* contact = w->contacts.data + contactId;
			int colorIndex = contact->colorIndex;
			int localIndex = contact->localIndex;
			o_contactSim* cs =
				colorIndex != B2_NULL_INDEX ? w->colors[colorIndex].contactSims.data + localIndex : w->awakeContactSims.data + localIndex;
			const o_shape* shapeA = w->shapes.data + contact->shapeIdA;
			const o_shape* shapeB = w->shapes.data + contact->shapeIdB;
			b2ShapeId shapeIdA = { shapeA->id + 1, w->worldId, shapeA->generation };
			b2ShapeId shapeIdB = { shapeB->id + 1, w->worldId, shapeB->generation };
			b2ContactId fullId;
			fullId.index1 = contactId + 1;
			fullId.world0 = w->worldId;
			fullId.padding = 0;
			fullId.generation = contact->generation;
			uint32_t flags = contact->flags;
			uint32_t simFlags = cs->simFlags;
			if ( simFlags & O_S_DISJOINT )
			{
				o_destroyContact( w, contact );
			}
			else if ( simFlags & O_S_STARTED )
			{
				if ( flags & O_C_ENABLE_EVENTS )
				{
					b2ContactBeginTouchEvent ev = { shapeIdA, shapeIdB, fullId };
					o_push( w->beginEvents, ev );
				}
				contact->flags |= O_C_TOUCHING;
				cs->simFlags &= ~O_S_STARTED;
				o_addContactToGraph( w, cs, contact );
				/* b2RemoveNonTouchingContact */
				int moved = o_removeSwap( w->awakeContactSims, localIndex );
				if ( moved != B2_NULL_INDEX )
					w->contacts.data[w->awakeContactSims.data[localIndex].contactId].localIndex = localIndex;
			}
			else if ( simFlags & O_S_STOPPED )
			{
				cs->simFlags &= ~O_S_STOPPED;
				contact->flags &= ~O_C_TOUCHING;
				if ( contact->flags & O_C_ENABLE_EVENTS )
				{
					b2ContactEndTouchEvent ev = { shapeIdA, shapeIdB, fullId };
					o_push( w->endEvents[endEventArrayIndex], ev );
				}
				int bodyIdA = contact->edges[0].bodyId, bodyIdB = contact->edges[1].bodyId;
				/* b2AddNonTouchingContact then b2RemoveContactFromGraph */
				contact->colorIndex = B2_NULL_INDEX;
				contact->localIndex = w->awakeContactSims.count;
				o_contactSim copy = *cs;
				o_push( w->awakeContactSims, copy );
				o_removeContactFromGraph( w, bodyIdA, bodyIdB, colorIndex, localIndex );
			}
			bits = bits & ( bits - 1 );
		}
	}
}

/* ---------------- b2World_Step (physics_world.c:845-1005) ---------------- */
void b2World_Step( b2WorldId worldId, float timeStep, int subStepCount )
{
	o_world* w = o_worldFromId( worldId );
	if ( w == NULL || w->locked ) return;
	w->moveEvents.count = 0;
	w->beginEvents.count = 0;
	memset( &w->profile, 0, sizeof( w->profile ) );
	w->locked = 1;
	uint64_t stepTicks = b2GetTicks();
	uint64_t t0 = b2GetTicks();
	o_updateBroadPhasePairs( w );
	w->profile.pairs = b2GetMilliseconds( t0 );
	o_stepContext ctx;
	memset( &ctx, 0, sizeof( ctx ) );
	ctx.dt = timeStep;
	ctx.subStepCount = o_maxi( 1, subStepCount );
	if ( timeStep > 0.0f )
	{
		ctx.inv_dt = 1.0f / timeStep;
		ctx.h = timeStep / ctx.subStepCount;
		ctx.inv_h = ctx.subStepCount * ctx.inv_dt;
	}
	float contactHertz = o_min( w->contactHertz, 0.125f * ctx.inv_h );
	ctx.contactSoftness = o_makeSoft( contactHertz, w->contactDampingRatio, ctx.h );
	ctx.staticSoftness = o_makeSoft( 2.0f * contactHertz, w->contactDampingRatio, ctx.h );
	ctx.restitutionThreshold = w->restitutionThreshold;
	ctx.maxLinearVelocity = w->maxLinearSpeed;
	ctx.enableWarmStarting = w->enableWarmStarting;
	t0 = b2GetTicks();
	o_collide( w, &ctx );
	w->profile.collide = b2GetMilliseconds( t0 );
	if ( timeStep > 0.0f )
	{
		t0 = b2GetTicks();
		o_solve( w, &ctx );
		w->profile.solve = b2GetMilliseconds( t0 );
	}
	w->profile.step = b2GetMilliseconds( stepTicks );
	w->endEventArrayIndex = 1 - w->endEventArrayIndex;
	w->endEvents[w->endEventArrayIndex].count = 0;
	w->locked = 0;
}
