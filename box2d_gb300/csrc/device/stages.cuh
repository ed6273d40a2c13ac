/*
 * Per-item bodies of the solver and finalize stages, shared by the per-stage kernels
 * (world.cu) and the persistent solver kernel (persistent.cu). Each function does the work
 * of one contact slot, joint or body exactly as the reference stage does for one lane.
 */
#pragma once

#include "ccd.cuh"
#include "joints.cuh"
#include "solver.cuh"

/* ======================= solver ======================= */
struct d_solveArgs
{
	int colorOffsets[B2_GRAPH_COLOR_COUNT + 1];
	b2gContact* contacts;
	const int* colorIds;
	b2gContactLane* lanes;
	b2gJoint* joints;
	float4* sv;
	float4* sd;
	const float* params;
	int awakeCount;
	b2gStepParams p;
};

/* contact_solver.c:1573-1809 (graph colors) and :20-160 (overflow), one thread per slot;
   the constraint is written to `out` */
static __device__ void d_prepareContactLane( const d_solveArgs& a, int slot, int overflowBegin, b2gContactLane* out )
{
	int contactId = a.colorIds[slot];
	const b2gContact* cs = a.contacts + contactId;
	const b2Manifold* m = &cs->manifold;
	b2gContactLane c;
	float warmStartScale = a.p.enableWarmStarting ? 1.0f : 0.0f;
	int indexA = cs->bodySimIndexA, indexB = cs->bodySimIndexB;
	c.indexA = indexA + 1;
	c.indexB = indexB + 1;
	b2Vec2 vA = { 0.0f, 0.0f }, vB = { 0.0f, 0.0f };
	float wA = 0.0f, wB = 0.0f;
	float mA = cs->invMassA, iA = cs->invIA, mB = cs->invMassB, iB = cs->invIB;
	if ( indexA != -1 )
	{
		float4 v = a.sv[indexA];
		vA = d_v( v.x, v.y );
		wA = v.z;
	}
	if ( indexB != -1 )
	{
		float4 v = a.sv[indexB];
		vB = d_v( v.x, v.y );
		wB = v.z;
	}
	c.invMassA = mA;
	c.invMassB = mB;
	c.invIA = iA;
	c.invIB = iB;
	{
		float k = iA + iB;
		c.rollingMass = k > 0.0f ? 1.0f / k : 0.0f;
	}
	bool isOverflow = slot >= overflowBegin;
	float biasRate = a.p.contactBiasRate, massScale = a.p.contactMassScale, impulseScale = a.p.contactImpulseScale;
	if ( indexA == -1 || indexB == -1 )
	{
		biasRate = a.p.staticBiasRate;
		massScale = a.p.staticMassScale;
		impulseScale = a.p.staticImpulseScale;
	}
	else if ( a.p.enableContactSoftening && isOverflow == false )
	{
		float contactHertz = d_min( a.p.contactHertz, 0.125f * a.p.inv_h );
		float ratio = 1.0f;
		if ( mA < mB ) ratio = d_max( 0.5f, mA / mB );
		else if ( mB < mA ) ratio = d_max( 0.5f, mB / mA );
		d_makeSoftInto( ratio * contactHertz, ratio * a.p.contactDampingRatio, a.p.h, &biasRate, &massScale, &impulseScale );
	}
	b2Vec2 normal = m->normal;
	c.normal = normal;
	c.friction = cs->friction;
	c.tangentSpeed = cs->tangentSpeed;
	c.restitution = cs->restitution;
	c.rollingResistance = cs->rollingResistance;
	c.rollingImpulse = warmStartScale * m->rollingImpulse;
	c.biasRate = biasRate;
	c.massScale = massScale;
	c.impulseScale = impulseScale;
	c.pointCount = m->pointCount;
	b2Vec2 tangent = d_rightPerp( normal );
	{
		const b2ManifoldPoint* mp = m->points + 0;
		b2Vec2 rA = mp->anchorA, rB = mp->anchorB;
		c.anchorA1 = rA;
		c.anchorB1 = rB;
		c.baseSeparation1 = mp->separation - d_dot( d_sub( rB, rA ), normal );
		c.normalImpulse1 = warmStartScale * mp->normalImpulse;
		c.tangentImpulse1 = warmStartScale * mp->tangentImpulse;
		c.totalNormalImpulse1 = 0.0f;
		float rnA = d_cross( rA, normal ), rnB = d_cross( rB, normal );
		float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		c.normalMass1 = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
		float rtA = d_cross( rA, tangent ), rtB = d_cross( rB, tangent );
		float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		c.tangentMass1 = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
		b2Vec2 vrA = d_add( vA, d_crossSV( wA, rA ) );
		b2Vec2 vrB = d_add( vB, d_crossSV( wB, rB ) );
		c.relativeVelocity1 = d_dot( normal, d_sub( vrB, vrA ) );
	}
	if ( m->pointCount == 2 )
	{
		const b2ManifoldPoint* mp = m->points + 1;
		b2Vec2 rA = mp->anchorA, rB = mp->anchorB;
		c.anchorA2 = rA;
		c.anchorB2 = rB;
		c.baseSeparation2 = mp->separation - d_dot( d_sub( rB, rA ), normal );
		c.normalImpulse2 = warmStartScale * mp->normalImpulse;
		c.tangentImpulse2 = warmStartScale * mp->tangentImpulse;
		c.totalNormalImpulse2 = 0.0f;
		float rnA = d_cross( rA, normal ), rnB = d_cross( rB, normal );
		float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		c.normalMass2 = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
		float rtA = d_cross( rA, tangent ), rtB = d_cross( rB, tangent );
		float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		c.tangentMass2 = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
		b2Vec2 vrA = d_add( vA, d_crossSV( wA, rA ) );
		b2Vec2 vrB = d_add( vB, d_crossSV( wB, rB ) );
		c.relativeVelocity2 = d_dot( normal, d_sub( vrB, vrA ) );
	}
	else
	{
		c.baseSeparation2 = 0.0f;
		c.normalImpulse2 = 0.0f;
		c.tangentImpulse2 = 0.0f;
		c.totalNormalImpulse2 = 0.0f;
		c.anchorA2 = d_v( 0.0f, 0.0f );
		c.anchorB2 = d_v( 0.0f, 0.0f );
		c.normalMass2 = 0.0f;
		c.tangentMass2 = 0.0f;
		c.relativeVelocity2 = 0.0f;
	}
	c.groupFlags = 0;
	if ( isOverflow == false )
	{
		/* 4-wide group of the slot's color: any lane with rolling resistance / restitution
		   (contact_solver.c:2021, :2131) */
		int color = 0;
		while ( a.colorOffsets[color + 1] <= slot ) color += 1;
		int colorBegin = a.colorOffsets[color], colorEnd = a.colorOffsets[color + 1];
		int g0 = colorBegin + ( ( slot - colorBegin ) / 4 ) * 4;
		for ( int k = g0; k < g0 + 4 && k < colorEnd; ++k )
		{
			const b2gContact* other = a.contacts + a.colorIds[k];
			c.groupFlags |= other->rollingResistance != 0.0f ? 1 : 0;
			c.groupFlags |= other->restitution != 0.0f ? 2 : 0;
		}
	}
	*out = c;
}

static __device__ __forceinline__ void d_prepareContactSlot( const d_solveArgs& a, int slot, int overflowBegin )
{
	d_prepareContactLane( a, slot, overflowBegin, a.lanes + slot );
}

static __device__ void d_prepareJointItem( const d_solveArgs& a, const d_jointBodies& bodies, int i )
{
	d_prepareJoint( a.joints + i, &bodies, a.p.h, a.p.inv_h, a.p.enableWarmStarting != 0 );
}

/* solver.c:66-112; pr = the body's 8 integration parameters (force, torque, damping,
   gravity scale, inverse mass, inverse inertia) */
static __device__ __forceinline__ void d_integrateVelocitiesState( const b2gStepParams& P, float4* sv, int i, const float* pr )
{
	float h = P.h;
	float4 s = sv[i];
	b2Vec2 v = { s.x, s.y };
	float w = s.z;
	float linearDamping = 1.0f / ( 1.0f + h * pr[3] );
	float angularDamping = 1.0f / ( 1.0f + h * pr[4] );
	float invMass = pr[6];
	float gravityScale = invMass > 0.0f ? pr[5] : 0.0f;
	b2Vec2 force = { pr[0], pr[1] };
	b2Vec2 gravity = { P.gravityX, P.gravityY };
	b2Vec2 lvd = d_add( d_mulSV( h * invMass, force ), d_mulSV( h * gravityScale, gravity ) );
	float avd = h * pr[7] * pr[2];
	v = d_mulAdd( lvd, linearDamping, v );
	w = avd + angularDamping * w;
	sv[i] = make_float4( v.x, v.y, w, s.w );
}

static __device__ __forceinline__ void d_integrateVelocitiesItem( const d_solveArgs& a, int i )
{
	d_integrateVelocitiesState( a.p, a.sv, i, a.params + 8 * i );
}

/* solver.c:114-162 */
static __device__ __forceinline__ void d_integratePositionsState( const b2gStepParams& P, float4* sv, float4* sd, int i )
{
	float h = P.h;
	float maxLinearSpeed = P.maxLinearVelocity;
	float maxAngularSpeed = D_MAX_ROTATION * P.inv_dt;
	float maxLinearSq = maxLinearSpeed * maxLinearSpeed;
	float maxAngularSq = maxAngularSpeed * maxAngularSpeed;
	float4 s = sv[i];
	float4 d = sd[i];
	uint32_t flags = __float_as_uint( s.w );
	b2Vec2 v = { s.x, s.y };
	float w = s.z;
	v.x = ( flags & B2G_LOCK_X ) ? 0.0f : v.x;
	v.y = ( flags & B2G_LOCK_Y ) ? 0.0f : v.y;
	w = ( flags & B2G_LOCK_Z ) ? 0.0f : w;
	if ( d_dot( v, v ) > maxLinearSq )
	{
		float ratio = maxLinearSpeed / d_length( v );
		v = d_mulSV( ratio, v );
		flags |= B2G_SPEED_CAPPED;
	}
	if ( w * w > maxAngularSq && ( flags & B2G_ALLOW_FAST_ROTATION ) == 0 )
	{
		float ratio = maxAngularSpeed / d_abs( w );
		w *= ratio;
		flags |= B2G_SPEED_CAPPED;
	}
	b2Vec2 dp = d_mulAdd( d_v( d.x, d.y ), h, v );
	b2Rot dq = d_integrateRotation( b2Rot{ d.z, d.w }, h * w );
	sv[i] = make_float4( v.x, v.y, w, __uint_as_float( flags ) );
	sd[i] = make_float4( dp.x, dp.y, dq.c, dq.s );
}

static __device__ __forceinline__ void d_integratePositionsItem( const d_solveArgs& a, int i )
{
	d_integratePositionsState( a.p, a.sv, a.sd, i );
}

enum
{
	STAGE_WARM = 0,
	STAGE_SOLVE = 1,
	STAGE_RELAX = 2,
	STAGE_RESTITUTION = 3,
};

/* one joint or one contact lane of a graph color at a stage, through a body accessor */
template <class TBodies>
static __device__ __forceinline__ void d_jointStageT( const b2gStepParams& P, b2gJoint* j, TBodies& bodies, int stage )
{
	if ( stage == STAGE_WARM ) d_warmStartJoint( j, bodies );
	else if ( stage == STAGE_SOLVE ) d_solveJoint( j, bodies, P.h, P.inv_h, true );
	else if ( stage == STAGE_RELAX ) d_solveJoint( j, bodies, P.h, P.inv_h, false );
}

template <class TBodies>
static __device__ __forceinline__ void d_laneStageT( const b2gStepParams& P, b2gContactLane* c, TBodies& bodies, int stage )
{
	if ( stage == STAGE_WARM ) d_warmStartLane( c, bodies );
	else if ( stage == STAGE_SOLVE ) d_solveLane( c, bodies, P.inv_h, -P.contactSpeed, true );
	else if ( stage == STAGE_RELAX ) d_solveLane( c, bodies, P.inv_h, -P.contactSpeed, false );
	else d_restitutionLane( c, bodies, P.restitutionThreshold );
}

/* the same with body state in two float4 arrays */
static __device__ __forceinline__ void d_jointStage( const b2gStepParams& P, b2gJoint* j, float4* sv, float4* sd, int stage )
{
	d_arrayBodies bodies = { sv, sd };
	d_jointStageT( P, j, bodies, stage );
}

static __device__ __forceinline__ void d_laneStage( const b2gStepParams& P, b2gContactLane* c, float4* sv, float4* sd, int stage )
{
	d_arrayBodies bodies = { sv, sd };
	d_laneStageT( P, c, bodies, stage );
}

/* one graph color: threads [0, jointCount) run joints, the rest run contact lanes */
static __device__ void d_colorStageItem( const d_solveArgs& a, int jointBegin, int jointCount, int laneBegin, int laneCount,
										 int stage, int i )
{
	if ( i < jointCount )
	{
		d_jointStage( a.p, a.joints + jointBegin + i, a.sv, a.sd, stage );
		return;
	}
	i -= jointCount;
	if ( i >= laneCount ) return;
	d_laneStage( a.p, a.lanes + laneBegin + i, a.sv, a.sd, stage );
}

/* overflow color: one thread walks joints then contacts in array order (joint.c:1542-1591,
   contact_solver.c:20-545) */
static __device__ void d_overflowStageAll( const d_solveArgs& a, int jointBegin, int jointCount, int laneBegin, int laneCount,
											int stage )
{
	d_arrayBodies bodies = { a.sv, a.sd };
	for ( int i = 0; i < jointCount; ++i ) d_jointStage( a.p, a.joints + jointBegin + i, a.sv, a.sd, stage );
	for ( int i = 0; i < laneCount; ++i )
	{
		b2gContactLane* c = a.lanes + laneBegin + i;
		if ( stage == STAGE_WARM ) d_warmStartOverflow( c, bodies );
		else if ( stage == STAGE_SOLVE ) d_solveOverflow( c, bodies, a.p.inv_h, a.p.contactSpeed, true );
		else if ( stage == STAGE_RELAX ) d_solveOverflow( c, bodies, a.p.inv_h, a.p.contactSpeed, false );
		else d_restitutionOverflow( c, bodies, a.p.restitutionThreshold );
	}
}

/* contact_solver.c:2238-2331 (colors) and :516-545 (overflow) */
static __device__ void d_storeLane( const b2gContactLane* c, b2Manifold* m, bool isOverflow )
{
	if ( isOverflow )
	{
		for ( int j = 0; j < m->pointCount; ++j )
		{
			m->points[j].normalImpulse = j == 0 ? c->normalImpulse1 : c->normalImpulse2;
			m->points[j].tangentImpulse = j == 0 ? c->tangentImpulse1 : c->tangentImpulse2;
			m->points[j].totalNormalImpulse = j == 0 ? c->totalNormalImpulse1 : c->totalNormalImpulse2;
			m->points[j].normalVelocity = j == 0 ? c->relativeVelocity1 : c->relativeVelocity2;
		}
		m->rollingImpulse = c->rollingImpulse;
		return;
	}
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

static __device__ __forceinline__ void d_storeSlot( const d_solveArgs& a, int slot, int overflowBegin )
{
	d_storeLane( a.lanes + slot, &a.contacts[a.colorIds[slot]].manifold, slot >= overflowBegin );
}

/* geometry.c:400-506 fat AABB (built in double, narrowed once) */
static __device__ float4 d_fatBox( double lx, double ly, double ux, double uy, double r )
{
	return make_float4( (float)__dsub_rn( lx, r ), (float)__dsub_rn( ly, r ), (float)__dadd_rn( ux, r ), (float)__dadd_rn( uy, r ) );
}

static __device__ float4 d_computeFatShapeAABB( const b2gShape* s, b2Transform xf, float extra )
{
	switch ( s->type )
	{
		case b2_circleShape:
		{
			b2Vec2 c = d_transformWorldPoint( xf, s->v[0] );
			double r = __dadd_rn( (double)s->radius, (double)extra );
			return d_fatBox( c.x, c.y, c.x, c.y, r );
		}
		case b2_capsuleShape:
		case b2_segmentShape:
		case b2_chainSegmentShape:
		{
			b2Vec2 v1 = d_transformWorldPoint( xf, s->v[0] );
			b2Vec2 v2 = d_transformWorldPoint( xf, s->v[1] );
			double r = s->type == b2_capsuleShape ? __dadd_rn( (double)s->radius, (double)extra ) : (double)extra;
			return d_fatBox( v1.x < v2.x ? v1.x : v2.x, v1.y < v2.y ? v1.y : v2.y, v1.x > v2.x ? v1.x : v2.x,
							 v1.y > v2.y ? v1.y : v2.y, r );
		}
		case b2_polygonShape:
		{
			b2Vec2 v = d_transformWorldPoint( xf, s->v[0] );
			double lx = v.x, ly = v.y, ux = v.x, uy = v.y;
			for ( int i = 1; i < s->count; ++i )
			{
				v = d_transformWorldPoint( xf, s->v[i] );
				lx = v.x < lx ? v.x : lx;
				ly = v.y < ly ? v.y : ly;
				ux = v.x > ux ? v.x : ux;
				uy = v.y > uy ? v.y : uy;
			}
			double r = __dadd_rn( (double)s->radius, (double)extra );
			return d_fatBox( lx, ly, ux, uy, r );
		}
		default:
			return make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	}
}

struct d_finalizeArgs
{
	float4* sv;
	float4* sd;
	float* params;
	float4* center0;
	const int* awakeBodyId;
	int awakeCount;
	float4* xf;
	float2* center;
	const float2* localCenter;
	const float* minExtent;
	const float* maxExtent;
	const float* sleepThreshold;
	const float* safetyFactor;
	const int* bodyType;
	uint32_t* bodyFlags;
	const int* shapeStart;
	const int* shapeCount;
	const int* shapeList;
	const b2gShape* shapes;
	float4* aabb;
	float4* fat;
	int* shapeEnlarged;
	int* enlargedRecs;
	float4* enlargedBoxes;
	int enlargedCap;
	b2gStepCounters* counters;
	float dt, inv_dt;
	int enableSleep, enableContinuous;
	d_ccdWorld ccd; /* static tree and filters for the continuous sweep */
	float* toi;		/* when recording: time-of-impact fraction per awake body (1 = none) */
	/* per awake index the sleep timer; islands (null when sleeping is disabled): per awake
	   index the island's index in the awake set, per awake island (island id, has removed
	   constraints); out: one bit per island that stays awake */
	float* sleepTime;
	const int* islandLocal;
	const int2* islandInfo;
	unsigned int* awakeIslandBits;
};

/* solver.c:384-550 b2SolveContinuous for a fast non-bullet body: sweep every non-sensor
   shape from the step's start pose (center0, rotation0) to the solved pose against the
   static tree, move the body back to the earliest time of impact, and refresh the shape
   boxes. Kept out of line: fast bodies are rare and the sweep needs a deep stack.
   Returns whether a shape's fat box was enlarged. */
static __device__ __noinline__ bool d_solveContinuous( const d_finalizeArgs& a, int simIndex, int bodyId, b2Vec2 center, b2Rot q,
														bool isBullet )
{
	float4 c0 = a.center0[simIndex];
	b2Vec2 base = { c0.x, c0.y };
	float2 lc2 = a.localCenter[bodyId];
	b2Vec2 localCenter = { lc2.x, lc2.y };
	d_sweep sweep = d_relativeSweep( base, b2Rot{ c0.z, c0.w }, center, q, localCenter, base );
	b2Transform xf1;
	xf1.q = sweep.q1;
	xf1.p = d_sub( sweep.c1, d_rotate( sweep.q1, sweep.localCenter ) );
	b2Transform xf2;
	xf2.q = sweep.q2;
	xf2.p = d_sub( sweep.c2, d_rotate( sweep.q2, sweep.localCenter ) );
	float fraction = 1.0f;
	bool hit = false, overflow = false;
	d_sensorHits sensorHits;
	sensorHits.count = 0;
	int start = a.shapeStart[bodyId], count = a.shapeCount[bodyId];
	for ( int k = 0; k < count; ++k )
	{
		int shapeId = a.shapeList[start + k];
		const b2gShape* fastShape = a.shapes + shapeId;
		float4 box1 = a.aabb[shapeId];
		float4 box2 = d_offsetAABB( d_computeFatShapeAABB( fastShape, xf2, 0.0f ), base );
		a.aabb[shapeId] = box2;
		if ( fastShape->isSensor ) continue;
		float4 swept = make_float4( d_min( box1.x, box2.x ), d_min( box1.y, box2.y ), d_max( box1.z, box2.z ),
									d_max( box1.w, box2.w ) );
		d_fastShape fast;
		fast.centroid1 = d_transformPoint( xf1, fastShape->ccdCentroid );
		fast.centroid2 = d_transformPoint( xf2, fastShape->ccdCentroid );
		fast.coreDistance = D_CORE_FRACTION * a.minExtent[bodyId];
		fraction = d_continuousQuery( a.ccd, a.ccd.staticTree, a.ccd.staticRoot, swept, shapeId, fastShape, sweep, base, fraction,
									  &hit, &overflow, fast, &sensorHits );
		if ( isBullet )
		{
			fraction = d_continuousQuery( a.ccd, a.ccd.kinematicTree, a.ccd.kinematicRoot, swept, shapeId, fastShape, sweep, base,
										  fraction, &hit, &overflow, fast, &sensorHits );
			fraction = d_continuousQuery( a.ccd, a.ccd.dynamicTree, a.ccd.dynamicRoot, swept, shapeId, fastShape, sweep, base,
										  fraction, &hit, &overflow, fast, &sensorHits );
		}
	}
	/* solver.c:539-547: the sensor hits before the solid time of impact */
	for ( int i = 0; i < sensorHits.count; ++i )
	{
		if ( sensorHits.fraction[i] >= fraction || a.ccd.sensorHits == nullptr ) continue;
		int k = atomicAdd( a.ccd.sensorHitCount, 1 );
		if ( k < a.ccd.sensorHitCap ) a.ccd.sensorHits[k] = make_int2( sensorHits.sensor[i], sensorHits.visitor[i] );
		else atomicOr( &a.counters->status, B2G_STATUS_CAPACITY );
	}
	atomicAdd( &a.counters->continuousSweeps, 1 );
	if ( overflow ) atomicOr( &a.counters->status, B2G_STATUS_CAPACITY );
	bool anyEnlarged = false;
	if ( fraction < 1.0f )
	{
		atomicAdd( &a.counters->continuousHits, 1 );
		if ( a.toi != nullptr ) a.toi[simIndex] = fraction;
		b2Rot qt = d_nlerp( sweep.q1, sweep.q2, fraction );
		b2Vec2 ct = d_lerp( sweep.c1, sweep.c2, fraction );
		b2Vec2 origin = d_sub( ct, d_rotate( qt, sweep.localCenter ) );
		b2Transform transform = { d_add( base, origin ), qt };
		b2Vec2 centerT = d_add( base, ct );
		a.xf[bodyId] = make_float4( transform.p.x, transform.p.y, qt.c, qt.s );
		a.center[bodyId] = make_float2( centerT.x, centerT.y );
		a.center0[simIndex] = make_float4( centerT.x, centerT.y, qt.c, qt.s );
		for ( int k = 0; k < count; ++k )
		{
			int shapeId = a.shapeList[start + k];
			const b2gShape* shape = a.shapes + shapeId;
			float4 aabb = d_computeFatShapeAABB( shape, transform, D_SPECULATIVE_DISTANCE );
			a.aabb[shapeId] = aabb;
			float4 fat = a.fat[shapeId];
			int enlarged = 0;
			if ( ( fat.x <= aabb.x && fat.y <= aabb.y && aabb.z <= fat.z && aabb.w <= fat.w ) == false )
			{
				float margin = shape->aabbMargin;
				a.fat[shapeId] = make_float4( aabb.x - margin, aabb.y - margin, aabb.z + margin, aabb.w + margin );
				enlarged = 1;
				anyEnlarged = true;
			}
			a.shapeEnlarged[shapeId] = enlarged;
		}
	}
	else
	{
		a.center0[simIndex] = make_float4( center.x, center.y, q.c, q.s );
		for ( int k = 0; k < count; ++k )
		{
			int shapeId = a.shapeList[start + k];
			float4 aabb = a.aabb[shapeId];
			float4 fat = a.fat[shapeId];
			int enlarged = 0;
			if ( ( fat.x <= aabb.x && fat.y <= aabb.y && aabb.z <= fat.z && aabb.w <= fat.w ) == false )
			{
				float margin = a.shapes[shapeId].aabbMargin;
				a.fat[shapeId] = make_float4( aabb.x - margin, aabb.y - margin, aabb.z + margin, aabb.w + margin );
				enlarged = 1;
				anyEnlarged = true;
			}
			a.shapeEnlarged[shapeId] = enlarged;
		}
	}
	if ( hit )
	{
		/* b2_hadTimeOfImpact lands in the body's sim flags, reported by the next finalize */
		float4 s = a.sv[simIndex];
		s.w = __uint_as_float( __float_as_uint( s.w ) | B2G_HAD_TOI );
		a.sv[simIndex] = s;
	}
	return anyEnlarged;
}

/* solver.c:553-743, one thread per awake body. A body with an enlarged shape (or a fast
   bullet) appends one record per shape, as one contiguous group:
   (awake index, shape id, enlarged, fast bullet) + fat box. */
static __device__ void d_finalizeBody( const d_finalizeArgs& a, int simIndex )
{
	int bodyId = a.awakeBodyId[simIndex];
	float4 s = a.sv[simIndex];
	float4 d = a.sd[simIndex];
	b2Vec2 v = { s.x, s.y };
	float w = s.z;
	uint32_t stateFlags = __float_as_uint( s.w );
	if ( isfinite( v.x ) == false || isfinite( v.y ) == false || isfinite( w ) == false )
		atomicOr( &a.counters->status, B2G_STATUS_NAN );
	float2 c2 = a.center[bodyId];
	float4 x4 = a.xf[bodyId];
	b2Vec2 center = { c2.x + d.x, c2.y + d.y };
	b2Rot q = d_normalizeRot( d_mulRot( b2Rot{ d.z, d.w }, b2Rot{ x4.z, x4.w } ) );
	float maxExtent = a.maxExtent[bodyId];
	float maxVelocity = d_length( v ) + d_abs( w ) * maxExtent;
	float maxDeltaPosition = d_length( d_v( d.x, d.y ) ) + d_abs( d.w ) * maxExtent;
	float positionSleepFactor = 0.5f;
	float sleepVelocity = d_max( maxVelocity, positionSleepFactor * a.inv_dt * maxDeltaPosition );
	float2 lc = a.localCenter[bodyId];
	b2Vec2 p = d_add( center, d_neg( d_rotate( q, d_v( lc.x, lc.y ) ) ) );
	a.xf[bodyId] = make_float4( p.x, p.y, q.c, q.s );
	a.center[bodyId] = make_float2( center.x, center.y );
	a.sd[simIndex] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
	float* pr = a.params + 8 * simIndex;
	pr[0] = 0.0f;
	pr[1] = 0.0f;
	pr[2] = 0.0f;
	uint32_t bodyFlags = a.bodyFlags[bodyId];
	bodyFlags &= ~B2G_TRANSIENT;
	bodyFlags |= ( stateFlags & ( B2G_SPEED_CAPPED | B2G_HAD_TOI ) );
	stateFlags &= ~B2G_TRANSIENT;
	a.sv[simIndex] = make_float4( v.x, v.y, w, __uint_as_float( stateFlags ) );
	bool isBullet = ( bodyFlags & B2G_IS_BULLET ) != 0;
	bool sweep = false;
	bool sleepy = !( a.enableSleep == 0 || ( bodyFlags & B2G_ENABLE_SLEEP ) == 0 || sleepVelocity > a.sleepThreshold[bodyId] );
	/* solver.c:637-695: the body's sleep timer, then its island stays awake or, when the
	   island must be split before it can sleep, becomes the split candidate (largest sleep
	   time, then largest island id) */
	float sleepTime = sleepy ? a.sleepTime[simIndex] + a.dt : 0.0f;
	a.sleepTime[simIndex] = sleepTime;
	if ( a.islandLocal != nullptr )
	{
		int islandIndex = a.islandLocal[simIndex];
		if ( sleepTime < D_TIME_TO_SLEEP )
		{
			atomicOr( a.awakeIslandBits + ( islandIndex >> 5 ), 1u << ( islandIndex & 31 ) );
		}
		else
		{
			int2 info = a.islandInfo[islandIndex];
			if ( info.y != 0 )
			{
				unsigned long long key = ( (unsigned long long)__float_as_uint( sleepTime ) << 32 ) | (unsigned int)info.x;
				atomicMax( &a.counters->splitKey, key );
			}
		}
	}
	if ( sleepy == false )
	{
		float maxMotion = d_max( maxDeltaPosition, maxVelocity * a.dt );
		if ( a.bodyType[bodyId] == b2_dynamicBody && a.enableContinuous && maxMotion > a.safetyFactor[bodyId] * a.minExtent[bodyId] )
		{
			/* fast body: non-bullets sweep against static shapes here; bullets advance like
			   a slow body and are re-inserted into the broadphase by the host */
			bodyFlags |= B2G_IS_FAST;
			atomicAdd( &a.counters->fastBodyCount, 1 );
			sweep = isBullet == false;
		}
	}
	a.bodyFlags[bodyId] = bodyFlags;
	if ( a.toi != nullptr ) a.toi[simIndex] = 1.0f;
	int start = a.shapeStart[bodyId], count = a.shapeCount[bodyId];
	bool anyEnlarged = false;
	bool fastBullet = ( bodyFlags & B2G_IS_FAST ) != 0 && isBullet;
	if ( sweep ) anyEnlarged = d_solveContinuous( a, simIndex, bodyId, center, q, false );
	else if ( fastBullet == false ) a.center0[simIndex] = make_float4( center.x, center.y, q.c, q.s );
	/* a fast bullet keeps its sweep start (center0) for the bullet pass after the broadphase
	   enlargement (solver.c:1917-1928) */
	bool isFast = ( bodyFlags & B2G_IS_FAST ) != 0;
	b2Transform transform = { p, q };
	for ( int k = 0; k < count && sweep == false; ++k )
	{
		int shapeId = a.shapeList[start + k];
		int enlarged = 0;
		if ( isFast == false )
		{
			const b2gShape* shape = a.shapes + shapeId;
			float4 aabb = d_computeFatShapeAABB( shape, transform, D_SPECULATIVE_DISTANCE );
			a.aabb[shapeId] = aabb;
			float4 fat = a.fat[shapeId];
			bool contains = fat.x <= aabb.x && fat.y <= aabb.y && aabb.z <= fat.z && aabb.w <= fat.w;
			if ( contains == false )
			{
				float margin = shape->aabbMargin;
				a.fat[shapeId] = make_float4( aabb.x - margin, aabb.y - margin, aabb.z + margin, aabb.w + margin );
				enlarged = 1;
				anyEnlarged = true;
			}
		}
		a.shapeEnlarged[shapeId] = enlarged;
	}
	if ( anyEnlarged || fastBullet )
	{
		int base = atomicAdd( &a.counters->enlargedBodyCount, count );
		for ( int k = 0; k < count && base + k < a.enlargedCap; ++k )
		{
			int shapeId = a.shapeList[start + k];
			int* r = a.enlargedRecs + 4 * ( base + k );
			r[0] = simIndex;
			r[1] = shapeId;
			r[2] = a.shapeEnlarged[shapeId];
			r[3] = fastBullet ? 1 : 0;
			a.enlargedBoxes[base + k] = a.fat[shapeId];
		}
	}
}

