/*
 * Device Soft Step constraint math for contacts (contact_solver.c in the reference).
 *
 * Graph-color contacts follow the SSE2 wide path lane by lane (one thread = one lane):
 * the second point of a one-point manifold runs on the zeroed dummy data exactly as the
 * reference does, min/max are SSE-ordered selects, and rolling resistance / restitution
 * are switched per 4-wide group of the color's contact array (contact_solver.c:2021,
 * :2131). Overflow contacts follow the scalar path (contact_solver.c:20-545).
 */
#pragma once

#include "math.cuh"

typedef struct d_body
{
	float vx, vy, w;
	uint32_t flags;
	float dpx, dpy, dqc, dqs;
} d_body;

/* body-state access of the solver functions: awake state in two float4 arrays, indexed by
   awake index (global memory, or a shared-memory copy with bin-local indices) */
struct d_arrayBodies
{
	float4* sv;
	float4* sd;
	__device__ __forceinline__ float4& v( int i ) const { return sv[i]; }
	__device__ __forceinline__ float4& d( int i ) const { return sd[i]; }
};

static __device__ __forceinline__ float w_min( float a, float b ) { return a < b ? a : b; }
static __device__ __forceinline__ float w_max( float a, float b ) { return a > b ? a : b; }
static __device__ __forceinline__ float w_symClamp( float a, float b )
{
	float nb = -b;
	return w_max( nb, w_min( a, b ) );
}

template <class TBodies> static __device__ __forceinline__ d_body d_gather( TBodies& bodies, int index1 )
{
	d_body b;
	if ( index1 == 0 )
	{
		b.vx = 0.0f;
		b.vy = 0.0f;
		b.w = 0.0f;
		b.flags = 0;
		b.dpx = 0.0f;
		b.dpy = 0.0f;
		b.dqc = 1.0f;
		b.dqs = 0.0f;
		return b;
	}
	float4 v = bodies.v( index1 - 1 );
	float4 d = bodies.d( index1 - 1 );
	b.vx = v.x;
	b.vy = v.y;
	b.w = v.z;
	b.flags = __float_as_uint( v.w );
	b.dpx = d.x;
	b.dpy = d.y;
	b.dqc = d.z;
	b.dqs = d.w;
	return b;
}

/* writes only velocities, only for dynamic bodies (contact_solver.c:1526-1562) */
template <class TBodies> static __device__ __forceinline__ void d_scatter( TBodies& bodies, int index1, const d_body* b )
{
	if ( index1 == 0 ) return;
	if ( ( b->flags & B2G_DYNAMIC_FLAG ) == 0 ) return;
	float4 v;
	v.x = b->vx;
	v.y = b->vy;
	v.z = b->w;
	v.w = __uint_as_float( b->flags );
	bodies.v( index1 - 1 ) = v;
}

/* contact_solver.c:1811-1871 */
template <class TBodies> static __device__ void d_warmStartLane( b2gContactLane* c, TBodies& bodies )
{
	d_body bA = d_gather( bodies, c->indexA ), bB = d_gather( bodies, c->indexB );
	float tangentX = c->normal.y;
	float tangentY = 0.0f - c->normal.x;
	{
		b2Vec2 rA = c->anchorA1, rB = c->anchorB1;
		float Px = c->normalImpulse1 * c->normal.x + c->tangentImpulse1 * tangentX;
		float Py = c->normalImpulse1 * c->normal.y + c->tangentImpulse1 * tangentY;
		bA.w = bA.w - c->invIA * ( rA.x * Py - rA.y * Px );
		bA.vx = bA.vx - c->invMassA * Px;
		bA.vy = bA.vy - c->invMassA * Py;
		bB.w = bB.w + c->invIB * ( rB.x * Py - rB.y * Px );
		bB.vx = bB.vx + c->invMassB * Px;
		bB.vy = bB.vy + c->invMassB * Py;
		c->totalNormalImpulse1 = c->totalNormalImpulse1 + c->normalImpulse1;
	}
	{
		b2Vec2 rA = c->anchorA2, rB = c->anchorB2;
		float Px = c->normalImpulse2 * c->normal.x + c->tangentImpulse2 * tangentX;
		float Py = c->normalImpulse2 * c->normal.y + c->tangentImpulse2 * tangentY;
		bA.w = bA.w - c->invIA * ( rA.x * Py - rA.y * Px );
		bA.vx = bA.vx - c->invMassA * Px;
		bA.vy = bA.vy - c->invMassA * Py;
		bB.w = bB.w + c->invIB * ( rB.x * Py - rB.y * Px );
		bB.vx = bB.vx + c->invMassB * Px;
		bB.vy = bB.vy + c->invMassB * Py;
		c->totalNormalImpulse2 = c->totalNormalImpulse2 + c->normalImpulse2;
	}
	bA.w = bA.w - c->invIA * c->rollingImpulse;
	bB.w = bB.w + c->invIB * c->rollingImpulse;
	d_scatter( bodies, c->indexA, &bA );
	d_scatter( bodies, c->indexB, &bB );
}

static __device__ __forceinline__ void d_normalPoint( const b2gContactLane* c, d_body* bA, d_body* bB, float dpx, float dpy,
													  b2Vec2 rA, b2Vec2 rB, float baseSeparation, float normalMass,
													  float* normalImpulse, float* totalImpulse, float biasRate,
													  float massScale, float impulseScale, float inv_h, float contactSpeed,
													  float* totalNormalImpulse )
{
	float rsAx = bA->dqc * rA.x - bA->dqs * rA.y;
	float rsAy = bA->dqs * rA.x + bA->dqc * rA.y;
	float rsBx = bB->dqc * rB.x - bB->dqs * rB.y;
	float rsBy = bB->dqs * rB.x + bB->dqc * rB.y;
	float dsx = dpx + ( rsBx - rsAx );
	float dsy = dpy + ( rsBy - rsAy );
	float s = ( c->normal.x * dsx + c->normal.y * dsy ) + baseSeparation;
	bool mask = s > 0.0f;
	float specBias = s * inv_h;
	float softBias = w_max( biasRate * s, contactSpeed );
	float bias = mask ? specBias : softBias;
	float pointMassScale = mask ? 1.0f : massScale;
	float pointImpulseScale = mask ? 0.0f : impulseScale;
	float dvx = ( bB->vx - bB->w * rB.y ) - ( bA->vx - bA->w * rA.y );
	float dvy = ( bB->vy + bB->w * rB.x ) - ( bA->vy + bA->w * rA.x );
	float vn = dvx * c->normal.x + dvy * c->normal.y;
	float negImpulse = normalMass * ( pointMassScale * vn + bias ) + pointImpulseScale * *normalImpulse;
	float newImpulse = w_max( *normalImpulse - negImpulse, 0.0f );
	float impulse = newImpulse - *normalImpulse;
	*normalImpulse = newImpulse;
	*totalImpulse = *totalImpulse + impulse;
	*totalNormalImpulse = *totalNormalImpulse + newImpulse;
	float Px = impulse * c->normal.x;
	float Py = impulse * c->normal.y;
	bA->vx = bA->vx - c->invMassA * Px;
	bA->vy = bA->vy - c->invMassA * Py;
	bA->w = bA->w - c->invIA * ( rA.x * Py - rA.y * Px );
	bB->vx = bB->vx + c->invMassB * Px;
	bB->vy = bB->vy + c->invMassB * Py;
	bB->w = bB->w + c->invIB * ( rB.x * Py - rB.y * Px );
}

static __device__ __forceinline__ void d_frictionPoint( const b2gContactLane* c, d_body* bA, d_body* bB, b2Vec2 rA, b2Vec2 rB,
														float tangentMass, float normalImpulse, float* tangentImpulse )
{
	float tangentX = c->normal.y;
	float tangentY = 0.0f - c->normal.x;
	float dvx = ( bB->vx - bB->w * rB.y ) - ( bA->vx - bA->w * rA.y );
	float dvy = ( bB->vy + bB->w * rB.x ) - ( bA->vy + bA->w * rA.x );
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
	bA->vx = bA->vx - c->invMassA * Px;
	bA->vy = bA->vy - c->invMassA * Py;
	bA->w = bA->w - c->invIA * ( rA.x * Py - rA.y * Px );
	bB->vx = bB->vx + c->invMassB * Px;
	bB->vy = bB->vy + c->invMassB * Py;
	bB->w = bB->w + c->invIB * ( rB.x * Py - rB.y * Px );
}

/* contact_solver.c:1873-2116 */
template <class TBodies> static __device__ void d_solveLane( b2gContactLane* c, TBodies& bodies, float inv_h, float contactSpeedNeg,
									bool useBias )
{
	d_body bA = d_gather( bodies, c->indexA ), bB = d_gather( bodies, c->indexB );
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
	float totalNormalImpulse = 0.0f;
	float dpx = bB.dpx - bA.dpx, dpy = bB.dpy - bA.dpy;
	d_normalPoint( c, &bA, &bB, dpx, dpy, c->anchorA1, c->anchorB1, c->baseSeparation1, c->normalMass1, &c->normalImpulse1,
				   &c->totalNormalImpulse1, biasRate, massScale, impulseScale, inv_h, contactSpeedNeg, &totalNormalImpulse );
	d_normalPoint( c, &bA, &bB, dpx, dpy, c->anchorA2, c->anchorB2, c->baseSeparation2, c->normalMass2, &c->normalImpulse2,
				   &c->totalNormalImpulse2, biasRate, massScale, impulseScale, inv_h, contactSpeedNeg, &totalNormalImpulse );
	if ( useBias == false )
	{
		if ( c->groupFlags & 1 )
		{
			float deltaLambda = c->rollingMass * ( bA.w - bB.w );
			float lambda = c->rollingImpulse;
			float maxLambda = c->rollingResistance * totalNormalImpulse;
			c->rollingImpulse = w_symClamp( lambda + deltaLambda, maxLambda );
			deltaLambda = c->rollingImpulse - lambda;
			bA.w = bA.w - c->invIA * deltaLambda;
			bB.w = bB.w + c->invIB * deltaLambda;
		}
		d_frictionPoint( c, &bA, &bB, c->anchorA1, c->anchorB1, c->tangentMass1, c->normalImpulse1, &c->tangentImpulse1 );
		d_frictionPoint( c, &bA, &bB, c->anchorA2, c->anchorB2, c->tangentMass2, c->normalImpulse2, &c->tangentImpulse2 );
	}
	d_scatter( bodies, c->indexA, &bA );
	d_scatter( bodies, c->indexB, &bB );
}

static __device__ __forceinline__ void d_restitutionPoint( const b2gContactLane* c, d_body* bA, d_body* bB, b2Vec2 rA, b2Vec2 rB,
														   float relativeVelocity, float totalImpulseIn, float normalMass,
														   float threshold, float* normalImpulse, float* totalImpulse )
{
	bool mask = ( relativeVelocity + threshold > 0.0f ) || ( totalImpulseIn == 0.0f ) || ( c->restitution == 0.0f );
	float mass = mask ? 0.0f : normalMass;
	float dvx = ( bB->vx - bB->w * rB.y ) - ( bA->vx - bA->w * rA.y );
	float dvy = ( bB->vy + bB->w * rB.x ) - ( bA->vy + bA->w * rA.x );
	float vn = dvx * c->normal.x + dvy * c->normal.y;
	float negImpulse = mass * ( vn + c->restitution * relativeVelocity );
	float newImpulse = w_max( *normalImpulse - negImpulse, 0.0f );
	float deltaImpulse = newImpulse - *normalImpulse;
	*normalImpulse = newImpulse;
	*totalImpulse = *totalImpulse + deltaImpulse;
	float Px = deltaImpulse * c->normal.x;
	float Py = deltaImpulse * c->normal.y;
	bA->vx = bA->vx - c->invMassA * Px;
	bA->vy = bA->vy - c->invMassA * Py;
	bA->w = bA->w - c->invIA * ( rA.x * Py - rA.y * Px );
	bB->vx = bB->vx + c->invMassB * Px;
	bB->vy = bB->vy + c->invMassB * Py;
	bB->w = bB->w + c->invIB * ( rB.x * Py - rB.y * Px );
}

/* contact_solver.c:2118-2228 */
template <class TBodies> static __device__ void d_restitutionLane( b2gContactLane* c, TBodies& bodies, float threshold )
{
	if ( ( c->groupFlags & 2 ) == 0 ) return;
	d_body bA = d_gather( bodies, c->indexA ), bB = d_gather( bodies, c->indexB );
	d_restitutionPoint( c, &bA, &bB, c->anchorA1, c->anchorB1, c->relativeVelocity1, c->totalNormalImpulse1, c->normalMass1,
						threshold, &c->normalImpulse1, &c->totalNormalImpulse1 );
	d_restitutionPoint( c, &bA, &bB, c->anchorA2, c->anchorB2, c->relativeVelocity2, c->totalNormalImpulse2, c->normalMass2,
						threshold, &c->normalImpulse2, &c->totalNormalImpulse2 );
	d_scatter( bodies, c->indexA, &bA );
	d_scatter( bodies, c->indexB, &bB );
}

/* ---------------- overflow contacts: scalar path (contact_solver.c:20-545) ---------------- */
template <class TBodies> static __device__ void d_warmStartOverflow( b2gContactLane* c, TBodies& bodies )
{
	d_body bA = d_gather( bodies, c->indexA ), bB = d_gather( bodies, c->indexB );
	b2Vec2 vA = { bA.vx, bA.vy }, vB = { bB.vx, bB.vy };
	float wA = bA.w, wB = bB.w;
	float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	b2Vec2 normal = c->normal, tangent = d_rightPerp( c->normal );
	for ( int j = 0; j < c->pointCount; ++j )
	{
		b2Vec2 rA = j == 0 ? c->anchorA1 : c->anchorA2;
		b2Vec2 rB = j == 0 ? c->anchorB1 : c->anchorB2;
		float ni = j == 0 ? c->normalImpulse1 : c->normalImpulse2;
		float ti = j == 0 ? c->tangentImpulse1 : c->tangentImpulse2;
		b2Vec2 P = d_add( d_mulSV( ni, normal ), d_mulSV( ti, tangent ) );
		if ( j == 0 ) c->totalNormalImpulse1 += c->normalImpulse1;
		else c->totalNormalImpulse2 += c->normalImpulse2;
		wA -= iA * d_cross( rA, P );
		vA = d_mulAdd( vA, -mA, P );
		wB += iB * d_cross( rB, P );
		vB = d_mulAdd( vB, mB, P );
	}
	wA -= iA * c->rollingImpulse;
	wB += iB * c->rollingImpulse;
	bA.vx = vA.x;
	bA.vy = vA.y;
	bA.w = wA;
	bB.vx = vB.x;
	bB.vy = vB.y;
	bB.w = wB;
	d_scatter( bodies, c->indexA, &bA );
	d_scatter( bodies, c->indexB, &bB );
}

template <class TBodies> static __device__ void d_solveOverflow( b2gContactLane* c, TBodies& bodies, float inv_h, float contactSpeed,
										bool useBias )
{
	d_body bA = d_gather( bodies, c->indexA ), bB = d_gather( bodies, c->indexB );
	float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	b2Vec2 vA = { bA.vx, bA.vy }, vB = { bB.vx, bB.vy };
	float wA = bA.w, wB = bB.w;
	b2Rot dqA = { bA.dqc, bA.dqs }, dqB = { bB.dqc, bB.dqs };
	b2Vec2 dp = { bB.dpx - bA.dpx, bB.dpy - bA.dpy };
	b2Vec2 normal = c->normal, tangent = d_rightPerp( normal );
	float friction = c->friction;
	/* overflow softness is stored in biasRate/massScale/impulseScale */
	float totalNormalImpulse = 0.0f;
	for ( int j = 0; j < c->pointCount; ++j )
	{
		b2Vec2 rA = j == 0 ? c->anchorA1 : c->anchorA2;
		b2Vec2 rB = j == 0 ? c->anchorB1 : c->anchorB2;
		float baseSeparation = j == 0 ? c->baseSeparation1 : c->baseSeparation2;
		float normalMass = j == 0 ? c->normalMass1 : c->normalMass2;
		float* normalImpulse = j == 0 ? &c->normalImpulse1 : &c->normalImpulse2;
		float* totalImpulse = j == 0 ? &c->totalNormalImpulse1 : &c->totalNormalImpulse2;
		b2Vec2 ds = d_add( dp, d_sub( d_rotate( dqB, rB ), d_rotate( dqA, rA ) ) );
		float s = baseSeparation + d_dot( ds, normal );
		float velocityBias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( s > 0.0f ) velocityBias = s * inv_h;
		else if ( useBias )
		{
			velocityBias = d_max( c->massScale * c->biasRate * s, -contactSpeed );
			massScale = c->massScale;
			impulseScale = c->impulseScale;
		}
		b2Vec2 vrA = d_add( vA, d_crossSV( wA, rA ) );
		b2Vec2 vrB = d_add( vB, d_crossSV( wB, rB ) );
		float vn = d_dot( d_sub( vrB, vrA ), normal );
		float impulse = -normalMass * ( massScale * vn + velocityBias ) - impulseScale * *normalImpulse;
		float newImpulse = d_max( *normalImpulse + impulse, 0.0f );
		impulse = newImpulse - *normalImpulse;
		*normalImpulse = newImpulse;
		*totalImpulse += impulse;
		totalNormalImpulse += newImpulse;
		b2Vec2 P = d_mulSV( impulse, normal );
		vA = d_mulSub( vA, mA, P );
		wA -= iA * d_cross( rA, P );
		vB = d_mulAdd( vB, mB, P );
		wB += iB * d_cross( rB, P );
	}
	if ( useBias == false )
	{
		for ( int j = 0; j < c->pointCount; ++j )
		{
			b2Vec2 rA = j == 0 ? c->anchorA1 : c->anchorA2;
			b2Vec2 rB = j == 0 ? c->anchorB1 : c->anchorB2;
			float tangentMass = j == 0 ? c->tangentMass1 : c->tangentMass2;
			float normalImpulse = j == 0 ? c->normalImpulse1 : c->normalImpulse2;
			float* tangentImpulse = j == 0 ? &c->tangentImpulse1 : &c->tangentImpulse2;
			b2Vec2 vrB = d_add( vB, d_crossSV( wB, rB ) );
			b2Vec2 vrA = d_add( vA, d_crossSV( wA, rA ) );
			float vt = d_dot( d_sub( vrB, vrA ), tangent ) - c->tangentSpeed;
			float impulse = tangentMass * ( -vt );
			float maxFriction = friction * normalImpulse;
			float newImpulse = d_clamp( *tangentImpulse + impulse, -maxFriction, maxFriction );
			impulse = newImpulse - *tangentImpulse;
			*tangentImpulse = newImpulse;
			b2Vec2 P = d_mulSV( impulse, tangent );
			vA = d_mulSub( vA, mA, P );
			wA -= iA * d_cross( rA, P );
			vB = d_mulAdd( vB, mB, P );
			wB += iB * d_cross( rB, P );
		}
		{
			float deltaLambda = -c->rollingMass * ( wB - wA );
			float lambda = c->rollingImpulse;
			float maxLambda = c->rollingResistance * totalNormalImpulse;
			c->rollingImpulse = d_clamp( lambda + deltaLambda, -maxLambda, maxLambda );
			deltaLambda = c->rollingImpulse - lambda;
			wA -= iA * deltaLambda;
			wB += iB * deltaLambda;
		}
	}
	bA.vx = vA.x;
	bA.vy = vA.y;
	bA.w = wA;
	bB.vx = vB.x;
	bB.vy = vB.y;
	bB.w = wB;
	d_scatter( bodies, c->indexA, &bA );
	d_scatter( bodies, c->indexB, &bB );
}

template <class TBodies> static __device__ void d_restitutionOverflow( b2gContactLane* c, TBodies& bodies, float threshold )
{
	float restitution = c->restitution;
	if ( restitution == 0.0f ) return;
	d_body bA = d_gather( bodies, c->indexA ), bB = d_gather( bodies, c->indexB );
	float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	b2Vec2 vA = { bA.vx, bA.vy }, vB = { bB.vx, bB.vy };
	float wA = bA.w, wB = bB.w;
	b2Vec2 normal = c->normal;
	for ( int j = 0; j < c->pointCount; ++j )
	{
		float relativeVelocity = j == 0 ? c->relativeVelocity1 : c->relativeVelocity2;
		float* totalImpulse = j == 0 ? &c->totalNormalImpulse1 : &c->totalNormalImpulse2;
		float* normalImpulse = j == 0 ? &c->normalImpulse1 : &c->normalImpulse2;
		float normalMass = j == 0 ? c->normalMass1 : c->normalMass2;
		if ( relativeVelocity > -threshold || *totalImpulse == 0.0f ) continue;
		b2Vec2 rA = j == 0 ? c->anchorA1 : c->anchorA2;
		b2Vec2 rB = j == 0 ? c->anchorB1 : c->anchorB2;
		b2Vec2 vrB = d_add( vB, d_crossSV( wB, rB ) );
		b2Vec2 vrA = d_add( vA, d_crossSV( wA, rA ) );
		float vn = d_dot( d_sub( vrB, vrA ), normal );
		float impulse = -normalMass * ( vn + restitution * relativeVelocity );
		float newImpulse = d_max( *normalImpulse + impulse, 0.0f );
		impulse = newImpulse - *normalImpulse;
		*normalImpulse = newImpulse;
		*totalImpulse += impulse;
		b2Vec2 P = d_mulSV( impulse, normal );
		vA = d_mulSub( vA, mA, P );
		wA -= iA * d_cross( rA, P );
		vB = d_mulAdd( vB, mB, P );
		wB += iB * d_cross( rB, P );
	}
	bA.vx = vA.x;
	bA.vy = vA.y;
	bA.w = wA;
	bB.vx = vB.x;
	bB.vy = vB.y;
	bB.w = wB;
	d_scatter( bodies, c->indexA, &bA );
	d_scatter( bodies, c->indexB, &bB );
}
