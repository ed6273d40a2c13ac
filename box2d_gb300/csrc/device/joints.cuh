/*
 * Device joint solvers: prepare / warm start / solve per joint, one thread per joint of a
 * graph color. Revolute follows revolute_joint.c:217-500 of the reference with the same
 * operation order. The parameter slots of b2gJoint are documented in host/joint.c.
 */
#pragma once

#include "math.cuh"

/* math_functions.c:96-136 */
static __device__ float d_atan2( float y, float x )
{
	if ( x == 0.0f && y == 0.0f ) return 0.0f;
	float ax = d_abs( x ), ay = d_abs( y );
	float mx = d_max( ay, ax ), mn = d_min( ay, ax );
	float a = mn / mx;
	float s = a * a;
	float c = s * a;
	float q = s * s;
	float r = 0.024840285f * q + 0.18681418f;
	float t = -0.094097948f * q - 0.33213072f;
	r = r * s + t;
	r = r * c + a;
	if ( ay > ax ) r = 1.57079637f - r;
	if ( x < 0 ) r = 3.14159274f - r;
	if ( y < 0 ) r = -r;
	return r;
}

/* math_functions.h:520-545 b2UnwindAngle (double arithmetic as in the reference) */
static __device__ float d_unwind( float radians )
{
	float x = d_clamp( radians, -1.0e6f, 1.0e6f );
	double twoPi = 2.0f * B2_PI;
	double roundToNearest = 6755399441055744.0;
	double a = x;
	double k = __dsub_rn( __dadd_rn( __ddiv_rn( a, twoPi ), roundToNearest ), roundToNearest );
	return (float)__dsub_rn( a, __dmul_rn( k, twoPi ) );
}

static __device__ b2Vec2 d_solve22( float a11, float a12, float a21, float a22, b2Vec2 b )
{
	float det = a11 * a22 - a12 * a21;
	if ( det != 0.0f ) det = 1.0f / det;
	b2Vec2 x = { det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) };
	return x;
}

static __device__ __forceinline__ void d_makeSoftInto( float hertz, float zeta, float h, float* biasRate, float* massScale,
													   float* impulseScale )
{
	if ( hertz == 0.0f )
	{
		*biasRate = 0.0f;
		*massScale = 0.0f;
		*impulseScale = 0.0f;
		return;
	}
	float omega = 2.0f * B2_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	*biasRate = omega / a1;
	*massScale = a2 * a3;
	*impulseScale = a3;
}

typedef struct d_jointBodies
{
	const float4* xf;
	const float2* center;
	const float2* localCenter;
	const float* invMass;
	const float* invI;
	const int* awakeIndex;
} d_jointBodies;

/* revolute_joint.c:217-281 */
static __device__ void d_prepareRevolute( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	int idA = j->bodyIdA, idB = j->bodyIdB;
	float4 xfA = bodies->xf[idA], xfB = bodies->xf[idB];
	b2Rot qA = { xfA.z, xfA.w }, qB = { xfB.z, xfB.w };
	float2 lcA = bodies->localCenter[idA], lcB = bodies->localCenter[idB];
	float2 cA = bodies->center[idA], cB = bodies->center[idB];
	float mA = bodies->invMass[idA], iA = bodies->invI[idA], mB = bodies->invMass[idB], iB = bodies->invI[idB];
	j->invMassA = mA;
	j->invMassB = mB;
	j->invIA = iA;
	j->invIB = iB;
	j->indexA = bodies->awakeIndex[idA];
	j->indexB = bodies->awakeIndex[idB];
	j->frameA.q = d_mulRot( qA, j->localFrameA.q );
	j->frameA.p = d_rotate( qA, d_sub( j->localFrameA.p, d_v( lcA.x, lcA.y ) ) );
	j->frameB.q = d_mulRot( qB, j->localFrameB.q );
	j->frameB.p = d_rotate( qB, d_sub( j->localFrameB.p, d_v( lcB.x, lcB.y ) ) );
	j->deltaCenter = d_v( cB.x - cA.x, cB.y - cA.y );
	float k = iA + iB;
	j->s[6] = k > 0.0f ? 1.0f / k : 0.0f;
	d_makeSoftInto( j->p[1], j->p[2], h, j->s + 7, j->s + 8, j->s + 9 );
	if ( warmStart == false )
	{
		j->s[0] = 0.0f;
		j->s[1] = 0.0f;
		j->s[2] = 0.0f;
		j->s[3] = 0.0f;
		j->s[4] = 0.0f;
		j->s[5] = 0.0f;
	}
}

struct d_stateRef
{
	float4 v;
	float4 d;
	bool dynamic;
};

static __device__ __forceinline__ d_stateRef d_loadState( const float4* sv, const float4* sd, int index )
{
	d_stateRef r;
	if ( index < 0 )
	{
		r.v = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		r.d = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		r.dynamic = false;
		return r;
	}
	r.v = sv[index];
	r.d = sd[index];
	r.dynamic = ( __float_as_uint( r.v.w ) & B2G_DYNAMIC_FLAG ) != 0;
	return r;
}

/* revolute_joint.c:283-315 */
static __device__ void d_warmStartRevolute( b2gJoint* j, float4* sv, const float4* sd )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( sv, sd, j->indexA ), B = d_loadState( sv, sd, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 linearImpulse = { j->s[0], j->s[1] };
	float axialImpulse = j->s[2] + j->s[3] + j->s[4] - j->s[5];
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, linearImpulse );
		float w = A.v.z;
		w -= iA * ( d_cross( rA, linearImpulse ) + axialImpulse );
		sv[j->indexA] = make_float4( v.x, v.y, w, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, linearImpulse );
		float w = B.v.z;
		w += iB * ( d_cross( rB, linearImpulse ) + axialImpulse );
		sv[j->indexB] = make_float4( v.x, v.y, w, B.v.w );
	}
}

/* revolute_joint.c:317-500 */
static __device__ void d_solveRevolute( b2gJoint* j, float4* sv, const float4* sd, float h, float inv_h, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( sv, sd, j->indexA ), B = d_loadState( sv, sd, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Rot qA = d_mulRot( dqA, j->frameA.q );
	b2Rot qB = d_mulRot( dqB, j->frameB.q );
	b2Rot relQ = d_invMulRot( qA, qB );
	bool fixedRotation = ( iA + iB == 0.0f );
	float axialMass = j->s[6];
	if ( j->enableSpring && fixedRotation == false )
	{
		float jointAngle = d_atan2( relQ.s, relQ.c );
		float C = d_unwind( jointAngle - j->p[0] );
		float bias = j->s[7] * C;
		float massScale = j->s[8];
		float impulseScale = j->s[9];
		float Cdot = wB - wA;
		float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * j->s[2];
		j->s[2] += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableMotor && fixedRotation == false )
	{
		float Cdot = wB - wA - j->p[6];
		float impulse = -axialMass * Cdot;
		float oldImpulse = j->s[3];
		float maxImpulse = h * j->p[5];
		j->s[3] = d_clamp( j->s[3] + impulse, -maxImpulse, maxImpulse );
		impulse = j->s[3] - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableLimit && fixedRotation == false )
	{
		float jointAngle = d_atan2( relQ.s, relQ.c );
		{
			float C = jointAngle - j->p[3];
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->softBias * C;
				massScale = j->softMass;
				impulseScale = j->softImpulse;
			}
			float Cdot = wB - wA;
			float oldImpulse = j->s[4];
			float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->s[4] = d_max( oldImpulse + impulse, 0.0f );
			impulse = j->s[4] - oldImpulse;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		{
			float C = j->p[4] - jointAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->softBias * C;
				massScale = j->softMass;
				impulseScale = j->softImpulse;
			}
			float Cdot = wA - wB;
			float oldImpulse = j->s[5];
			float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->s[5] = d_max( oldImpulse + impulse, 0.0f );
			impulse = j->s[5] - oldImpulse;
			wA += iA * impulse;
			wB -= iB * impulse;
		}
	}
	{
		b2Vec2 rA = d_rotate( dqA, j->frameA.p );
		b2Vec2 rB = d_rotate( dqB, j->frameB.p );
		b2Vec2 Cdot = d_sub( d_add( vB, d_crossSV( wB, rB ) ), d_add( vA, d_crossSV( wA, rA ) ) );
		b2Vec2 bias = { 0.0f, 0.0f };
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			b2Vec2 dcA = { A.d.x, A.d.y }, dcB = { B.d.x, B.d.y };
			b2Vec2 separation = d_add( d_add( d_sub( dcB, dcA ), d_sub( rB, rA ) ), j->deltaCenter );
			bias = d_mulSV( j->softBias, separation );
			massScale = j->softMass;
			impulseScale = j->softImpulse;
		}
		float k11 = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		float k12 = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		float k22 = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		b2Vec2 b = d_solve22( k11, k12, k12, k22, d_add( Cdot, bias ) );
		b2Vec2 impulse;
		impulse.x = -massScale * b.x - impulseScale * j->s[0];
		impulse.y = -massScale * b.y - impulseScale * j->s[1];
		j->s[0] += impulse.x;
		j->s[1] += impulse.y;
		vA = d_mulSub( vA, mA, impulse );
		wA -= iA * d_cross( rA, impulse );
		vB = d_mulAdd( vB, mB, impulse );
		wB += iB * d_cross( rB, impulse );
	}
	if ( A.dynamic ) sv[j->indexA] = make_float4( vA.x, vA.y, wA, A.v.w );
	if ( B.dynamic ) sv[j->indexB] = make_float4( vB.x, vB.y, wB, B.v.w );
}

/* joint.c:1406-1540 dispatch */
static __device__ void d_prepareJoint( b2gJoint* j, const d_jointBodies* bodies, float h, float inv_h, bool warmStart )
{
	float hertz = d_min( j->constraintHertz, 0.25f * inv_h );
	d_makeSoftInto( hertz, j->constraintDampingRatio, h, &j->softBias, &j->softMass, &j->softImpulse );
	switch ( j->type )
	{
		case b2_revoluteJoint: d_prepareRevolute( j, bodies, h, warmStart ); break;
		default: break;
	}
}

static __device__ void d_warmStartJoint( b2gJoint* j, float4* sv, const float4* sd )
{
	switch ( j->type )
	{
		case b2_revoluteJoint: d_warmStartRevolute( j, sv, sd ); break;
		default: break;
	}
}

static __device__ void d_solveJoint( b2gJoint* j, float4* sv, const float4* sd, float h, float inv_h, bool useBias )
{
	switch ( j->type )
	{
		case b2_revoluteJoint: d_solveRevolute( j, sv, sd, h, inv_h, useBias ); break;
		default: break;
	}
}
