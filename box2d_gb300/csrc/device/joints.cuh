/*
 * Device joint solvers: prepare / warm start / solve per joint, one thread per joint of a
 * graph color, with the reference's operation order: revolute_joint.c:217-500,
 * prismatic_joint.c:295-667, weld_joint.c:148-454 (non-block solver), wheel_joint.c:197-525,
 * distance_joint.c:250-543, motor_joint.c:180-436 and pogo_joint.c:98-281. The parameter slots
 * of b2gJoint are documented in host/joint.c.
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

/* the part of every b2Prepare*Joint shared by all types: masses, awake indices, joint frames
   relative to the centers of mass, and the center delta (revolute_joint.c:217-262 and the
   same lines of the other joint files) */
static __device__ void d_prepareJointFrames( b2gJoint* j, const d_jointBodies* bodies )
{
	int idA = j->bodyIdA, idB = j->bodyIdB;
	float4 xfA = bodies->xf[idA], xfB = bodies->xf[idB];
	b2Rot qA = { xfA.z, xfA.w }, qB = { xfB.z, xfB.w };
	float2 lcA = bodies->localCenter[idA], lcB = bodies->localCenter[idB];
	float2 cA = bodies->center[idA], cB = bodies->center[idB];
	j->invMassA = bodies->invMass[idA];
	j->invMassB = bodies->invMass[idB];
	j->invIA = bodies->invI[idA];
	j->invIB = bodies->invI[idB];
	j->indexA = bodies->awakeIndex[idA];
	j->indexB = bodies->awakeIndex[idB];
	j->frameA.q = d_mulRot( qA, j->localFrameA.q );
	j->frameA.p = d_rotate( qA, d_sub( j->localFrameA.p, d_v( lcA.x, lcA.y ) ) );
	j->frameB.q = d_mulRot( qB, j->localFrameB.q );
	j->frameB.p = d_rotate( qB, d_sub( j->localFrameB.p, d_v( lcB.x, lcB.y ) ) );
	j->deltaCenter = d_v( cB.x - cA.x, cB.y - cA.y );
}

/* revolute_joint.c:217-281 */
static __device__ void d_prepareRevolute( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	float k = j->invIA + j->invIB;
	j->s[6] = k > 0.0f ? 1.0f / k : 0.0f;
	d_makeSoftInto( j->p[1], j->p[2], h, j->s + 7, j->s + 8, j->s + 9 );
	if ( warmStart == false )
	{
		for ( int i = 0; i < 6; ++i ) j->s[i] = 0.0f;
	}
}

struct d_stateRef
{
	float4 v;
	float4 d;
	bool dynamic;
};

template <class TBodies> static __device__ __forceinline__ d_stateRef d_loadState( const TBodies& bodies, int index )
{
	d_stateRef r;
	if ( index < 0 )
	{
		r.v = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		r.d = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		r.dynamic = false;
		return r;
	}
	r.v = bodies.v( index );
	r.d = bodies.d( index );
	r.dynamic = ( __float_as_uint( r.v.w ) & B2G_DYNAMIC_FLAG ) != 0;
	return r;
}

/* revolute_joint.c:283-315 */
template <class TBodies> static __device__ void d_warmStartRevolute( b2gJoint* j, TBodies& bodies )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
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
		bodies.v( j->indexA ) = make_float4( v.x, v.y, w, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, linearImpulse );
		float w = B.v.z;
		w += iB * ( d_cross( rB, linearImpulse ) + axialImpulse );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, w, B.v.w );
	}
}

/* revolute_joint.c:317-500 */
template <class TBodies> static __device__ void d_solveRevolute( b2gJoint* j, TBodies& bodies, float h, float inv_h, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
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
	if ( A.dynamic ) bodies.v( j->indexA ) = make_float4( vA.x, vA.y, wA, A.v.w );
	if ( B.dynamic ) bodies.v( j->indexB ) = make_float4( vB.x, vB.y, wB, B.v.w );
}

/* velocity update of one axial row: P = impulse * axis with lever arms a1, a2 */
static __device__ __forceinline__ void d_applyAxial( b2Vec2* vA, float* wA, b2Vec2* vB, float* wB, float mA, float iA, float mB,
													 float iB, b2Vec2 axis, float a1, float a2, float impulse )
{
	b2Vec2 P = d_mulSV( impulse, axis );
	float LA = impulse * a1;
	float LB = impulse * a2;
	*vA = d_mulSub( *vA, mA, P );
	*wA -= iA * LA;
	*vB = d_mulAdd( *vB, mB, P );
	*wB += iB * LB;
}

template <class TBodies> static __device__ __forceinline__ void d_storeVelocities( TBodies& bodies, const b2gJoint* j, const d_stateRef& A, const d_stateRef& B,
														  b2Vec2 vA, float wA, b2Vec2 vB, float wB )
{
	if ( A.dynamic ) bodies.v( j->indexA ) = make_float4( vA.x, vA.y, wA, A.v.w );
	if ( B.dynamic ) bodies.v( j->indexB ) = make_float4( vB.x, vB.y, wB, B.v.w );
}

/* ---- prismatic (prismatic_joint.c:295-667)
   p: hertz, dampingRatio, targetTranslation, lowerTranslation, upperTranslation,
      maxMotorForce, motorSpeed
   s: impulse.x, impulse.y, springImpulse, motorImpulse, lowerImpulse, upperImpulse,
      spring softness (3) ---- */
static __device__ void d_preparePrismatic( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	d_makeSoftInto( j->p[0], j->p[1], h, j->s + 6, j->s + 7, j->s + 8 );
	if ( warmStart == false )
	{
		for ( int i = 0; i < 6; ++i ) j->s[i] = 0.0f;
	}
}

template <class TBodies> static __device__ void d_warmStartPrismatic( b2gJoint* j, TBodies& bodies )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 d = d_add( d_add( d_sub( d_v( B.d.x, B.d.y ), d_v( A.d.x, A.d.y ) ), j->deltaCenter ), d_sub( rB, rA ) );
	b2Vec2 axisA = d_rotate( j->frameA.q, d_v( 1.0f, 0.0f ) );
	axisA = d_rotate( dqA, axisA );
	float a1 = d_cross( d_add( rA, d ), axisA );
	float a2 = d_cross( rB, axisA );
	float axialImpulse = j->s[2] + j->s[3] + j->s[4] - j->s[5];
	b2Vec2 perpA = d_leftPerp( axisA );
	float s1 = d_cross( d_add( rA, d ), perpA );
	float s2 = d_cross( rB, perpA );
	float perpImpulse = j->s[0];
	float angleImpulse = j->s[1];
	b2Vec2 P = d_add( d_mulSV( axialImpulse, axisA ), d_mulSV( perpImpulse, perpA ) );
	float LA = axialImpulse * a1 + perpImpulse * s1 + angleImpulse;
	float LB = axialImpulse * a2 + perpImpulse * s2 + angleImpulse;
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, P );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, A.v.z - iA * LA, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, P );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, B.v.z + iB * LB, B.v.w );
	}
}

template <class TBodies> static __device__ void d_solvePrismatic( b2gJoint* j, TBodies& bodies, float h, float inv_h, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Rot qA = d_mulRot( dqA, j->frameA.q );
	b2Rot qB = d_mulRot( dqB, j->frameB.q );
	b2Rot relQ = d_invMulRot( qA, qB );
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 d = d_add( d_add( d_sub( d_v( B.d.x, B.d.y ), d_v( A.d.x, A.d.y ) ), j->deltaCenter ), d_sub( rB, rA ) );
	b2Vec2 axisA = d_rotate( j->frameA.q, d_v( 1.0f, 0.0f ) );
	axisA = d_rotate( dqA, axisA );
	float translation = d_dot( axisA, d );
	float a1 = d_cross( d_add( rA, d ), axisA );
	float a2 = d_cross( rB, axisA );
	float k = mA + mB + iA * a1 * a1 + iB * a2 * a2;
	float axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	if ( j->enableSpring )
	{
		float C = translation - j->p[2];
		float bias = j->s[6] * C;
		float massScale = j->s[7];
		float impulseScale = j->s[8];
		float Cdot = d_dot( axisA, d_sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float deltaImpulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * j->s[2];
		j->s[2] += deltaImpulse;
		d_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, deltaImpulse );
	}
	if ( j->enableMotor )
	{
		float Cdot = d_dot( axisA, d_sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = axialMass * ( j->p[6] - Cdot );
		float oldImpulse = j->s[3];
		float maxImpulse = h * j->p[5];
		j->s[3] = d_clamp( j->s[3] + impulse, -maxImpulse, maxImpulse );
		impulse = j->s[3] - oldImpulse;
		d_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, impulse );
	}
	if ( j->enableLimit )
	{
		float speculativeDistance = 0.25f * ( j->p[4] - j->p[3] );
		{
			float C = translation - j->p[3];
			if ( C < speculativeDistance )
			{
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f ) bias = d_min( C, 1.0f ) * inv_h;
				else if ( useBias )
				{
					bias = j->softBias * C;
					massScale = j->softMass;
					impulseScale = j->softImpulse;
				}
				float oldImpulse = j->s[4];
				float Cdot = d_dot( axisA, d_sub( vB, vA ) ) + a2 * wB - a1 * wA;
				float deltaImpulse = -axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
				j->s[4] = d_max( oldImpulse + deltaImpulse, 0.0f );
				deltaImpulse = j->s[4] - oldImpulse;
				d_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, deltaImpulse );
			}
			else
			{
				j->s[4] = 0.0f;
			}
		}
		{
			float C = j->p[4] - translation;
			if ( C < speculativeDistance )
			{
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f ) bias = d_min( C, 1.0f ) * inv_h;
				else if ( useBias )
				{
					bias = j->softBias * C;
					massScale = j->softMass;
					impulseScale = j->softImpulse;
				}
				float oldImpulse = j->s[5];
				float Cdot = d_dot( axisA, d_sub( vA, vB ) ) + a1 * wA - a2 * wB;
				float deltaImpulse = -axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
				j->s[5] = d_max( oldImpulse + deltaImpulse, 0.0f );
				deltaImpulse = j->s[5] - oldImpulse;
				b2Vec2 P = d_mulSV( deltaImpulse, axisA );
				float LA = deltaImpulse * a1;
				float LB = deltaImpulse * a2;
				vA = d_mulAdd( vA, mA, P );
				wA += iA * LA;
				vB = d_mulSub( vB, mB, P );
				wB -= iB * LB;
			}
			else
			{
				j->s[5] = 0.0f;
			}
		}
	}
	{
		b2Vec2 perpA = d_leftPerp( axisA );
		float s1 = d_cross( d_add( d, rA ), perpA );
		float s2 = d_cross( rB, perpA );
		b2Vec2 Cdot;
		Cdot.x = d_dot( perpA, d_sub( vB, vA ) ) + s2 * wB - s1 * wA;
		Cdot.y = wB - wA;
		b2Vec2 bias = { 0.0f, 0.0f };
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			b2Vec2 C;
			C.x = d_dot( perpA, d );
			C.y = d_atan2( relQ.s, relQ.c );
			bias = d_mulSV( j->softBias, C );
			massScale = j->softMass;
			impulseScale = j->softImpulse;
		}
		float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
		float k12 = iA * s1 + iB * s2;
		float k22 = iA + iB;
		if ( k22 == 0.0f ) k22 = 1.0f;
		b2Vec2 b = d_solve22( k11, k12, k12, k22, d_add( Cdot, bias ) );
		b2Vec2 deltaImpulse;
		deltaImpulse.x = -massScale * b.x - impulseScale * j->s[0];
		deltaImpulse.y = -massScale * b.y - impulseScale * j->s[1];
		j->s[0] += deltaImpulse.x;
		j->s[1] += deltaImpulse.y;
		b2Vec2 P = d_mulSV( deltaImpulse.x, perpA );
		float LA = deltaImpulse.x * s1 + deltaImpulse.y;
		float LB = deltaImpulse.x * s2 + deltaImpulse.y;
		vA = d_mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = d_mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	d_storeVelocities( bodies, j, A, B, vA, wA, vB, wB );
}

/* ---- weld (weld_joint.c:148-454, the non-block solver)
   p: linearHertz, linearDampingRatio, angularHertz, angularDampingRatio
   s: linearImpulse.x, linearImpulse.y, angularImpulse, axialMass, linear softness (3),
      angular softness (3) ---- */
static __device__ void d_prepareWeld( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	float ka = j->invIA + j->invIB;
	j->s[3] = ka > 0.0f ? 1.0f / ka : 0.0f;
	if ( j->p[0] == 0.0f )
	{
		j->s[4] = j->softBias;
		j->s[5] = j->softMass;
		j->s[6] = j->softImpulse;
	}
	else
	{
		d_makeSoftInto( j->p[0], j->p[1], h, j->s + 4, j->s + 5, j->s + 6 );
	}
	if ( j->p[2] == 0.0f )
	{
		j->s[7] = j->softBias;
		j->s[8] = j->softMass;
		j->s[9] = j->softImpulse;
	}
	else
	{
		d_makeSoftInto( j->p[2], j->p[3], h, j->s + 7, j->s + 8, j->s + 9 );
	}
	if ( warmStart == false )
	{
		j->s[0] = 0.0f;
		j->s[1] = 0.0f;
		j->s[2] = 0.0f;
	}
}

template <class TBodies> static __device__ void d_warmStartWeld( b2gJoint* j, TBodies& bodies )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 linearImpulse = { j->s[0], j->s[1] };
	float angularImpulse = j->s[2];
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, linearImpulse );
		float w = A.v.z - iA * ( d_cross( rA, linearImpulse ) + angularImpulse );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, w, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, linearImpulse );
		float w = B.v.z + iB * ( d_cross( rB, linearImpulse ) + angularImpulse );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, w, B.v.w );
	}
}

template <class TBodies> static __device__ void d_solveWeld( b2gJoint* j, TBodies& bodies, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	{
		b2Rot qA = d_mulRot( dqA, j->frameA.q );
		b2Rot qB = d_mulRot( dqB, j->frameB.q );
		b2Rot relQ = d_invMulRot( qA, qB );
		float jointAngle = d_atan2( relQ.s, relQ.c );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->p[2] > 0.0f )
		{
			float C = jointAngle;
			bias = j->s[7] * C;
			massScale = j->s[8];
			impulseScale = j->s[9];
		}
		float Cdot = wB - wA;
		float impulse = -massScale * j->s[3] * ( Cdot + bias ) - impulseScale * j->s[2];
		j->s[2] += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		b2Vec2 rA = d_rotate( dqA, j->frameA.p );
		b2Vec2 rB = d_rotate( dqB, j->frameB.p );
		b2Vec2 bias = { 0.0f, 0.0f };
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->p[0] > 0.0f )
		{
			b2Vec2 dcA = { A.d.x, A.d.y }, dcB = { B.d.x, B.d.y };
			b2Vec2 C = d_add( d_add( d_sub( dcB, dcA ), d_sub( rB, rA ) ), j->deltaCenter );
			bias = d_mulSV( j->s[4], C );
			massScale = j->s[5];
			impulseScale = j->s[6];
		}
		b2Vec2 Cdot = d_sub( d_add( vB, d_crossSV( wB, rB ) ), d_add( vA, d_crossSV( wA, rA ) ) );
		float k11 = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		float k12 = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		float k22 = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		b2Vec2 b = d_solve22( k11, k12, k12, k22, d_add( Cdot, bias ) );
		b2Vec2 impulse = { -massScale * b.x - impulseScale * j->s[0], -massScale * b.y - impulseScale * j->s[1] };
		j->s[0] += impulse.x;
		j->s[1] += impulse.y;
		vA = d_mulSub( vA, mA, impulse );
		wA -= iA * d_cross( rA, impulse );
		vB = d_mulAdd( vB, mB, impulse );
		wB += iB * d_cross( rB, impulse );
	}
	d_storeVelocities( bodies, j, A, B, vA, wA, vB, wB );
}

/* ---- wheel (wheel_joint.c:197-525)
   p: lowerTranslation, upperTranslation, maxMotorTorque, motorSpeed, hertz, dampingRatio
   s: perpImpulse, motorImpulse, springImpulse, lowerImpulse, upperImpulse, perpMass,
      motorMass, axialMass, spring softness (3) ---- */
static __device__ void d_prepareWheel( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2Vec2 rA = j->frameA.p, rB = j->frameB.p;
	b2Vec2 d = d_add( j->deltaCenter, d_sub( rB, rA ) );
	b2Vec2 axisA = d_rotate( j->frameA.q, d_v( 1.0f, 0.0f ) );
	b2Vec2 perpA = d_leftPerp( axisA );
	float s1 = d_cross( d_add( d, rA ), perpA );
	float s2 = d_cross( rB, perpA );
	float kp = mA + mB + iA * s1 * s1 + iB * s2 * s2;
	j->s[5] = kp > 0.0f ? 1.0f / kp : 0.0f;
	float a1 = d_cross( d_add( d, rA ), axisA );
	float a2 = d_cross( rB, axisA );
	float ka = mA + mB + iA * a1 * a1 + iB * a2 * a2;
	j->s[7] = ka > 0.0f ? 1.0f / ka : 0.0f;
	d_makeSoftInto( j->p[4], j->p[5], h, j->s + 8, j->s + 9, j->s + 10 );
	float km = iA + iB;
	j->s[6] = km > 0.0f ? 1.0f / km : 0.0f;
	if ( warmStart == false )
	{
		for ( int i = 0; i < 5; ++i ) j->s[i] = 0.0f;
	}
}

template <class TBodies> static __device__ void d_warmStartWheel( b2gJoint* j, TBodies& bodies )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 d = d_add( d_add( d_sub( d_v( B.d.x, B.d.y ), d_v( A.d.x, A.d.y ) ), j->deltaCenter ), d_sub( rB, rA ) );
	b2Vec2 axisA = d_rotate( j->frameA.q, d_v( 1.0f, 0.0f ) );
	axisA = d_rotate( dqA, axisA );
	b2Vec2 perpA = d_leftPerp( axisA );
	float a1 = d_cross( d_add( d, rA ), axisA );
	float a2 = d_cross( rB, axisA );
	float s1 = d_cross( d_add( d, rA ), perpA );
	float s2 = d_cross( rB, perpA );
	float axialImpulse = j->s[2] + j->s[3] - j->s[4];
	b2Vec2 P = d_add( d_mulSV( axialImpulse, axisA ), d_mulSV( j->s[0], perpA ) );
	float LA = axialImpulse * a1 + j->s[0] * s1 + j->s[1];
	float LB = axialImpulse * a2 + j->s[0] * s2 + j->s[1];
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, P );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, A.v.z - iA * LA, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, P );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, B.v.z + iB * LB, B.v.w );
	}
}

template <class TBodies> static __device__ void d_solveWheel( b2gJoint* j, TBodies& bodies, float h, float inv_h, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	bool fixedRotation = ( iA + iB == 0.0f );
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 d = d_add( d_add( d_sub( d_v( B.d.x, B.d.y ), d_v( A.d.x, A.d.y ) ), j->deltaCenter ), d_sub( rB, rA ) );
	b2Vec2 axisA = d_rotate( j->frameA.q, d_v( 1.0f, 0.0f ) );
	axisA = d_rotate( dqA, axisA );
	float translation = d_dot( axisA, d );
	float a1 = d_cross( d_add( d, rA ), axisA );
	float a2 = d_cross( rB, axisA );
	if ( j->enableMotor && fixedRotation == false )
	{
		float Cdot = wB - wA - j->p[3];
		float impulse = -j->s[6] * Cdot;
		float oldImpulse = j->s[1];
		float maxImpulse = h * j->p[2];
		j->s[1] = d_clamp( j->s[1] + impulse, -maxImpulse, maxImpulse );
		impulse = j->s[1] - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableSpring )
	{
		float C = translation;
		float bias = j->s[8] * C;
		float massScale = j->s[9];
		float impulseScale = j->s[10];
		float Cdot = d_dot( axisA, d_sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = -massScale * j->s[7] * ( Cdot + bias ) - impulseScale * j->s[2];
		j->s[2] += impulse;
		d_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, impulse );
	}
	if ( j->enableLimit )
	{
		{
			float C = translation - j->p[0];
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->softBias * C;
				massScale = j->softMass;
				impulseScale = j->softImpulse;
			}
			float Cdot = d_dot( axisA, d_sub( vB, vA ) ) + a2 * wB - a1 * wA;
			float impulse = -massScale * j->s[7] * ( Cdot + bias ) - impulseScale * j->s[3];
			float oldImpulse = j->s[3];
			j->s[3] = d_max( oldImpulse + impulse, 0.0f );
			impulse = j->s[3] - oldImpulse;
			d_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, axisA, a1, a2, impulse );
		}
		{
			float C = j->p[1] - translation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f ) bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->softBias * C;
				massScale = j->softMass;
				impulseScale = j->softImpulse;
			}
			float Cdot = d_dot( axisA, d_sub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -massScale * j->s[7] * ( Cdot + bias ) - impulseScale * j->s[4];
			float oldImpulse = j->s[4];
			j->s[4] = d_max( oldImpulse + impulse, 0.0f );
			impulse = j->s[4] - oldImpulse;
			b2Vec2 P = d_mulSV( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = d_mulAdd( vA, mA, P );
			wA += iA * LA;
			vB = d_mulSub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		b2Vec2 perpA = d_leftPerp( axisA );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			float C = d_dot( perpA, d );
			bias = j->softBias * C;
			massScale = j->softMass;
			impulseScale = j->softImpulse;
		}
		float s1 = d_cross( d_add( d, rA ), perpA );
		float s2 = d_cross( rB, perpA );
		float Cdot = d_dot( perpA, d_sub( vB, vA ) ) + s2 * wB - s1 * wA;
		float impulse = -massScale * j->s[5] * ( Cdot + bias ) - impulseScale * j->s[0];
		j->s[0] += impulse;
		d_applyAxial( &vA, &wA, &vB, &wB, mA, iA, mB, iB, perpA, s1, s2, impulse );
	}
	d_storeVelocities( bodies, j, A, B, vA, wA, vB, wB );
}

/* ---- distance (distance_joint.c:250-543); the anchors are the frames' origins
   p: length, hertz, dampingRatio, lowerSpringForce, upperSpringForce, minLength,
      maxLength, maxMotorForce, motorSpeed
   s: impulse, lowerImpulse, upperImpulse, motorImpulse, axialMass, distance softness (3) ---- */
static __device__ void d_prepareDistance( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2Vec2 rA = j->frameA.p, rB = j->frameB.p;
	b2Vec2 separation = d_add( d_sub( rB, rA ), j->deltaCenter );
	b2Vec2 axis = d_normalize( separation );
	float crA = d_cross( rA, axis );
	float crB = d_cross( rB, axis );
	float k = mA + mB + iA * crA * crA + iB * crB * crB;
	j->s[4] = k > 0.0f ? 1.0f / k : 0.0f;
	d_makeSoftInto( j->p[1], j->p[2], h, j->s + 5, j->s + 6, j->s + 7 );
	if ( warmStart == false )
	{
		for ( int i = 0; i < 4; ++i ) j->s[i] = 0.0f;
	}
}

template <class TBodies> static __device__ void d_warmStartDistance( b2gJoint* j, TBodies& bodies )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 ds = d_add( d_sub( d_v( B.d.x, B.d.y ), d_v( A.d.x, A.d.y ) ), d_sub( rB, rA ) );
	b2Vec2 separation = d_add( j->deltaCenter, ds );
	b2Vec2 axis = d_normalize( separation );
	float axialImpulse = j->s[0] + j->s[1] - j->s[2] + j->s[3];
	b2Vec2 P = d_mulSV( axialImpulse, axis );
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, P );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, A.v.z - iA * d_cross( rA, P ), A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, P );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, B.v.z + iB * d_cross( rB, P ), B.v.w );
	}
}

static __device__ __forceinline__ void d_applyLinear( b2Vec2* vA, float* wA, b2Vec2* vB, float* wB, float mA, float iA, float mB,
													  float iB, b2Vec2 rA, b2Vec2 rB, b2Vec2 P )
{
	*vA = d_mulSub( *vA, mA, P );
	*wA -= iA * d_cross( rA, P );
	*vB = d_mulAdd( *vB, mB, P );
	*wB += iB * d_cross( rB, P );
}

template <class TBodies> static __device__ void d_solveDistance( b2gJoint* j, TBodies& bodies, float h, float inv_h, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 ds = d_add( d_sub( d_v( B.d.x, B.d.y ), d_v( A.d.x, A.d.y ) ), d_sub( rB, rA ) );
	b2Vec2 separation = d_add( j->deltaCenter, ds );
	float length = d_length( separation );
	b2Vec2 axis = d_normalize( separation );
	float axialMass = j->s[4];
	if ( j->enableSpring && ( j->p[5] < j->p[6] || j->enableLimit == 0 ) )
	{
		if ( j->p[1] > 0.0f )
		{
			b2Vec2 vr = d_add( d_sub( vB, vA ), d_sub( d_crossSV( wB, rB ), d_crossSV( wA, rA ) ) );
			float cdot = d_dot( axis, vr );
			float c = length - j->p[0];
			float bias = j->s[5] * c;
			float m = j->s[6] * axialMass;
			float oldImpulse = j->s[0];
			float impulse = -m * ( cdot + bias ) - j->s[7] * oldImpulse;
			j->s[0] = d_clamp( j->s[0] + impulse, j->p[3] * h, j->p[4] * h );
			impulse = j->s[0] - oldImpulse;
			d_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, d_mulSV( impulse, axis ) );
		}
		if ( j->enableMotor )
		{
			b2Vec2 vr = d_add( d_sub( vB, vA ), d_sub( d_crossSV( wB, rB ), d_crossSV( wA, rA ) ) );
			float Cdot = d_dot( axis, vr );
			float impulse = axialMass * ( j->p[8] - Cdot );
			float oldImpulse = j->s[3];
			float maxImpulse = h * j->p[7];
			j->s[3] = d_clamp( j->s[3] + impulse, -maxImpulse, maxImpulse );
			impulse = j->s[3] - oldImpulse;
			d_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, d_mulSV( impulse, axis ) );
		}
		if ( j->enableLimit )
		{
			{
				b2Vec2 vr = d_add( d_sub( vB, vA ), d_sub( d_crossSV( wB, rB ), d_crossSV( wA, rA ) ) );
				float cdot = d_dot( axis, vr );
				float c = length - j->p[5];
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( c > 0.0f ) bias = c * inv_h;
				else if ( useBias )
				{
					bias = j->softBias * c;
					massScale = j->softMass;
					impulseScale = j->softImpulse;
				}
				float impulse = -massScale * axialMass * ( cdot + bias ) - impulseScale * j->s[1];
				float newImpulse = d_max( 0.0f, j->s[1] + impulse );
				impulse = newImpulse - j->s[1];
				j->s[1] = newImpulse;
				d_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, d_mulSV( impulse, axis ) );
			}
			{
				b2Vec2 vr = d_add( d_sub( vA, vB ), d_sub( d_crossSV( wA, rA ), d_crossSV( wB, rB ) ) );
				float Cdot = d_dot( axis, vr );
				float C = j->p[6] - length;
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f ) bias = C * inv_h;
				else if ( useBias )
				{
					bias = j->softBias * C;
					massScale = j->softMass;
					impulseScale = j->softImpulse;
				}
				float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * j->s[2];
				float newImpulse = d_max( 0.0f, j->s[2] + impulse );
				impulse = newImpulse - j->s[2];
				j->s[2] = newImpulse;
				d_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, d_mulSV( -impulse, axis ) );
			}
		}
	}
	else
	{
		b2Vec2 vr = d_add( d_sub( vB, vA ), d_sub( d_crossSV( wB, rB ), d_crossSV( wA, rA ) ) );
		float Cdot = d_dot( axis, vr );
		float C = length - j->p[0];
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			bias = j->softBias * C;
			massScale = j->softMass;
			impulseScale = j->softImpulse;
		}
		float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * j->s[0];
		j->s[0] += impulse;
		d_applyLinear( &vA, &wA, &vB, &wB, mA, iA, mB, iB, rA, rB, d_mulSV( impulse, axis ) );
	}
	d_storeVelocities( bodies, j, A, B, vA, wA, vB, wB );
}

/* ---- motor (motor_joint.c:180-436)
   p: linearVelocity (2), maxVelocityForce, angularVelocity, maxVelocityTorque, linearHertz,
      linearDampingRatio, maxSpringForce, angularHertz, angularDampingRatio, maxSpringTorque,
      angular spring softness (3, written by prepare)
   s: linearVelocityImpulse (2), angularVelocityImpulse, linearSpringImpulse (2),
      angularSpringImpulse, linearMass (b2Mat22 cx, cy), angularMass, linear spring softness (3) ---- */
static __device__ __forceinline__ void d_motorLinearMass( b2gJoint* j, float mA, float mB, float iA, float iB, b2Vec2 rA, b2Vec2 rB )
{
	/* math_functions.h b2GetInverse22 of the point-to-point mass */
	float a = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
	float c = -rA.y * rA.x * iA - rB.y * rB.x * iB;
	float b = c;
	float d = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
	float det = a * d - b * c;
	if ( det != 0.0f ) det = 1.0f / det;
	j->s[6] = det * d;
	j->s[7] = -det * c;
	j->s[8] = -det * b;
	j->s[9] = det * a;
}

/* math_functions.h b2MulMV with the stored linear mass */
static __device__ __forceinline__ b2Vec2 d_motorMulMass( const b2gJoint* j, b2Vec2 v )
{
	return d_v( j->s[6] * v.x + j->s[8] * v.y, j->s[7] * v.x + j->s[9] * v.y );
}

static __device__ void d_prepareMotor( b2gJoint* j, const d_jointBodies* bodies, float h, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	d_makeSoftInto( j->p[5], j->p[6], h, j->s + 11, j->s + 12, j->s + 13 );
	d_makeSoftInto( j->p[8], j->p[9], h, j->p + 11, j->p + 12, j->p + 13 );
	d_motorLinearMass( j, j->invMassA, j->invMassB, j->invIA, j->invIB, j->frameA.p, j->frameB.p );
	float ka = j->invIA + j->invIB;
	j->s[10] = ka > 0.0f ? 1.0f / ka : 0.0f;
	if ( warmStart == false )
	{
		for ( int i = 0; i < 6; ++i ) j->s[i] = 0.0f;
	}
}

template <class TBodies> static __device__ void d_warmStartMotor( b2gJoint* j, TBodies& bodies )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 linearImpulse = d_add( d_v( j->s[0], j->s[1] ), d_v( j->s[3], j->s[4] ) );
	float angularImpulse = j->s[2] + j->s[5];
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, linearImpulse );
		float w = A.v.z - iA * ( d_cross( rA, linearImpulse ) + angularImpulse );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, w, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, linearImpulse );
		float w = B.v.z + iB * ( d_cross( rB, linearImpulse ) + angularImpulse );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, w, B.v.w );
	}
}

/* add `impulse` to the accumulated impulse at s[k], s[k + 1] and clamp its length to
   maxImpulse (motor_joint.c:383-392); returns the applied change */
static __device__ __forceinline__ b2Vec2 d_motorAccumulate( b2gJoint* j, int k, b2Vec2 impulse, float maxImpulse )
{
	b2Vec2 old = d_v( j->s[k], j->s[k + 1] );
	b2Vec2 acc = d_add( old, impulse );
	if ( d_lengthSq( acc ) > maxImpulse * maxImpulse )
	{
		acc = d_normalize( acc );
		acc.x *= maxImpulse;
		acc.y *= maxImpulse;
	}
	j->s[k] = acc.x;
	j->s[k + 1] = acc.y;
	return d_sub( acc, old );
}

/* solve and relax are the same pass for the motor joint (joint.c:1506-1508) */
template <class TBodies> static __device__ void d_solveMotor( b2gJoint* j, TBodies& bodies, float h )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	if ( j->p[10] > 0.0f && j->p[8] > 0.0f )
	{
		b2Rot qA = d_mulRot( dqA, j->frameA.q );
		b2Rot qB = d_mulRot( dqB, j->frameB.q );
		b2Rot relQ = d_invMulRot( qA, qB );
		float c = d_atan2( relQ.s, relQ.c );
		float bias = j->p[11] * c;
		float massScale = j->p[12];
		float impulseScale = j->p[13];
		float cdot = wB - wA;
		float maxImpulse = h * j->p[10];
		float oldImpulse = j->s[5];
		float impulse = -massScale * j->s[10] * ( cdot + bias ) - impulseScale * oldImpulse;
		j->s[5] = d_clamp( oldImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->s[5] - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->p[4] > 0.0f )
	{
		float cdot = wB - wA - j->p[3];
		float impulse = -j->s[10] * cdot;
		float maxImpulse = h * j->p[4];
		float oldImpulse = j->s[2];
		j->s[2] = d_clamp( oldImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->s[2] - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	if ( j->p[7] > 0.0f && j->p[5] > 0.0f )
	{
		b2Vec2 dcA = { A.d.x, A.d.y }, dcB = { B.d.x, B.d.y };
		b2Vec2 c = d_add( d_add( d_sub( dcB, dcA ), d_sub( rB, rA ) ), j->deltaCenter );
		b2Vec2 bias = d_mulSV( j->s[11], c );
		float massScale = j->s[12];
		float impulseScale = j->s[13];
		b2Vec2 cdot = d_sub( d_add( vB, d_crossSV( wB, rB ) ), d_add( vA, d_crossSV( wA, rA ) ) );
		cdot = d_add( cdot, bias );
		d_motorLinearMass( j, mA, mB, iA, iB, rA, rB );
		b2Vec2 b = d_motorMulMass( j, cdot );
		b2Vec2 impulse = d_v( -massScale * b.x - impulseScale * j->s[3], -massScale * b.y - impulseScale * j->s[4] );
		impulse = d_motorAccumulate( j, 3, impulse, h * j->p[7] );
		vA = d_mulSub( vA, mA, impulse );
		wA -= iA * d_cross( rA, impulse );
		vB = d_mulAdd( vB, mB, impulse );
		wB += iB * d_cross( rB, impulse );
	}
	if ( j->p[2] > 0.0f )
	{
		b2Vec2 cdot = d_sub( d_add( vB, d_crossSV( wB, rB ) ), d_add( vA, d_crossSV( wA, rA ) ) );
		cdot = d_sub( cdot, d_v( j->p[0], j->p[1] ) );
		b2Vec2 b = d_motorMulMass( j, cdot );
		b2Vec2 impulse = d_motorAccumulate( j, 0, d_v( -b.x, -b.y ), h * j->p[2] );
		vA = d_mulSub( vA, mA, impulse );
		wA -= iA * d_cross( rA, impulse );
		vB = d_mulAdd( vB, mB, impulse );
		wB += iB * d_cross( rB, impulse );
	}
	d_storeVelocities( bodies, j, A, B, vA, wA, vB, wB );
}

/* ---- mover (mover_joint.c:43-170): linear velocity only, the bodies' rotation untouched
   p: linearVelocity (2), maxVelocityForce (2)
   s: linearVelocityImpulse (2), linearMass ---- */
static __device__ void d_prepareMover( b2gJoint* j, const d_jointBodies* bodies, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	j->invIA = 0.0f;
	j->invIB = 0.0f;
	float k = j->invMassA + j->invMassB;
	j->s[2] = k > 0.0f ? 1.0f / k : 0.0f;
	if ( warmStart == false )
	{
		j->s[0] = 0.0f;
		j->s[1] = 0.0f;
	}
}

template <class TBodies> static __device__ void d_warmStartMover( b2gJoint* j, TBodies& bodies )
{
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 P = { j->s[0], j->s[1] };
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), j->invMassA, P );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, A.v.z, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), j->invMassB, P );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, B.v.z, B.v.w );
	}
}

template <class TBodies> static __device__ void d_solveMover( b2gJoint* j, TBodies& bodies, float h )
{
	float mA = j->invMassA, mB = j->invMassB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	if ( j->p[2] > 0.0f || j->p[3] > 0.0f )
	{
		b2Vec2 cdot = d_sub( d_sub( vB, vA ), d_v( j->p[0], j->p[1] ) );
		b2Vec2 b = d_mulSV( j->s[2], cdot );
		b2Vec2 old = { j->s[0], j->s[1] };
		b2Vec2 acc = d_add( old, d_v( -b.x, -b.y ) );
		/* x and y clamped separately (math_functions.h b2Clamp) */
		float mx = h * j->p[2], my = h * j->p[3];
		acc.x = d_clamp( acc.x, -mx, mx );
		acc.y = d_clamp( acc.y, -my, my );
		j->s[0] = acc.x;
		j->s[1] = acc.y;
		b2Vec2 impulse = d_sub( acc, old );
		vA = d_mulSub( vA, mA, impulse );
		vB = d_mulAdd( vB, mB, impulse );
	}
	else
	{
		j->s[0] = 0.0f;
		j->s[1] = 0.0f;
	}
	if ( A.dynamic ) bodies.v( j->indexA ) = make_float4( vA.x, vA.y, A.v.z, A.v.w );
	if ( B.dynamic ) bodies.v( j->indexB ) = make_float4( vB.x, vB.y, B.v.z, B.v.w );
}

/* ---- pogo (pogo_joint.c:98-281)
   p: normal (2), hertz, dampingRatio, restLength, maxTensionForce, maxCompressionForce
   s: impulse, velocity (the spring's internal velocity), linearMass ---- */
static __device__ void d_preparePogo( b2gJoint* j, const d_jointBodies* bodies, bool warmStart )
{
	d_prepareJointFrames( j, bodies );
	b2Vec2 normal = { j->p[0], j->p[1] };
	float crA = d_cross( j->frameA.p, normal );
	float crB = d_cross( j->frameB.p, normal );
	float k = j->invMassA + j->invMassB + j->invIA * crA * crA + j->invIB * crB * crB;
	j->s[2] = k > 0.0f ? 1.0f / k : 0.0f;
	if ( warmStart == false ) j->s[0] = 0.0f;
}

template <class TBodies> static __device__ void d_warmStartPogo( b2gJoint* j, TBodies& bodies )
{
	if ( j->p[2] == 0.0f )
	{
		j->s[0] = 0.0f;
		return;
	}
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 P = d_mulSV( j->s[0], d_v( j->p[0], j->p[1] ) );
	if ( A.dynamic )
	{
		b2Vec2 v = d_mulSub( d_v( A.v.x, A.v.y ), mA, P );
		float w = A.v.z - iA * d_cross( rA, P );
		bodies.v( j->indexA ) = make_float4( v.x, v.y, w, A.v.w );
	}
	if ( B.dynamic )
	{
		b2Vec2 v = d_mulAdd( d_v( B.v.x, B.v.y ), mB, P );
		float w = B.v.z + iB * d_cross( rB, P );
		bodies.v( j->indexB ) = make_float4( v.x, v.y, w, B.v.w );
	}
}

template <class TBodies> static __device__ void d_solvePogo( b2gJoint* j, TBodies& bodies, float h, bool useBias )
{
	if ( j->p[2] == 0.0f )
	{
		j->s[0] = 0.0f;
		return;
	}
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	d_stateRef A = d_loadState( bodies, j->indexA ), B = d_loadState( bodies, j->indexB );
	b2Vec2 vA = { A.v.x, A.v.y }, vB = { B.v.x, B.v.y };
	float wA = A.v.z, wB = B.v.z;
	b2Rot dqA = { A.d.z, A.d.w }, dqB = { B.d.z, B.d.w };
	b2Vec2 rA = d_rotate( dqA, j->frameA.p );
	b2Vec2 rB = d_rotate( dqB, j->frameB.p );
	b2Vec2 normal = { j->p[0], j->p[1] };
	float bias = 0.0f;
	if ( useBias )
	{
		b2Vec2 dcA = { A.d.x, A.d.y }, dcB = { B.d.x, B.d.y };
		b2Vec2 d = d_add( d_add( d_sub( dcB, dcA ), d_sub( rB, rA ) ), j->deltaCenter );
		/* the pogo axis is frame B's y axis (pogo_joint.c:14) */
		b2Vec2 pogoAxis = d_rotate( j->frameB.q, d_v( 0.0f, 1.0f ) );
		float c = d_dot( pogoAxis, d ) - j->p[4];
		/* math_functions.h b2SpringDamper */
		float omega = 2.0f * B2_PI * j->p[2];
		float omegaH = omega * h;
		j->s[1] = ( j->s[1] - omega * omegaH * c ) / ( 1.0f + 2.0f * j->p[3] * omegaH + omegaH * omegaH );
		bias = -j->s[1];
	}
	b2Vec2 vr = d_sub( d_add( vB, d_crossSV( wB, rB ) ), d_add( vA, d_crossSV( wA, rA ) ) );
	float cdot = d_dot( normal, vr );
	float maxTensionImpulse = h * j->p[5];
	float maxCompressionImpulse = h * j->p[6];
	float oldImpulse = j->s[0];
	float impulse = -j->s[2] * ( cdot + bias );
	j->s[0] = d_clamp( j->s[0] + impulse, -maxTensionImpulse, maxCompressionImpulse );
	impulse = j->s[0] - oldImpulse;
	b2Vec2 P = d_mulSV( impulse, normal );
	vA = d_mulSub( vA, mA, P );
	wA -= iA * d_cross( rA, P );
	vB = d_mulAdd( vB, mB, P );
	wB += iB * d_cross( rB, P );
	d_storeVelocities( bodies, j, A, B, vA, wA, vB, wB );
}

/* joint.c:1406-1540 dispatch */
static __device__ void d_prepareJoint( b2gJoint* j, const d_jointBodies* bodies, float h, float inv_h, bool warmStart )
{
	float hertz = d_min( j->constraintHertz, 0.25f * inv_h );
	d_makeSoftInto( hertz, j->constraintDampingRatio, h, &j->softBias, &j->softMass, &j->softImpulse );
	switch ( j->type )
	{
		case b2_distanceJoint: d_prepareDistance( j, bodies, h, warmStart ); break;
		case b2_prismaticJoint: d_preparePrismatic( j, bodies, h, warmStart ); break;
		case b2_revoluteJoint: d_prepareRevolute( j, bodies, h, warmStart ); break;
		case b2_weldJoint: d_prepareWeld( j, bodies, h, warmStart ); break;
		case b2_wheelJoint: d_prepareWheel( j, bodies, h, warmStart ); break;
		case b2_motorJoint: d_prepareMotor( j, bodies, h, warmStart ); break;
		case b2_pogoJoint: d_preparePogo( j, bodies, warmStart ); break;
		case b2_moverJoint: d_prepareMover( j, bodies, warmStart ); break;
		default: break; /* filter joints have no constraint */
	}
}

template <class TBodies> static __device__ void d_warmStartJoint( b2gJoint* j, TBodies& bodies )
{
	switch ( j->type )
	{
		case b2_distanceJoint: d_warmStartDistance( j, bodies ); break;
		case b2_prismaticJoint: d_warmStartPrismatic( j, bodies ); break;
		case b2_revoluteJoint: d_warmStartRevolute( j, bodies ); break;
		case b2_weldJoint: d_warmStartWeld( j, bodies ); break;
		case b2_wheelJoint: d_warmStartWheel( j, bodies ); break;
		case b2_motorJoint: d_warmStartMotor( j, bodies ); break;
		case b2_pogoJoint: d_warmStartPogo( j, bodies ); break;
		case b2_moverJoint: d_warmStartMover( j, bodies ); break;
		default: break;
	}
}

template <class TBodies> static __device__ void d_solveJoint( b2gJoint* j, TBodies& bodies, float h, float inv_h, bool useBias )
{
	switch ( j->type )
	{
		case b2_distanceJoint: d_solveDistance( j, bodies, h, inv_h, useBias ); break;
		case b2_prismaticJoint: d_solvePrismatic( j, bodies, h, inv_h, useBias ); break;
		case b2_revoluteJoint: d_solveRevolute( j, bodies, h, inv_h, useBias ); break;
		case b2_weldJoint: d_solveWeld( j, bodies, useBias ); break;
		case b2_wheelJoint: d_solveWheel( j, bodies, h, inv_h, useBias ); break;
		case b2_motorJoint: d_solveMotor( j, bodies, h ); break;
		case b2_pogoJoint: d_solvePogo( j, bodies, h, useBias ); break;
		case b2_moverJoint: d_solveMover( j, bodies, h ); break;
		default: break;
	}
}
