/*
 * Adjoint of the recorded Soft Step (differentiable stepping, box2d_gb300_diff.h).
 *
 * One CTA per world and one launch per recorded step, last step first. For step n a CTA
 *   1. rebuilds the contact constraints from the recorded manifolds with the forward's own
 *      prepare function and replays the substeps with the forward's lane functions
 *      (bit-identical: same code, same color order), keeping a checkpoint of body and
 *      constraint state at the start of every substep;
 *   2. runs the adjoint of finalize (solver.c:553-600), store and restitution;
 *   3. for each substep, last first: replays it from its checkpoint keeping the inputs of
 *      every color stage, then sweeps relax, integrate positions, solve, warm start and
 *      integrate velocities backwards, colors in reverse order (contact_solver.c:1811-2228,
 *      solver.c:66-162);
 *   4. runs the adjoint of prepare (contact_solver.c:1573-1809) and of the narrowphase
 *      (contact.c:519-698 through a dual-number evaluation of b2CollidePolygons,
 *      b2CollidePolygonAndCircle or b2CollideCircles; for a
 *      recycled manifold, the separation update of physics_world.c:508-560), and hands the
 *      manifold and warm-start adjoints of each contact to step n - 1 by contact id.
 * Branches (clamps, speculative or soft contact, friction cone, speed caps, clip and edge
 * choices) follow the recorded trajectory: the derivative is that of the branch taken.
 */
#include "box2d_gb300_diff.h"
#include "diff_collide.h"
#include "stages.cuh"

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define B2G_ADJ_THREADS 128
#define B2G_ADJ_MAX_SUBSTEPS 16

/* impulses of one contact constraint (both points), as snapshots and checkpoints hold them */
struct d_laneImp
{
	float n1, n2, t1, t2, tot1, tot2, roll;
};

/* adjoint of a contact constraint's fields */
struct d_laneAdj
{
	float rA1x, rA1y, rB1x, rB1y, rA2x, rA2y, rB2x, rB2y;
	float nx, ny;
	float base1, base2, nm1, nm2, tm1, tm2, rv1, rv2;
	float n1, n2, t1, t2;
	float friction;
	float roll; /* rolling impulse */
};

/* adjoint handed from step n to step n - 1 for one contact id: manifold geometry (normal,
   anchors, base separation), warm-start impulses and the cached rotations of recycling */
struct d_carry
{
	float nx, ny;
	float aA[2][2], aB[2][2];
	float base[2];
	float ni[2], ti[2];
	float qA[2], qB[2];
	float roll; /* the manifold's rolling impulse */
};

static __device__ __forceinline__ d_laneImp d_getImp( const b2gContactLane* c )
{
	d_laneImp m = { c->normalImpulse1, c->normalImpulse2, c->tangentImpulse1, c->tangentImpulse2,
					c->totalNormalImpulse1, c->totalNormalImpulse2, c->rollingImpulse };
	return m;
}

static __device__ __forceinline__ void d_setImp( b2gContactLane* c, const d_laneImp& m )
{
	c->normalImpulse1 = m.n1;
	c->normalImpulse2 = m.n2;
	c->tangentImpulse1 = m.t1;
	c->tangentImpulse2 = m.t2;
	c->totalNormalImpulse1 = m.tot1;
	c->totalNormalImpulse2 = m.tot2;
	c->rollingImpulse = m.roll;
}

/* body velocity and its adjoint in the reverse sweep */
struct d_vel
{
	float vx, vy, w;
};

/* ---------------- adjoints of the contact lane functions (solver.cuh) ---------------- */

/* the impulse P applied at anchors rA, rB: adjoint of P from the velocity adjoints, and the
   anchor adjoints of the angular terms */
static __device__ __forceinline__ void d_adjApply( const b2gContactLane* c, b2Vec2 rA, b2Vec2 rB, float Px, float Py,
												   const d_vel& gA, const d_vel& gB, float* gPx, float* gPy, float* grAx,
												   float* grAy, float* grBx, float* grBy )
{
	/* vA -= mA P; wA -= iA (rA x P); vB += mB P; wB += iB (rB x P) */
	*gPx = -c->invMassA * gA.vx + c->invMassB * gB.vx + c->invIA * rA.y * gA.w - c->invIB * rB.y * gB.w;
	*gPy = -c->invMassA * gA.vy + c->invMassB * gB.vy - c->invIA * rA.x * gA.w + c->invIB * rB.x * gB.w;
	*grAx += -c->invIA * Py * gA.w;
	*grAy += c->invIA * Px * gA.w;
	*grBx += c->invIB * Py * gB.w;
	*grBy += -c->invIB * Px * gB.w;
}

/* relative velocity dv = (vB + wB x rB) - (vA + wA x rA): accumulate the adjoint of dv */
static __device__ __forceinline__ void d_adjRelVel( float gdx, float gdy, const d_vel& A, const d_vel& B, b2Vec2 rA, b2Vec2 rB,
													d_vel* gA, d_vel* gB, float* grAx, float* grAy, float* grBx, float* grBy )
{
	gB->vx += gdx;
	gB->vy += gdy;
	gA->vx -= gdx;
	gA->vy -= gdy;
	gB->w += -rB.y * gdx + rB.x * gdy;
	gA->w -= -rA.y * gdx + rA.x * gdy;
	*grBy += -B.w * gdx;
	*grBx += B.w * gdy;
	*grAy += A.w * gdx;
	*grAx += -A.w * gdy;
}

/* contact_solver.c:1811-1871 warm start, reversed. gA/gB hold the adjoint of the body
   velocities after the stage and receive the adjoint before it (the map is the identity
   plus terms that do not depend on velocity). */
static __device__ void d_adjWarmStart( const b2gContactLane* c, const d_laneImp& imp, d_vel* gA, d_vel* gB, d_laneAdj* g )
{
	float tx = c->normal.y, ty = 0.0f - c->normal.x;
	float gtx = 0.0f, gty = 0.0f;
	for ( int p = 0; p < 2; ++p )
	{
		b2Vec2 rA = p == 0 ? c->anchorA1 : c->anchorA2;
		b2Vec2 rB = p == 0 ? c->anchorB1 : c->anchorB2;
		float ni = p == 0 ? imp.n1 : imp.n2;
		float ti = p == 0 ? imp.t1 : imp.t2;
		float Px = ni * c->normal.x + ti * tx;
		float Py = ni * c->normal.y + ti * ty;
		float gPx, gPy;
		float* grAx = p == 0 ? &g->rA1x : &g->rA2x;
		float* grAy = p == 0 ? &g->rA1y : &g->rA2y;
		float* grBx = p == 0 ? &g->rB1x : &g->rB2x;
		float* grBy = p == 0 ? &g->rB1y : &g->rB2y;
		d_adjApply( c, rA, rB, Px, Py, *gA, *gB, &gPx, &gPy, grAx, grAy, grBx, grBy );
		float gn = gPx * c->normal.x + gPy * c->normal.y;
		float gt = gPx * tx + gPy * ty;
		if ( p == 0 )
		{
			g->n1 += gn;
			g->t1 += gt;
		}
		else
		{
			g->n2 += gn;
			g->t2 += gt;
		}
		g->nx += ni * gPx;
		g->ny += ni * gPy;
		gtx += ti * gPx;
		gty += ti * gPy;
	}
	/* tangent = (n.y, -n.x) */
	g->ny += gtx;
	g->nx -= gty;
	/* wA -= iA roll, wB += iB roll (contact_solver.c:1863-1864) */
	g->roll += -c->invIA * gA->w + c->invIB * gB->w;
}

/* accumulators of one lane point's geometric adjoints */
struct d_pointAdj
{
	float rAx, rAy, rBx, rBy;
};

static __device__ __forceinline__ d_vel d_velOf( const d_body& b )
{
	d_vel v = { b.vx, b.vy, b.w };
	return v;
}

/* rotation of an anchor by a body's delta rotation (rs = dq r): adjoint */
static __device__ __forceinline__ void d_adjRotate( float dqc, float dqs, b2Vec2 r, float grsx, float grsy, float* gdqc, float* gdqs,
													float* grx, float* gry )
{
	*gdqc += r.x * grsx + r.y * grsy;
	*gdqs += -r.y * grsx + r.x * grsy;
	*grx += dqc * grsx + dqs * grsy;
	*gry += -dqs * grsx + dqc * grsy;
}

/* d_normalPoint reversed (contact_solver.c:1930-1990). A and B are the body states the point
   saw; gA/gB hold the velocity adjoints after it and receive those before it; *gLambda
   holds the adjoint of the new accumulated impulse and receives that of the old one. */
static __device__ void d_adjNormalPoint( const b2gContactLane* c, const d_body& A, const d_body& B, float dpx, float dpy, b2Vec2 rA,
										 b2Vec2 rB, float baseSeparation, float normalMass, float lambda, float biasRate,
										 float massScale, float impulseScale, float inv_h, float contactSpeed, d_vel* gA, d_vel* gB,
										 float* gLambda, d_pointAdj* gr, float* gnx, float* gny, float* gBase, float* gNormalMass,
										 float* gdpx, float* gdpy, float* gdqA, float* gdqB )
{
	float rsAx = A.dqc * rA.x - A.dqs * rA.y;
	float rsAy = A.dqs * rA.x + A.dqc * rA.y;
	float rsBx = B.dqc * rB.x - B.dqs * rB.y;
	float rsBy = B.dqs * rB.x + B.dqc * rB.y;
	float dsx = dpx + ( rsBx - rsAx );
	float dsy = dpy + ( rsBy - rsAy );
	float s = ( c->normal.x * dsx + c->normal.y * dsy ) + baseSeparation;
	bool mask = s > 0.0f;
	float specBias = s * inv_h;
	float soft = biasRate * s;
	bool softActive = soft > contactSpeed;
	float softBias = softActive ? soft : contactSpeed;
	float bias = mask ? specBias : softBias;
	float pointMassScale = mask ? 1.0f : massScale;
	float pointImpulseScale = mask ? 0.0f : impulseScale;
	float dvx = ( B.vx - B.w * rB.y ) - ( A.vx - A.w * rA.y );
	float dvy = ( B.vy + B.w * rB.x ) - ( A.vy + A.w * rA.x );
	float vn = dvx * c->normal.x + dvy * c->normal.y;
	float negImpulse = normalMass * ( pointMassScale * vn + bias ) + pointImpulseScale * lambda;
	float x = lambda - negImpulse;
	float newImpulse = x > 0.0f ? x : 0.0f;
	float impulse = newImpulse - lambda;
	float Px = impulse * c->normal.x;
	float Py = impulse * c->normal.y;

	float gPx, gPy;
	d_adjApply( c, rA, rB, Px, Py, *gA, *gB, &gPx, &gPy, &gr->rAx, &gr->rAy, &gr->rBx, &gr->rBy );
	float gImpulse = gPx * c->normal.x + gPy * c->normal.y;
	*gnx += impulse * gPx;
	*gny += impulse * gPy;
	float gNew = *gLambda + gImpulse;
	float gl = -gImpulse;
	float gx = x > 0.0f ? gNew : 0.0f;
	gl += gx;
	float gNeg = -gx;
	*gNormalMass += ( pointMassScale * vn + bias ) * gNeg;
	float gvn = normalMass * pointMassScale * gNeg;
	float gBias = normalMass * gNeg;
	gl += pointImpulseScale * gNeg;
	float gs = mask ? inv_h * gBias : ( softActive ? biasRate * gBias : 0.0f );
	*gBase += gs;
	*gnx += dsx * gs;
	*gny += dsy * gs;
	float gdsx = c->normal.x * gs, gdsy = c->normal.y * gs;
	*gdpx += gdsx;
	*gdpy += gdsy;
	d_adjRotate( B.dqc, B.dqs, rB, gdsx, gdsy, gdqB, gdqB + 1, &gr->rBx, &gr->rBy );
	d_adjRotate( A.dqc, A.dqs, rA, -gdsx, -gdsy, gdqA, gdqA + 1, &gr->rAx, &gr->rAy );
	*gnx += dvx * gvn;
	*gny += dvy * gvn;
	d_vel vA = d_velOf( A ), vB = d_velOf( B );
	d_adjRelVel( c->normal.x * gvn, c->normal.y * gvn, vA, vB, rA, rB, gA, gB, &gr->rAx, &gr->rAy, &gr->rBx, &gr->rBy );
	*gLambda = gl;
}

/* d_frictionPoint reversed (contact_solver.c:2050-2109); lambdaN is the point's normal
   impulse after the normal solve, whose adjoint *gLambdaN receives the friction cone term */
static __device__ void d_adjFrictionPoint( const b2gContactLane* c, const d_body& A, const d_body& B, b2Vec2 rA, b2Vec2 rB,
										   float tangentMass, float lambdaN, float tau, d_vel* gA, d_vel* gB, float* gTau,
										   float* gLambdaN, d_pointAdj* gr, float* gnx, float* gny, float* gTangentMass,
										   float* gFriction )
{
	float tx = c->normal.y;
	float ty = 0.0f - c->normal.x;
	float dvx = ( B.vx - B.w * rB.y ) - ( A.vx - A.w * rA.y );
	float dvy = ( B.vy + B.w * rB.x ) - ( A.vy + A.w * rA.x );
	float vt = dvx * tx + dvy * ty;
	vt = vt - c->tangentSpeed;
	float negImpulse = tangentMass * vt;
	float maxFriction = c->friction * lambdaN;
	float x = tau - negImpulse;
	float inner = x < maxFriction ? x : maxFriction;
	float lo = 0.0f - maxFriction;
	bool atLower = lo > inner;
	float newImpulse = atLower ? lo : inner;
	float impulse = newImpulse - tau;
	float Px = impulse * tx;
	float Py = impulse * ty;

	float gPx, gPy;
	d_adjApply( c, rA, rB, Px, Py, *gA, *gB, &gPx, &gPy, &gr->rAx, &gr->rAy, &gr->rBx, &gr->rBy );
	float gImpulse = gPx * tx + gPy * ty;
	float gtx = impulse * gPx, gty = impulse * gPy;
	float gRes = *gTau + gImpulse;
	float gt = -gImpulse;
	float gx = 0.0f, gMax = 0.0f;
	if ( atLower ) gMax = -gRes;
	else if ( x < maxFriction ) gx = gRes;
	else gMax = gRes;
	gt += gx;
	float gNeg = -gx;
	*gTangentMass += vt * gNeg;
	float gvt = tangentMass * gNeg;
	gtx += dvx * gvt;
	gty += dvy * gvt;
	d_vel vA = d_velOf( A ), vB = d_velOf( B );
	d_adjRelVel( tx * gvt, ty * gvt, vA, vB, rA, rB, gA, gB, &gr->rAx, &gr->rAy, &gr->rBx, &gr->rBy );
	*gFriction += lambdaN * gMax;
	*gLambdaN += c->friction * gMax;
	*gny += gtx;
	*gnx -= gty;
	*gTau = gt;
}

/* d_restitutionPoint reversed (contact_solver.c:2140-2220); *gRelVel receives the adjoint of
   the relative normal velocity recorded at prepare */
static __device__ void d_adjRestitutionPoint( const b2gContactLane* c, const d_body& A, const d_body& B, b2Vec2 rA, b2Vec2 rB,
											  float relativeVelocity, float totalImpulseIn, float normalMass, float threshold,
											  float lambda, d_vel* gA, d_vel* gB, float* gLambda, d_pointAdj* gr, float* gnx,
											  float* gny, float* gNormalMass, float* gRelVel )
{
	bool mask = ( relativeVelocity + threshold > 0.0f ) || ( totalImpulseIn == 0.0f ) || ( c->restitution == 0.0f );
	float mass = mask ? 0.0f : normalMass;
	float dvx = ( B.vx - B.w * rB.y ) - ( A.vx - A.w * rA.y );
	float dvy = ( B.vy + B.w * rB.x ) - ( A.vy + A.w * rA.x );
	float vn = dvx * c->normal.x + dvy * c->normal.y;
	float negImpulse = mass * ( vn + c->restitution * relativeVelocity );
	float x = lambda - negImpulse;
	float newImpulse = x > 0.0f ? x : 0.0f;
	float impulse = newImpulse - lambda;
	float Px = impulse * c->normal.x;
	float Py = impulse * c->normal.y;

	float gPx, gPy;
	d_adjApply( c, rA, rB, Px, Py, *gA, *gB, &gPx, &gPy, &gr->rAx, &gr->rAy, &gr->rBx, &gr->rBy );
	float gImpulse = gPx * c->normal.x + gPy * c->normal.y;
	*gnx += impulse * gPx;
	*gny += impulse * gPy;
	float gNew = *gLambda + gImpulse;
	float gl = -gImpulse;
	float gx = x > 0.0f ? gNew : 0.0f;
	gl += gx;
	float gNeg = -gx;
	if ( mask == false )
	{
		*gNormalMass += ( vn + c->restitution * relativeVelocity ) * gNeg;
		float gvn = normalMass * gNeg;
		*gRelVel += normalMass * c->restitution * gNeg;
		*gnx += dvx * gvn;
		*gny += dvy * gvn;
		d_vel vA = d_velOf( A ), vB = d_velOf( B );
		d_adjRelVel( c->normal.x * gvn, c->normal.y * gvn, vA, vB, rA, rB, gA, gB, &gr->rAx, &gr->rAy, &gr->rBx, &gr->rBy );
	}
	*gLambda = gl;
}

/* the adjoint of the body quantities a lane stage touches: velocities, and the position
   and rotation deltas the separation reads */
struct d_bodyAdj
{
	d_vel v;
	float dpx, dpy, dqc, dqs;
};

/* d_solveLane reversed (contact_solver.c:1873-2116): A0/B0 and imp are the body states and
   impulses the lane saw; the forward is recomputed with the forward's own point functions
   to recover the state between points. */
static __device__ void d_adjSolveLane( const b2gContactLane* c, const d_laneImp& imp, const d_body& A0, const d_body& B0,
									   const b2gStepParams& P, bool useBias, d_bodyAdj* gA, d_bodyAdj* gB, d_laneAdj* g )
{
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
	float inv_h = P.inv_h, contactSpeed = -P.contactSpeed;
	float dpx = B0.dpx - A0.dpx, dpy = B0.dpy - A0.dpy;
	/* forward, keeping the states between the points */
	d_body A1 = A0, B1 = B0;
	float l1 = imp.n1, l2 = imp.n2, tot1 = imp.tot1, tot2 = imp.tot2, total = 0.0f;
	d_normalPoint( c, &A1, &B1, dpx, dpy, c->anchorA1, c->anchorB1, c->baseSeparation1, c->normalMass1, &l1, &tot1, biasRate,
				   massScale, impulseScale, inv_h, contactSpeed, &total );
	d_body A2 = A1, B2 = B1;
	d_normalPoint( c, &A2, &B2, dpx, dpy, c->anchorA2, c->anchorB2, c->baseSeparation2, c->normalMass2, &l2, &tot2, biasRate,
				   massScale, impulseScale, inv_h, contactSpeed, &total );
	d_pointAdj g1 = { 0.0f, 0.0f, 0.0f, 0.0f }, g2 = { 0.0f, 0.0f, 0.0f, 0.0f };
	float gdqA[2] = { 0.0f, 0.0f }, gdqB[2] = { 0.0f, 0.0f };
	float gdpx = 0.0f, gdpy = 0.0f;
	if ( useBias == false )
	{
		/* rolling resistance (contact_solver.c:2021-2031) between the normal points and the
		   friction: symClamp(lambda + rollingMass (wA - wB), rollingResistance total) */
		d_body AR = A2, BR = B2;
		const bool rolling = ( c->groupFlags & 1 ) != 0;
		float rx = 0.0f, rmax = 0.0f, rinner = 0.0f;
		if ( rolling )
		{
			float deltaLambda = c->rollingMass * ( A2.w - B2.w );
			rx = imp.roll + deltaLambda;
			rmax = c->rollingResistance * total;
			rinner = w_min( rx, rmax );
			float newRoll = w_symClamp( rx, rmax );
			deltaLambda = newRoll - imp.roll;
			AR.w = A2.w - c->invIA * deltaLambda;
			BR.w = B2.w + c->invIB * deltaLambda;
		}
		d_body A3 = AR, B3 = BR;
		float t1 = imp.t1;
		d_frictionPoint( c, &A3, &B3, c->anchorA1, c->anchorB1, c->tangentMass1, l1, &t1 );
		/* friction point 2 saw (A3, B3), point 1 saw (AR, BR) */
		d_adjFrictionPoint( c, A3, B3, c->anchorA2, c->anchorB2, c->tangentMass2, l2, imp.t2, &gA->v, &gB->v, &g->t2, &g->n2, &g2,
							&g->nx, &g->ny, &g->tm2, &g->friction );
		d_adjFrictionPoint( c, AR, BR, c->anchorA1, c->anchorB1, c->tangentMass1, l1, imp.t1, &gA->v, &gB->v, &g->t1, &g->n1, &g1,
							&g->nx, &g->ny, &g->tm1, &g->friction );
		if ( rolling )
		{
			/* the branch the forward took: the bound -max, the bound max, or the sum */
			float gDelta = -c->invIA * gA->v.w + c->invIB * gB->v.w;
			float gNew = g->roll + gDelta;
			float gLambda = -gDelta;
			float gMax = 0.0f;
			if ( -rmax > rinner ) gMax = -gNew;
			else if ( rinner == rmax && !( rx < rmax ) ) gMax = gNew;
			else
			{
				gLambda += gNew;
				gA->v.w += c->rollingMass * gNew;
				gB->v.w -= c->rollingMass * gNew;
			}
			g->roll = gLambda;
			/* total = the two points' new normal impulses */
			float gTotal = c->rollingResistance * gMax;
			g->n1 += gTotal;
			g->n2 += gTotal;
		}
	}
	d_adjNormalPoint( c, A1, B1, dpx, dpy, c->anchorA2, c->anchorB2, c->baseSeparation2, c->normalMass2, imp.n2, biasRate, massScale,
					  impulseScale, inv_h, contactSpeed, &gA->v, &gB->v, &g->n2, &g2, &g->nx, &g->ny, &g->base2, &g->nm2, &gdpx, &gdpy,
					  gdqA, gdqB );
	d_adjNormalPoint( c, A0, B0, dpx, dpy, c->anchorA1, c->anchorB1, c->baseSeparation1, c->normalMass1, imp.n1, biasRate, massScale,
					  impulseScale, inv_h, contactSpeed, &gA->v, &gB->v, &g->n1, &g1, &g->nx, &g->ny, &g->base1, &g->nm1, &gdpx, &gdpy,
					  gdqA, gdqB );
	g->rA1x += g1.rAx;
	g->rA1y += g1.rAy;
	g->rB1x += g1.rBx;
	g->rB1y += g1.rBy;
	g->rA2x += g2.rAx;
	g->rA2y += g2.rAy;
	g->rB2x += g2.rBx;
	g->rB2y += g2.rBy;
	/* dp = dpB - dpA */
	gB->dpx += gdpx;
	gB->dpy += gdpy;
	gA->dpx -= gdpx;
	gA->dpy -= gdpy;
	gA->dqc += gdqA[0];
	gA->dqs += gdqA[1];
	gB->dqc += gdqB[0];
	gB->dqs += gdqB[1];
}

/* d_restitutionLane reversed (contact_solver.c:2118-2228) */
static __device__ void d_adjRestitutionLane( const b2gContactLane* c, const d_laneImp& imp, const d_body& A0, const d_body& B0,
											 float threshold, d_bodyAdj* gA, d_bodyAdj* gB, d_laneAdj* g )
{
	d_body A1 = A0, B1 = B0;
	float l1 = imp.n1, tot1 = imp.tot1;
	d_restitutionPoint( c, &A1, &B1, c->anchorA1, c->anchorB1, c->relativeVelocity1, imp.tot1, c->normalMass1, threshold, &l1, &tot1 );
	d_pointAdj g1 = { 0.0f, 0.0f, 0.0f, 0.0f }, g2 = { 0.0f, 0.0f, 0.0f, 0.0f };
	d_adjRestitutionPoint( c, A1, B1, c->anchorA2, c->anchorB2, c->relativeVelocity2, imp.tot2, c->normalMass2, threshold, imp.n2,
						   &gA->v, &gB->v, &g->n2, &g2, &g->nx, &g->ny, &g->nm2, &g->rv2 );
	d_adjRestitutionPoint( c, A0, B0, c->anchorA1, c->anchorB1, c->relativeVelocity1, imp.tot1, c->normalMass1, threshold, imp.n1,
						   &gA->v, &gB->v, &g->n1, &g1, &g->nx, &g->ny, &g->nm1, &g->rv1 );
	g->rA1x += g1.rAx;
	g->rA1y += g1.rAy;
	g->rB1x += g1.rBx;
	g->rB1y += g1.rBy;
	g->rA2x += g2.rAx;
	g->rA2y += g2.rAy;
	g->rB2x += g2.rBx;
	g->rB2y += g2.rBy;
}

/* ---------------- body stages ---------------- */

/* solver.c:66-112 reversed: v' = lvd + v / (1 + h linearDamping), likewise w */
static __device__ __forceinline__ void d_adjIntegrateVelocities( const b2gStepParams& P, const float* pr, d_vel* g )
{
	float h = P.h;
	float linearDamping = 1.0f / ( 1.0f + h * pr[3] );
	float angularDamping = 1.0f / ( 1.0f + h * pr[4] );
	g->vx *= linearDamping;
	g->vy *= linearDamping;
	g->w *= angularDamping;
}

/* solver.c:114-162 reversed; s/d are the body state before the stage */
static __device__ void d_adjIntegratePositions( const b2gStepParams& P, float4 s, float4 d, d_bodyAdj* g )
{
	float h = P.h;
	float maxLinearSpeed = P.maxLinearVelocity;
	float maxAngularSpeed = D_MAX_ROTATION * P.inv_dt;
	float maxLinearSq = maxLinearSpeed * maxLinearSpeed;
	float maxAngularSq = maxAngularSpeed * maxAngularSpeed;
	uint32_t flags = __float_as_uint( s.w );
	b2Vec2 v = { s.x, s.y };
	float w = s.z;
	v.x = ( flags & B2G_LOCK_X ) ? 0.0f : v.x;
	v.y = ( flags & B2G_LOCK_Y ) ? 0.0f : v.y;
	w = ( flags & B2G_LOCK_Z ) ? 0.0f : w;
	bool linearCap = d_dot( v, v ) > maxLinearSq;
	b2Vec2 vc = v;
	float length = 0.0f;
	if ( linearCap )
	{
		length = d_length( v );
		float ratio = maxLinearSpeed / length;
		vc = d_mulSV( ratio, v );
	}
	bool angularCap = w * w > maxAngularSq && ( flags & B2G_ALLOW_FAST_ROTATION ) == 0;
	float wc = w;
	if ( angularCap ) wc *= maxAngularSpeed / d_abs( w );
	/* dq' = normalize( dq.c - da dq.s, dq.s + da dq.c ), da = h wc */
	float da = h * wc;
	float q2c = d.z - da * d.w, q2s = d.w + da * d.z;
	float mag = sqrtf( q2s * q2s + q2c * q2c );
	float gq2c = 0.0f, gq2s = 0.0f;
	if ( mag > 0.0f )
	{
		float inv = 1.0f / mag;
		float oc = q2c * inv, os = q2s * inv;
		float dot = oc * g->dqc + os * g->dqs;
		gq2c = ( g->dqc - oc * dot ) * inv;
		gq2s = ( g->dqs - os * dot ) * inv;
	}
	float gdqc = gq2c + da * gq2s;
	float gdqs = -da * gq2c + gq2s;
	float gda = -d.w * gq2c + d.z * gq2s;
	/* dp' = dp + h vc; the velocity written back is vc */
	float gvcx = g->v.vx + h * g->dpx;
	float gvcy = g->v.vy + h * g->dpy;
	float gwc = g->v.w + h * gda;
	float gvx = gvcx, gvy = gvcy;
	if ( linearCap )
	{
		float ratio = maxLinearSpeed / length;
		float ux = v.x / length, uy = v.y / length;
		float dot = ux * gvcx + uy * gvcy;
		gvx = ratio * ( gvcx - ux * dot );
		gvy = ratio * ( gvcy - uy * dot );
	}
	float gw = angularCap ? 0.0f : gwc;
	g->v.vx = ( flags & B2G_LOCK_X ) ? 0.0f : gvx;
	g->v.vy = ( flags & B2G_LOCK_Y ) ? 0.0f : gvy;
	g->v.w = ( flags & B2G_LOCK_Z ) ? 0.0f : gw;
	g->dqc = gdqc;
	g->dqs = gdqs;
}

/* ---------------- per-world scratch ---------------- */

/* sizes every world's scratch is carved for */
struct d_adjSizes
{
	int maxAwake, maxSlots, maxBodies, maxContacts, maxShapes, substeps;
};

/* one world's view of the backward pass */
struct d_adjWorld
{
	const unsigned char* arena;
	const long long* stepOffsets; /* device copy */
	const b2gShape* shapes;
	int shapeCount, bodyCount, contactCapacity;
	/* inputs/outputs by body id (world slice of the concatenated host arrays) */
	int bodyBase, shapeBase;
};

struct d_adjScratch
{
	float4 *sv, *sd, *ckV, *ckD, *snapV, *ipV, *sdPost, *restV;
	b2gContactLane* lanes;
	d_laneImp *ckImp, *snapImp, *restImp;
	d_bodyAdj* gV;
	d_laneAdj* gL;
	float2 *gC, *gQ;		  /* pose adjoint of the step's start, by body id */
	float2 *endC, *endQ;	  /* pose adjoint of the step's end, by body id */
	float4* endV;			  /* velocity adjoint of the step's end, by body id */
	d_carry *carry, *carryNext; /* by contact id */
	int* prevSlot;			  /* contact id -> slot in the previous step, -1 */
	int* awakeBody;			  /* awake index -> body id */
	int* identity;			  /* 0, 1, 2, ... (slot -> record index) */
	float* gFriction;		  /* by shape id */
	int* status;			  /* B2_DIFF_* of the world (0 = fine), then the step, the check and its item */
};

static __host__ __device__ inline size_t d_alignUp( size_t x ) { return ( x + 255 ) & ~(size_t)255; }

/* carve one world's scratch from a base pointer; returns the bytes used */
static __host__ __device__ size_t d_carveScratch( unsigned char* base, const d_adjSizes& z, d_adjScratch* s )
{
	size_t o = 0;
	size_t na = (size_t)( z.maxAwake > 0 ? z.maxAwake : 1 ), nc = (size_t)( z.maxSlots > 0 ? z.maxSlots : 1 );
	size_t nb = (size_t)( z.maxBodies > 0 ? z.maxBodies : 1 ), ncap = (size_t)( z.maxContacts > 0 ? z.maxContacts : 1 );
	size_t ns = (size_t)( z.maxShapes > 0 ? z.maxShapes : 1 ), S = (size_t)z.substeps;
	const size_t colors = B2G_OVERFLOW_INDEX;
#define D_CARVE( field, type, count )                                                                                           \
	s->field = (type*)( base + o );                                                                                              \
	o = d_alignUp( o + sizeof( type ) * ( count ) )
	D_CARVE( sv, float4, na );
	D_CARVE( sd, float4, na );
	D_CARVE( ckV, float4, S * na );
	D_CARVE( ckD, float4, S * na );
	D_CARVE( snapV, float4, 3 * colors * na );
	D_CARVE( ipV, float4, na );
	D_CARVE( sdPost, float4, na );
	D_CARVE( restV, float4, colors * na );
	D_CARVE( lanes, b2gContactLane, nc );
	D_CARVE( ckImp, d_laneImp, S * nc );
	D_CARVE( snapImp, d_laneImp, 3 * nc );
	D_CARVE( restImp, d_laneImp, nc );
	D_CARVE( gV, d_bodyAdj, na );
	D_CARVE( gL, d_laneAdj, nc );
	D_CARVE( gC, float2, nb );
	D_CARVE( gQ, float2, nb );
	D_CARVE( endC, float2, nb );
	D_CARVE( endQ, float2, nb );
	D_CARVE( endV, float4, nb );
	D_CARVE( carry, d_carry, ncap );
	D_CARVE( carryNext, d_carry, ncap );
	D_CARVE( prevSlot, int, ncap );
	D_CARVE( awakeBody, int, na );
	D_CARVE( identity, int, nc );
	D_CARVE( gFriction, float, ns );
	D_CARVE( status, int, 4 );
#undef D_CARVE
	return o;
}

/* parts of one recorded step */
struct d_tapeView
{
	const b2gTapeStep* h;
	const b2gTapeBody* bodies;
	const float* params;
	const float* toi;
	const int* ids;
	const b2gContact* contacts;
};

static __device__ __forceinline__ d_tapeView d_viewStep( const unsigned char* rec )
{
	d_tapeView v;
	v.h = (const b2gTapeStep*)rec;
	int nb = v.h->bodyCount, na = v.h->awakeCount, nc = v.h->slotCount;
	v.bodies = (const b2gTapeBody*)( rec + b2gTapeBodiesOffset() );
	v.params = (const float*)( rec + b2gTapeParamsOffset( nb ) );
	v.toi = (const float*)( rec + b2gTapeToiOffset( nb, na ) );
	v.ids = (const int*)( rec + b2gTapeIdsOffset( nb, na ) );
	v.contacts = (const b2gContact*)( rec + b2gTapeContactsOffset( nb, na, nc ) );
	return v;
}

static __device__ __forceinline__ d_body d_bodyFrom( float4 v, float4 d )
{
	d_body b;
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

static __device__ __forceinline__ d_body d_staticBody( void )
{
	d_body b;
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

static __device__ __forceinline__ void d_zeroBodyAdj( d_bodyAdj* g )
{
	g->v.vx = 0.0f;
	g->v.vy = 0.0f;
	g->v.w = 0.0f;
	g->dpx = 0.0f;
	g->dpy = 0.0f;
	g->dqc = 0.0f;
	g->dqs = 0.0f;
}

/* records the first failure of a world: code, step, check (1 narrowphase, 2 finalize,
   3 unsupported shape) and the slot or body index */
static __device__ void d_fail( int* status, int code, int step, int check, int index )
{
	if ( atomicCAS( status, 0, code ) == 0 )
	{
		status[1] = step;
		status[2] = check;
		status[3] = index;
	}
}

/* ---------------- prepare and narrowphase adjoints ---------------- */

/* pose adjoint of a transform (p, q) moved to the body's center of mass and rotation:
   p = c - R(q) lc */
static __device__ __forceinline__ void d_adjPoseToCenter( float gpx, float gpy, float gqc, float gqs, b2Vec2 lc, float2* gC, float2* gQ )
{
	atomicAdd( &gC->x, gpx );
	atomicAdd( &gC->y, gpy );
	/* d(R(q) lc)/dq.c = lc, d/dq.s = (-lc.y, lc.x) */
	atomicAdd( &gQ->x, gqc - ( lc.x * gpx + lc.y * gpy ) );
	atomicAdd( &gQ->y, gqs - ( -lc.y * gpx + lc.x * gpy ) );
}

typedef b2dDual<float, 8> d_dual8;

static __device__ void d_dualPoly( const b2gShape* s, b2dPoly<d_dual8>* p )
{
	p->count = s->count;
	p->radius = s->radius;
	for ( int i = 0; i < s->count; ++i )
	{
		p->v[i] = b2dV( d_dual8::make( s->v[i].x ), d_dual8::make( s->v[i].y ) );
		p->n[i] = b2dV( d_dual8::make( s->n[i].x ), d_dual8::make( s->n[i].y ) );
	}
}

/* a capsule (or a segment, radius 0) as the two-vertex polygon the narrowphase collides
   it as (manifold.c:16-34 b2MakeCapsule, the same float operations) */
static __device__ void d_dualCapsule( b2Vec2 p1, b2Vec2 p2, float radius, b2dPoly<d_dual8>* p )
{
	b2Vec2 axis = d_normalize( d_sub( p2, p1 ) );
	b2Vec2 normal = d_rightPerp( axis );
	b2Vec2 neg = d_neg( normal );
	p->count = 2;
	p->radius = radius;
	p->v[0] = b2dV( d_dual8::make( p1.x ), d_dual8::make( p1.y ) );
	p->v[1] = b2dV( d_dual8::make( p2.x ), d_dual8::make( p2.y ) );
	p->n[0] = b2dV( d_dual8::make( normal.x ), d_dual8::make( normal.y ) );
	p->n[1] = b2dV( d_dual8::make( neg.x ), d_dual8::make( neg.y ) );
}

static __device__ __forceinline__ d_dual8 d_seed( float v, int k )
{
	d_dual8 r = d_dual8::make( v );
	r.d[k] = 1.0f;
	return r;
}

static __device__ __forceinline__ float d_contract( const d_dual8& x, float g, int j ) { return g * x.d[j]; }

/* adjoint of prepare (contact_solver.c:1573-1809) and of the narrowphase for one colored
   slot; writes the contact's adjoint for the previous step and accumulates pose, velocity
   and friction adjoints */
static __device__ void d_adjPrepareCollide( const d_tapeView& V, const d_tapeView& prev, bool hasPrev, const d_adjWorld& W,
											d_adjScratch& s, int slot, int step )
{
	const b2gContact* cs = V.contacts + slot;
	const b2gContactLane* L = s.lanes + slot;
	const d_laneAdj g = s.gL[slot];
	const int k = V.ids[slot];
	const d_carry cin = s.carry[k];
	const b2Manifold& m = cs->manifold;
	const int pc = m.pointCount;
	const float iA = cs->invIA, iB = cs->invIB;
	const b2Vec2 n = m.normal;
	const float warmScale = V.h->params.enableWarmStarting ? 1.0f : 0.0f;
	const b2gShape* shapeA = W.shapes + cs->shapeIdA;
	const b2gShape* shapeB = W.shapes + cs->shapeIdB;
	const int bodyA = shapeA->bodyId, bodyB = shapeB->bodyId;
	const int awA = cs->bodySimIndexA, awB = cs->bodySimIndexB;
	float gnx = g.nx, gny = g.ny;
	float gaA[2][2] = { { 0.0f, 0.0f }, { 0.0f, 0.0f } }, gaB[2][2] = { { 0.0f, 0.0f }, { 0.0f, 0.0f } };
	float gSep[2] = { 0.0f, 0.0f }, gNI[2] = { 0.0f, 0.0f }, gTI[2] = { 0.0f, 0.0f };
	for ( int p = 0; p < pc && p < 2; ++p )
	{
		b2Vec2 rA = m.points[p].anchorA, rB = m.points[p].anchorB;
		float grAx = p == 0 ? g.rA1x : g.rA2x, grAy = p == 0 ? g.rA1y : g.rA2y;
		float grBx = p == 0 ? g.rB1x : g.rB2x, grBy = p == 0 ? g.rB1y : g.rB2y;
		/* baseSeparation = separation - dot(rB - rA, n) */
		float gBase = p == 0 ? g.base1 : g.base2;
		gSep[p] += gBase;
		float ddx = rB.x - rA.x, ddy = rB.y - rA.y;
		gnx -= ddx * gBase;
		gny -= ddy * gBase;
		grAx += n.x * gBase;
		grAy += n.y * gBase;
		grBx -= n.x * gBase;
		grBy -= n.y * gBase;
		/* normal mass 1 / (mA + mB + iA rnA^2 + iB rnB^2), rn = r x n */
		float nm = p == 0 ? L->normalMass1 : L->normalMass2;
		float gnm = p == 0 ? g.nm1 : g.nm2;
		if ( nm > 0.0f && gnm != 0.0f )
		{
			float gk = -nm * nm * gnm;
			float rnA = rA.x * n.y - rA.y * n.x, rnB = rB.x * n.y - rB.y * n.x;
			float grnA = 2.0f * iA * rnA * gk, grnB = 2.0f * iB * rnB * gk;
			grAx += n.y * grnA;
			grAy -= n.x * grnA;
			gny += rA.x * grnA;
			gnx -= rA.y * grnA;
			grBx += n.y * grnB;
			grBy -= n.x * grnB;
			gny += rB.x * grnB;
			gnx -= rB.y * grnB;
		}
		/* tangent mass, tangent t = (n.y, -n.x) */
		float tm = p == 0 ? L->tangentMass1 : L->tangentMass2;
		float gtm = p == 0 ? g.tm1 : g.tm2;
		if ( tm > 0.0f && gtm != 0.0f )
		{
			float tx = n.y, ty = -n.x;
			float gk = -tm * tm * gtm;
			float rtA = rA.x * ty - rA.y * tx, rtB = rB.x * ty - rB.y * tx;
			float grtA = 2.0f * iA * rtA * gk, grtB = 2.0f * iB * rtB * gk;
			float gtx = 0.0f, gty = 0.0f;
			grAx += ty * grtA;
			grAy -= tx * grtA;
			gty += rA.x * grtA;
			gtx -= rA.y * grtA;
			grBx += ty * grtB;
			grBy -= tx * grtB;
			gty += rB.x * grtB;
			gtx -= rB.y * grtB;
			gny += gtx;
			gnx -= gty;
		}
		/* relative normal velocity at the step's start (restitution) */
		float grv = p == 0 ? g.rv1 : g.rv2;
		if ( grv != 0.0f )
		{
			d_vel vA = { 0.0f, 0.0f, 0.0f }, vB = { 0.0f, 0.0f, 0.0f };
			if ( awA >= 0 ) vA = { s.ckV[awA].x, s.ckV[awA].y, s.ckV[awA].z };
			if ( awB >= 0 ) vB = { s.ckV[awB].x, s.ckV[awB].y, s.ckV[awB].z };
			float dvx = ( vB.vx - vB.w * rB.y ) - ( vA.vx - vA.w * rA.y );
			float dvy = ( vB.vy + vB.w * rB.x ) - ( vA.vy + vA.w * rA.x );
			gnx += dvx * grv;
			gny += dvy * grv;
			d_vel gA = { 0.0f, 0.0f, 0.0f }, gB = { 0.0f, 0.0f, 0.0f };
			d_adjRelVel( n.x * grv, n.y * grv, vA, vB, rA, rB, &gA, &gB, &grAx, &grAy, &grBx, &grBy );
			if ( awA >= 0 )
			{
				atomicAdd( &s.gV[awA].v.vx, gA.vx );
				atomicAdd( &s.gV[awA].v.vy, gA.vy );
				atomicAdd( &s.gV[awA].v.w, gA.w );
			}
			if ( awB >= 0 )
			{
				atomicAdd( &s.gV[awB].v.vx, gB.vx );
				atomicAdd( &s.gV[awB].v.vy, gB.vy );
				atomicAdd( &s.gV[awB].v.w, gB.w );
			}
		}
		gNI[p] = warmScale * ( p == 0 ? g.n1 : g.n2 );
		gTI[p] = warmScale * ( p == 0 ? g.t1 : g.t2 );
		gaA[p][0] = grAx;
		gaA[p][1] = grAy;
		gaB[p][0] = grBx;
		gaB[p][1] = grBy;
	}
	/* friction = sqrt(fA fB) (contact.c b2MixFriction) */
	if ( g.friction != 0.0f && cs->friction > 0.0f )
	{
		if ( shapeA->friction > 0.0f ) atomicAdd( s.gFriction + cs->shapeIdA, g.friction * 0.5f * cs->friction / shapeA->friction );
		if ( shapeB->friction > 0.0f ) atomicAdd( s.gFriction + cs->shapeIdB, g.friction * 0.5f * cs->friction / shapeB->friction );
	}
	/* the manifold as the next step read it */
	gnx += cin.nx;
	gny += cin.ny;
	for ( int p = 0; p < 2; ++p )
	{
		gaA[p][0] += cin.aA[p][0];
		gaA[p][1] += cin.aA[p][1];
		gaB[p][0] += cin.aB[p][0];
		gaB[p][1] += cin.aB[p][1];
	}
	const b2gTapeBody& TA = V.bodies[bodyA];
	const b2gTapeBody& TB = V.bodies[bodyB];
	d_carry out;
	memset( &out, 0, sizeof( out ) );
	if ( cs->simFlags & B2G_S_RECYCLED )
	{
		/* physics_world.c:530-552: sep = base + dot(dc + R(qB cB^-1) aB - R(qA cA^-1) aA, n) */
		b2Rot cA = cs->cachedRotationA, cB = cs->cachedRotationB;
		b2Rot dqA = d_mulRot( TA.xf.q, d_invertRot( cA ) );
		b2Rot dqB = d_mulRot( TB.xf.q, d_invertRot( cB ) );
		b2Vec2 dc = { TB.center.x - TA.center.x, TB.center.y - TA.center.y };
		float gdqA[2] = { 0.0f, 0.0f }, gdqB[2] = { 0.0f, 0.0f }, gdcx = 0.0f, gdcy = 0.0f;
		for ( int p = 0; p < pc && p < 2; ++p )
		{
			b2Vec2 aA = m.points[p].anchorA, aB = m.points[p].anchorB;
			b2Vec2 rA = d_rotate( dqA, aA ), rB = d_rotate( dqB, aB );
			b2Vec2 dp = d_add( dc, d_sub( rB, rA ) );
			float gs = gSep[p];
			out.base[p] = gs + cin.base[p];
			gnx += dp.x * gs;
			gny += dp.y * gs;
			float gx = n.x * gs, gy = n.y * gs;
			gdcx += gx;
			gdcy += gy;
			d_adjRotate( dqB.c, dqB.s, aB, gx, gy, gdqB, gdqB + 1, &gaB[p][0], &gaB[p][1] );
			d_adjRotate( dqA.c, dqA.s, aA, -gx, -gy, gdqA, gdqA + 1, &gaA[p][0], &gaA[p][1] );
		}
		/* dq = q * inverse(cached): r = (cached.c, -cached.s) */
		float gqA[2], gqB[2], gcA[2], gcB[2];
		{
			float rc = cA.c, rs = -cA.s;
			gqA[0] = gdqA[1] * rs + gdqA[0] * rc;
			gqA[1] = gdqA[1] * rc - gdqA[0] * rs;
			float grc = gdqA[1] * TA.xf.q.s + gdqA[0] * TA.xf.q.c;
			float grs = gdqA[1] * TA.xf.q.c - gdqA[0] * TA.xf.q.s;
			gcA[0] = grc;
			gcA[1] = -grs;
		}
		{
			float rc = cB.c, rs = -cB.s;
			gqB[0] = gdqB[1] * rs + gdqB[0] * rc;
			gqB[1] = gdqB[1] * rc - gdqB[0] * rs;
			float grc = gdqB[1] * TB.xf.q.s + gdqB[0] * TB.xf.q.c;
			float grs = gdqB[1] * TB.xf.q.c - gdqB[0] * TB.xf.q.s;
			gcB[0] = grc;
			gcB[1] = -grs;
		}
		if ( TA.type != b2_staticBody )
		{
			atomicAdd( &s.gC[bodyA].x, -gdcx );
			atomicAdd( &s.gC[bodyA].y, -gdcy );
			atomicAdd( &s.gQ[bodyA].x, gqA[0] );
			atomicAdd( &s.gQ[bodyA].y, gqA[1] );
		}
		if ( TB.type != b2_staticBody )
		{
			atomicAdd( &s.gC[bodyB].x, gdcx );
			atomicAdd( &s.gC[bodyB].y, gdcy );
			atomicAdd( &s.gQ[bodyB].x, gqB[0] );
			atomicAdd( &s.gQ[bodyB].y, gqB[1] );
		}
		out.nx = gnx;
		out.ny = gny;
		for ( int p = 0; p < 2; ++p )
		{
			out.aA[p][0] = gaA[p][0];
			out.aA[p][1] = gaA[p][1];
			out.aB[p][0] = gaB[p][0];
			out.aB[p][1] = gaB[p][1];
			out.ni[p] = gNI[p];
			out.ti[p] = gTI[p];
		}
		out.qA[0] = cin.qA[0] + gcA[0];
		out.qA[1] = cin.qA[1] + gcA[1];
		out.qB[0] = cin.qB[0] + gcB[0];
		out.qB[1] = cin.qB[1] + gcB[1];
		/* a kept manifold keeps its rolling impulse */
		out.roll = warmScale * g.roll;
		s.carryNext[k] = out;
		return;
	}
	/* computed this step (contact.c:519-698): the manifold is a function of both poses, and
	   takes the old manifold's rolling impulse when it has points (contact.c:609-612) */
	if ( pc > 0 )
	{
		out.roll = warmScale * g.roll;
		/* the pairs contact.c registers with polygon manifolds (polygon-polygon,
		   polygon-capsule, segment-polygon: a capsule or segment as a two-vertex polygon),
		   polygon-circle and circle-circle; shape A is the registered first type */
		const int tA = shapeA->type, tB = shapeB->type;
		const bool polyPair = ( tA == b2_polygonShape && ( tB == b2_polygonShape || tB == b2_capsuleShape ) ) ||
							  ( tA == b2_segmentShape && tB == b2_polygonShape );
		const int kindA = polyPair ? 1 : ( tA == b2_polygonShape ? 1 : ( tA == b2_circleShape ? 0 : -1 ) );
		const int kindB = polyPair ? 1 : ( tB == b2_circleShape ? 0 : -1 );
		if ( kindA < 0 || kindB < 0 || ( kindA == 0 && kindB == 1 ) )
		{
			d_fail( s.status, B2_DIFF_UNSUPPORTED, step, 3, slot );
			return;
		}
		b2dPoly<d_dual8> polyA, polyB;
		if ( kindA == 1 )
		{
			if ( tA == b2_segmentShape ) d_dualCapsule( shapeA->v[0], shapeA->v[1], 0.0f, &polyA );
			else d_dualPoly( shapeA, &polyA );
		}
		if ( kindB == 1 )
		{
			if ( tB == b2_capsuleShape ) d_dualCapsule( shapeB->v[0], shapeB->v[1], shapeB->radius, &polyB );
			else d_dualPoly( shapeB, &polyB );
		}
		const b2dVec2<d_dual8> centerA = b2dV( d_dual8::make( shapeA->v[0].x ), d_dual8::make( shapeA->v[0].y ) );
		const b2dVec2<d_dual8> centerB = b2dV( d_dual8::make( shapeB->v[0].x ), d_dual8::make( shapeB->v[0].y ) );
		b2dXf<d_dual8> xfA, xfB;
		xfA.p = b2dV( d_seed( TA.xf.p.x, 0 ), d_seed( TA.xf.p.y, 1 ) );
		xfA.q.c = d_seed( TA.xf.q.c, 2 );
		xfA.q.s = d_seed( TA.xf.q.s, 3 );
		xfB.p = b2dV( d_seed( TB.xf.p.x, 4 ), d_seed( TB.xf.p.y, 5 ) );
		xfB.q.c = d_seed( TB.xf.q.c, 6 );
		xfB.q.s = d_seed( TB.xf.q.s, 7 );
		b2dContactGeometry<d_dual8> cg =
			kindA == 1 && kindB == 1
				? b2dContactManifold( &polyA, &polyB, xfA, xfB, TA.localCenter.x, TA.localCenter.y, TB.localCenter.x, TB.localCenter.y )
			: kindA == 1 ? b2dContactPolygonCircle( &polyA, centerB, shapeB->radius, xfA, xfB, TA.localCenter.x, TA.localCenter.y,
													  TB.localCenter.x, TB.localCenter.y )
						 : b2dContactCircles( centerA, shapeA->radius, centerB, shapeB->radius, xfA, xfB, TA.localCenter.x,
											  TA.localCenter.y, TB.localCenter.x, TB.localCenter.y );
		/* the recomputed manifold must be the recorded one */
		bool same = cg.count == pc && cg.normal.x.v == n.x && cg.normal.y.v == n.y;
		for ( int p = 0; p < pc && same; ++p )
		{
			same = cg.id[p] == m.points[p].id && cg.separation[p].v == m.points[p].separation &&
				   cg.anchorA[p].x.v == m.points[p].anchorA.x && cg.anchorA[p].y.v == m.points[p].anchorA.y &&
				   cg.anchorB[p].x.v == m.points[p].anchorB.x && cg.anchorB[p].y.v == m.points[p].anchorB.y;
		}
		if ( same == false )
		{
			d_fail( s.status, B2_DIFF_REPLAY_MISMATCH, step, 1, slot );
			return;
		}
		float gPose[8];
		for ( int j = 0; j < 8; ++j )
		{
			float acc = d_contract( cg.normal.x, gnx, j ) + d_contract( cg.normal.y, gny, j );
			for ( int p = 0; p < pc; ++p )
			{
				/* baseSeparation = separation when the manifold is computed */
				float gs = gSep[p] + cin.base[p];
				acc += d_contract( cg.anchorA[p].x, gaA[p][0], j ) + d_contract( cg.anchorA[p].y, gaA[p][1], j );
				acc += d_contract( cg.anchorB[p].x, gaB[p][0], j ) + d_contract( cg.anchorB[p].y, gaB[p][1], j );
				acc += d_contract( cg.separation[p], gs, j );
			}
			gPose[j] = acc;
		}
		/* the cached rotations of recycling are the poses' rotations */
		if ( TA.type != b2_staticBody )
			d_adjPoseToCenter( gPose[0], gPose[1], gPose[2] + cin.qA[0], gPose[3] + cin.qA[1], TA.localCenter, s.gC + bodyA, s.gQ + bodyA );
		if ( TB.type != b2_staticBody )
			d_adjPoseToCenter( gPose[4], gPose[5], gPose[6] + cin.qB[0], gPose[7] + cin.qB[1], TB.localCenter, s.gC + bodyB, s.gQ + bodyB );
		/* warm start: impulses of the previous manifold's point with the same id (contact.c:655-672) */
		if ( hasPrev )
		{
			int ps = s.prevSlot[k];
			if ( ps >= 0 )
			{
				const b2Manifold& old = prev.contacts[ps].manifold;
				for ( int p = 0; p < pc; ++p )
				{
					for ( int j = 0; j < old.pointCount; ++j )
					{
						if ( old.points[j].id == m.points[p].id )
						{
							out.ni[j] += gNI[p];
							out.ti[j] += gTI[p];
							break;
						}
					}
				}
			}
		}
	}
	s.carryNext[k] = out;
}

/* solver.c:583-600 and, after a time of impact, :495-512: the pose a body ends the step
   with, from its start pose (c, q) and its accumulated deltas d */
static __device__ __forceinline__ void d_finalPose( b2Vec2 c, b2Rot q, float4 d, float toi, b2Vec2* c2, b2Rot* q2 )
{
	b2Vec2 center = { c.x + d.x, c.y + d.y };
	b2Rot qEnd = d_normalizeRot( d_mulRot( b2Rot{ d.z, d.w }, q ) );
	if ( toi < 1.0f )
	{
		/* the sweep is relative to the start center; the start rotation is rotation0 */
		b2Vec2 c1 = d_sub( c, c ), cs2 = d_sub( center, c );
		b2Rot qt = d_nlerp( q, qEnd, toi );
		b2Vec2 ct = d_lerp( c1, cs2, toi );
		*c2 = d_add( c, ct );
		*q2 = qt;
		return;
	}
	*c2 = center;
	*q2 = qEnd;
}

/* adjoint of normalize: u = r / |r| */
static __device__ __forceinline__ void d_adjNormalize( b2Rot r, float gx, float gy, float* grc, float* grs )
{
	float mag = sqrtf( r.s * r.s + r.c * r.c );
	*grc = 0.0f;
	*grs = 0.0f;
	if ( mag > 0.0f )
	{
		float inv = 1.0f / mag;
		float oc = r.c * inv, os = r.s * inv;
		float dot = oc * gx + os * gy;
		*grc = ( gx - oc * dot ) * inv;
		*grs = ( gy - os * dot ) * inv;
	}
}

/* ---------------- the backward pass of one recorded step, one CTA per world ---------------- */

static __device__ __forceinline__ d_body d_snapBody( const float4* v, const float4* d, int index1 )
{
	if ( index1 == 0 ) return d_staticBody();
	return d_bodyFrom( v[index1 - 1], d[index1 - 1] );
}

/* the active colors of a step (overflow excluded) */
static __device__ int d_activeColors( const int* colorOffsets, int* list )
{
	int n = 0;
	for ( int c = 0; c < B2G_OVERFLOW_INDEX; ++c )
		if ( colorOffsets[c + 1] > colorOffsets[c] ) list[n++] = c;
	return n;
}

__global__ void __launch_bounds__( B2G_ADJ_THREADS ) k_adjointStep( const d_adjWorld* worlds, d_adjSizes z, unsigned char* scratch,
																	 size_t stride, int step, int stepCount )
{
	const int wi = blockIdx.x;
	const int tid = threadIdx.x, nt = blockDim.x;
	const d_adjWorld W = worlds[wi];
	d_adjScratch s;
	d_carveScratch( scratch + stride * (size_t)wi, z, &s );
	if ( *s.status != 0 ) return;
	const d_tapeView V = d_viewStep( W.arena + W.stepOffsets[step] );
	const bool hasPrev = step > 0;
	d_tapeView prev;
	if ( hasPrev ) prev = d_viewStep( W.arena + W.stepOffsets[step - 1] );
	else prev = V;
	const b2gStepParams P = V.h->params;
	const int nb = V.h->bodyCount, na = V.h->awakeCount, nc = V.h->slotCount;
	const int* colorOffsets = V.h->colorOffsets;
	const int S = P.subStepCount;
	__shared__ int s_colors[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_colorCount, s_restitution, s_bad;
	if ( tid == 0 )
	{
		s_colorCount = d_activeColors( colorOffsets, s_colors );
		s_restitution = 0;
		int bad = 0;
		if ( V.h->jointCount > 0 || colorOffsets[B2_GRAPH_COLOR_COUNT] > colorOffsets[B2G_OVERFLOW_INDEX] ) bad = B2_DIFF_UNSUPPORTED;
		if ( na > z.maxAwake || nc > z.maxSlots || nb > z.maxBodies || S > z.substeps || S < 1 ) bad = B2_DIFF_UNSUPPORTED;
		s_bad = bad;
	}
	__syncthreads();
	if ( s_bad != 0 )
	{
		if ( tid == 0 ) d_fail( s.status, s_bad, step, 4, 0 );
		return;
	}
	const int C = s_colorCount;

	/* ---- setup: awake map, start state, previous-step slot map, cleared adjoints ---- */
	for ( int b = tid; b < nb; b += nt )
	{
		const b2gTapeBody& T = V.bodies[b];
		if ( T.awakeIndex >= 0 )
		{
			s.awakeBody[T.awakeIndex] = b;
			s.sv[T.awakeIndex] = make_float4( T.vx, T.vy, T.w, __uint_as_float( T.flags ) );
			s.sd[T.awakeIndex] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		}
	}
	for ( int k = tid; k < W.contactCapacity; k += nt )
	{
		s.prevSlot[k] = -1;
		memset( s.carryNext + k, 0, sizeof( d_carry ) );
	}
	for ( int i = tid; i < nc; i += nt ) memset( s.gL + i, 0, sizeof( d_laneAdj ) );
	__syncthreads();
	if ( hasPrev )
		for ( int i = tid; i < prev.h->slotCount; i += nt ) s.prevSlot[prev.ids[i]] = i;

	/* ---- prepare (the forward's own function) ---- */
	d_solveArgs a;
	memcpy( a.colorOffsets, colorOffsets, sizeof( a.colorOffsets ) );
	a.contacts = (b2gContact*)V.contacts;
	a.colorIds = s.identity;
	a.lanes = s.lanes;
	a.joints = NULL;
	a.sv = s.sv;
	a.sd = s.sd;
	a.params = V.params;
	a.awakeCount = na;
	a.p = P;
	const int overflowBegin = colorOffsets[B2G_OVERFLOW_INDEX];
	for ( int i = tid; i < nc; i += nt )
	{
		d_prepareContactLane( a, i, overflowBegin, s.lanes + i );
		if ( s.lanes[i].groupFlags & 2 ) s_restitution = 1;
	}
	__syncthreads();

	/* ---- forward replay with a checkpoint per substep ---- */
	for ( int sub = 0; sub < S; ++sub )
	{
		for ( int i = tid; i < na; i += nt )
		{
			s.ckV[sub * na + i] = s.sv[i];
			s.ckD[sub * na + i] = s.sd[i];
		}
		for ( int i = tid; i < nc; i += nt ) s.ckImp[sub * nc + i] = d_getImp( s.lanes + i );
		__syncthreads();
		for ( int i = tid; i < na; i += nt ) d_integrateVelocitiesState( P, s.sv, i, V.params + 8 * i );
		__syncthreads();
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int i = tid; i < na; i += nt ) d_integratePositionsState( P, s.sv, s.sd, i );
				__syncthreads();
			}
			for ( int ci = 0; ci < C; ++ci )
			{
				int c = s_colors[ci];
				for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt ) d_laneStage( P, s.lanes + i, s.sv, s.sd, stage );
				__syncthreads();
			}
		}
	}
	if ( s_restitution )
	{
		for ( int ci = 0; ci < C; ++ci )
		{
			int c = s_colors[ci];
			for ( int i = tid; i < na; i += nt ) s.restV[ci * na + i] = s.sv[i];
			for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt ) s.restImp[i] = d_getImp( s.lanes + i );
			__syncthreads();
			for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt )
				d_laneStage( P, s.lanes + i, s.sv, s.sd, STAGE_RESTITUTION );
			__syncthreads();
		}
	}
	/* the replay must land on the next recorded step's start (solver.c:583-600) */
	if ( step + 1 < stepCount )
	{
		const d_tapeView N = d_viewStep( W.arena + W.stepOffsets[step + 1] );
		for ( int i = tid; i < na; i += nt )
		{
			int b = s.awakeBody[i];
			const b2gTapeBody& T = V.bodies[b];
			const b2gTapeBody& T2 = N.bodies[b];
			float4 d = s.sd[i], v = s.sv[i];
			b2Vec2 c2;
			b2Rot q2;
			d_finalPose( T.center, T.xf.q, d, V.toi[i], &c2, &q2 );
			bool ok = c2.x == T2.center.x && c2.y == T2.center.y && q2.c == T2.xf.q.c && q2.s == T2.xf.q.s;
			if ( T2.awakeIndex >= 0 ) ok = ok && v.x == T2.vx && v.y == T2.vy && v.z == T2.w;
			if ( ok == false ) d_fail( s.status, B2_DIFF_REPLAY_MISMATCH, step, 2, b );
		}
	}
	__syncthreads();

	/* ---- adjoint of finalize (solver.c:583-600): c' = c + dp, q' = normalize(dq q) ---- */
	for ( int b = tid; b < nb; b += nt )
	{
		const b2gTapeBody& T = V.bodies[b];
		if ( T.awakeIndex < 0 )
		{
			s.gC[b] = s.endC[b];
			s.gQ[b] = s.endQ[b];
			continue;
		}
		int i = T.awakeIndex;
		float2 gc = s.endC[b], gq = s.endQ[b];
		float4 gv = s.endV[b];
		float4 d = s.sd[i];
		b2Rot q0 = T.xf.q;
		b2Rot r = d_mulRot( b2Rot{ d.z, d.w }, q0 );
		/* a time of impact (fraction held as recorded): c' = c + t dp, q' = nlerp(q0, qEnd, t) */
		float t = V.toi[i];
		float gq0c = 0.0f, gq0s = 0.0f, gEndc = gq.x, gEnds = gq.y, tp = 1.0f;
		if ( t < 1.0f )
		{
			b2Rot qEnd = d_normalizeRot( r );
			b2Rot rt = { ( 1.0f - t ) * q0.c + t * qEnd.c, ( 1.0f - t ) * q0.s + t * qEnd.s };
			float gtc, gts;
			d_adjNormalize( rt, gq.x, gq.y, &gtc, &gts );
			gq0c = ( 1.0f - t ) * gtc;
			gq0s = ( 1.0f - t ) * gts;
			gEndc = t * gtc;
			gEnds = t * gts;
			tp = t;
		}
		float grc, grs;
		d_adjNormalize( r, gEndc, gEnds, &grc, &grs );
		/* r.c = dq.c q.c - dq.s q.s, r.s = dq.s q.c + dq.c q.s */
		d_bodyAdj g;
		g.v.vx = gv.x;
		g.v.vy = gv.y;
		g.v.w = gv.z;
		g.dpx = tp * gc.x;
		g.dpy = tp * gc.y;
		g.dqc = grc * q0.c + grs * q0.s;
		g.dqs = -grc * q0.s + grs * q0.c;
		s.gV[i] = g;
		s.gC[b] = gc;
		s.gQ[b] = make_float2( gq0c + grc * d.z + grs * d.w, gq0s - grc * d.w + grs * d.z );
	}
	/* ---- adjoint of store: the next step's warm start read the final impulses ---- */
	for ( int i = tid; i < nc; i += nt )
	{
		const d_carry& cin = s.carry[V.ids[i]];
		s.gL[i].n1 = cin.ni[0];
		s.gL[i].n2 = cin.ni[1];
		s.gL[i].t1 = cin.ti[0];
		s.gL[i].t2 = cin.ti[1];
		s.gL[i].roll = cin.roll;
	}
	__syncthreads();

	/* ---- restitution, colors in reverse ---- */
	if ( s_restitution )
	{
		for ( int ci = C - 1; ci >= 0; --ci )
		{
			int c = s_colors[ci];
			for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt )
			{
				const b2gContactLane* L = s.lanes + i;
				if ( ( L->groupFlags & 2 ) == 0 ) continue;
				d_body A0 = d_snapBody( s.restV + ci * na, s.sd, L->indexA );
				d_body B0 = d_snapBody( s.restV + ci * na, s.sd, L->indexB );
				d_bodyAdj gA, gB;
				d_zeroBodyAdj( &gA );
				d_zeroBodyAdj( &gB );
				if ( L->indexA ) gA = s.gV[L->indexA - 1];
				if ( L->indexB ) gB = s.gV[L->indexB - 1];
				d_adjRestitutionLane( L, s.restImp[i], A0, B0, P.restitutionThreshold, &gA, &gB, s.gL + i );
				if ( L->indexA ) s.gV[L->indexA - 1] = gA;
				if ( L->indexB ) s.gV[L->indexB - 1] = gB;
			}
			__syncthreads();
		}
	}

	/* ---- substeps in reverse, each replayed from its checkpoint ---- */
	for ( int sub = S - 1; sub >= 0; --sub )
	{
		for ( int i = tid; i < na; i += nt )
		{
			s.sv[i] = s.ckV[sub * na + i];
			s.sd[i] = s.ckD[sub * na + i];
		}
		for ( int i = tid; i < nc; i += nt ) d_setImp( s.lanes + i, s.ckImp[sub * nc + i] );
		__syncthreads();
		for ( int i = tid; i < na; i += nt ) d_integrateVelocitiesState( P, s.sv, i, V.params + 8 * i );
		__syncthreads();
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int i = tid; i < na; i += nt ) s.ipV[i] = s.sv[i];
				__syncthreads();
				for ( int i = tid; i < na; i += nt ) d_integratePositionsState( P, s.sv, s.sd, i );
				__syncthreads();
				for ( int i = tid; i < na; i += nt ) s.sdPost[i] = s.sd[i];
			}
			for ( int ci = 0; ci < C; ++ci )
			{
				int c = s_colors[ci];
				float4* snap = s.snapV + ( stage * B2G_OVERFLOW_INDEX + ci ) * na;
				for ( int i = tid; i < na; i += nt ) snap[i] = s.sv[i];
				for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt ) s.snapImp[stage * nc + i] = d_getImp( s.lanes + i );
				__syncthreads();
				for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt ) d_laneStage( P, s.lanes + i, s.sv, s.sd, stage );
				__syncthreads();
			}
		}
		/* relax and solve, colors in reverse; integrate positions between them */
		for ( int stage = STAGE_RELAX; stage >= STAGE_SOLVE; --stage )
		{
			const float4* dState = stage == STAGE_RELAX ? s.sdPost : s.ckD + sub * na;
			for ( int ci = C - 1; ci >= 0; --ci )
			{
				int c = s_colors[ci];
				const float4* snap = s.snapV + ( stage * B2G_OVERFLOW_INDEX + ci ) * na;
				for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt )
				{
					const b2gContactLane* L = s.lanes + i;
					d_body A0 = d_snapBody( snap, dState, L->indexA );
					d_body B0 = d_snapBody( snap, dState, L->indexB );
					d_bodyAdj gA, gB;
					d_zeroBodyAdj( &gA );
					d_zeroBodyAdj( &gB );
					if ( L->indexA ) gA = s.gV[L->indexA - 1];
					if ( L->indexB ) gB = s.gV[L->indexB - 1];
					d_adjSolveLane( L, s.snapImp[stage * nc + i], A0, B0, P, stage == STAGE_SOLVE, &gA, &gB, s.gL + i );
					if ( L->indexA ) s.gV[L->indexA - 1] = gA;
					if ( L->indexB ) s.gV[L->indexB - 1] = gB;
				}
				__syncthreads();
			}
			if ( stage == STAGE_RELAX )
			{
				for ( int i = tid; i < na; i += nt ) d_adjIntegratePositions( P, s.ipV[i], s.ckD[sub * na + i], s.gV + i );
				__syncthreads();
			}
		}
		/* warm start, colors in reverse */
		for ( int ci = C - 1; ci >= 0; --ci )
		{
			int c = s_colors[ci];
			for ( int i = colorOffsets[c] + tid; i < colorOffsets[c + 1]; i += nt )
			{
				const b2gContactLane* L = s.lanes + i;
				d_vel gA = { 0.0f, 0.0f, 0.0f }, gB = { 0.0f, 0.0f, 0.0f };
				if ( L->indexA ) gA = s.gV[L->indexA - 1].v;
				if ( L->indexB ) gB = s.gV[L->indexB - 1].v;
				d_adjWarmStart( L, s.snapImp[STAGE_WARM * nc + i], &gA, &gB, s.gL + i );
				if ( L->indexA ) s.gV[L->indexA - 1].v = gA;
				if ( L->indexB ) s.gV[L->indexB - 1].v = gB;
			}
			__syncthreads();
		}
		for ( int i = tid; i < na; i += nt ) d_adjIntegrateVelocities( P, V.params + 8 * i, &s.gV[i].v );
		__syncthreads();
	}

	/* ---- prepare and narrowphase adjoints, then hand over to the previous step ---- */
	for ( int i = tid; i < nc; i += nt ) d_adjPrepareCollide( V, prev, hasPrev, W, s, i, step );
	__syncthreads();
	for ( int b = tid; b < nb; b += nt )
	{
		s.endC[b] = s.gC[b];
		s.endQ[b] = s.gQ[b];
		int i = V.bodies[b].awakeIndex;
		if ( i >= 0 ) s.endV[b] = make_float4( s.gV[i].v.vx, s.gV[i].v.vy, s.gV[i].v.w, 0.0f );
	}
	for ( int k = tid; k < W.contactCapacity; k += nt ) s.carry[k] = s.carryNext[k];
}

/* inputs of the last step's end, cleared carries and friction adjoints */
__global__ void k_adjointInit( const d_adjWorld* worlds, d_adjSizes z, unsigned char* scratch, size_t stride, const float* adjCenter,
							   const float* adjRotation, const float* adjVelocity )
{
	const int wi = blockIdx.x;
	const d_adjWorld W = worlds[wi];
	d_adjScratch s;
	d_carveScratch( scratch + stride * (size_t)wi, z, &s );
	for ( int b = threadIdx.x; b < W.bodyCount; b += blockDim.x )
	{
		int g = W.bodyBase + b;
		s.endC[b] = make_float2( adjCenter[2 * g], adjCenter[2 * g + 1] );
		s.endQ[b] = adjRotation ? make_float2( adjRotation[2 * g], adjRotation[2 * g + 1] ) : make_float2( 0.0f, 0.0f );
		s.endV[b] = adjVelocity ? make_float4( adjVelocity[3 * g], adjVelocity[3 * g + 1], adjVelocity[3 * g + 2], 0.0f )
								: make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	}
	for ( int k = threadIdx.x; k < W.contactCapacity; k += blockDim.x ) memset( s.carry + k, 0, sizeof( d_carry ) );
	for ( int i = threadIdx.x; i < z.maxSlots; i += blockDim.x ) s.identity[i] = i;
	for ( int i = threadIdx.x; i < W.shapeCount; i += blockDim.x ) s.gFriction[i] = 0.0f;
	if ( threadIdx.x < 4 ) s.status[threadIdx.x] = 0;
}

__global__ void k_adjointOutputs( const d_adjWorld* worlds, d_adjSizes z, unsigned char* scratch, size_t stride, float* gradVelocity,
								  float* gradCenter, float* gradFriction, int* status )
{
	const int wi = blockIdx.x;
	const d_adjWorld W = worlds[wi];
	d_adjScratch s;
	d_carveScratch( scratch + stride * (size_t)wi, z, &s );
	for ( int b = threadIdx.x; b < W.bodyCount; b += blockDim.x )
	{
		int g = W.bodyBase + b;
		float4 v = s.endV[b];
		gradVelocity[3 * g] = v.x;
		gradVelocity[3 * g + 1] = v.y;
		gradVelocity[3 * g + 2] = v.z;
		gradCenter[2 * g] = s.endC[b].x;
		gradCenter[2 * g + 1] = s.endC[b].y;
	}
	for ( int i = threadIdx.x; i < W.shapeCount; i += blockDim.x ) gradFriction[W.shapeBase + i] = s.gFriction[i];
	if ( threadIdx.x < 4 ) status[4 * wi + threadIdx.x] = s.status[threadIdx.x];
}

#define CKA( x )                                                                                                               \
	do                                                                                                                           \
	{                                                                                                                            \
		cudaError_t e_ = ( x );                                                                                                  \
		if ( e_ != cudaSuccess )                                                                                                 \
		{                                                                                                                        \
			rc = (int)e_;                                                                                                        \
			goto done;                                                                                                           \
		}                                                                                                                        \
	} while ( 0 )

extern "C" int b2gDev_AdjointRun( const b2gAdjointWorld* worlds, int worldCount, int stepCount, const int* bodyOffsets,
								   const int* shapeOffsets, const float* adjCenter, const float* adjRotation, const float* adjVelocity,
								   float* gradVelocity, float* gradCenter, float* gradFriction, float* ms, int* launches,
								   int* failure )
{
	if ( failure ) memset( failure, 0, 5 * sizeof( int ) );
	if ( worldCount <= 0 || stepCount <= 0 ) return B2_DIFF_EMPTY;
	int rc = 0;
	d_adjSizes z;
	memset( &z, 0, sizeof( z ) );
	z.substeps = 1;
	for ( int w = 0; w < worldCount; ++w )
	{
		const b2gAdjointWorld& W = worlds[w];
		z.maxAwake = W.maxAwake > z.maxAwake ? W.maxAwake : z.maxAwake;
		z.maxSlots = W.maxSlots > z.maxSlots ? W.maxSlots : z.maxSlots;
		z.maxBodies = W.bodyCount > z.maxBodies ? W.bodyCount : z.maxBodies;
		z.maxContacts = W.contactCapacity > z.maxContacts ? W.contactCapacity : z.maxContacts;
		z.maxShapes = W.shapeCount > z.maxShapes ? W.shapeCount : z.maxShapes;
		z.substeps = W.maxSubsteps > z.substeps ? W.maxSubsteps : z.substeps;
	}
	int totalBodies = bodyOffsets[worldCount], totalShapes = shapeOffsets[worldCount];
	d_adjScratch probe;
	size_t stride = d_alignUp( d_carveScratch( (unsigned char*)0, z, &probe ) );
	unsigned char* scratch = NULL;
	d_adjWorld* dWorlds = NULL;
	long long* dOffsets = NULL;
	float *dIn = NULL, *dOut = NULL;
	int* dStatus = NULL;
	int* hStatus = NULL;
	d_adjWorld* hWorlds = (d_adjWorld*)calloc( (size_t)worldCount, sizeof( d_adjWorld ) );
	long long* hOffsets = (long long*)malloc( (size_t)worldCount * stepCount * sizeof( long long ) );
	cudaStream_t stream = NULL;
	cudaEvent_t e0 = NULL, e1 = NULL;
	size_t inFloats = (size_t)totalBodies * 7, outFloats = (size_t)totalBodies * 5 + (size_t)totalShapes;
	CKA( cudaDeviceSynchronize() );
	CKA( cudaStreamCreateWithFlags( &stream, cudaStreamNonBlocking ) );
	CKA( cudaEventCreate( &e0 ) );
	CKA( cudaEventCreate( &e1 ) );
	CKA( cudaMalloc( (void**)&scratch, stride * (size_t)worldCount ) );
	CKA( cudaMalloc( (void**)&dWorlds, sizeof( d_adjWorld ) * (size_t)worldCount ) );
	CKA( cudaMalloc( (void**)&dOffsets, sizeof( long long ) * (size_t)worldCount * stepCount ) );
	CKA( cudaMalloc( (void**)&dIn, sizeof( float ) * ( inFloats > 0 ? inFloats : 1 ) ) );
	CKA( cudaMalloc( (void**)&dOut, sizeof( float ) * ( outFloats > 0 ? outFloats : 1 ) ) );
	CKA( cudaMalloc( (void**)&dStatus, sizeof( int ) * 4 * (size_t)worldCount ) );
	for ( int w = 0; w < worldCount; ++w )
	{
		const b2gAdjointWorld& W = worlds[w];
		memcpy( hOffsets + (size_t)w * stepCount, W.stepOffsets, sizeof( long long ) * (size_t)stepCount );
		d_adjWorld& D = hWorlds[w];
		D.arena = (const unsigned char*)W.arena;
		D.stepOffsets = dOffsets + (size_t)w * stepCount;
		D.shapes = W.shapes;
		D.shapeCount = W.shapeCount;
		D.bodyCount = W.bodyCount;
		D.contactCapacity = W.contactCapacity;
		D.bodyBase = bodyOffsets[w];
		D.shapeBase = shapeOffsets[w];
	}
	CKA( cudaMemcpyAsync( dWorlds, hWorlds, sizeof( d_adjWorld ) * (size_t)worldCount, cudaMemcpyHostToDevice, stream ) );
	CKA( cudaMemcpyAsync( dOffsets, hOffsets, sizeof( long long ) * (size_t)worldCount * stepCount, cudaMemcpyHostToDevice, stream ) );
	{
		float* in = dIn;
		CKA( cudaMemcpyAsync( in, adjCenter, sizeof( float ) * 2 * totalBodies, cudaMemcpyHostToDevice, stream ) );
		if ( adjRotation )
			CKA( cudaMemcpyAsync( in + 2 * totalBodies, adjRotation, sizeof( float ) * 2 * totalBodies, cudaMemcpyHostToDevice, stream ) );
		if ( adjVelocity )
			CKA( cudaMemcpyAsync( in + 4 * totalBodies, adjVelocity, sizeof( float ) * 3 * totalBodies, cudaMemcpyHostToDevice, stream ) );
	}
	CKA( cudaEventRecord( e0, stream ) );
	k_adjointInit<<<worldCount, B2G_ADJ_THREADS, 0, stream>>>( dWorlds, z, scratch, stride, dIn, adjRotation ? dIn + 2 * totalBodies : NULL,
															  adjVelocity ? dIn + 4 * totalBodies : NULL );
	CKA( cudaGetLastError() );
	for ( int step = stepCount - 1; step >= 0; --step )
	{
		k_adjointStep<<<worldCount, B2G_ADJ_THREADS, 0, stream>>>( dWorlds, z, scratch, stride, step, stepCount );
		CKA( cudaGetLastError() );
	}
	k_adjointOutputs<<<worldCount, B2G_ADJ_THREADS, 0, stream>>>( dWorlds, z, scratch, stride, dOut, dOut + 3 * totalBodies,
																 dOut + 5 * totalBodies, dStatus );
	CKA( cudaGetLastError() );
	CKA( cudaEventRecord( e1, stream ) );
	CKA( cudaStreamSynchronize( stream ) );
	if ( ms ) CKA( cudaEventElapsedTime( ms, e0, e1 ) );
	if ( launches ) *launches = stepCount + 2;
	CKA( cudaMemcpy( gradVelocity, dOut, sizeof( float ) * 3 * totalBodies, cudaMemcpyDeviceToHost ) );
	if ( gradCenter ) CKA( cudaMemcpy( gradCenter, dOut + 3 * totalBodies, sizeof( float ) * 2 * totalBodies, cudaMemcpyDeviceToHost ) );
	if ( gradFriction ) CKA( cudaMemcpy( gradFriction, dOut + 5 * totalBodies, sizeof( float ) * totalShapes, cudaMemcpyDeviceToHost ) );
	hStatus = (int*)malloc( sizeof( int ) * 4 * (size_t)worldCount );
	CKA( cudaMemcpy( hStatus, dStatus, sizeof( int ) * 4 * (size_t)worldCount, cudaMemcpyDeviceToHost ) );
	for ( int w = 0; w < worldCount && rc == 0; ++w )
	{
		if ( hStatus[4 * w] != 0 )
		{
			rc = hStatus[4 * w];
			if ( failure )
			{
				failure[0] = rc;
				failure[1] = w;
				failure[2] = hStatus[4 * w + 1];
				failure[3] = hStatus[4 * w + 2];
				failure[4] = hStatus[4 * w + 3];
			}
		}
	}
done:
	free( hStatus );
	free( hWorlds );
	free( hOffsets );
	if ( scratch ) cudaFree( scratch );
	if ( dWorlds ) cudaFree( dWorlds );
	if ( dOffsets ) cudaFree( dOffsets );
	if ( dIn ) cudaFree( dIn );
	if ( dOut ) cudaFree( dOut );
	if ( dStatus ) cudaFree( dStatus );
	if ( e0 ) cudaEventDestroy( e0 );
	if ( e1 ) cudaEventDestroy( e1 );
	if ( stream ) cudaStreamDestroy( stream );
	return rc;
}

extern "C" int b2gDev_DownloadArena( const void* arena, long long bytes, void* out )
{
	cudaError_t e = cudaDeviceSynchronize();
	if ( e == cudaSuccess ) e = cudaMemcpy( out, arena, (size_t)bytes, cudaMemcpyDeviceToHost );
	return (int)e;
}
