/*
 * Oracle (test checker only): FP64 tangent-linear model of recorded GB300 steps, the
 * reference for the adjoint of box2d_gb300_diff.h.
 *
 * Input is one world's tape as b2Diff_DownloadTape returns it. The recorded trajectory is
 * replayed on the host in float, operation for operation as the step computes it
 * (contact_solver.c:1573-2331, solver.c:66-162 and :583-600, contact.c:519-698,
 * physics_world.c:508-560), so every branch (clamp, speculative or soft contact, friction
 * cone, speed cap, clip and edge choice) is the recorded one; each float carries one tangent
 * in double, propagated forward from a direction in (initial velocity, friction) space.
 * Every step's replay must land bit for bit on the next recorded step.
 */
#include "../box2d_gb300/csrc/b2g_device_abi.h"
#include "../box2d_gb300/csrc/device/diff_collide.h"

#include <string.h>

#include <vector>

typedef b2dDual<double, 1> T1;
typedef b2dVec2<T1> V1;
typedef b2dRot<T1> R1;

static inline T1 t_c( float x ) { return T1::make( x ); }
static inline T1 t_v( float x, double d )
{
	T1 r = T1::make( x );
	r.d[0] = d;
	return r;
}
static inline V1 t_vec( b2Vec2 a ) { return b2dV( t_c( a.x ), t_c( a.y ) ); }
static inline T1 t_max( const T1& a, const T1& b ) { return a.v > b.v ? a : b; }
static inline T1 t_min( const T1& a, const T1& b ) { return a.v < b.v ? a : b; }
static inline T1 t_cross( V1 a, V1 b ) { return a.x * b.y - a.y * b.x; }

/* body state of the substep loop */
struct t_body
{
	T1 vx, vy, w;
	uint32_t flags;
	T1 dpx, dpy, dqc, dqs;
};

/* contact constraint lane (the fields of b2gContactLane the stages read) */
struct t_lane
{
	int indexA, indexB;
	float invMassA, invMassB, invIA, invIB;
	V1 normal;
	T1 friction;
	float tangentSpeed, restitution;
	float biasRate, massScale, impulseScale;
	V1 anchorA[2], anchorB[2];
	T1 normalMass[2], tangentMass[2], baseSeparation[2], normalImpulse[2], tangentImpulse[2], totalNormalImpulse[2];
	T1 relativeVelocity[2];
	int groupFlags;
	int pointCount;
};

/* manifold state carried by contact id between steps */
struct t_manifold
{
	V1 normal;
	V1 anchorA[2], anchorB[2];
	T1 baseSeparation[2], separation[2], normalImpulse[2], tangentImpulse[2];
	R1 cachedA, cachedB;
	uint16_t id[2];
	int pointCount;
	bool valid;
};

static t_body t_static( void )
{
	t_body b;
	b.vx = t_c( 0.0f );
	b.vy = t_c( 0.0f );
	b.w = t_c( 0.0f );
	b.flags = 0;
	b.dpx = t_c( 0.0f );
	b.dpy = t_c( 0.0f );
	b.dqc = t_c( 1.0f );
	b.dqs = t_c( 0.0f );
	return b;
}

/* ---------------- stages (the device's operation order) ---------------- */

static void t_apply( const t_lane& c, t_body* A, t_body* B, V1 rA, V1 rB, T1 Px, T1 Py )
{
	A->vx = A->vx - c.invMassA * Px;
	A->vy = A->vy - c.invMassA * Py;
	A->w = A->w - c.invIA * ( rA.x * Py - rA.y * Px );
	B->vx = B->vx + c.invMassB * Px;
	B->vy = B->vy + c.invMassB * Py;
	B->w = B->w + c.invIB * ( rB.x * Py - rB.y * Px );
}

static void t_warmStart( t_lane& c, t_body* A, t_body* B )
{
	T1 tx = c.normal.y, ty = 0.0f - c.normal.x;
	for ( int p = 0; p < 2; ++p )
	{
		V1 rA = c.anchorA[p], rB = c.anchorB[p];
		T1 Px = c.normalImpulse[p] * c.normal.x + c.tangentImpulse[p] * tx;
		T1 Py = c.normalImpulse[p] * c.normal.y + c.tangentImpulse[p] * ty;
		A->w = A->w - c.invIA * ( rA.x * Py - rA.y * Px );
		A->vx = A->vx - c.invMassA * Px;
		A->vy = A->vy - c.invMassA * Py;
		B->w = B->w + c.invIB * ( rB.x * Py - rB.y * Px );
		B->vx = B->vx + c.invMassB * Px;
		B->vy = B->vy + c.invMassB * Py;
		c.totalNormalImpulse[p] = c.totalNormalImpulse[p] + c.normalImpulse[p];
	}
}

static void t_normalPoint( t_lane& c, int p, t_body* A, t_body* B, T1 dpx, T1 dpy, float biasRate, float massScale, float impulseScale,
						   float inv_h, float contactSpeed )
{
	V1 rA = c.anchorA[p], rB = c.anchorB[p];
	T1 rsAx = A->dqc * rA.x - A->dqs * rA.y;
	T1 rsAy = A->dqs * rA.x + A->dqc * rA.y;
	T1 rsBx = B->dqc * rB.x - B->dqs * rB.y;
	T1 rsBy = B->dqs * rB.x + B->dqc * rB.y;
	T1 dsx = dpx + ( rsBx - rsAx );
	T1 dsy = dpy + ( rsBy - rsAy );
	T1 s = ( c.normal.x * dsx + c.normal.y * dsy ) + c.baseSeparation[p];
	bool mask = s.v > 0.0f;
	T1 specBias = s * inv_h;
	T1 softBias = t_max( biasRate * s, t_c( contactSpeed ) );
	T1 bias = mask ? specBias : softBias;
	float pointMassScale = mask ? 1.0f : massScale;
	float pointImpulseScale = mask ? 0.0f : impulseScale;
	T1 dvx = ( B->vx - B->w * rB.y ) - ( A->vx - A->w * rA.y );
	T1 dvy = ( B->vy + B->w * rB.x ) - ( A->vy + A->w * rA.x );
	T1 vn = dvx * c.normal.x + dvy * c.normal.y;
	T1 negImpulse = c.normalMass[p] * ( pointMassScale * vn + bias ) + pointImpulseScale * c.normalImpulse[p];
	T1 newImpulse = t_max( c.normalImpulse[p] - negImpulse, t_c( 0.0f ) );
	T1 impulse = newImpulse - c.normalImpulse[p];
	c.normalImpulse[p] = newImpulse;
	c.totalNormalImpulse[p] = c.totalNormalImpulse[p] + impulse;
	t_apply( c, A, B, rA, rB, impulse * c.normal.x, impulse * c.normal.y );
}

static void t_frictionPoint( t_lane& c, int p, t_body* A, t_body* B )
{
	V1 rA = c.anchorA[p], rB = c.anchorB[p];
	T1 tx = c.normal.y;
	T1 ty = 0.0f - c.normal.x;
	T1 dvx = ( B->vx - B->w * rB.y ) - ( A->vx - A->w * rA.y );
	T1 dvy = ( B->vy + B->w * rB.x ) - ( A->vy + A->w * rA.x );
	T1 vt = dvx * tx + dvy * ty;
	vt = vt - c.tangentSpeed;
	T1 negImpulse = c.tangentMass[p] * vt;
	T1 maxFriction = c.friction * c.normalImpulse[p];
	T1 newImpulse = c.tangentImpulse[p] - negImpulse;
	newImpulse = t_max( 0.0f - maxFriction, t_min( newImpulse, maxFriction ) );
	T1 impulse = newImpulse - c.tangentImpulse[p];
	c.tangentImpulse[p] = newImpulse;
	t_apply( c, A, B, rA, rB, impulse * tx, impulse * ty );
}

static void t_solve( t_lane& c, t_body* A, t_body* B, float inv_h, float contactSpeedNeg, bool useBias )
{
	float biasRate, massScale, impulseScale;
	if ( useBias )
	{
		biasRate = c.massScale * c.biasRate;
		massScale = c.massScale;
		impulseScale = c.impulseScale;
	}
	else
	{
		biasRate = 0.0f;
		massScale = 1.0f;
		impulseScale = 0.0f;
	}
	T1 dpx = B->dpx - A->dpx, dpy = B->dpy - A->dpy;
	t_normalPoint( c, 0, A, B, dpx, dpy, biasRate, massScale, impulseScale, inv_h, contactSpeedNeg );
	t_normalPoint( c, 1, A, B, dpx, dpy, biasRate, massScale, impulseScale, inv_h, contactSpeedNeg );
	if ( useBias == false )
	{
		t_frictionPoint( c, 0, A, B );
		t_frictionPoint( c, 1, A, B );
	}
}

static void t_restitution( t_lane& c, t_body* A, t_body* B, float threshold )
{
	if ( ( c.groupFlags & 2 ) == 0 ) return;
	for ( int p = 0; p < 2; ++p )
	{
		V1 rA = c.anchorA[p], rB = c.anchorB[p];
		bool mask = ( c.relativeVelocity[p].v + threshold > 0.0f ) || ( c.totalNormalImpulse[p].v == 0.0f ) || ( c.restitution == 0.0f );
		T1 mass = mask ? t_c( 0.0f ) : c.normalMass[p];
		T1 dvx = ( B->vx - B->w * rB.y ) - ( A->vx - A->w * rA.y );
		T1 dvy = ( B->vy + B->w * rB.x ) - ( A->vy + A->w * rA.x );
		T1 vn = dvx * c.normal.x + dvy * c.normal.y;
		T1 negImpulse = mass * ( vn + c.restitution * c.relativeVelocity[p] );
		T1 newImpulse = t_max( c.normalImpulse[p] - negImpulse, t_c( 0.0f ) );
		T1 deltaImpulse = newImpulse - c.normalImpulse[p];
		c.normalImpulse[p] = newImpulse;
		c.totalNormalImpulse[p] = c.totalNormalImpulse[p] + deltaImpulse;
		t_apply( c, A, B, rA, rB, deltaImpulse * c.normal.x, deltaImpulse * c.normal.y );
	}
}

static void t_integrateVelocities( const b2gStepParams& P, t_body* b, const float* pr )
{
	float h = P.h;
	float linearDamping = 1.0f / ( 1.0f + h * pr[3] );
	float angularDamping = 1.0f / ( 1.0f + h * pr[4] );
	float invMass = pr[6];
	float gravityScale = invMass > 0.0f ? pr[5] : 0.0f;
	float lvdx = ( h * invMass ) * pr[0] + ( h * gravityScale ) * P.gravityX;
	float lvdy = ( h * invMass ) * pr[1] + ( h * gravityScale ) * P.gravityY;
	float avd = h * pr[7] * pr[2];
	b->vx = lvdx + linearDamping * b->vx;
	b->vy = lvdy + linearDamping * b->vy;
	b->w = avd + angularDamping * b->w;
}

static void t_integratePositions( const b2gStepParams& P, t_body* b )
{
	float h = P.h;
	float maxLinearSpeed = P.maxLinearVelocity;
	float maxAngularSpeed = ( 0.25f * B2_PI ) * P.inv_dt;
	float maxLinearSq = maxLinearSpeed * maxLinearSpeed;
	float maxAngularSq = maxAngularSpeed * maxAngularSpeed;
	uint32_t flags = b->flags;
	T1 vx = ( flags & B2G_LOCK_X ) ? t_c( 0.0f ) : b->vx;
	T1 vy = ( flags & B2G_LOCK_Y ) ? t_c( 0.0f ) : b->vy;
	T1 w = ( flags & B2G_LOCK_Z ) ? t_c( 0.0f ) : b->w;
	if ( ( vx * vx + vy * vy ).v > maxLinearSq )
	{
		T1 ratio = maxLinearSpeed / b2dSqrt( vx * vx + vy * vy );
		vx = ratio * vx;
		vy = ratio * vy;
		flags |= B2G_SPEED_CAPPED;
	}
	if ( ( w * w ).v > maxAngularSq && ( flags & B2G_ALLOW_FAST_ROTATION ) == 0 )
	{
		T1 aw = w.v < 0.0f ? -w : w;
		T1 ratio = maxAngularSpeed / aw;
		w = w * ratio;
		flags |= B2G_SPEED_CAPPED;
	}
	b->dpx = b->dpx + h * vx;
	b->dpy = b->dpy + h * vy;
	T1 da = h * w;
	T1 q2c = b->dqc - da * b->dqs, q2s = b->dqs + da * b->dqc;
	T1 mag = b2dSqrt( q2s * q2s + q2c * q2c );
	T1 inv = mag.v > 0.0f ? 1.0f / mag : t_c( 0.0f );
	b->dqc = q2c * inv;
	b->dqs = q2s * inv;
	b->vx = vx;
	b->vy = vy;
	b->w = w;
	b->flags = flags;
}

static void t_makeSoft( float hertz, float zeta, float h, float* biasRate, float* massScale, float* impulseScale )
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

/* contact_solver.c:1573-1809 for one colored slot; v0 are the awake bodies' velocities at
   the step's start */
static t_lane t_prepare( const b2gStepParams& P, const b2gContact* cs, const t_manifold& m, T1 friction, const std::vector<t_body>& v0 )
{
	t_lane c;
	memset( &c, 0, sizeof( c ) );
	float warmStartScale = P.enableWarmStarting ? 1.0f : 0.0f;
	int indexA = cs->bodySimIndexA, indexB = cs->bodySimIndexB;
	c.indexA = indexA + 1;
	c.indexB = indexB + 1;
	t_body zero = t_static();
	const t_body& A = indexA != -1 ? v0[indexA] : zero;
	const t_body& B = indexB != -1 ? v0[indexB] : zero;
	float mA = cs->invMassA, iA = cs->invIA, mB = cs->invMassB, iB = cs->invIB;
	c.invMassA = mA;
	c.invMassB = mB;
	c.invIA = iA;
	c.invIB = iB;
	float biasRate = P.contactBiasRate, massScale = P.contactMassScale, impulseScale = P.contactImpulseScale;
	if ( indexA == -1 || indexB == -1 )
	{
		biasRate = P.staticBiasRate;
		massScale = P.staticMassScale;
		impulseScale = P.staticImpulseScale;
	}
	else if ( P.enableContactSoftening )
	{
		float contactHertz = ( P.contactHertz < 0.125f * P.inv_h ) ? P.contactHertz : 0.125f * P.inv_h;
		float ratio = 1.0f;
		if ( mA < mB ) ratio = ( 0.5f > mA / mB ) ? 0.5f : mA / mB;
		else if ( mB < mA ) ratio = ( 0.5f > mB / mA ) ? 0.5f : mB / mA;
		t_makeSoft( ratio * contactHertz, ratio * P.contactDampingRatio, P.h, &biasRate, &massScale, &impulseScale );
	}
	V1 normal = m.normal;
	c.normal = normal;
	c.friction = friction;
	c.tangentSpeed = cs->tangentSpeed;
	c.restitution = cs->restitution;
	c.biasRate = biasRate;
	c.massScale = massScale;
	c.impulseScale = impulseScale;
	c.pointCount = m.pointCount;
	V1 tangent = b2dV( normal.y, -normal.x );
	for ( int p = 0; p < 2; ++p )
	{
		if ( p >= m.pointCount )
		{
			c.anchorA[p] = b2dV( t_c( 0.0f ), t_c( 0.0f ) );
			c.anchorB[p] = c.anchorA[p];
			c.baseSeparation[p] = t_c( 0.0f );
			c.normalImpulse[p] = t_c( 0.0f );
			c.tangentImpulse[p] = t_c( 0.0f );
			c.totalNormalImpulse[p] = t_c( 0.0f );
			c.normalMass[p] = t_c( 0.0f );
			c.tangentMass[p] = t_c( 0.0f );
			c.relativeVelocity[p] = t_c( 0.0f );
			continue;
		}
		V1 rA = m.anchorA[p], rB = m.anchorB[p];
		c.anchorA[p] = rA;
		c.anchorB[p] = rB;
		c.baseSeparation[p] = m.separation[p] - b2dDot( b2dSub( rB, rA ), normal );
		c.normalImpulse[p] = warmStartScale * m.normalImpulse[p];
		c.tangentImpulse[p] = warmStartScale * m.tangentImpulse[p];
		c.totalNormalImpulse[p] = t_c( 0.0f );
		T1 rnA = t_cross( rA, normal ), rnB = t_cross( rB, normal );
		T1 kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		c.normalMass[p] = kNormal.v > 0.0f ? 1.0f / kNormal : t_c( 0.0f );
		T1 rtA = t_cross( rA, tangent ), rtB = t_cross( rB, tangent );
		T1 kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		c.tangentMass[p] = kTangent.v > 0.0f ? 1.0f / kTangent : t_c( 0.0f );
		V1 vrA = b2dV( A.vx - A.w * rA.y, A.vy + A.w * rA.x );
		V1 vrB = b2dV( B.vx - B.w * rB.y, B.vy + B.w * rB.x );
		c.relativeVelocity[p] = b2dDot( normal, b2dSub( vrB, vrA ) );
	}
	return c;
}

/* pose of a body as a dual transform: p = c - R(q) lc */
struct t_pose
{
	V1 c;
	R1 q;
};

static b2dXf<T1> t_transform( const t_pose& b, b2Vec2 lc, b2Transform recorded )
{
	b2dXf<T1> xf;
	xf.q = b.q;
	V1 off = b2dRotate( b.q, t_vec( lc ) );
	xf.p = b2dV( b.c.x - off.x, b.c.y - off.y );
	/* the primal is the recorded transform (the step stores p, not c - R(q) lc) */
	xf.p.x.v = recorded.p.x;
	xf.p.y.v = recorded.p.y;
	return xf;
}

static t_manifold t_invalid( void )
{
	t_manifold m;
	memset( &m, 0, sizeof( m ) );
	m.valid = false;
	return m;
}

static inline bool t_same( float a, float b ) { return memcmp( &a, &b, 4 ) == 0; }

/* colored-slot group flags of the wide path: bit 0 rolling resistance, bit 1 restitution in
   the slot's 4-wide group (contact_solver.c:2021, :2131) */
static int t_groupFlags( const b2gTapeStep* h, const b2gContact* contacts, int slot )
{
	int color = 0;
	while ( h->colorOffsets[color + 1] <= slot ) color += 1;
	int begin = h->colorOffsets[color], end = h->colorOffsets[color + 1];
	int g0 = begin + ( ( slot - begin ) / 4 ) * 4;
	int flags = 0;
	for ( int k = g0; k < g0 + 4 && k < end; ++k )
	{
		flags |= contacts[k].rollingResistance != 0.0f ? 1 : 0;
		flags |= contacts[k].restitution != 0.0f ? 2 : 0;
	}
	return flags;
}

extern "C" __attribute__( ( visibility( "default" ) ) ) int b2t_tangent( const void* tape, long long bytes, const float* dirVelocity,
																		  const float* dirFriction, double* centerTangent,
																		  double* velocityTangent )
{
	const unsigned char* base = (const unsigned char*)tape;
	if ( bytes < 16 ) return -4;
	const b2gTapeHeader* H = (const b2gTapeHeader*)base;
	const int stepCount = H->stepCount, bodyCount = H->bodyCount, cap = H->contactCapacity;
	const long long headerBytes = b2gTapeAlign( 16 + 8LL * stepCount );
	const b2gShape* shapes = (const b2gShape*)( base + headerBytes );
	/* tangents of the state at the start of the current step, by body id */
	std::vector<double> dC( 2 * bodyCount, 0.0 ), dQ( 2 * bodyCount, 0.0 ), dV( 3 * bodyCount, 0.0 );
	for ( int b = 0; b < bodyCount; ++b )
		for ( int k = 0; k < 3; ++k ) dV[3 * b + k] = dirVelocity[3 * b + k];
	std::vector<t_manifold> carry( cap > 0 ? cap : 1, t_invalid() ), next( cap > 0 ? cap : 1, t_invalid() );
	for ( int n = 0; n < stepCount; ++n )
	{
		const unsigned char* rec = base + H->stepOffsets[n];
		const b2gTapeStep* h = (const b2gTapeStep*)rec;
		const int nb = h->bodyCount, na = h->awakeCount, nc = h->slotCount;
		if ( nb != bodyCount || h->jointCount > 0 || h->colorOffsets[B2_GRAPH_COLOR_COUNT] > h->colorOffsets[B2G_OVERFLOW_INDEX] )
			return -1;
		const b2gStepParams& P = h->params;
		const b2gTapeBody* bodies = (const b2gTapeBody*)( rec + b2gTapeBodiesOffset() );
		const float* params = (const float*)( rec + b2gTapeParamsOffset( nb ) );
		const float* toi = (const float*)( rec + b2gTapeToiOffset( nb, na ) );
		const int* ids = (const int*)( rec + b2gTapeIdsOffset( nb, na ) );
		const b2gContact* contacts = (const b2gContact*)( rec + b2gTapeContactsOffset( nb, na, nc ) );
		std::vector<t_pose> pose( nb );
		std::vector<int> awakeBody( na > 0 ? na : 1 );
		std::vector<t_body> v0( na > 0 ? na : 1 );
		for ( int b = 0; b < nb; ++b )
		{
			const b2gTapeBody& T = bodies[b];
			pose[b].c = b2dV( t_v( T.center.x, dC[2 * b] ), t_v( T.center.y, dC[2 * b + 1] ) );
			pose[b].q.c = t_v( T.xf.q.c, dQ[2 * b] );
			pose[b].q.s = t_v( T.xf.q.s, dQ[2 * b + 1] );
			if ( T.awakeIndex >= 0 )
			{
				t_body& s = v0[T.awakeIndex];
				s = t_static();
				s.vx = t_v( T.vx, dV[3 * b] );
				s.vy = t_v( T.vy, dV[3 * b + 1] );
				s.w = t_v( T.w, dV[3 * b + 2] );
				s.flags = T.flags;
				awakeBody[T.awakeIndex] = b;
			}
		}
		/* ---- narrowphase (contact.c:519-698, physics_world.c:508-560) ---- */
		std::vector<t_manifold> man( nc > 0 ? nc : 1 );
		std::vector<t_lane> lanes( nc > 0 ? nc : 1 );
		for ( int s = 0; s < nc; ++s )
		{
			const b2gContact* cs = contacts + s;
			const b2Manifold& rm = cs->manifold;
			const b2gShape* shapeA = shapes + cs->shapeIdA;
			const b2gShape* shapeB = shapes + cs->shapeIdB;
			int bA = shapeA->bodyId, bB = shapeB->bodyId;
			const t_manifold& old = carry[ids[s]];
			t_manifold m = t_invalid();
			m.valid = true;
			m.pointCount = rm.pointCount;
			if ( cs->simFlags & B2G_S_RECYCLED )
			{
				if ( old.valid == false || old.pointCount != rm.pointCount ) return -2;
				m = old;
				R1 qA = pose[bA].q, qB = pose[bB].q;
				R1 iA = { old.cachedA.c, -old.cachedA.s }, iB = { old.cachedB.c, -old.cachedB.s };
				R1 dqA = { qA.c * iA.c - qA.s * iA.s, qA.s * iA.c + qA.c * iA.s };
				R1 dqB = { qB.c * iB.c - qB.s * iB.s, qB.s * iB.c + qB.c * iB.s };
				V1 dc = b2dV( pose[bB].c.x - pose[bA].c.x, pose[bB].c.y - pose[bA].c.y );
				for ( int p = 0; p < m.pointCount; ++p )
				{
					V1 rA = b2dRotate( dqA, old.anchorA[p] );
					V1 rB = b2dRotate( dqB, old.anchorB[p] );
					V1 dp = b2dAdd( dc, b2dSub( rB, rA ) );
					m.separation[p] = old.baseSeparation[p] + b2dDot( dp, old.normal );
					if ( t_same( m.separation[p].v, rm.points[p].separation ) == false ) return -2;
				}
			}
			else if ( rm.pointCount > 0 )
			{
				if ( shapeA->type != b2_polygonShape || shapeB->type != b2_polygonShape ) return -1;
				b2dPoly<T1> polyA, polyB;
				b2dMakePoly( &polyA, &shapeA->v[0].x, &shapeA->n[0].x, shapeA->count, shapeA->radius );
				b2dMakePoly( &polyB, &shapeB->v[0].x, &shapeB->n[0].x, shapeB->count, shapeB->radius );
				b2dXf<T1> xfA = t_transform( pose[bA], bodies[bA].localCenter, bodies[bA].xf );
				b2dXf<T1> xfB = t_transform( pose[bB], bodies[bB].localCenter, bodies[bB].xf );
				b2dContactGeometry<T1> g = b2dContactManifold( &polyA, &polyB, xfA, xfB, bodies[bA].localCenter.x, bodies[bA].localCenter.y,
															   bodies[bB].localCenter.x, bodies[bB].localCenter.y );
				if ( g.count != rm.pointCount || t_same( g.normal.x.v, rm.normal.x ) == false || t_same( g.normal.y.v, rm.normal.y ) == false )
					return -2;
				m.normal = g.normal;
				for ( int p = 0; p < g.count; ++p )
				{
					if ( g.id[p] != rm.points[p].id || t_same( g.separation[p].v, rm.points[p].separation ) == false ||
						 t_same( g.anchorA[p].x.v, rm.points[p].anchorA.x ) == false ||
						 t_same( g.anchorB[p].y.v, rm.points[p].anchorB.y ) == false )
						return -2;
					m.anchorA[p] = g.anchorA[p];
					m.anchorB[p] = g.anchorB[p];
					m.separation[p] = g.separation[p];
					m.baseSeparation[p] = g.separation[p];
					m.id[p] = g.id[p];
					m.normalImpulse[p] = t_c( 0.0f );
					m.tangentImpulse[p] = t_c( 0.0f );
					if ( old.valid )
					{
						for ( int j = 0; j < old.pointCount; ++j )
						{
							if ( old.id[j] == g.id[p] )
							{
								m.normalImpulse[p] = old.normalImpulse[j];
								m.tangentImpulse[p] = old.tangentImpulse[j];
								break;
							}
						}
					}
					if ( t_same( m.normalImpulse[p].v, rm.points[p].normalImpulse ) == false ||
						 t_same( m.tangentImpulse[p].v, rm.points[p].tangentImpulse ) == false )
						return -2;
				}
				m.cachedA = pose[bA].q;
				m.cachedB = pose[bB].q;
			}
			/* friction = sqrt(fA fB) (b2MixFriction) */
			T1 fA = t_v( shapeA->friction, dirFriction[cs->shapeIdA] ), fB = t_v( shapeB->friction, dirFriction[cs->shapeIdB] );
			T1 friction = b2dSqrt( fA * fB );
			if ( t_same( friction.v, cs->friction ) == false ) return -2;
			man[s] = m;
			lanes[s] = t_prepare( P, cs, m, friction, v0 );
			lanes[s].groupFlags = t_groupFlags( h, contacts, s );
			if ( lanes[s].groupFlags & 1 ) return -1;
		}
		/* ---- substeps (solver.c:1010-1198), colors in order ---- */
		std::vector<t_body> sb( v0 );
		for ( int i = 0; i < na; ++i )
		{
			sb[i].dpx = t_c( 0.0f );
			sb[i].dpy = t_c( 0.0f );
			sb[i].dqc = t_c( 1.0f );
			sb[i].dqs = t_c( 0.0f );
		}
		const float contactSpeedNeg = -P.contactSpeed;
		bool restitution = false;
		for ( int s = 0; s < nc; ++s ) restitution = restitution || ( lanes[s].groupFlags & 2 ) != 0;
		for ( int sub = 0; sub < P.subStepCount; ++sub )
		{
			for ( int i = 0; i < na; ++i ) t_integrateVelocities( P, &sb[i], params + 8 * i );
			for ( int stage = 0; stage < 3; ++stage )
			{
				if ( stage == 2 )
					for ( int i = 0; i < na; ++i ) t_integratePositions( P, &sb[i] );
				for ( int c = 0; c < B2G_OVERFLOW_INDEX; ++c )
				{
					for ( int s = h->colorOffsets[c]; s < h->colorOffsets[c + 1]; ++s )
					{
						t_lane& L = lanes[s];
						t_body sA = t_static(), sBd = t_static();
						t_body* A = L.indexA ? &sb[L.indexA - 1] : &sA;
						t_body* B = L.indexB ? &sb[L.indexB - 1] : &sBd;
						t_body a0 = *A, b0 = *B;
						if ( stage == 0 ) t_warmStart( L, A, B );
						else t_solve( L, A, B, P.inv_h, contactSpeedNeg, stage == 1 );
						/* static and non-dynamic bodies keep their state (contact_solver.c:1526-1562) */
						if ( L.indexA == 0 || ( a0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *A = a0;
						if ( L.indexB == 0 || ( b0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *B = b0;
					}
				}
			}
		}
		if ( restitution )
		{
			for ( int c = 0; c < B2G_OVERFLOW_INDEX; ++c )
			{
				for ( int s = h->colorOffsets[c]; s < h->colorOffsets[c + 1]; ++s )
				{
					t_lane& L = lanes[s];
					t_body sA = t_static(), sBd = t_static();
					t_body* A = L.indexA ? &sb[L.indexA - 1] : &sA;
					t_body* B = L.indexB ? &sb[L.indexB - 1] : &sBd;
					t_body a0 = *A, b0 = *B;
					t_restitution( L, A, B, P.restitutionThreshold );
					if ( L.indexA == 0 || ( a0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *A = a0;
					if ( L.indexB == 0 || ( b0.flags & B2G_DYNAMIC_FLAG ) == 0 ) *B = b0;
				}
			}
		}
		/* ---- store impulses: the manifold the next step reads ---- */
		for ( int k = 0; k < cap; ++k ) next[k] = t_invalid();
		for ( int s = 0; s < nc; ++s )
		{
			t_manifold m = man[s];
			for ( int p = 0; p < m.pointCount; ++p )
			{
				m.normalImpulse[p] = lanes[s].normalImpulse[p];
				m.tangentImpulse[p] = lanes[s].tangentImpulse[p];
			}
			next[ids[s]] = m;
		}
		carry.swap( next );
		/* ---- finalize (solver.c:583-600) and the next step's start ---- */
		const b2gTapeBody* nextBodies = NULL;
		if ( n + 1 < stepCount ) nextBodies = (const b2gTapeBody*)( base + H->stepOffsets[n + 1] + b2gTapeBodiesOffset() );
		for ( int i = 0; i < na; ++i )
		{
			int b = awakeBody[i];
			const t_body& s = sb[i];
			V1 c2 = b2dV( pose[b].c.x + s.dpx, pose[b].c.y + s.dpy );
			R1 r = { s.dqc * pose[b].q.c - s.dqs * pose[b].q.s, s.dqs * pose[b].q.c + s.dqc * pose[b].q.s };
			T1 mag = b2dSqrt( r.s * r.s + r.c * r.c );
			T1 inv = mag.v > 0.0f ? 1.0f / mag : t_c( 0.0f );
			R1 q2 = { r.c * inv, r.s * inv };
			float t = toi[i];
			if ( t < 1.0f )
			{
				/* solver.c:495-512 with the recorded fraction: the sweep is relative to the start center */
				V1 base = pose[b].c;
				V1 c1 = b2dSub( base, base ), cs2 = b2dSub( c2, base );
				V1 ct = b2dLerpF( c1, cs2, t );
				float omt = 1.0f - t;
				R1 qt = { omt * pose[b].q.c + t * q2.c, omt * pose[b].q.s + t * q2.s };
				T1 m2 = b2dSqrt( qt.s * qt.s + qt.c * qt.c );
				T1 i2 = m2.v > 0.0f ? 1.0f / m2 : t_c( 0.0f );
				q2 = { qt.c * i2, qt.s * i2 };
				c2 = b2dAdd( base, ct );
			}
			if ( nextBodies != NULL )
			{
				const b2gTapeBody& T2 = nextBodies[b];
				bool ok = t_same( c2.x.v, T2.center.x ) && t_same( c2.y.v, T2.center.y ) && t_same( q2.c.v, T2.xf.q.c ) &&
						  t_same( q2.s.v, T2.xf.q.s );
				if ( T2.awakeIndex >= 0 ) ok = ok && t_same( s.vx.v, T2.vx ) && t_same( s.vy.v, T2.vy ) && t_same( s.w.v, T2.w );
				if ( ok == false ) return -2;
			}
			dC[2 * b] = c2.x.d[0];
			dC[2 * b + 1] = c2.y.d[0];
			dQ[2 * b] = q2.c.d[0];
			dQ[2 * b + 1] = q2.s.d[0];
			dV[3 * b] = s.vx.d[0];
			dV[3 * b + 1] = s.vy.d[0];
			dV[3 * b + 2] = s.w.d[0];
		}
	}
	for ( int b = 0; b < bodyCount; ++b )
	{
		centerTangent[2 * b] = dC[2 * b];
		centerTangent[2 * b + 1] = dC[2 * b + 1];
		if ( velocityTangent )
			for ( int k = 0; k < 3; ++k ) velocityTangent[3 * b + k] = dV[3 * b + k];
	}
	return 0;
}
