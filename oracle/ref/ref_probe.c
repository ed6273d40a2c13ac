/*
 * Contact-table probe compiled into the reference build (oracle/_ref, development
 * container only). It reads the reference's internal contact array so parity fixtures
 * can record contact ids, shape pairs, graph colors and manifold feature ids.
 * Row layout (8 ints per live contact, ascending contact id):
 *   contactId, shapeIdA, shapeIdB, colorIndex, pointCount, id0, id1, touching
 */
#include "contact.h"
#include "physics_world.h"
#include "solver_set.h"
#include "constraint_graph.h"
#include "body.h"
#include "joint.h"
#include "id_pool.h"

#include <string.h>

#define B2P_EXPORT __attribute__( ( visibility( "default" ) ) )

B2P_EXPORT int b2p_contacts( uint32_t packedWorldId, int* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	b2World* world = b2GetWorldFromId( id );
	int n = 0;
	for ( int i = 0; i < world->contacts.count; ++i )
	{
		b2Contact* c = world->contacts.data + i;
		if ( c->contactId != i ) continue;
		if ( n < capacity )
		{
			b2ContactSim* sim = b2GetContactSim( world, c );
			int* o = out + 8 * n;
			o[0] = c->contactId;
			o[1] = c->shapeIdA;
			o[2] = c->shapeIdB;
			o[3] = c->colorIndex;
			o[4] = sim->manifold.pointCount;
			o[5] = sim->manifold.pointCount > 0 ? sim->manifold.points[0].id : -1;
			o[6] = sim->manifold.pointCount > 1 ? sim->manifold.points[1].id : -1;
			o[7] = ( c->flags & b2_contactTouchingFlag ) ? 1 : 0;
		}
		n += 1;
	}
	return n;
}

/* 12 floats per live contact: normal.x, normal.y, then per point: separation,
   normalImpulse, tangentImpulse, anchorA.x, anchorA.y (unused points are zero) */
B2P_EXPORT int b2p_contact_floats( uint32_t packedWorldId, float* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	b2World* world = b2GetWorldFromId( id );
	int n = 0;
	for ( int i = 0; i < world->contacts.count; ++i )
	{
		b2Contact* c = world->contacts.data + i;
		if ( c->contactId != i ) continue;
		if ( n < capacity )
		{
			b2ContactSim* sim = b2GetContactSim( world, c );
			float* o = out + 12 * n;
			o[0] = sim->manifold.normal.x;
			o[1] = sim->manifold.normal.y;
			for ( int p = 0; p < 2; ++p )
			{
				const b2ManifoldPoint* mp = sim->manifold.points + p;
				int live = p < sim->manifold.pointCount;
				o[2 + 5 * p] = live ? mp->separation : 0.0f;
				o[3 + 5 * p] = live ? mp->normalImpulse : 0.0f;
				o[4 + 5 * p] = live ? mp->tangentImpulse : 0.0f;
				o[5 + 5 * p] = live ? mp->anchorA.x : 0.0f;
				o[6 + 5 * p] = live ? mp->anchorA.y : 0.0f;
			}
		}
		n += 1;
	}
	return n;
}

/* The values the reference's b2World_GetStateHash (world_snapshot.c:1025-1181) mixes into its
   FNV hash, in the same order, one 32-bit value per mix (bytes one by one); returns the
   count. Used to locate a bookkeeping difference between the GB300 library and the
   reference. */
typedef struct rp_words
{
	uint32_t* out;
	int count, capacity;
} rp_words;

static void rp_word( rp_words* w, uint32_t v )
{
	if ( w->count < w->capacity ) w->out[w->count] = v;
	w->count += 1;
}
static void rp_float( rp_words* w, float f )
{
	uint32_t b;
	memcpy( &b, &f, 4 );
	rp_word( w, b );
}
static void rp_int( rp_words* w, int v ) { rp_word( w, (uint32_t)v ); }
static void rp_bytes( rp_words* w, const void* p, int n )
{
	for ( int i = 0; i < n; ++i ) rp_word( w, ( (const uint8_t*)p )[i] );
}
static void rp_pool( rp_words* w, b2IdPool* pool )
{
	rp_int( w, pool->nextIndex );
	rp_int( w, b2GetIdCount( pool ) );
}

B2P_EXPORT int b2p_state_words( uint32_t packedWorldId, uint32_t* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	b2World* world = b2GetWorldFromId( id );
	rp_words w = { out, 0, capacity };
	for ( int i = 0; i < world->bodies.count; ++i )
	{
		b2Body* body = world->bodies.data + i;
		if ( body->id != i ) continue;
		b2BodySim* sim = b2GetBodySim( world, body );
		rp_float( &w, (float)sim->transform.p.x );
		rp_float( &w, (float)sim->transform.p.y );
		rp_float( &w, sim->transform.q.c );
		rp_float( &w, sim->transform.q.s );
		b2BodyState* state = b2GetBodyState( world, body );
		if ( state != NULL )
		{
			rp_float( &w, state->linearVelocity.x );
			rp_float( &w, state->linearVelocity.y );
			rp_float( &w, state->angularVelocity );
		}
		rp_int( &w, body->setIndex );
		rp_int( &w, body->localIndex );
	}
	for ( int i = 0; i < world->contacts.count; ++i )
	{
		b2Contact* contact = world->contacts.data + i;
		if ( contact->contactId != i ) continue;
		rp_int( &w, contact->setIndex );
		rp_int( &w, contact->colorIndex );
		rp_int( &w, contact->localIndex );
		b2ContactSim* sim = b2GetContactSim( world, contact );
		if ( sim != NULL )
		{
			rp_int( &w, sim->manifold.pointCount );
			for ( int p = 0; p < sim->manifold.pointCount; ++p )
			{
				rp_float( &w, sim->manifold.points[p].normalImpulse );
				rp_float( &w, sim->manifold.points[p].tangentImpulse );
				rp_float( &w, sim->manifold.points[p].totalNormalImpulse );
			}
		}
	}
	for ( int i = 0; i < world->joints.count; ++i )
	{
		b2Joint* joint = world->joints.data + i;
		if ( joint->jointId != i ) continue;
		rp_int( &w, joint->setIndex );
		rp_int( &w, joint->colorIndex );
		rp_int( &w, joint->localIndex );
		b2JointSim* sim = b2GetJointSim( world, joint );
		if ( sim == NULL ) continue;
		switch ( sim->type )
		{
			case b2_distanceJoint:
				rp_float( &w, sim->distanceJoint.impulse );
				rp_float( &w, sim->distanceJoint.lowerImpulse );
				rp_float( &w, sim->distanceJoint.upperImpulse );
				rp_float( &w, sim->distanceJoint.motorImpulse );
				break;
			case b2_moverJoint:
				rp_float( &w, sim->moverJoint.linearVelocityImpulse.x );
				rp_float( &w, sim->moverJoint.linearVelocityImpulse.y );
				break;
			case b2_motorJoint:
				rp_float( &w, sim->motorJoint.linearVelocityImpulse.x );
				rp_float( &w, sim->motorJoint.linearVelocityImpulse.y );
				rp_float( &w, sim->motorJoint.angularVelocityImpulse );
				rp_float( &w, sim->motorJoint.linearSpringImpulse.x );
				rp_float( &w, sim->motorJoint.linearSpringImpulse.y );
				rp_float( &w, sim->motorJoint.angularSpringImpulse );
				break;
			case b2_pogoJoint:
				rp_float( &w, sim->pogoJoint.impulse );
				rp_float( &w, sim->pogoJoint.velocity );
				break;
			case b2_prismaticJoint:
				rp_bytes( &w, &sim->prismaticJoint.impulse, (int)sizeof( b2Vec2 ) );
				rp_float( &w, sim->prismaticJoint.springImpulse );
				rp_float( &w, sim->prismaticJoint.motorImpulse );
				rp_float( &w, sim->prismaticJoint.lowerImpulse );
				rp_float( &w, sim->prismaticJoint.upperImpulse );
				break;
			case b2_revoluteJoint:
				rp_bytes( &w, &sim->revoluteJoint.linearImpulse, (int)sizeof( b2Vec2 ) );
				rp_float( &w, sim->revoluteJoint.springImpulse );
				rp_float( &w, sim->revoluteJoint.motorImpulse );
				rp_float( &w, sim->revoluteJoint.lowerImpulse );
				rp_float( &w, sim->revoluteJoint.upperImpulse );
				break;
			case b2_weldJoint:
				rp_bytes( &w, &sim->weldJoint.linearImpulse, (int)sizeof( b2Vec2 ) );
				rp_float( &w, sim->weldJoint.angularImpulse );
				break;
			case b2_wheelJoint:
				rp_float( &w, sim->wheelJoint.perpImpulse );
				rp_float( &w, sim->wheelJoint.motorImpulse );
				rp_float( &w, sim->wheelJoint.springImpulse );
				rp_float( &w, sim->wheelJoint.lowerImpulse );
				rp_float( &w, sim->wheelJoint.upperImpulse );
				break;
			default:
				break;
		}
	}
	rp_pool( &w, &world->bodyIdPool );
	rp_pool( &w, &world->shapeIdPool );
	rp_pool( &w, &world->chainIdPool );
	rp_pool( &w, &world->contactIdPool );
	rp_pool( &w, &world->jointIdPool );
	rp_pool( &w, &world->islandIdPool );
	rp_pool( &w, &world->solverSetIdPool );
	rp_int( &w, world->solverSets.count );
	return w.count;
}
