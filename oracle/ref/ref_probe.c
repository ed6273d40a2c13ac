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
