/*
 * Oracle (test checker only): contact-table probe with the same row layout as the
 * probe compiled into the reference build and the GB300 library's b2p_contacts.
 */
#include "o_core.h"

#define B2P_EXPORT __attribute__( ( visibility( "default" ) ) )

static o_contactSim* o_contactSimOf( o_world* w, o_contact* c )
{
	if ( c->colorIndex != B2_NULL_INDEX ) return w->colors[c->colorIndex].contactSims.data + c->localIndex;
	return w->awakeContactSims.data + c->localIndex;
}

B2P_EXPORT int b2p_contacts( uint32_t packedWorldId, int* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	o_world* w = o_worldFromId( id );
	int n = 0;
	for ( int i = 0; i < w->contacts.count; ++i )
	{
		o_contact* c = w->contacts.data + i;
		if ( c->contactId != i ) continue;
		if ( n < capacity )
		{
			o_contactSim* sim = o_contactSimOf( w, c );
			int* o = out + 8 * n;
			o[0] = c->contactId;
			o[1] = c->shapeIdA;
			o[2] = c->shapeIdB;
			o[3] = c->colorIndex;
			o[4] = sim->manifold.pointCount;
			o[5] = sim->manifold.pointCount > 0 ? sim->manifold.points[0].id : -1;
			o[6] = sim->manifold.pointCount > 1 ? sim->manifold.points[1].id : -1;
			o[7] = ( c->flags & O_C_TOUCHING ) ? 1 : 0;
		}
		n += 1;
	}
	return n;
}

B2P_EXPORT int b2p_contact_floats( uint32_t packedWorldId, float* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	o_world* w = o_worldFromId( id );
	int n = 0;
	for ( int i = 0; i < w->contacts.count; ++i )
	{
		o_contact* c = w->contacts.data + i;
		if ( c->contactId != i ) continue;
		if ( n < capacity )
		{
			o_contactSim* sim = o_contactSimOf( w, c );
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

extern int o_continuousSkipped;

/* continuous collision of one world since its creation: fast bodies swept, sweeps that hit */
B2P_EXPORT void b2p_continuous_counts( uint32_t packedWorldId, int* out )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	o_world* w = o_worldFromId( id );
	out[0] = w->continuousSweeps;
	out[1] = w->continuousHits;
}

/* number of fast-body continuous steps the oracle could not restate (0 when exact) */
B2P_EXPORT int b2p_oracle_unsupported( void ) { return o_continuousSkipped; }

/* threads of the oracle's data-parallel loops (1 = serial, the default) */
B2P_EXPORT void b2o_set_threads( int n ) { o_setThreads( n ); }
