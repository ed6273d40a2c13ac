/*
 * Parity probes of the GB300 step library: the live contact table with the same row
 * layout as the probe compiled into the reference build and the oracle
 * (contactId, shapeIdA, shapeIdB, colorIndex, pointCount, id0, id1, touching), and the
 * per-step device status. Declared in include/b2g_probe.h.
 */
#include "b2g_world.h"

#include <stdio.h>

#define B2P_EXPORT __attribute__( ( visibility( "default" ) ) )

static b2gContact* h_downloadContacts( h_world* w )
{
	int n = w->contactIdPool.nextIndex;
	b2gContact* dc = malloc( (size_t)( n > 0 ? n : 1 ) * sizeof( b2gContact ) );
	int rc = b2gDev_DownloadContacts( w->dev, dc, n );
	if ( rc != 0 ) h_fail( w, "contact download", rc );
	return dc;
}

B2P_EXPORT int b2p_contacts( uint32_t packedWorldId, int* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	if ( w == NULL ) return -1;
	b2gContact* dc = h_downloadContacts( w );
	int n = 0;
	for ( int i = 0; i < w->contacts.count; ++i )
	{
		h_contact* c = w->contacts.data + i;
		if ( c->contactId != i ) continue;
		if ( n < capacity )
		{
			const b2Manifold* m = &dc[i].manifold;
			int* o = out + 8 * n;
			o[0] = c->contactId;
			o[1] = c->shapeIdA;
			o[2] = c->shapeIdB;
			o[3] = c->colorIndex;
			o[4] = m->pointCount;
			o[5] = m->pointCount > 0 ? m->points[0].id : -1;
			o[6] = m->pointCount > 1 ? m->points[1].id : -1;
			o[7] = ( c->flags & B2G_C_TOUCHING ) ? 1 : 0;
		}
		n += 1;
	}
	free( dc );
	return n;
}

B2P_EXPORT int b2p_contact_floats( uint32_t packedWorldId, float* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	if ( w == NULL ) return -1;
	b2gContact* dc = h_downloadContacts( w );
	int n = 0;
	for ( int i = 0; i < w->contacts.count; ++i )
	{
		h_contact* c = w->contacts.data + i;
		if ( c->contactId != i ) continue;
		if ( n < capacity )
		{
			const b2Manifold* m = &dc[i].manifold;
			float* o = out + 12 * n;
			o[0] = m->normal.x;
			o[1] = m->normal.y;
			for ( int p = 0; p < 2; ++p )
			{
				const b2ManifoldPoint* mp = m->points + p;
				int live = p < m->pointCount;
				o[2 + 5 * p] = live ? mp->separation : 0.0f;
				o[3 + 5 * p] = live ? mp->normalImpulse : 0.0f;
				o[4 + 5 * p] = live ? mp->tangentImpulse : 0.0f;
				o[5 + 5 * p] = live ? mp->anchorA.x : 0.0f;
				o[6 + 5 * p] = live ? mp->anchorA.y : 0.0f;
			}
		}
		n += 1;
	}
	free( dc );
	return n;
}

/* the values b2World_GetStateHash mixes, in order (to locate a bookkeeping difference) */
B2P_EXPORT int b2p_state_words( uint32_t packedWorldId, uint32_t* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	return w == NULL ? -1 : h_stateHashWords( w, out, capacity );
}

/* device status of the last step (0 ok, 1 non-finite velocity, 2 capacity) */
B2P_EXPORT int b2p_status( uint32_t packedWorldId )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	return w == NULL ? -1 : w->lastStatus;
}

/* continuous collision of one world since its creation: fast bodies swept, sweeps that hit */
B2P_EXPORT void b2p_continuous_counts( uint32_t packedWorldId, int* out )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	out[0] = w == NULL ? 0 : w->continuousSweeps;
	out[1] = w == NULL ? 0 : w->continuousHits;
}

/* accumulated device stage times (ms: pairs, narrowphase, solver, finalize) and
   host<->device traffic (bytes: to device, to host) and the number of kernels launched since the last reset */
B2P_EXPORT int b2p_timings( uint32_t packedWorldId, float* stageMs, long long* traffic, int reset )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	if ( w == NULL ) return -1;
	b2gDev_Timings( w->dev, stageMs, traffic, reset );
	return 0;
}

/* the CUDA stream every kernel of this world is launched on (cudaStream_t) */
B2P_EXPORT void* b2p_stream( uint32_t packedWorldId )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	return w == NULL ? NULL : b2gDev_Stream( w->dev );
}

/* accumulated host time per step phase since the last reset, in ms: tree upload, pair
   query, contact creation, tree rebuild, narrowphase, contact-state pass, contact / color /
   joint uploads, solver, proxy enlargement, (unused) */
B2P_EXPORT int b2p_host_profile( uint32_t packedWorldId, float* out, int reset )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	if ( w == NULL ) return -1;
	memcpy( out, w->hostMs, sizeof( w->hostMs ) );
	if ( reset ) memset( w->hostMs, 0, sizeof( w->hostMs ) );
	return 0;
}

/* b2p_contacts without any allocation: the table is built on the device in a fixed scratch
   array (see noalloc.cu for its limit and rules). Needs a world that has been stepped with
   a positive time step since its last change; returns the row count (may exceed
   capacity), -1 for an unknown or never-stepped world, -2 when the world has more contact
   ids than the scratch holds, or -(1000 + CUDA error code). */
B2P_EXPORT int b2p_contacts_noalloc( uint32_t packedWorldId, int* out, int capacity )
{
	b2WorldId id = { (uint16_t)( packedWorldId >> 16 ), (uint16_t)( packedWorldId & 0xFFFF ) };
	h_world* w = h_worldFromId( id );
	if ( w == NULL || w->devReady == 0 ) return -1;
	int rc = b2gDev_ContactTableNoAlloc( w->dev, w->contactIdPool.nextIndex, out, capacity );
	if ( rc == -2 )
		fprintf( stderr, "b2p_contacts_noalloc: the world has %d contact ids, more than the fixed scratch holds; use b2p_contacts\n",
				 w->contactIdPool.nextIndex );
	else if ( rc <= -1000 )
		fprintf( stderr, "b2p_contacts_noalloc: %s\n", b2gDev_ErrorString( -1000 - rc ) );
	return rc;
}
