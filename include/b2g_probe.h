/*
 * b2g_probe.h -- parity probes and scene builders exported by the GB300 step library.
 * These have no counterpart in the reference's public API: they exist so tests can read
 * the contact table and drive the benchmark scenes through the same C ABI on every
 * build (GB300 library, CPU oracle, and the reference build in the development container).
 */
#ifndef B2G_PROBE_H
#define B2G_PROBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

/* Live contact table, ascending contact id, 8 ints per row:
   contactId, shapeIdA, shapeIdB, colorIndex, pointCount, featureId0, featureId1, touching.
   packedWorldId = (index1 << 16) | generation. Returns the row count (may exceed capacity). */
int b2p_contacts( uint32_t packedWorldId, int* out, int capacity );

/* The table of b2p_contacts built without allocating anything (no counterpart in the
   reference). For callers that may not allocate while they run, such as a real-time loop
   that must not stall in cudaMalloc/cudaFree or host malloc. Limit: 32768 contact ids per
   world (-2 and a message above it). The scratch is one fixed device array per device:
   calls whose GPU work overlaps race on it. A call waits for the world's stream and copies
   into the caller's host array, so it cannot be made inside a CUDA stream capture.
   Returns the row count (may exceed capacity); -1 for an unknown world or one that has not
   been stepped with a positive time step since its last change made through the API (a
   body, shape or joint created or destroyed, a body woken, moved or given a velocity while
   asleep); or -(1000 + CUDA error code). */
int b2p_contacts_noalloc( uint32_t packedWorldId, int* out, int capacity );

/* 12 floats per live contact: normal (2), then per point: separation, normalImpulse,
   tangentImpulse, anchorA (2). Returns the row count. */
int b2p_contact_floats( uint32_t packedWorldId, float* out, int capacity );

/* The 32-bit values b2World_GetStateHash mixes into its hash, in order, up to capacity
   (bytes mixed one by one appear one per value); returns their count. For locating where
   two worlds' state or bookkeeping differ. */
int b2p_state_words( uint32_t packedWorldId, uint32_t* out, int capacity );

/* Device status bits of every step since the world was created (or restored from a
   snapshot): 0 ok, 1 non-finite body velocity, 2 a query ran out of traversal stack,
   4 the persistent solver's grid barrier gave up. */
int b2p_status( uint32_t packedWorldId );

/* Accumulated device time per stage since the last reset, in ms: pair query, narrowphase
   kernel, solver (prepare through store), finalize; and host<->device traffic in bytes
   (to device, to host) and kernels launched, as traffic[0..2]. reset != 0 zeroes them after reading. */
int b2p_timings( uint32_t packedWorldId, float* stageMs, long long* traffic, int reset );

/* Accumulated host time per step phase since the last reset, in ms, 10 floats: tree
   upload, pair query, contact creation, tree rebuild, narrowphase, contact-state pass,
   contact/color/joint uploads, solver, proxy enlargement, unused. Device waits are
   included in the phase that waits. reset != 0 zeroes them after reading. */
int b2p_host_profile( uint32_t packedWorldId, float* out, int reset );

/* The CUDA stream (cudaStream_t) the world's kernels are launched on. */
void* b2p_stream( uint32_t packedWorldId );

/* Batched stepping (b2World_StepBatch) since the last reset, in milliseconds: out[0..3]
   the begin, pairs, collide and finish phases on the host threads, out[4] the flushes;
   out[5] the kernels the flushes launched since the library loaded; out[6], out[7] the
   flushes' host assembly and their wait for the device; out[8..11] the four phases' thread
   time summed over worlds; out[12..16] the flushes' planning, table layout, staging, issue
   and delivery (17 floats). */
void b2p_batch_profile( float* out, int reset );

/* Continuous collision of one world since its creation: out[0] = fast non-bullet bodies
   swept against static shapes, out[1] = sweeps that moved the body back to a time of
   impact (solver.c:384-550). */
void b2p_continuous_counts( uint32_t packedWorldId, int* out );

/* Scene builders (box2d_gb300/scenes/scenes.c). kind: 0 large pyramid, 1 many pyramids
   with rain, 2 joint grid with mixed shapes, 3 one batched world, 4 one ramp world,
   5 reference many_pyramids, 6 reference joint_grid, 7 hello world, 8 shape zoo,
   9 joint zoo (prismatic, weld, wheel, distance and revolute mechanisms).
   flags bit 0 disables continuous collision, bit 1 warm starting, bit 2 contact recycling
   (ramp scene). Returns a handle or -1. */
int b2s_create( int kind, int a, int b, int c, uint32_t seed, int flags );
/* worker threads put in the world definition (b2WorldDef.workerCount) of scenes created
   afterwards; 0 keeps the default. Only a library with its own task system uses it. */
void b2s_set_workers( int count );
void b2s_destroy( int handle );
/* a scripted change to scene body `bodyIndex` between steps: 0 b2Body_ApplyForce (force
   (a, b) at the center of mass + (c, d)), 1 ApplyForceToCenter, 2 ApplyTorque (a),
   3 ApplyLinearImpulse, 4 ApplyLinearImpulseToCenter, 5 ApplyAngularImpulse (a),
   6 SetTransform (position (a, b), angle c), 7 SetTargetTransform (also time step d),
   8 b2DestroyBody, 9 b2DestroyShape of its first shape */
void b2s_body_action( int handle, int kind, int bodyIndex, float a, float b, float c, float d );
void b2s_step( int handle, float timeStep, int subStepCount, int count );
/* step `count` scenes `steps` times, one b2World_StepBatch call (up to `threads` host
   threads) per step on the GB300 library, one world after the other elsewhere */
void b2s_step_batch( const int* handles, int count, float timeStep, int subStepCount, int steps, int threads );
int b2s_body_count( int handle );
int b2s_dynamic_count( int handle );
uint32_t b2s_world_id( int handle );
/* 7 floats per body in creation order: p.x, p.y, q.c, q.s, v.x, v.y, w */
void b2s_get_state( int handle, float* out );
/* the last step's body move events (b2World_GetBodyEvents), 4 floats per event:
   p.x, p.y, q.c, q.s, up to capacity; returns the event count */
int b2s_move_events( int handle, float* out, int capacity );
/* the same for `count` scenes, their events one after the other (capacity events in all);
   returns the event count */
int b2s_move_events_many( const int* handles, int count, float* out, int capacity );
/* the last step's contact begin/end touch events (b2World_GetContactEvents), 5 ints per
   event, begin events first: kind (0 begin, 1 end), shape A id, shape B id, contact id
   (index1 - 1), contact generation, up to capacity; returns the event count */
int b2s_contact_events( int handle, int* out, int capacity );
/* the last step's sensor begin/end touch events (b2World_GetSensorEvents), 5 ints per
   event, begin events first: kind (0 begin, 1 end), sensor shape id, visitor shape id,
   sensor generation, visitor generation; returns the event count (not in the oracle) */
int b2s_sensor_events( int handle, int* out, int capacity );
/* b2World_GetStateHash of the scene's world (not in the oracle, which has no islands) */
uint64_t b2s_world_state_hash( int handle );
/* FNV-1a 64 over the bit patterns of b2s_get_state */
uint64_t b2s_state_hash( int handle );
void b2s_set_velocities( int handle, const float* in );
void b2s_target( int handle, float* out );
void b2s_counters( int handle, int* out );
/* friction of every shape on the scene's bodies, indexed by shape id (count entries) */
void b2s_set_friction( int handle, const float* byShape, int count );
void b2s_get_friction( int handle, float* byShape, int count );
/* world center of mass of each scene body (2 floats), in the order of b2s_get_state */
void b2s_get_centers( int handle, float* out );
/* body id of each scene body, in the order of b2s_get_state */
void b2s_body_ids( int handle, int* out );

#ifdef __cplusplus
}
#endif

#endif
