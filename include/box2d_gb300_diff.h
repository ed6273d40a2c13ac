/*
 * Differentiable stepping for box2d_gb300 (no counterpart in the reference's box2d.h).
 *
 * A tape records, for a set of worlds, every b2World_Step taken while recording is on:
 * the contact set, its graph coloring and manifolds after the narrowphase, and every
 * body's pose and velocity at the start of the step. b2Diff_Backward then runs the
 * adjoint of the recorded Soft Steps on the GPU, all worlds in one launch per step, with
 * the active contact set, the coloring and every branch (clamps, speculative/soft contact
 * switch, reference edge and clip decisions of the manifold) held as recorded. Colors are
 * swept in reverse; each substep is recomputed from a per-substep checkpoint to get the
 * inputs of every constraint solve, so memory stays bounded by one substep per world.
 *
 * Differentiated: contacts between polygons (boxes and convex polygons, rounded or not),
 * polygon-capsule, segment-polygon, polygon-circle and circle-circle contacts (the
 * manifold's dependence on both poses, and contact recycling), restitution, rolling
 * resistance, speed clamping, gravity and damping. Not differentiated (b2Diff_Backward
 * returns B2_DIFF_UNSUPPORTED for a tape that contains them): joints, capsule-capsule,
 * capsule-circle, segment-circle and segment-capsule contacts, chains, constraints in the
 * overflow color, and islands that fall asleep or wake while recording.
 */
#ifndef BOX2D_GB300_DIFF_H
#define BOX2D_GB300_DIFF_H

#include "box2d_gb300.h"

#ifdef __cplusplus
extern "C"
{
#endif

typedef struct b2DiffTape b2DiffTape;

enum
{
	B2_DIFF_OK = 0,
	B2_DIFF_UNSUPPORTED = -1,	  /* a recorded step holds something the adjoint does not differentiate */
	B2_DIFF_REPLAY_MISMATCH = -2, /* recomputing a recorded step did not reproduce the recorded result */
	B2_DIFF_EMPTY = -3,			  /* no step recorded */
	B2_DIFF_BAD_ARGUMENT = -4,
};

/* A tape over `worldCount` worlds of this library. Recording starts switched off. */
B2G_API b2DiffTape* b2Diff_CreateTape( const b2WorldId* worlds, int worldCount );
B2G_API void b2Diff_DestroyTape( b2DiffTape* tape );

/* While on, every b2World_Step (or b2World_StepBatch) of the tape's worlds appends one
   recorded step. Switching it on clears what was recorded before. */
B2G_API void b2Diff_Record( b2DiffTape* tape, bool on );
B2G_API int b2Diff_StepCount( const b2DiffTape* tape );

/* Reverse pass over every recorded step, all worlds together.
   Inputs, per world w and body id b (bodies of world w start at bodyOffsets[w]):
     adjCenter[2 * (off + b)]   dL/d(center of mass) after the last step
     adjRotation[2 * (off + b)] dL/d(rotation cosine, sine) after the last step (may be NULL)
     adjVelocity[3 * (off + b)] dL/d(linear velocity, angular velocity) after the last step (may be NULL)
   Outputs:
     gradVelocity[3 * (off + b)] dL/d(linear, angular velocity) before the first step
     gradCenter[2 * (off + b)]   dL/d(center of mass) before the first step (may be NULL)
     gradFriction[shapeOffsets[w] + s] dL/d(friction of shape s) (may be NULL)
   bodyOffsets and shapeOffsets have worldCount + 1 entries (prefix sums of the worlds'
   body and shape id counts, b2Diff_Sizes). All arrays are host memory. */
B2G_API int b2Diff_Backward( b2DiffTape* tape, const float* adjCenter, const float* adjRotation, const float* adjVelocity,
							 float* gradVelocity, float* gradCenter, float* gradFriction );

/* body and shape id counts of each world (worldCount entries each) */
B2G_API void b2Diff_Sizes( const b2DiffTape* tape, int* bodyCounts, int* shapeCounts );

/* Where the last b2Diff_Backward failed: code, world, step, check (1 narrowphase replay,
   2 step replay, 3 unsupported shape, 4 unsupported step, 6 an island slept or woke
   while recording) and the contact slot or body id. All zero after a success. */
B2G_API void b2Diff_LastFailure( const b2DiffTape* tape, int* out );

/* Device time of the last b2Diff_Backward (ms) and the kernels it launched. */
B2G_API float b2Diff_LastBackwardMs( const b2DiffTape* tape, int* launches );

/* The recorded bytes of one world (the format of b2g_device_abi.h b2gTapeHeader /
   b2gTapeStep), for checking the adjoint on the host. Returns the size; copies when
   `out` is not NULL and `capacity` is large enough. */
B2G_API long long b2Diff_DownloadTape( b2DiffTape* tape, int world, void* out, long long capacity );

#ifdef __cplusplus
}
#endif

#endif
