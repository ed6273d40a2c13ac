/*
 * Differentiable stepping, host side (box2d_gb300_diff.h): a tape owns, per world, a device
 * arena of step records appended by b2World_Step while recording, and runs the adjoint
 * kernels (adjoint.cu) over all of its worlds at once.
 */
#include "b2g_world.h"
#include "box2d_gb300_diff.h"

#include <stdio.h>

typedef struct h_tapeWorld
{
	b2DiffTape* tape;
	h_world* world;
	void* arena;
	long long capacity, used;
	long long* offsets;
	int stepCount, offsetCapacity;
	int maxAwake, maxSlots, maxSubsteps;
	int bodyCount, shapeCount;
	int setChanges; /* the world's set-change count at the first recorded step */
} h_tapeWorld;

struct b2DiffTape
{
	int worldCount;
	int recording;
	h_tapeWorld* worlds;
	float lastMs;
	int lastLaunches;
	int lastFailure[5];
};

b2DiffTape* b2Diff_CreateTape( const b2WorldId* worlds, int worldCount )
{
	if ( worldCount <= 0 ) return NULL;
	b2DiffTape* t = calloc( 1, sizeof( b2DiffTape ) );
	t->worldCount = worldCount;
	t->worlds = calloc( (size_t)worldCount, sizeof( h_tapeWorld ) );
	for ( int i = 0; i < worldCount; ++i )
	{
		h_world* w = h_worldFromId( worlds[i] );
		if ( w == NULL || w->tape != NULL )
		{
			for ( int j = 0; j < i; ++j ) t->worlds[j].world->tape = NULL;
			free( t->worlds );
			free( t );
			return NULL;
		}
		t->worlds[i].tape = t;
		t->worlds[i].world = w;
		w->tape = t->worlds + i;
	}
	return t;
}

static void h_tapeClear( h_tapeWorld* tw )
{
	tw->used = 0;
	tw->stepCount = 0;
	tw->maxAwake = 0;
	tw->maxSlots = 0;
	tw->maxSubsteps = 0;
}

void b2Diff_DestroyTape( b2DiffTape* t )
{
	if ( t == NULL ) return;
	for ( int i = 0; i < t->worldCount; ++i )
	{
		h_tapeWorld* tw = t->worlds + i;
		if ( tw->world != NULL ) tw->world->tape = NULL;
		if ( tw->world != NULL ) b2gDev_Synchronize( tw->world->dev );
		b2gDev_FreeTapeArena( tw->arena );
		free( tw->offsets );
	}
	free( t->worlds );
	free( t );
}

void h_tapeDetach( h_world* w )
{
	if ( w->tape == NULL ) return;
	b2gDev_Synchronize( w->dev );
	w->tape->world = NULL;
	w->tape = NULL;
}

void b2Diff_Record( b2DiffTape* t, bool on )
{
	if ( t == NULL ) return;
	if ( on && t->recording == 0 )
		for ( int i = 0; i < t->worldCount; ++i ) h_tapeClear( t->worlds + i );
	t->recording = on ? 1 : 0;
}

int b2Diff_StepCount( const b2DiffTape* t )
{
	if ( t == NULL || t->worldCount == 0 ) return 0;
	int n = t->worlds[0].stepCount;
	for ( int i = 1; i < t->worldCount; ++i )
		if ( t->worlds[i].stepCount < n ) n = t->worlds[i].stepCount;
	return n;
}

void h_tapeCapture( h_world* w, const b2gStepParams* params )
{
	h_tapeWorld* tw = w->tape;
	if ( tw->tape->recording == 0 ) return;
	if ( tw->stepCount == tw->offsetCapacity )
	{
		tw->offsetCapacity = tw->offsetCapacity ? 2 * tw->offsetCapacity : 64;
		tw->offsets = realloc( tw->offsets, (size_t)tw->offsetCapacity * sizeof( long long ) );
	}
	int awake = w->awakeBodyIds.count;
	int slots = 0;
	for ( int i = 0; i < B2_GRAPH_COLOR_COUNT; ++i ) slots += w->colors[i].contactIds.count;
	long long offset = 0;
	if ( tw->stepCount == 0 ) tw->setChanges = w->setChangeCount;
	int rc = b2gDev_CaptureTape( w->dev, params, w->bodies.count, awake, w->joints.count, &tw->arena, &tw->capacity, &tw->used,
								 &offset );
	if ( rc != 0 ) h_fail( w, "tape capture", rc );
	tw->offsets[tw->stepCount++] = offset;
	tw->maxAwake = awake > tw->maxAwake ? awake : tw->maxAwake;
	tw->maxSlots = slots > tw->maxSlots ? slots : tw->maxSlots;
	tw->maxSubsteps = params->subStepCount > tw->maxSubsteps ? params->subStepCount : tw->maxSubsteps;
	tw->bodyCount = w->bodies.count;
	tw->shapeCount = w->shapes.count;
}

void b2Diff_Sizes( const b2DiffTape* t, int* bodyCounts, int* shapeCounts )
{
	for ( int i = 0; i < t->worldCount; ++i )
	{
		const h_tapeWorld* tw = t->worlds + i;
		bodyCounts[i] = tw->world ? tw->world->bodies.count : tw->bodyCount;
		shapeCounts[i] = tw->world ? tw->world->shapes.count : tw->shapeCount;
	}
}

int b2Diff_Backward( b2DiffTape* t, const float* adjCenter, const float* adjRotation, const float* adjVelocity, float* gradVelocity,
					 float* gradCenter, float* gradFriction )
{
	if ( t == NULL || adjCenter == NULL || gradVelocity == NULL ) return B2_DIFF_BAD_ARGUMENT;
	int steps = b2Diff_StepCount( t );
	if ( steps == 0 ) return B2_DIFF_EMPTY;
	memset( t->lastFailure, 0, sizeof( t->lastFailure ) );
	int n = t->worldCount;
	b2gAdjointWorld* aw = calloc( (size_t)n, sizeof( b2gAdjointWorld ) );
	int* bodyOffsets = malloc( (size_t)( n + 1 ) * sizeof( int ) );
	int* shapeOffsets = malloc( (size_t)( n + 1 ) * sizeof( int ) );
	bodyOffsets[0] = 0;
	shapeOffsets[0] = 0;
	int rc = 0;
	for ( int i = 0; i < n; ++i )
	{
		h_tapeWorld* tw = t->worlds + i;
		if ( tw->world == NULL || tw->stepCount != steps )
		{
			rc = B2_DIFF_BAD_ARGUMENT;
			break;
		}
		if ( tw->world->setChangeCount != tw->setChanges )
		{
			/* an island fell asleep or woke while recording: the awake set of the recorded
			   steps no longer describes one trajectory */
			rc = B2_DIFF_UNSUPPORTED;
			t->lastFailure[0] = rc;
			t->lastFailure[1] = i;
			t->lastFailure[3] = 6;
			break;
		}
		int shapeCount = 0;
		aw[i].arena = tw->arena;
		aw[i].stepOffsets = tw->offsets;
		aw[i].shapes = b2gDev_ShapeArray( tw->world->dev, &shapeCount );
		aw[i].shapeCount = tw->world->shapes.count;
		aw[i].bodyCount = tw->world->bodies.count;
		aw[i].contactCapacity = b2gDev_ContactCapacity( tw->world->dev );
		aw[i].maxAwake = tw->maxAwake;
		aw[i].maxSlots = tw->maxSlots;
		aw[i].maxSubsteps = tw->maxSubsteps;
		bodyOffsets[i + 1] = bodyOffsets[i] + aw[i].bodyCount;
		shapeOffsets[i + 1] = shapeOffsets[i] + aw[i].shapeCount;
	}
	float* center = gradCenter;
	float* friction = gradFriction;
	if ( rc == 0 )
	{
		if ( center == NULL ) center = malloc( sizeof( float ) * 2 * (size_t)( bodyOffsets[n] > 0 ? bodyOffsets[n] : 1 ) );
		if ( friction == NULL ) friction = malloc( sizeof( float ) * (size_t)( shapeOffsets[n] > 0 ? shapeOffsets[n] : 1 ) );
		rc = b2gDev_AdjointRun( aw, n, steps, bodyOffsets, shapeOffsets, adjCenter, adjRotation, adjVelocity, gradVelocity, center,
								friction, &t->lastMs, &t->lastLaunches, t->lastFailure );
		if ( rc > 0 ) fprintf( stderr, "box2d_gb300: adjoint failed: %s\n", b2gDev_ErrorString( rc ) );
	}
	if ( center != gradCenter ) free( center );
	if ( friction != gradFriction ) free( friction );
	free( aw );
	free( bodyOffsets );
	free( shapeOffsets );
	return rc;
}

void b2Diff_LastFailure( const b2DiffTape* t, int* out )
{
	memcpy( out, t->lastFailure, sizeof( t->lastFailure ) );
}

float b2Diff_LastBackwardMs( const b2DiffTape* t, int* launches )
{
	if ( launches ) *launches = t->lastLaunches;
	return t->lastMs;
}

long long b2Diff_DownloadTape( b2DiffTape* t, int world, void* out, long long capacity )
{
	if ( t == NULL || world < 0 || world >= t->worldCount ) return -1;
	h_tapeWorld* tw = t->worlds + world;
	if ( tw->world == NULL ) return -1;
	int shapeCount = 0;
	const b2gShape* shapes = b2gDev_ShapeArray( tw->world->dev, &shapeCount );
	shapeCount = tw->world->shapes.count;
	long long headerBytes = b2gTapeAlign( 16 + 8LL * tw->stepCount );
	long long shapeBytes = b2gTapeAlign( (long long)shapeCount * (long long)sizeof( b2gShape ) );
	long long total = headerBytes + shapeBytes + tw->used;
	if ( out == NULL || capacity < total ) return total;
	unsigned char* o = out;
	memset( o, 0, (size_t)headerBytes );
	b2gTapeHeader* h = (b2gTapeHeader*)o;
	h->stepCount = tw->stepCount;
	h->shapeCount = shapeCount;
	h->bodyCount = tw->world->bodies.count;
	h->contactCapacity = b2gDev_ContactCapacity( tw->world->dev );
	for ( int i = 0; i < tw->stepCount; ++i ) h->stepOffsets[i] = headerBytes + shapeBytes + tw->offsets[i];
	int rc = b2gDev_DownloadArena( shapes, (long long)shapeCount * (long long)sizeof( b2gShape ), o + headerBytes );
	if ( rc == 0 && tw->used > 0 ) rc = b2gDev_DownloadArena( tw->arena, tw->used, o + headerBytes + shapeBytes );
	return rc == 0 ? total : -1;
}
