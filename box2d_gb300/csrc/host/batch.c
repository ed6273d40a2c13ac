/*
 * Batched stepping of many independent worlds (b2World_StepBatch; no counterpart in the
 * reference API, whose worlds are stepped one call at a time).
 *
 * The step has three waits (pair query, narrowphase, solver). Batched, every world runs
 * each of the step's four phases (step.c) on a pool of host threads while its device work
 * is recorded instead of issued; between phases one flush replays the records of all
 * worlds with one launch per kernel kind and position (b2gDev_BatchFlush). A world whose
 * solve is not a one-CTA solve issues it on its own stream in the last phase.
 * The result of every world is exactly what b2World_Step alone produces.
 *
 * B2G_BATCH=streams selects the other strategy: every world steps on its own stream, from
 * a pool of threads that wait on their worlds in turn.
 */
#include "b2g_world.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <unistd.h>

/* ---- a fork-join pool of host threads, kept across calls ---- */
typedef struct h_pool
{
	pthread_mutex_t runMu; /* held by the thread that runs the pool */
	pthread_mutex_t mu;
	pthread_cond_t start, done;
	pthread_t threads[256];
	int threadCount;
	unsigned generation;
	int finished;
	void ( *fn )( void* ctx, int index );
	void* ctx;
	int count;
	atomic_int next;
} h_pool;

static h_pool h_thePool = { .runMu = PTHREAD_MUTEX_INITIALIZER,
							 .mu = PTHREAD_MUTEX_INITIALIZER,
							 .start = PTHREAD_COND_INITIALIZER,
							 .done = PTHREAD_COND_INITIALIZER };

static void h_poolDrain( h_pool* p )
{
	for ( ;; )
	{
		int i = atomic_fetch_add( &p->next, 1 );
		if ( i >= p->count ) break;
		p->fn( p->ctx, i );
	}
}

static void* h_poolMain( void* arg )
{
	h_pool* p = arg;
	unsigned seen = 0;
	pthread_mutex_lock( &p->mu );
	for ( ;; )
	{
		while ( p->generation == seen ) pthread_cond_wait( &p->start, &p->mu );
		seen = p->generation;
		pthread_mutex_unlock( &p->mu );
		h_poolDrain( p );
		pthread_mutex_lock( &p->mu );
		p->finished += 1;
		pthread_cond_broadcast( &p->done );
	}
	return NULL;
}

static void h_poolRunLocked( h_pool* p, int threads, void ( *fn )( void*, int ), void* ctx, int count )
{
	pthread_mutex_lock( &p->mu );
	while ( p->threadCount < threads - 1 && p->threadCount < 256 )
	{
		if ( pthread_create( p->threads + p->threadCount, NULL, h_poolMain, p ) != 0 ) break;
		pthread_detach( p->threads[p->threadCount] );
		p->threadCount += 1;
	}
	p->fn = fn;
	p->ctx = ctx;
	p->count = count;
	atomic_store( &p->next, 0 );
	p->finished = 0;
	p->generation += 1;
	int helpers = p->threadCount;
	pthread_cond_broadcast( &p->start );
	pthread_mutex_unlock( &p->mu );
	h_poolDrain( p );
	pthread_mutex_lock( &p->mu );
	while ( p->finished < helpers ) pthread_cond_wait( &p->done, &p->mu );
	pthread_mutex_unlock( &p->mu );
}

/* run fn(ctx, i) for i in [0, count) on `threads` threads (the caller is one of them) */
static void h_poolRun( int threads, void ( *fn )( void*, int ), void* ctx, int count )
{
	h_pool* p = &h_thePool;
	pthread_mutex_lock( &p->runMu );
	h_poolRunLocked( p, threads, fn, ctx, count );
	pthread_mutex_unlock( &p->runMu );
}

int h_parallelFor( int threads, void ( *fn )( void*, int ), void* ctx, int count )
{
	h_pool* p = &h_thePool;
	if ( pthread_mutex_trylock( &p->runMu ) != 0 ) return 0;
	h_poolRunLocked( p, threads, fn, ctx, count );
	pthread_mutex_unlock( &p->runMu );
	return 1;
}

int h_hostThreads( void )
{
	static int threads = 0;
	if ( threads == 0 )
	{
		long n = sysconf( _SC_NPROCESSORS_ONLN );
		threads = n > 8 ? 8 : ( n < 1 ? 1 : (int)n );
	}
	return threads;
}

/* ---- batched stepping ---- */
typedef struct h_lockstep
{
	h_world** worlds;
	float timeStep;
	int subStepCount;
} h_lockstep;

/* thread time of the phases summed over worlds (microseconds), beside their wall time */
static _Atomic long long h_phaseThreadUs[4];

static void h_phaseBegin( void* ctx, int i )
{
	h_lockstep* L = ctx;
	uint64_t t0 = b2GetTicks();
	h_stepBegin( L->worlds[i], L->timeStep, L->subStepCount );
	atomic_fetch_add( &h_phaseThreadUs[0], (long long)( 1e3 * b2GetMilliseconds( t0 ) ) );
}

static void h_phasePairs( void* ctx, int i )
{
	h_lockstep* L = ctx;
	uint64_t t0 = b2GetTicks();
	h_stepPairs( L->worlds[i] );
	atomic_fetch_add( &h_phaseThreadUs[1], (long long)( 1e3 * b2GetMilliseconds( t0 ) ) );
}

static void h_phaseCollide( void* ctx, int i )
{
	h_lockstep* L = ctx;
	uint64_t t0 = b2GetTicks();
	h_stepCollide( L->worlds[i], 1 );
	atomic_fetch_add( &h_phaseThreadUs[2], (long long)( 1e3 * b2GetMilliseconds( t0 ) ) );
}

static void h_phaseFinishWorld( h_lockstep* L, int i );

static void h_phaseFinish( void* ctx, int i )
{
	uint64_t t0 = b2GetTicks();
	h_phaseFinishWorld( ctx, i );
	atomic_fetch_add( &h_phaseThreadUs[3], (long long)( 1e3 * b2GetMilliseconds( t0 ) ) );
}

static void h_phaseFinishWorld( h_lockstep* L, int i )
{
	h_world* w = L->worlds[i];
	if ( w->stepSolveLate )
	{
		/* not a one-CTA solve: issue it on the world's own stream (nothing is recorded for
		   the world since the last flush) */
		b2gDev_BatchRecord( w->dev, 0 );
		h_stepSolveIssue( w );
		b2gDev_Synchronize( w->dev );
		h_stepFinish( w );
		b2gDev_BatchRecord( w->dev, 1 );
		return;
	}
	h_stepFinish( w );
}

static void h_phaseEvents( void* ctx, int i )
{
	h_lockstep* L = ctx;
	h_world* w = L->worlds[i];
	if ( w->moveEventsValid == 0 && w->stepIndex > 0 ) h_buildMoveEvents( w );
}

static pthread_mutex_t h_batchMu = PTHREAD_MUTEX_INITIALIZER;
static b2gDevBatch* h_batchDevice = NULL;

/* accumulated milliseconds of batched stepping: the four host phases, the flushes, and the
   kernels the flushes launched */
static double h_batchMs[6];
static long long h_batchFlushLaunches;

static void h_poolFor( void* pool, int count, void ( *fn )( void*, int ), void* ctx )
{
	h_poolRun( *(int*)pool, fn, ctx, count );
}

static void h_flushAll( b2gDevBatch* batch, b2gDeviceWorld** devs, int n, int threads )
{
	uint64_t t0 = b2GetTicks();
	int rc = b2gDev_BatchFlush( batch, devs, n, h_poolFor, &threads );
	h_batchMs[4] += b2GetMilliseconds( t0 );
	if ( rc != 0 )
	{
		fprintf( stderr, "box2d_gb300: batched flush failed: %s\n", b2gDev_ErrorString( rc ) );
		abort();
	}
}

/* the other strategy: each world steps alone on its stream */
typedef struct h_streamJob
{
	h_world** worlds;
	float timeStep;
	int subStepCount;
	int blocking;
} h_streamJob;

static void h_streamStep( void* ctx, int i )
{
	h_streamJob* job = ctx;
	h_world* w = job->worlds[i];
	b2gDev_SetBlockingSync( w->dev, job->blocking );
	b2World_Step( ( b2WorldId ){ (uint16_t)( w->worldId + 1 ), w->generation }, job->timeStep, job->subStepCount );
	b2gDev_SetBlockingSync( w->dev, 0 );
}

void b2World_StepBatch( const b2WorldId* worldIds, int worldCount, float timeStep, int subStepCount, int threadCount )
{
	if ( worldIds == NULL || worldCount <= 0 ) return;
	h_world** worlds = malloc( (size_t)worldCount * sizeof( h_world* ) );
	b2gDeviceWorld** devs = malloc( (size_t)worldCount * sizeof( b2gDeviceWorld* ) );
	int n = 0;
	for ( int i = 0; i < worldCount; ++i )
	{
		h_world* w = h_worldFromId( worldIds[i] );
		if ( w == NULL || w->locked ) continue;
		worlds[n] = w;
		devs[n] = w->dev;
		n += 1;
	}
	int threads = threadCount > 0 ? threadCount : 1;
	const char* mode = getenv( "B2G_BATCH" );
	int batched = mode == NULL || strcmp( mode, "streams" ) != 0;
	/* the phases never wait on the device: more threads than cores only contend */
	long cores = sysconf( _SC_NPROCESSORS_ONLN );
	if ( batched && cores > 0 && threads > cores ) threads = (int)cores;
	if ( batched == 0 )
	{
		h_streamJob job = { worlds, timeStep, subStepCount, threads > 1 };
		h_poolRun( threads, h_streamStep, &job, n );
	}
	else if ( n > 0 )
	{
		pthread_mutex_lock( &h_batchMu );
		if ( h_batchDevice == NULL && b2gDev_BatchCreate( &h_batchDevice ) != 0 )
		{
			fprintf( stderr, "box2d_gb300: batched stepping unavailable\n" );
			abort();
		}
		/* every world's earlier work is done: recorded work replays on the flush stream */
		b2gDev_DeviceSynchronize();
		for ( int i = 0; i < n; ++i ) b2gDev_BatchRecord( devs[i], 1 );
		h_lockstep L = { worlds, timeStep, subStepCount };
		void ( *phases[4] )( void*, int ) = { h_phaseBegin, h_phasePairs, h_phaseCollide, h_phaseFinish };
		for ( int k = 0; k < 4; ++k )
		{
			uint64_t t0 = b2GetTicks();
			h_poolRun( threads, phases[k], &L, n );
			h_batchMs[k] += b2GetMilliseconds( t0 );
			/* after the last phase, whatever it recorded replays so every world ends idle */
			h_flushAll( h_batchDevice, devs, n, threads );
		}
		h_batchFlushLaunches = b2gDev_BatchLaunches( h_batchDevice );
		for ( int i = 0; i < n; ++i ) b2gDev_BatchRecord( devs[i], 0 );
		/* sensor overlaps of the worlds that have sensors, on the final state; their end
		   events go to the buffer the step just completed (the one the reader uses) */
		for ( int i = 0; i < n; ++i )
			if ( worlds[i]->sensors.count > 0 && worlds[i]->sensorStep != worlds[i]->stepIndex )
				h_overlapSensors( worlds[i], 1 - worlds[i]->endEventArrayIndex );
		/* the move events of every world, from the state the last flush delivered, as the
		   reference's finalize builds them inside the step */
		uint64_t t0 = b2GetTicks();
		h_poolRun( threads, h_phaseEvents, &L, n );
		h_batchMs[3] += b2GetMilliseconds( t0 );
		pthread_mutex_unlock( &h_batchMu );
	}
	free( worlds );
	free( devs );
}

/* milliseconds spent by batched stepping since the last reset: begin, pairs, collide and
   finish phases (host), flushes (host assembly, copies and device work); out[5] = kernels
   launched by flushes since the library loaded; out[6..7] flush assembly and wait, out[8..11]
   thread-time of the four phases, out[12..16] the flush's planning, layout, staging, issue
   and delivery (17 floats) */
__attribute__( ( visibility( "default" ) ) ) void b2p_batch_profile( float* out, int reset )
{
	pthread_mutex_lock( &h_batchMu );
	for ( int k = 0; k < 5; ++k ) out[k] = (float)h_batchMs[k];
	out[5] = (float)h_batchFlushLaunches;
	double assembleMs = 0.0, waitMs = 0.0;
	if ( h_batchDevice ) b2gDev_BatchTimes( h_batchDevice, &assembleMs, &waitMs, reset );
	out[6] = (float)assembleMs;
	out[7] = (float)waitMs;
	for ( int k = 0; k < 4; ++k ) out[8 + k] = (float)( 1e-3 * (double)atomic_load( &h_phaseThreadUs[k] ) );
	double parts[5] = { 0.0, 0.0, 0.0, 0.0, 0.0 };
	if ( h_batchDevice ) b2gDev_BatchPartTimes( h_batchDevice, parts, reset );
	for ( int k = 0; k < 5; ++k ) out[12 + k] = (float)parts[k];
	if ( reset )
	{
		for ( int k = 0; k < 5; ++k ) h_batchMs[k] = 0.0;
		for ( int k = 0; k < 4; ++k ) atomic_store( &h_phaseThreadUs[k], 0 );
	}
	pthread_mutex_unlock( &h_batchMu );
}
