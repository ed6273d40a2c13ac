/*
 * Batched stepping of many independent worlds (b2World_StepBatch; no counterpart in the
 * reference API, whose worlds are stepped one call at a time).
 *
 * Each world keeps its own host bookkeeping, device buffers and CUDA stream, so worlds
 * share nothing but the GPU: a pool of host threads pulls world indices from an atomic
 * counter and runs b2World_Step on each. While one world's thread waits for its device
 * work, the others keep the GPU fed, so the device work of many small worlds overlaps.
 * With more than one thread the waits block (sleep) instead of spinning, so the thread
 * count can exceed the host's cores.
 * The result of every world is exactly what b2World_Step alone produces.
 */
#include "b2g_world.h"

#include <pthread.h>
#include <stdatomic.h>

typedef struct h_batchJob
{
	const b2WorldId* worldIds;
	int worldCount;
	float timeStep;
	int subStepCount;
	int blocking; /* waits sleep: more stepping threads than host cores */
	atomic_int next;
} h_batchJob;

static void h_batchRun( h_batchJob* job )
{
	for ( ;; )
	{
		int i = atomic_fetch_add( &job->next, 1 );
		if ( i >= job->worldCount ) break;
		h_world* w = h_worldFromId( job->worldIds[i] );
		if ( w == NULL ) continue;
		b2gDev_SetBlockingSync( w->dev, job->blocking );
		b2World_Step( job->worldIds[i], job->timeStep, job->subStepCount );
		b2gDev_SetBlockingSync( w->dev, 0 );
	}
}

static void* h_batchWorker( void* arg )
{
	h_batchRun( (h_batchJob*)arg );
	return NULL;
}

#define H_BATCH_MAX_THREADS 256

void b2World_StepBatch( const b2WorldId* worldIds, int worldCount, float timeStep, int subStepCount, int threadCount )
{
	if ( worldIds == NULL || worldCount <= 0 ) return;
	h_batchJob job;
	job.worldIds = worldIds;
	job.worldCount = worldCount;
	job.timeStep = timeStep;
	job.subStepCount = subStepCount;
	job.blocking = threadCount > 1;
	atomic_init( &job.next, 0 );
	int helpers = threadCount - 1;
	if ( helpers > worldCount - 1 ) helpers = worldCount - 1;
	if ( helpers > H_BATCH_MAX_THREADS ) helpers = H_BATCH_MAX_THREADS;
	pthread_t threads[H_BATCH_MAX_THREADS];
	int started = 0;
	for ( int t = 0; t < helpers; ++t )
	{
		if ( pthread_create( threads + t, NULL, h_batchWorker, &job ) != 0 ) break;
		started += 1;
	}
	h_batchRun( &job );
	for ( int t = 0; t < started; ++t ) pthread_join( threads[t], NULL );
}
