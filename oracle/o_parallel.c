/*
 * Oracle (test checker and CPU baseline only): a fork-join pool for the data-parallel
 * loops of the step. The reference runs the same loops as tasks on its worker threads
 * (b2CollideTask, the solver stage blocks, b2FinalizeBodiesTask); every item is computed
 * exactly as in the serial loop and items of one loop touch disjoint data, so the result
 * does not depend on the thread count. One thread (the default) runs everything inline.
 */
#include "o_core.h"

#include <pthread.h>
#include <sched.h>
#include <stdatomic.h>

#define O_MAX_THREADS 256

static int o_threadCount = 1;
static pthread_t o_workers[O_MAX_THREADS];
static int o_workerCount = 0;

static pthread_mutex_t o_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t o_cv = PTHREAD_COND_INITIALIZER;
static atomic_uint o_generation;
static atomic_int o_next;
static atomic_int o_finished; /* workers done with the current generation */
static o_rangeFcn* o_fcn;
static void* o_ctx;
static int o_count, o_chunk;

static void o_runChunks( void )
{
	for ( ;; )
	{
		int begin = atomic_fetch_add( &o_next, o_chunk );
		if ( begin >= o_count ) break;
		int end = begin + o_chunk < o_count ? begin + o_chunk : o_count;
		o_fcn( o_ctx, begin, end );
	}
}

/* A worker takes part in every generation and reports when it is done with it; the caller
   of o_parallelFor waits for every worker before returning, so no worker can still be
   inside a loop when the next one is set up. */
static void* o_workerMain( void* arg )
{
	(void)arg;
	unsigned seen = atomic_load( &o_generation );
	for ( ;; )
	{
		int spins = 0;
		unsigned g;
		while ( ( g = atomic_load( &o_generation ) ) == seen )
		{
			if ( ++spins < 20000 ) sched_yield();
			else
			{
				pthread_mutex_lock( &o_mu );
				while ( atomic_load( &o_generation ) == seen ) pthread_cond_wait( &o_cv, &o_mu );
				pthread_mutex_unlock( &o_mu );
			}
		}
		seen = g;
		o_runChunks();
		atomic_fetch_add( &o_finished, 1 );
	}
	return NULL;
}

void o_setThreads( int n )
{
	if ( n < 1 ) n = 1;
	if ( n > O_MAX_THREADS ) n = O_MAX_THREADS;
	while ( o_workerCount < n - 1 )
	{
		if ( pthread_create( o_workers + o_workerCount, NULL, o_workerMain, NULL ) != 0 ) break;
		o_workerCount += 1;
	}
	o_threadCount = n;
}

void o_parallelFor( int count, int minParallel, o_rangeFcn* fcn, void* ctx )
{
	if ( count <= 0 ) return;
	if ( o_threadCount <= 1 || o_workerCount == 0 || count < minParallel )
	{
		fcn( ctx, 0, count );
		return;
	}
	int chunk = count / ( 4 * ( o_workerCount + 1 ) );
	o_fcn = fcn;
	o_ctx = ctx;
	o_count = count;
	o_chunk = chunk < 16 ? 16 : chunk;
	atomic_store( &o_next, 0 );
	atomic_store( &o_finished, 0 );
	pthread_mutex_lock( &o_mu );
	atomic_fetch_add( &o_generation, 1u );
	pthread_cond_broadcast( &o_cv );
	pthread_mutex_unlock( &o_mu );
	o_runChunks();
	while ( atomic_load( &o_finished ) < o_workerCount ) sched_yield();
}
