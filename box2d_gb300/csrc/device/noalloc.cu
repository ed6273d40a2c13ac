/*
 * Contact table without any allocation (b2p_contacts_noalloc in include/b2g_probe.h).
 *
 * The same table as b2p_contacts -- one row per live contact in ascending contact id:
 * (contactId, shapeIdA, shapeIdB, colorIndex, pointCount, featureId0, featureId1,
 * touching) -- built on the device by one kernel whose scratch (the contact-id -> graph
 * color map and the compacted rows) lives in a fixed file-scope device array, so a call
 * makes no cudaMalloc / cudaFree / host malloc at all.
 *
 * Limits and rules:
 *   - at most B2G_NOALLOC_MAX_CONTACT_IDS contact ids (the world's contact-id capacity);
 *     larger worlds are refused with -2 and a message;
 *   - the scratch is shared by every caller in the process: calls whose GPU work overlaps
 *     (two threads, two streams) race on it and must be serialized by the caller;
 *   - the first call on each device resolves the scratch address (cudaGetSymbolAddress,
 *     with the world's device current);
 *   - a call waits for the world's stream and copies the table into the caller's (pageable)
 *     host array, so it must be made outside any CUDA stream capture;
 *   - the kernel writes every scratch word it reads (the color map is reset inside the
 *     kernel, the row count is stored, not accumulated), so nothing has to be zeroed
 *     between calls.
 */
#include "../b2g_device_abi.h"

#include <cuda_runtime.h>
#include <pthread.h>
#include <stdio.h>

#define B2G_NOALLOC_MAX_CONTACT_IDS 32768
#define B2G_NOALLOC_THREADS 1024
#define B2G_NOALLOC_HEADER_BYTES 256
#define B2G_NOALLOC_SCRATCH_BYTES ( B2G_NOALLOC_HEADER_BYTES + B2G_NOALLOC_MAX_CONTACT_IDS * ( 4 + 32 ) )
#define B2G_NOALLOC_MAX_DEVICES 64

/* header (row count) | color of each contact id | rows, 8 ints each */
static __device__ __align__( 256 ) unsigned char g_contactTableScratch[B2G_NOALLOC_SCRATCH_BYTES];

struct d_colorOffsets
{
	int v[B2_GRAPH_COLOR_COUNT + 1];
};

__global__ void __launch_bounds__( B2G_NOALLOC_THREADS )
	k_contactTableNoAlloc( const b2gContact* __restrict__ contacts, int capacity, const int* __restrict__ colorIds,
						   d_colorOffsets colorOffsets, unsigned char* scratch )
{
	__shared__ int s_scan[B2G_NOALLOC_THREADS];
	int* rowCount = (int*)scratch;
	int* colorOf = (int*)( scratch + B2G_NOALLOC_HEADER_BYTES );
	int* rows = colorOf + B2G_NOALLOC_MAX_CONTACT_IDS;
	const int tid = threadIdx.x, nt = blockDim.x;
	const int total = colorOffsets.v[B2_GRAPH_COLOR_COUNT];

	for ( int i = tid; i < capacity; i += nt ) colorOf[i] = B2_NULL_INDEX;
	__syncthreads();
	for ( int s = tid; s < total; s += nt )
	{
		int color = 0;
		while ( color < B2_GRAPH_COLOR_COUNT - 1 && colorOffsets.v[color + 1] <= s ) color += 1;
		int contactId = colorIds[s];
		if ( contactId >= 0 && contactId < capacity ) colorOf[contactId] = color;
	}
	__syncthreads();

	/* each thread owns a run of consecutive contact ids; a block scan of the live counts
	   places the rows in ascending id order */
	const int per = ( capacity + nt - 1 ) / nt;
	const int begin = tid * per;
	const int end = begin + per < capacity ? begin + per : capacity;
	int live = 0;
	for ( int i = begin; i < end; ++i ) live += ( contacts[i].simFlags & B2G_S_LIVE ) ? 1 : 0;
	s_scan[tid] = live;
	__syncthreads();
	for ( int offset = 1; offset < nt; offset <<= 1 )
	{
		int add = tid >= offset ? s_scan[tid - offset] : 0;
		__syncthreads();
		s_scan[tid] += add;
		__syncthreads();
	}
	int row = s_scan[tid] - live;
	for ( int i = begin; i < end; ++i )
	{
		const b2gContact* c = contacts + i;
		if ( ( c->simFlags & B2G_S_LIVE ) == 0 ) continue;
		const b2Manifold* m = &c->manifold;
		int* o = rows + 8 * row;
		o[0] = i;
		o[1] = c->shapeIdA;
		o[2] = c->shapeIdB;
		/* a contact of a sleeping island is in no graph color (its id may still sit in a
		   color list that is refreshed at the next step) */
		o[3] = ( c->simFlags & B2G_S_ASLEEP ) ? B2_NULL_INDEX : colorOf[i];
		o[4] = m->pointCount;
		o[5] = m->pointCount > 0 ? (int)m->points[0].id : -1;
		o[6] = m->pointCount > 1 ? (int)m->points[1].id : -1;
		o[7] = ( c->simFlags & B2G_S_TOUCHING ) ? 1 : 0;
		row += 1;
	}
	if ( tid == nt - 1 ) *rowCount = s_scan[tid];
}

static pthread_mutex_t s_setupLock = PTHREAD_MUTEX_INITIALIZER;
static unsigned char* s_scratch[B2G_NOALLOC_MAX_DEVICES];

/* the scratch address on `dev` (the current device), resolved once per device */
static int noallocScratch( int dev, unsigned char** out )
{
	if ( dev < 0 || dev >= B2G_NOALLOC_MAX_DEVICES ) return (int)cudaErrorInvalidDevice;
	cudaError_t e = cudaSuccess;
	pthread_mutex_lock( &s_setupLock );
	if ( s_scratch[dev] == NULL )
	{
		void* p = NULL;
		e = cudaGetSymbolAddress( &p, g_contactTableScratch );
		if ( e == cudaSuccess ) s_scratch[dev] = (unsigned char*)p;
	}
	unsigned char* p = s_scratch[dev];
	pthread_mutex_unlock( &s_setupLock );
	if ( e != cudaSuccess ) return (int)e;
	*out = p;
	return 0;
}

/* Build the contact table of `dw` (contact-id capacity `capacity`) into the host array `out`
   (8 ints per row, at most `outCapacity` rows). Returns the row count (which may exceed
   outCapacity), -2 when capacity exceeds the fixed scratch, or -(1000 + CUDA error). */
extern "C" int b2gDev_ContactTableNoAlloc( b2gDeviceWorld* dw, int capacity, int* out, int outCapacity )
{
	if ( capacity > B2G_NOALLOC_MAX_CONTACT_IDS ) return -2;
	if ( capacity <= 0 ) return 0;
	const b2gContact* contacts = NULL;
	const int* colorIds = NULL;
	d_colorOffsets offsets;
	void* stream = NULL;
	int device = 0, current = 0;
	b2gDev_ContactView( dw, &contacts, &colorIds, offsets.v, &stream, &device );
	/* the world's device is current for the call (the scratch symbol and the kernel are
	   per device); the caller's current device is restored afterwards */
	cudaError_t e = cudaGetDevice( &current );
	if ( e == cudaSuccess && current != device ) e = cudaSetDevice( device );
	if ( e != cudaSuccess ) return -( 1000 + (int)e );
	unsigned char* scratch = NULL;
	int rc = noallocScratch( device, &scratch );
	int count = 0;
	if ( rc != 0 ) e = (cudaError_t)rc;
	cudaStream_t s = (cudaStream_t)stream;
	if ( e == cudaSuccess )
	{
		k_contactTableNoAlloc<<<1, B2G_NOALLOC_THREADS, 0, s>>>( contacts, capacity, colorIds, offsets, scratch );
		e = cudaGetLastError();
	}
	if ( e == cudaSuccess ) e = cudaMemcpyAsync( &count, scratch, sizeof( int ), cudaMemcpyDeviceToHost, s );
	if ( e == cudaSuccess ) e = cudaStreamSynchronize( s );
	int copy = count < outCapacity ? count : outCapacity;
	if ( e == cudaSuccess && copy > 0 )
		e = cudaMemcpyAsync( out, scratch + B2G_NOALLOC_HEADER_BYTES + (size_t)B2G_NOALLOC_MAX_CONTACT_IDS * 4,
							 (size_t)copy * 8 * sizeof( int ), cudaMemcpyDeviceToHost, s );
	if ( e == cudaSuccess ) e = cudaStreamSynchronize( s );
	if ( current != device ) cudaSetDevice( current );
	if ( e != cudaSuccess ) return -( 1000 + (int)e );
	return count;
}
