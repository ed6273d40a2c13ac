/*
 * Component solver (see components.cuh): connected components of the awake constraint
 * graph by lock-free union-find, packing of the small components into shared-memory bins,
 * one CTA per bin running the whole Soft Step of solver.c:1010-1198 for its bodies, and
 * the global per-color path for components too large for a bin.
 *
 * Kernels:
 *   k_compInit / k_compUnion / k_compRoots   union-find over colored contacts and joints
 *   k_compCountCons / k_compAssign           per-component sizes, bin packing
 *   k_compScatter                            component-contiguous body / constraint lists
 *   k_solveBins                              one bin per CTA, state in shared memory
 *   k_big*                                   global path restricted to big components
 */
#include "components.cuh"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define B2G_COMP_THREADS 256
#define B2G_BIN_THREADS 256
#define B2G_BIN_EMPTY 0x7f7f7f7f

/* per-root record in compData */
enum
{
	CD_COUNT = 0,
	CD_OFFSET = 3,
	CD_FILL = 6,
	CD_BIN = 9,
	CD_ROOT = 10, /* root of body i, in record i */
	CD_STRIDE = 11,
};

struct d_offsets
{
	int v[B2_GRAPH_COLOR_COUNT + 1];
};

static __device__ __forceinline__ int d_colorOf( const int* offsets, int index )
{
	int c = 0;
	while ( c < B2_GRAPH_COLOR_COUNT - 1 && offsets[c + 1] <= index ) c += 1;
	return c;
}

/* representative with path halving; parents always have smaller indices, so every walk ends */
static __device__ int d_find( int* parent, int x )
{
	volatile int* p = parent;
	int cur = p[x];
	if ( cur != x )
	{
		int prev = x, next;
		while ( cur > ( next = p[cur] ) )
		{
			p[prev] = next;
			prev = cur;
			cur = next;
		}
	}
	return cur;
}

/* link the larger root under the smaller one; the larger of the pair strictly decreases on
   every failed attempt, so the loop ends */
static __device__ void d_unite( int* parent, int a, int b )
{
	int ra = d_find( parent, a ), rb = d_find( parent, b );
	while ( ra != rb )
	{
		if ( ra < rb )
		{
			int t = ra;
			ra = rb;
			rb = t;
		}
		int old = atomicCAS( parent + ra, ra, rb );
		if ( old == ra ) break;
		ra = old;
	}
}

/* the two awake indices (-1 = not in the awake set) of constraint i: contact slots first,
   then joints in color order */
static __device__ __forceinline__ void d_constraintBodies( const d_solveArgs& a, const int* awakeIndex, int total, int i,
															int* ia, int* ib )
{
	if ( i < total )
	{
		const b2gContact* c = a.contacts + a.colorIds[i];
		*ia = c->bodySimIndexA;
		*ib = c->bodySimIndexB;
	}
	else
	{
		const b2gJoint* j = a.joints + ( i - total );
		*ia = awakeIndex[j->bodyIdA];
		*ib = awakeIndex[j->bodyIdB];
	}
}

__global__ void k_compInit( int* parent, int* compData, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	parent[i] = i;
	for ( int k = 0; k < CD_STRIDE; ++k ) compData[CD_STRIDE * i + k] = 0;
}

/* unions of the constraints [begin, end) (contact slots, then joints) */
__global__ void k_compUnion( d_solveArgs a, const int* awakeIndex, int* parent, int total, int begin, int end )
{
	int i = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= end ) return;
	int ia, ib;
	d_constraintBodies( a, awakeIndex, total, i, &ia, &ib );
	if ( ia >= 0 && ib >= 0 ) d_unite( parent, ia, ib );
}

/* unions of the live, awake contacts the narrowphase left touching (their awake indices
   are the narrowphase's, current for every contact it processed) */
__global__ void k_compUnionTouching( const b2gContact* contacts, int capacity, int* parent, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= capacity ) return;
	const b2gContact* c = contacts + i;
	uint32_t f = c->simFlags;
	if ( ( f & B2G_S_LIVE ) == 0 || ( f & B2G_S_TOUCHING ) == 0 || ( f & B2G_S_ASLEEP ) != 0 ) return;
	int ia = c->bodySimIndexA, ib = c->bodySimIndexB;
	if ( ia < 0 || ib < 0 || ia >= n || ib >= n ) return;
	d_unite( parent, ia, ib );
}

/* the forest over the joints, every body pointing at its root (no union runs meanwhile, so
   each root is final), kept for later analyses */
__global__ void k_compFlatten( int* parent, int* forest, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	forest[i] = d_find( parent, i );
}

/* the union-find starts from the kept joint forest */
__global__ void k_compInitFrom( int* parent, const int* forest, int* compData, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	parent[i] = forest[i];
	for ( int k = 0; k < CD_STRIDE; ++k ) compData[CD_STRIDE * i + k] = 0;
}

/* one atomic add of `1` per distinct address in the warp: lanes with the same address
   combine, and the lowest of them adds their count (a big component otherwise sends every
   one of its bodies or constraints to the same counter) */
static __device__ __forceinline__ void d_warpCountAdd( int* counter )
{
	unsigned peers = __match_any_sync( __activemask(), (unsigned long long)(uintptr_t)counter );
	if ( ( threadIdx.x & 31 ) == __ffs( peers ) - 1 ) atomicAdd( counter, __popc( peers ) );
}

/* the root goes to its own field: path halving by other threads may still rewrite parent[i]
   with a non-root ancestor during this kernel */
__global__ void k_compRoots( int* parent, int* compData, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	int r = d_find( parent, i );
	d_warpCountAdd( compData + CD_STRIDE * r + CD_COUNT );
	compData[CD_STRIDE * i + CD_ROOT] = r;
}

__global__ void k_compCountCons( d_solveArgs a, const int* awakeIndex, int* compData, int total, int count )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= count ) return;
	int ia, ib;
	d_constraintBodies( a, awakeIndex, total, i, &ia, &ib );
	int x = ia >= 0 ? ia : ib;
	if ( x < 0 ) return;
	int r = compData[CD_STRIDE * x + CD_ROOT];
	d_warpCountAdd( compData + CD_STRIDE * r + ( i < total ? 1 : 2 ) );
}

extern "C" int b2gBinCapBytes( void )
{
	static int cap = 0;
	if ( cap == 0 )
	{
		const char* e = getenv( "B2G_BIN_CAP_KB" );
		int kb = e != NULL ? atoi( e ) : 0;
		cap = kb >= 16 && kb <= 100 ? kb * 1024 : B2G_BIN_CAP_BYTES;
	}
	return cap;
}

__global__ void k_compAssign( int* compData, int* binRange, int binCap, b2gCompSummary* summary, int n, int forceBig,
							  long long capBytes )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	int* cd = compData + CD_STRIDE * i;
	if ( cd[CD_ROOT] != i ) return;
	int nb = cd[0], nc = cd[1], nj = cd[2];
	long long weight = (long long)B2G_BIN_BODY_BYTES * nb + (long long)B2G_BIN_CONTACT_BYTES * nc +
					   (long long)B2G_BIN_JOINT_BYTES * nj;
	if ( forceBig || weight > capBytes )
	{
		cd[CD_BIN] = -1;
		atomicAdd( &summary->bigComponents, 1 );
		atomicAdd( &summary->bigBodies, nb );
		return;
	}
	unsigned long long pack = ( (unsigned long long)nb << ( B2G_CURSOR_CONTACT_BITS + B2G_CURSOR_JOINT_BITS ) ) |
							  ( (unsigned long long)nc << B2G_CURSOR_JOINT_BITS ) | (unsigned long long)nj;
	unsigned long long old = atomicAdd( &summary->cursor, pack );
	int bo = (int)( old >> ( B2G_CURSOR_CONTACT_BITS + B2G_CURSOR_JOINT_BITS ) );
	int co = (int)( ( old >> B2G_CURSOR_JOINT_BITS ) & ( ( 1ull << B2G_CURSOR_CONTACT_BITS ) - 1 ) );
	int jo = (int)( old & ( ( 1ull << B2G_CURSOR_JOINT_BITS ) - 1 ) );
	cd[CD_OFFSET] = bo;
	cd[CD_OFFSET + 1] = co;
	cd[CD_OFFSET + 2] = jo;
	long long start = (long long)B2G_BIN_BODY_BYTES * bo + (long long)B2G_BIN_CONTACT_BYTES * co +
					  (long long)B2G_BIN_JOINT_BYTES * jo;
	int bin = (int)( start / capBytes );
	cd[CD_BIN] = bin;
	int* begin = binRange;
	int* end = binRange + 3 * binCap;
	atomicMin( begin + bin, bo );
	atomicMin( begin + binCap + bin, co );
	atomicMin( begin + 2 * binCap + bin, jo );
	atomicMax( end + bin, bo + nb );
	atomicMax( end + binCap + bin, co + nc );
	atomicMax( end + 2 * binCap + bin, jo + nj );
	atomicAdd( &summary->smallComponents, 1 );
}

struct d_compArgs
{
	int* compData;
	int* bodyList;
	int* localIndex;
	int* slotList;
	int* jointList;
	const int* binRange;
	int binCap;
	int* bigBodyList;
	int* bigSlotList;
	int* bigJointList;
	b2gCompSummary* summary;
	const int* awakeIndex;
	d_offsets jointOffsets;
	int identity; /* one bin holding the whole world: lists and local indices are the identity */
};

__global__ void k_compScatter( d_solveArgs a, d_compArgs c, int n, int total, int jointTotal )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n + total + jointTotal ) return;
	if ( i < n )
	{
		int r = c.compData[CD_STRIDE * i + CD_ROOT];
		int* cd = c.compData + CD_STRIDE * r;
		int bin = cd[CD_BIN];
		if ( bin >= 0 )
		{
			int pos = cd[CD_OFFSET] + atomicAdd( cd + CD_FILL, 1 );
			c.bodyList[pos] = i;
			c.localIndex[i] = pos - c.binRange[bin];
		}
		else
		{
			int pos = atomicAdd( &c.summary->bigBodyCount, 1 );
			c.bigBodyList[pos] = i;
			c.localIndex[i] = pos; /* position in the big-body list */
		}
		return;
	}
	int k = i - n;
	int ia, ib;
	d_constraintBodies( a, c.awakeIndex, total, k, &ia, &ib );
	int x = ia >= 0 ? ia : ib;
	if ( x < 0 ) return;
	int r = c.compData[CD_STRIDE * x + CD_ROOT];
	int* cd = c.compData + CD_STRIDE * r;
	bool small = cd[CD_BIN] >= 0;
	if ( k < total )
	{
		if ( small ) c.slotList[cd[CD_OFFSET + 1] + atomicAdd( cd + CD_FILL + 1, 1 )] = k;
		else
		{
			int color = d_colorOf( a.colorOffsets, k );
			c.bigSlotList[a.colorOffsets[color] + atomicAdd( &c.summary->bigContactCount[color], 1 )] = k;
		}
	}
	else
	{
		int j = k - total;
		if ( small ) c.jointList[cd[CD_OFFSET + 2] + atomicAdd( cd + CD_FILL + 2, 1 )] = j;
		else
		{
			int color = d_colorOf( c.jointOffsets.v, j );
			c.bigJointList[c.jointOffsets.v[color] + atomicAdd( &c.summary->bigJointCount[color], 1 )] = j;
		}
	}
}

/* One bin per CTA: bodies, contact constraints and joints of the bin's components live in
   shared memory for the whole step; colors run in ascending index order with a CTA barrier
   between them, exactly the stage sequence of solver.c:1010-1198 without an overflow color. */
#define D_BODY( x ) ( c.identity ? ( x ) : c.bodyList[x] )
#define D_SLOT( x ) ( c.identity ? ( x ) : c.slotList[x] )
#define D_JOINT( x ) ( c.identity ? ( x ) : c.jointList[x] )
#define D_LOCAL( x ) ( c.identity ? ( x ) : c.localIndex[x] )

static __device__ __forceinline__ void d_solveBin( const d_solveArgs& a, const d_compArgs& c, const d_jointBodies& jb,
													b2gStepCounters* counters, int smemBytes, const int bin )
{
	extern __shared__ float4 s_mem[];
	__shared__ int s_count[B2_GRAPH_COLOR_COUNT], s_start[B2_GRAPH_COLOR_COUNT + 1], s_fill[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_restitution;
	int bb, cb, jbeg, nb, nc, nj;
	if ( c.identity )
	{
		bb = 0;
		cb = 0;
		jbeg = 0;
		nb = a.awakeCount;
		nc = a.colorOffsets[B2_GRAPH_COLOR_COUNT];
		nj = c.jointOffsets.v[B2_GRAPH_COLOR_COUNT];
	}
	else
	{
		const int binCap = c.binCap;
		bb = c.binRange[bin];
		if ( bb == B2G_BIN_EMPTY ) return;
		cb = c.binRange[binCap + bin];
		jbeg = c.binRange[2 * binCap + bin];
		nb = c.binRange[3 * binCap + bin] - bb;
		nc = c.binRange[4 * binCap + bin] - cb;
		nj = c.binRange[5 * binCap + bin] - jbeg;
	}
	long long bytes = (long long)B2G_BIN_BODY_BYTES * nb + (long long)B2G_BIN_CONTACT_BYTES * nc + (long long)B2G_BIN_JOINT_BYTES * nj;
	if ( bytes > smemBytes )
	{
		if ( threadIdx.x == 0 ) atomicOr( &counters->status, B2G_STATUS_CAPACITY );
		return;
	}
	float4* sv = s_mem;
	float4* sd = sv + nb;
	b2gContactLane* lanes = (b2gContactLane*)( sd + nb );
	b2gJoint* joints = (b2gJoint*)( lanes + nc );
	int* order = (int*)( joints + nj );
	const int tid = threadIdx.x, nt = blockDim.x;
	const b2gStepParams& P = a.p;
	const int overflowBegin = a.colorOffsets[B2G_OVERFLOW_INDEX];

	if ( tid < B2_GRAPH_COLOR_COUNT ) s_count[tid] = 0;
	if ( tid == 0 ) s_restitution = 0;
	for ( int i = tid; i < nb; i += nt )
	{
		int ai = D_BODY( bb + i );
		sv[i] = a.sv[ai];
		sd[i] = a.sd[ai];
	}
	__syncthreads();

	/* prepare (contact_solver.c:1573-1809, joint.c:1593-1629) with bin-local body indices */
	for ( int k = tid; k < nc; k += nt )
	{
		int slot = D_SLOT( cb + k );
		b2gContactLane* L = lanes + k;
		d_prepareContactLane( a, slot, overflowBegin, L );
		L->indexA = L->indexA != 0 ? D_LOCAL( L->indexA - 1 ) + 1 : 0;
		L->indexB = L->indexB != 0 ? D_LOCAL( L->indexB - 1 ) + 1 : 0;
		if ( L->groupFlags & 2 ) s_restitution = 1;
		atomicAdd( s_count + d_colorOf( a.colorOffsets, slot ), 1 );
	}
	for ( int k = tid; k < nj; k += nt )
	{
		int g = D_JOINT( jbeg + k );
		b2gJoint* J = joints + k;
		*J = a.joints[g];
		d_prepareJoint( J, &jb, P.h, P.inv_h, P.enableWarmStarting != 0 );
		J->indexA = J->indexA >= 0 ? D_LOCAL( J->indexA ) : -1;
		J->indexB = J->indexB >= 0 ? D_LOCAL( J->indexB ) : -1;
		atomicAdd( s_count + d_colorOf( c.jointOffsets.v, g ), 1 );
	}
	__syncthreads();
	if ( tid == 0 )
	{
		int sum = 0;
		for ( int k = 0; k < B2_GRAPH_COLOR_COUNT; ++k )
		{
			s_start[k] = sum;
			s_fill[k] = sum;
			sum += s_count[k];
		}
		s_start[B2_GRAPH_COLOR_COUNT] = sum;
	}
	__syncthreads();
	/* color buckets: contact k as k, joint k as -(k + 1); order inside a color is free */
	for ( int k = tid; k < nc; k += nt ) order[atomicAdd( s_fill + d_colorOf( a.colorOffsets, D_SLOT( cb + k ) ), 1 )] = k;
	for ( int k = tid; k < nj; k += nt ) order[atomicAdd( s_fill + d_colorOf( c.jointOffsets.v, D_JOINT( jbeg + k ) ), 1 )] = -( k + 1 );
	__syncthreads();

	for ( int sub = 0; sub < P.subStepCount; ++sub )
	{
		for ( int i = tid; i < nb; i += nt ) d_integrateVelocitiesState( P, sv, i, a.params + 8 * D_BODY( bb + i ) );
		__syncthreads();
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int i = tid; i < nb; i += nt ) d_integratePositionsState( P, sv, sd, i );
				__syncthreads();
			}
			for ( int color = 0; color < B2G_OVERFLOW_INDEX; ++color )
			{
				int n = s_count[color];
				if ( n == 0 ) continue;
				int base = s_start[color];
				for ( int t = tid; t < n; t += nt )
				{
					int e = order[base + t];
					if ( e >= 0 ) d_laneStage( P, lanes + e, sv, sd, stage );
					else d_jointStage( P, joints + ( -e - 1 ), sv, sd, stage );
				}
				__syncthreads();
			}
		}
	}
	if ( s_restitution )
	{
		for ( int color = 0; color < B2G_OVERFLOW_INDEX; ++color )
		{
			int n = s_count[color];
			if ( n == 0 ) continue;
			int base = s_start[color];
			for ( int t = tid; t < n; t += nt )
			{
				int e = order[base + t];
				if ( e >= 0 ) d_laneStage( P, lanes + e, sv, sd, STAGE_RESTITUTION );
			}
			__syncthreads();
		}
	}

	/* store impulses (contact_solver.c:2238-2331), joint impulses and body state */
	for ( int k = tid; k < nc; k += nt )
		d_storeLane( lanes + k, &a.contacts[a.colorIds[D_SLOT( cb + k )]].manifold, false );
	for ( int k = tid; k < nj; k += nt )
	{
		b2gJoint* J = joints + k;
		J->indexA = J->indexA >= 0 ? D_BODY( bb + J->indexA ) : -1;
		J->indexB = J->indexB >= 0 ? D_BODY( bb + J->indexB ) : -1;
		a.joints[D_JOINT( jbeg + k )] = *J;
	}
	for ( int i = tid; i < nb; i += nt )
	{
		int ai = D_BODY( bb + i );
		a.sv[ai] = sv[i];
		a.sd[ai] = sd[i];
	}
}

__global__ void __launch_bounds__( B2G_BIN_THREADS ) k_solveBins( d_solveArgs a, d_compArgs c, d_jointBodies jb,
																   b2gStepCounters* counters, int smemBytes )
{
	d_solveBin( a, c, jb, counters, smemBytes, blockIdx.x );
}

/* one whole world per CTA, for many worlds at once (batched stepping): record r's
   arguments are at args + offsets[r] */
struct d_solveBinArgs
{
	d_solveArgs a;
	d_compArgs c;
	d_jointBodies jb;
	b2gStepCounters* counters;
	int smemBytes;
};

__global__ void __launch_bounds__( B2G_BIN_THREADS ) k_solveWorldBins( const long long* offsets, const unsigned char* args )
{
	const d_solveBinArgs& w = *(const d_solveBinArgs*)( args + offsets[blockIdx.x] );
	d_solveBin( w.a, w.c, w.jb, w.counters, w.smemBytes, 0 );
}

/* ---------------- global path restricted to big components ---------------- */
__global__ void k_bigPrepare( d_solveArgs a, d_jointBodies jb, d_offsets jointOffsets, const b2gCompSummary* summary,
							  const int* bigSlotList, const int* bigJointList, int total, int jointTotal )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < jointTotal )
	{
		int color = d_colorOf( jointOffsets.v, i );
		if ( i - jointOffsets.v[color] < summary->bigJointCount[color] ) d_prepareJointItem( a, jb, bigJointList[i] );
		return;
	}
	int s = i - jointTotal;
	if ( s >= total ) return;
	int color = d_colorOf( a.colorOffsets, s );
	if ( s - a.colorOffsets[color] < summary->bigContactCount[color] )
		d_prepareContactSlot( a, bigSlotList[s], a.colorOffsets[B2G_OVERFLOW_INDEX] );
}

__global__ void k_bigStore( d_solveArgs a, const b2gCompSummary* summary, const int* bigSlotList, int total )
{
	int s = blockIdx.x * blockDim.x + threadIdx.x;
	if ( s >= total ) return;
	int color = d_colorOf( a.colorOffsets, s );
	if ( s - a.colorOffsets[color] < summary->bigContactCount[color] )
		d_storeSlot( a, bigSlotList[s], a.colorOffsets[B2G_OVERFLOW_INDEX] );
}

__global__ void k_bigIntegrateVelocities( d_solveArgs a, const int* list, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < n ) d_integrateVelocitiesItem( a, list[i] );
}

__global__ void k_bigIntegratePositions( d_solveArgs a, const int* list, int n )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < n ) d_integratePositionsItem( a, list[i] );
}

/* one color of the big components; the list lengths were counted on the device */
__global__ void k_bigColorStage( d_solveArgs a, const b2gCompSummary* summary, int color, const int* jointList,
								 const int* slotList, int stage )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int nj = stage == STAGE_RESTITUTION ? 0 : summary->bigJointCount[color];
	int nl = summary->bigContactCount[color];
	if ( i < nj ) d_jointStage( a.p, a.joints + jointList[i], a.sv, a.sd, stage );
	else if ( i - nj < nl ) d_laneStage( a.p, a.lanes + slotList[i - nj], a.sv, a.sd, stage );
}

/* ---------------- host side ---------------- */
#define CKC( x )                                                                                                               \
	do                                                                                                                           \
	{                                                                                                                            \
		cudaError_t e_ = ( x );                                                                                                  \
		if ( e_ != cudaSuccess ) return (int)e_;                                                                                 \
	} while ( 0 )

static int compBlocks( int n ) { return ( n + B2G_COMP_THREADS - 1 ) / B2G_COMP_THREADS; }

/* grow two arrays of one capacity together */
static int growPair( int** p, int** q, int* cap, int need, int stride )
{
	if ( need <= *cap && *p != NULL ) return 0;
	int nc = *cap > 0 ? *cap : 256;
	while ( nc < need ) nc *= 2;
	if ( *p ) CKC( cudaFree( *p ) );
	if ( q && *q ) CKC( cudaFree( *q ) );
	*p = NULL;
	CKC( cudaMalloc( (void**)p, (size_t)nc * stride * sizeof( int ) ) );
	if ( q )
	{
		*q = NULL;
		CKC( cudaMalloc( (void**)q, (size_t)nc * sizeof( int ) ) );
	}
	*cap = nc;
	return 0;
}

extern "C" int b2gDev_CompReserve( b2gCompBuffers* b, int awake, int slots, int joints )
{
	awake = awake > 0 ? awake : 1;
	slots = slots > 0 ? slots : 1;
	joints = joints > 0 ? joints : 1;
	if ( awake > b->awakeCap || b->parent == NULL )
	{
		int cap = b->awakeCap, cap2 = b->awakeCap;
		int rc = growPair( &b->parent, &b->bodyList, &cap, awake, 1 );
		if ( rc == 0 ) rc = growPair( &b->localIndex, &b->bigBodyList, &cap2, awake, 1 );
		if ( rc ) return rc;
		if ( b->compData ) CKC( cudaFree( b->compData ) );
		b->compData = NULL;
		CKC( cudaMalloc( (void**)&b->compData, (size_t)cap * CD_STRIDE * sizeof( int ) ) );
		b->awakeCap = cap;
	}
	if ( slots > b->slotCap || b->slotList == NULL )
	{
		int rc = growPair( &b->slotList, &b->bigSlotList, &b->slotCap, slots, 1 );
		if ( rc ) return rc;
	}
	if ( joints > b->jointCap || b->jointList == NULL )
	{
		int rc = growPair( &b->jointList, &b->bigJointList, &b->jointCap, joints, 1 );
		if ( rc ) return rc;
	}
	if ( b->summary == NULL )
	{
		CKC( cudaMalloc( (void**)&b->summary, sizeof( b2gCompSummary ) ) );
		CKC( cudaMallocHost( (void**)&b->hSummary, sizeof( b2gCompSummary ) ) );
	}
	return 0;
}

extern "C" void b2gDev_CompFree( b2gCompBuffers* b )
{
	void* ptrs[] = { b->parent,		 b->compData,	 b->bodyList,	 b->localIndex,	  b->slotList, b->jointList,
					 b->binRange,	 b->bigBodyList, b->bigSlotList, b->bigJointList, b->summary,
					 b->clusterAssigned, b->clusterCounts, b->clusterJoints, b->jointForest };
	for ( size_t i = 0; i < sizeof( ptrs ) / sizeof( ptrs[0] ); ++i )
		if ( ptrs[i] ) cudaFree( ptrs[i] );
	if ( b->hSummary ) cudaFreeHost( b->hSummary );
	memset( b, 0, sizeof( *b ) );
}

static d_compArgs compArgs( b2gCompBuffers* b, const int* jointOffsets, const int* awakeIndex )
{
	d_compArgs c;
	c.compData = b->compData;
	c.bodyList = b->bodyList;
	c.localIndex = b->localIndex;
	c.slotList = b->slotList;
	c.jointList = b->jointList;
	c.binRange = b->binRange;
	c.binCap = b->binCap;
	c.bigBodyList = b->bigBodyList;
	c.bigSlotList = b->bigSlotList;
	c.bigJointList = b->bigJointList;
	c.summary = b->summary;
	c.awakeIndex = awakeIndex;
	memcpy( c.jointOffsets.v, jointOffsets, sizeof( c.jointOffsets.v ) );
	c.identity = 0;
	return c;
}

extern "C" int b2gDev_CompUnionEarly( b2gCompBuffers* b, const b2gContact* contacts, int capacity, const b2gJoint* joints,
									  const int* awakeIndex, int n, int jointTotal, long long jointEpoch, cudaStream_t stream,
									  long long* launches )
{
	b->earlyValid = 0;
	if ( n <= 0 || jointEpoch < 0 ) return 0;
	int rc = b2gDev_CompReserve( b, n, 1, jointTotal );
	if ( rc ) return rc;
	bool keptForest = jointTotal > 0 && b->jointForest != NULL && b->jointForestEpoch == jointEpoch && b->jointForestN == n &&
					  b->jointForestJoints == jointTotal;
	if ( keptForest == false && jointTotal > 0 )
	{
		if ( n > b->jointForestCap || b->jointForest == NULL )
		{
			int rc2 = growPair( &b->jointForest, NULL, &b->jointForestCap, n, 1 );
			if ( rc2 ) return rc2;
		}
		d_solveArgs ja;
		memset( &ja, 0, sizeof( ja ) );
		ja.joints = (b2gJoint*)joints;
		k_compInit<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->compData, n );
		k_compUnion<<<compBlocks( jointTotal ), B2G_COMP_THREADS, 0, stream>>>( ja, awakeIndex, b->parent, 0, 0, jointTotal );
		k_compFlatten<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->jointForest, n );
		*launches += 3;
		b->jointForestEpoch = jointEpoch;
		b->jointForestN = n;
		b->jointForestJoints = jointTotal;
		keptForest = true;
	}
	if ( keptForest ) k_compInitFrom<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->jointForest, b->compData, n );
	else k_compInit<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->compData, n );
	*launches += 1;
	if ( capacity > 0 )
	{
		k_compUnionTouching<<<compBlocks( capacity ), B2G_COMP_THREADS, 0, stream>>>( contacts, capacity, b->parent, n );
		*launches += 1;
	}
	k_compRoots<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->compData, n );
	*launches += 1;
	CKC( cudaGetLastError() );
	b->earlyValid = 1;
	b->earlyN = n;
	b->earlyJoints = jointTotal;
	b->earlyEpoch = jointEpoch;
	return 0;
}

extern "C" int b2gDev_CompAnalyze( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const int* awakeIndex,
								   int total, int jointTotal, int forceBig, long long jointEpoch, cudaStream_t stream,
								   long long* launches )
{
	int n = a->awakeCount;
	int rc = b2gDev_CompReserve( b, n, total, jointTotal );
	if ( rc ) return rc;
	long long upper = (long long)B2G_BIN_BODY_BYTES * n + (long long)B2G_BIN_CONTACT_BYTES * total +
					  (long long)B2G_BIN_JOINT_BYTES * jointTotal;
	int bins = (int)( upper / b2gBinCapBytes() ) + 2;
	if ( bins > b->binCap || b->binRange == NULL )
	{
		rc = growPair( &b->binRange, NULL, &b->binCap, bins, 6 );
		if ( rc ) return rc;
	}
	b->n = n;
	b->total = total;
	b->jointTotal = jointTotal;
	b->awakeIndex = awakeIndex;
	CKC( cudaMemsetAsync( b->binRange, 0x7f, (size_t)3 * b->binCap * sizeof( int ), stream ) );
	CKC( cudaMemsetAsync( b->binRange + 3 * b->binCap, 0, (size_t)3 * b->binCap * sizeof( int ), stream ) );
	CKC( cudaMemsetAsync( b->summary, 0, sizeof( b2gCompSummary ), stream ) );
	int cons = total + jointTotal;
	const bool early = b->earlyValid && jointEpoch >= 0 && b->earlyEpoch == jointEpoch && b->earlyN == n &&
					   b->earlyJoints == jointTotal;
	b->earlyValid = 0;
	/* Roots are the smallest index of each component whatever the order of the unions, so
	   the joints' unions can be done once and kept: later analyses start from that forest
	   and add the contacts. Joints change rarely; contacts begin and end every step. */
	bool keptForest = jointTotal > 0 && jointEpoch >= 0 && b->jointForest != NULL && b->jointForestEpoch == jointEpoch &&
					  b->jointForestN == n && b->jointForestJoints == jointTotal;
	if ( early == false && keptForest == false && jointTotal > 0 && jointEpoch >= 0 )
	{
		if ( n > b->jointForestCap || b->jointForest == NULL )
		{
			int rc2 = growPair( &b->jointForest, NULL, &b->jointForestCap, n, 1 );
			if ( rc2 ) return rc2;
		}
		k_compInit<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->compData, n );
		k_compUnion<<<compBlocks( jointTotal ), B2G_COMP_THREADS, 0, stream>>>( *a, awakeIndex, b->parent, total, total, cons );
		k_compFlatten<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->jointForest, n );
		*launches += 3;
		b->jointForestEpoch = jointEpoch;
		b->jointForestN = n;
		b->jointForestJoints = jointTotal;
		keptForest = true;
	}
	if ( early )
	{
		/* the roots and body counts are the early pass's */
	}
	else if ( keptForest )
	{
		k_compInitFrom<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->jointForest, b->compData, n );
		*launches += 1;
		if ( total > 0 )
		{
			k_compUnion<<<compBlocks( total ), B2G_COMP_THREADS, 0, stream>>>( *a, awakeIndex, b->parent, total, 0, total );
			*launches += 1;
		}
	}
	else
	{
		k_compInit<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->compData, n );
		*launches += 1;
		if ( cons > 0 )
		{
			k_compUnion<<<compBlocks( cons ), B2G_COMP_THREADS, 0, stream>>>( *a, awakeIndex, b->parent, total, 0, cons );
			*launches += 1;
		}
	}
	if ( early == false )
	{
		k_compRoots<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->parent, b->compData, n );
		*launches += 1;
	}
	if ( cons > 0 )
	{
		k_compCountCons<<<compBlocks( cons ), B2G_COMP_THREADS, 0, stream>>>( *a, awakeIndex, b->compData, total, cons );
		*launches += 1;
	}
	k_compAssign<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( b->compData, b->binRange, b->binCap, b->summary, n, forceBig,
													  (long long)b2gBinCapBytes() );
	*launches += 1;
	CKC( cudaGetLastError() );
	/* the lists now, so the summary read below carries the big components' per-color counts */
	d_compArgs c = compArgs( b, jointOffsets, awakeIndex );
	k_compScatter<<<compBlocks( n + cons ), B2G_COMP_THREADS, 0, stream>>>( *a, c, n, total, jointTotal );
	*launches += 1;
	CKC( cudaGetLastError() );
	CKC( cudaMemcpyAsync( b->hSummary, b->summary, sizeof( b2gCompSummary ), cudaMemcpyDeviceToHost, stream ) );
	CKC( cudaStreamSynchronize( stream ) );
	return 0;
}

static cudaError_t s_binsConfigured = cudaSuccess;

/* once per process: allow the bins kernel its dynamic shared memory */
static void configureBins( void )
{
	s_binsConfigured = cudaFuncSetAttribute( k_solveBins, cudaFuncAttributeMaxDynamicSharedMemorySize, B2G_WORLD_BIN_MAX_BYTES );
	if ( s_binsConfigured == cudaSuccess )
		s_binsConfigured =
			cudaFuncSetAttribute( k_solveWorldBins, cudaFuncAttributeMaxDynamicSharedMemorySize, B2G_WORLD_BIN_MAX_BYTES );
}

extern "C" int b2gDev_CompSolveBins( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets,
									 const d_jointBodies* jb, b2gStepCounters* counters, cudaStream_t stream,
									 long long* launches )
{
	static pthread_once_t s_once = PTHREAD_ONCE_INIT;
	const int smemBytes = 2 * b2gBinCapBytes();
	pthread_once( &s_once, configureBins );
	CKC( s_binsConfigured );
	d_compArgs c = compArgs( b, jointOffsets, b->awakeIndex );
	unsigned long long cur = b->hSummary->cursor;
	long long bo = (long long)( cur >> ( B2G_CURSOR_CONTACT_BITS + B2G_CURSOR_JOINT_BITS ) );
	long long co = (long long)( ( cur >> B2G_CURSOR_JOINT_BITS ) & ( ( 1ull << B2G_CURSOR_CONTACT_BITS ) - 1 ) );
	long long jo = (long long)( cur & ( ( 1ull << B2G_CURSOR_JOINT_BITS ) - 1 ) );
	long long weight = B2G_BIN_BODY_BYTES * bo + B2G_BIN_CONTACT_BYTES * co + B2G_BIN_JOINT_BYTES * jo;
	int bins = (int)( weight / b2gBinCapBytes() ) + 1;
	if ( bins > b->binCap ) bins = b->binCap;
	k_solveBins<<<bins, B2G_BIN_THREADS, smemBytes, stream>>>( *a, c, *jb, counters, smemBytes );
	*launches += 1;
	return (int)cudaGetLastError();
}

extern "C" int b2gDev_CompSolveBig( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									const int* activeColors, int activeColorCount, int total, int jointTotal,
									cudaStream_t stream, long long* launches )
{
	const b2gCompSummary* hs = b->hSummary;
	d_offsets jo;
	memcpy( jo.v, jointOffsets, sizeof( jo.v ) );
	int items = total + jointTotal;
	if ( items > 0 )
	{
		k_bigPrepare<<<compBlocks( items ), B2G_COMP_THREADS, 0, stream>>>( *a, *jb, jo, b->summary, b->bigSlotList,
																			 b->bigJointList, total, jointTotal );
		*launches += 1;
	}
	int nBodies = hs->bigBodies;
	for ( int sub = 0; sub < a->p.subStepCount; ++sub )
	{
		if ( nBodies > 0 )
		{
			k_bigIntegrateVelocities<<<compBlocks( nBodies ), B2G_COMP_THREADS, 0, stream>>>( *a, b->bigBodyList, nBodies );
			*launches += 1;
		}
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX && nBodies > 0 )
			{
				k_bigIntegratePositions<<<compBlocks( nBodies ), B2G_COMP_THREADS, 0, stream>>>( *a, b->bigBodyList, nBodies );
				*launches += 1;
			}
			for ( int k = 0; k < activeColorCount; ++k )
			{
				int color = activeColors[k];
				/* launched for the whole color; threads past the big lists return */
				int n = jointOffsets[color + 1] - jointOffsets[color] + a->colorOffsets[color + 1] - a->colorOffsets[color];
				if ( n == 0 ) continue;
				k_bigColorStage<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>(
					*a, b->summary, color, b->bigJointList + jointOffsets[color], b->bigSlotList + a->colorOffsets[color], stage );
				*launches += 1;
			}
		}
	}
	for ( int k = 0; k < activeColorCount; ++k )
	{
		int color = activeColors[k];
		int n = a->colorOffsets[color + 1] - a->colorOffsets[color];
		if ( n == 0 ) continue;
		k_bigColorStage<<<compBlocks( n ), B2G_COMP_THREADS, 0, stream>>>( *a, b->summary, color, b->bigJointList,
																			 b->bigSlotList + a->colorOffsets[color],
																			 STAGE_RESTITUTION );
		*launches += 1;
	}
	if ( total > 0 )
	{
		k_bigStore<<<compBlocks( total ), B2G_COMP_THREADS, 0, stream>>>( *a, b->summary, b->bigSlotList, total );
		*launches += 1;
	}
	return (int)cudaGetLastError();
}

/* a whole world that fits one CTA's shared memory: one bin, no component analysis */
extern "C" int b2gDev_SolveWorldBinArgs( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
										 const int* awakeIndex, int bytes, b2gStepCounters* counters, void* out, int* outBytes )
{
	if ( bytes > B2G_WORLD_BIN_MAX_BYTES ) return (int)cudaErrorInvalidValue;
	d_solveBinArgs w;
	w.a = *a;
	w.c = compArgs( b, jointOffsets, awakeIndex );
	w.c.identity = 1;
	w.jb = *jb;
	w.counters = counters;
	w.smemBytes = bytes > 16 ? bytes : 16;
	if ( out != NULL ) memcpy( out, &w, sizeof( w ) );
	*outBytes = (int)sizeof( w );
	return 0;
}

extern "C" int b2gDev_SolveWorldBinBatch( const long long* offsets, const unsigned char* args, int count, int smemBytes,
										  cudaStream_t stream )
{
	static pthread_once_t s_once = PTHREAD_ONCE_INIT;
	pthread_once( &s_once, configureBins );
	CKC( s_binsConfigured );
	if ( count <= 0 ) return 0;
	k_solveWorldBins<<<count, B2G_BIN_THREADS, smemBytes > 16 ? smemBytes : 16, stream>>>( offsets, args );
	return (int)cudaGetLastError();
}

extern "C" int b2gDev_SolveWorldBin( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									 const int* awakeIndex, int bytes, b2gStepCounters* counters, cudaStream_t stream,
									 long long* launches )
{
	static pthread_once_t s_once = PTHREAD_ONCE_INIT;
	pthread_once( &s_once, configureBins );
	CKC( s_binsConfigured );
	if ( bytes > B2G_WORLD_BIN_MAX_BYTES ) return (int)cudaErrorInvalidValue;
	d_compArgs c = compArgs( b, jointOffsets, awakeIndex );
	c.identity = 1;
	int smem = bytes > 16 ? bytes : 16;
	k_solveBins<<<1, B2G_BIN_THREADS, smem, stream>>>( *a, c, *jb, counters, smem );
	*launches += 1;
	return (int)cudaGetLastError();
}
