/*
 * GB300 (sm_103a) kernels of the Box2D v3.2 step and the thin C ABI the C17 host calls
 * (b2g_device_abi.h). One CUDA stream per world; all buffers are device-resident and grow
 * by doubling. Kernels:
 *   k_markMoved / k_findPairs / k_clearMoved  broadphase pair query (broad_phase.c:172-399)
 *   k_initContacts / k_killContacts           contact slot lifecycle
 *   k_collide                                 narrowphase + recycling (physics_world.c:451-609)
 *   k_prepareContacts / k_prepareJoints       constraint preparation
 *   k_integrateVelocities / k_integratePositions (solver.c:66-162)
 *   k_colorStage                              warm start / solve / relax / restitution per color
 *   k_overflowStage                           ordered scalar pass over the overflow color
 *   k_storeImpulses                           (contact_solver.c:2238-2331)
 *   k_finalizeBodies                          transforms, sleep metric, fat AABBs (solver.c:553-743)
 * Bit-exact mode: compiled with --fmad=false, IEEE division/sqrt, no flush-to-zero.
 */
#include "components.cuh"
#include "manifold.cuh"

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <vector>

#define B2G_THREADS 128
#define B2G_PAIR_STACK 256

/* the pair query's traversal stack depth in use (at most B2G_PAIR_STACK); the environment
   variable B2G_PAIR_STACK_LIMIT lowers it so that a test can exhaust it and check the
   capacity status */
static __device__ int d_pairStackLimit = B2G_PAIR_STACK;

/* solver strategies, chosen per world from the B2G_SOLVER environment variable at creation:
   "components" (default) solves small connected components one CTA each out of shared
   memory and the rest in one thread-block cluster (or, when they do not fit one, with one
   launch per color stage); "launches" uses the per-stage
   launches for everything; "persistent" runs all stages in one cooperative launch. All
   three produce identical results. */
enum
{
	B2G_SOLVER_COMPONENTS = 0,
	B2G_SOLVER_LAUNCHES = 1,
	B2G_SOLVER_PERSISTENT = 2,
};

/* device work of one world recorded instead of issued (batched stepping): uploads carry
   their bytes, kernels their argument blocks; b2gDev_BatchFlush replays the records of
   many worlds with one launch per kernel kind and level */
enum
{
	D_OP_H2D = 0,
	D_OP_D2H = 1,
	D_OP_MEMSET = 2,
	D_OP_KERNEL = 3,
	D_OP_D2D = 4, /* device copy: dev <- host (a device address here) */
};

enum
{
	DK_MARK_MOVED = 0,
	DK_FIND_PAIRS,
	DK_PAIR_SET,
	DK_CONVERT_TREE,
	DK_INIT_CONTACTS,
	DK_KILL_CONTACTS,
	DK_COLLIDE,
	DK_FINALIZE,
	DK_CAPTURE,
	DK_SOLVE_BIN,
	DK_ISLAND_OP,
	DK_COUNT
};

struct d_deferredOp
{
	int kind, kernel;
	void* dev;		 /* upload/memset destination, download source */
	void* host;		 /* download destination */
	long long bytes; /* copy/memset size; kernel argument size */
	long long at;	 /* offset of the upload bytes / kernel arguments in the world's records */
	int value;		 /* memset byte */
	int grid, smem;
};

struct d_deferred
{
	std::vector<d_deferredOp> ops;
	std::vector<unsigned char> up;	 /* upload bytes */
	std::vector<unsigned char> args; /* kernel argument blocks */
};

struct b2gDeviceWorld
{
	cudaStream_t stream;
	int device; /* the CUDA device the world's buffers and stream live on */
	d_deferred* defer;			 /* non-NULL: record device work for a batched flush */
	std::vector<void*> retired; /* device buffers recorded work may name, freed after the flush */
	cudaEvent_t ev[10];
	float pairsMs, collideMs, solveMs, finalizeMs; /* accumulated device time per stage */
	long long h2dBytes, d2hBytes;				   /* accumulated host<->device traffic */
	long long launches;							   /* kernels launched */
	int solverMode;								   /* B2G_SOLVER_* */
	int compSkip;								   /* steps left before the next component analysis */
	int compValid;								   /* the component lists match the current constraint graph */
	int topologyDirty;							   /* colors, joints or the awake set changed since the analysis */
	long long topologyEpoch;					   /* counts those changes and every component analysis */
	long long jointEpoch;						   /* counts changes of the joints or the awake set */
	b2gCompBuffers comp;						   /* component solver scratch */
	void* persistentScratch;					   /* barrier counter, generation, error, restitution flag */
	/* bodies by id */
	int bodyCap, bodyCount;
	float4* xf;
	float2* center;
	float2* localCenter;
	float* invMass;
	float* invI;
	float* minExtent;
	float* maxExtent;
	float* sleepThreshold;
	float* safetyFactor;
	int* awakeIndex;
	int* bodyType;
	uint32_t* bodyFlags;
	int* shapeStart;
	int* shapeCount;
	int* shapeList;
	int shapeListCap;
	/* awake bodies */
	int awakeCap, awakeCount;
	int* awakeBodyId;
	float4* stateV;
	float4* stateD;
	float* params; /* 8 per body: force.x, force.y, torque, linDamp, angDamp, gravityScale, invMass, invI */
	float4* center0; /* center0.x, center0.y, rotation0.c, rotation0.s */
	int* enlargedBody;
	float* sleepTime; /* seconds each awake body has been still (body.h b2Body.sleepTime) */
	/* islands of the finalize (sleeping enabled) */
	int islandsOn, islandCount;
	int* islandLocal;
	int islandLocalCap;
	int2* islandInfo;
	int islandInfoCap;
	unsigned int* islandBits;
	int islandBitsCap;
	unsigned int* hIslandBits;
	int hIslandBitsCap;
	int pendingIslandWords; /* island bits the solve awaiting its results reads back */
	int stageStatus;		/* status bits of the step's pair query, reported with the solve's */
	/* shapes */
	int shapeCap, shapeCountTotal;
	b2gShape* shapes;
	float4* aabb;
	float4* fat;
	int* shapeEnlarged;
	/* contacts */
	int contactCap;
	int contactSlots; /* contact ids in use at most (the host's id pool high-water mark) */
	b2gContact* contacts;
	/* the shape-pair keys of the live contact slots (open addressing, linear probing, at
	   most half full counting removed keys); the pair query drops pairs found here */
	unsigned long long* pairSet;
	int pairSetCap;		   /* a power of two, or 0 before the first contact */
	long long pairSetUsed; /* keys written since the last rebuild, live or removed */
	int pairSetStale;	   /* the slots changed behind the set (a snapshot restore) */
	int* colorIds;
	int colorIdsCap;
	int colorOffsets[B2_GRAPH_COLOR_COUNT + 1];
	b2gContactLane* lanes;
	int laneCap;
	/* joints in color order */
	b2gJoint* joints;
	int jointCap, jointCount;
	int jointOffsets[B2_GRAPH_COLOR_COUNT + 1];
	/* per body: the bodies a non-colliding joint connects it to (continuous collision filter) */
	int* partnerOffsets;
	int* partnerList;
	int partnerOffsetsCap, partnerListCap;
	int partnerCount; /* 0: no such joint */
	float* tapeToi;	  /* time-of-impact slot of the step being recorded, consumed by the next solve */
	int pendingMoves;	  /* moves of the pair query awaiting its results */
	int pendingCapacity; /* contact id capacity of the narrowphase awaiting its results */
	int pendingRecWindow, pendingShapeTotal, pendingSolved; /* the solve awaiting its results */
	/* broadphase */
	b2gTreeNode* tree[3];
	int treeCap[3], treeRoot[3];
	int treeNodes[3]; /* nodes of the last upload (the host tree's capacity) */
	b2gHostTreeNode* treeRaw[3]; /* host node arrays as uploaded */
	int treeRawCap[3];
	unsigned char* moved[3];
	int movedCap[3];
	int* moveKeys;
	float4* moveBoxes;
	int* moveShapes;
	int moveCap;
	void* moveStage; /* device: boxes, keys, shapes of the moved proxies */
	int moveStageCap;
	void* hMoveStage; /* pinned host staging of the same */
	int hMoveStageCap;
	int* pairPacked; /* pairs packed per move at atomically claimed offsets */
	int pairPackedCap;
	int* hPairPacked;
	int hPairPackedCap;
	int pairWindow;	  /* pairs copied back with the counters */
	int changeWindow; /* state changes copied back with the counters */
	int recWindow;	  /* enlarged-proxy records copied back with the counters */
	int pairsTimingPending;
	cudaEvent_t syncEvent; /* blocking-sync event for waits of batched steps */
	cudaEvent_t treeEvent; /* after the tree uploads that precede a device enlargement */
	/* small components' bins solved beside the cluster: a second stream, its fork and join
	   events, and the mapped word the cluster kernel sets once it is resident */
	cudaStream_t sideStream;
	cudaEvent_t forkEvent, joinEvent;
	cudaEvent_t enlargeEvent; /* after a tree enlargement run on the second stream */
	int enlargeOnSide;		  /* that enlargement is not yet ordered before the world's stream */
	int* hClusterStarted;
	int* dClusterStarted;
	int clusterToken;
	int blockingSync;
	/* bullet pass: bullet body slots in, shape records out */
	int* bulletSims;
	int bulletSimsCap;
	int* bulletRecs; /* 2 ints per bullet shape: shape id, enlarged */
	int bulletRecsCap;
	float4* bulletBoxes;
	int bulletBoxesCap;
	int* bulletCount;
	int* hBulletRecs;
	int hBulletRecsCap;
	float4* hBulletBoxes;
	int hBulletBoxesCap;
	/* sensor hits of the continuous sweeps, (sensor shape, visitor shape) */
	int2* sensorHits;
	int sensorHitsCap;
	int2* hSensorHits;
	int hSensorHitsCap;
	/* sensor overlap pass: sensor shape ids in, (sensor, shape) pairs out */
	int* sensorIds;
	int sensorIdsCap;
	int2* sensorPairs;
	int sensorPairsCap;
	int* sensorCount;
	int2* hSensorPairs;
	int hSensorPairsCap;
	/* upload arena (page-locked host + device) */
	void* upHost;
	void* upDev;
	int upCap;
	size_t upUsed;
	int* pairBuf;
	int* pairCounts; /* per move: pair counts at [0, n), packed offsets at [n, 2n) */
	int pairPerMove;
	int pairBufCap;
	/* outputs */
	int* changes;
	int changeCap;
	int* enlargedRecs;
	float4* enlargedBoxes;
	int enlargedCap, enlargedBoxesCap;
	b2gStepCounters* counters;
	/* pinned host staging */
	b2gStepCounters* hCounters;
	int* hChanges;
	int hChangesCap;
	int* hRecs;
	float* hBoxes;
	int hRecsCap, hBoxesCap;
	int* hPairs;
	int* hPairCounts;
	int hPairsCap, hPairCountsCap;
	int* hSortTmp; /* counting-sort buckets of the enlarged-proxy records (malloc) */
	int hSortTmpCap;
	int* hRecsRaw;
	float* hBoxesRaw;
	int hRecsRawCap, hBoxesRawCap;
	float4* hXf;
	float2* hCenter;
	uint32_t* hFlags;
	float4* hStateV;
	int hXfCap, hCenterCap, hFlagsCap, hStateVCap;
	/* the host mirrors above hold (or will hold after the next wait) the state as of the
	   last prefetch, and no device work was issued or recorded since */
	int prefetchValid, prefetchBodies, prefetchAwake;
	int prefetchWait; /* the prefetch copies were issued on the world's stream (not delivered by a flush) */
	cudaEvent_t prefetchEvent; /* after the prefetch copies: work queued behind them is not waited for */
	float* hSleepTime;
	int hSleepTimeCap;
};

#define CK( x )                                                                                                                \
	do                                                                                                                           \
	{                                                                                                                            \
		cudaError_t e_ = ( x );                                                                                                  \
		if ( e_ != cudaSuccess ) return (int)e_;                                                                                 \
	} while ( 0 )

/* capacity for `need` elements with room to grow: allocations (cudaMalloc, cudaMallocHost)
   take a process-wide lock and cost far more than the step's own work, so a buffer that
   grows gets twice what it needs */
static int growCapacity( int cap, int need )
{
	int nc = cap > 0 ? cap : 64;
	long long target = 2LL * need;
	if ( target > 0x7fffffffLL ) target = need;
	while ( nc < target && nc < 0x40000000 ) nc *= 2;
	return nc < need ? need : nc;
}

static int grow( b2gDeviceWorld* dw, void** ptr, int* cap, int need, size_t elem )
{
	if ( need <= *cap && *ptr != NULL ) return 0;
	int nc = growCapacity( *cap, need );
	void* p = NULL;
	CK( cudaMalloc( &p, (size_t)nc * elem ) );
	CK( cudaMemset( p, 0, (size_t)nc * elem ) );
	if ( *ptr != NULL )
	{
		if ( dw->defer )
		{
			/* recorded work may still write the old buffer: its contents move in order at the
			   flush, and the buffer is freed after it */
			if ( *cap > 0 )
			{
				d_deferredOp op;
				memset( &op, 0, sizeof( op ) );
				op.kind = D_OP_D2D;
				op.dev = p;
				op.host = *ptr;
				op.bytes = (long long)( *cap ) * (long long)elem;
				dw->defer->ops.push_back( op );
			}
			dw->retired.push_back( *ptr );
		}
		else
		{
			if ( *cap > 0 ) CK( cudaMemcpy( p, *ptr, (size_t)( *cap ) * elem, cudaMemcpyDeviceToDevice ) );
			CK( cudaFree( *ptr ) );
		}
	}
	*ptr = p;
	*cap = nc;
	return 0;
}

static int growHost( void** ptr, int* cap, int need, size_t elem )
{
	if ( need <= *cap && *ptr != NULL ) return 0;
	int nc = growCapacity( *cap, need );
	void* p = NULL;
	CK( cudaMallocHost( &p, (size_t)nc * elem ) );
	if ( *ptr != NULL )
	{
		if ( *cap > 0 ) memcpy( p, *ptr, (size_t)( *cap ) * elem );
		CK( cudaFreeHost( *ptr ) );
	}
	*ptr = p;
	*cap = nc;
	return 0;
}

static inline int blocks( int n ) { return ( n + B2G_THREADS - 1 ) / B2G_THREADS; }

/* ---- device work, issued or recorded ---- */

/* a kernel written as a body over (arguments, block, grid): one launch for one world, or one
   launch for the records of many worlds, whose blocks are laid end to end */
struct d_batchRec
{
	long long args;
	int blockBase, blocks;
};

template <class Args, void ( *Body )( const Args&, int, int ), int MinBlocks>
__global__ void __launch_bounds__( B2G_THREADS, MinBlocks ) k_single( Args a )
{
	Body( a, blockIdx.x, gridDim.x );
}

template <class Args, void ( *Body )( const Args&, int, int ), int MinBlocks>
__global__ void __launch_bounds__( B2G_THREADS, MinBlocks ) k_batched( const d_batchRec* __restrict__ recs, int count,
																	   const unsigned char* __restrict__ args )
{
	int lo = 0, hi = count - 1;
	while ( lo < hi )
	{
		int mid = ( lo + hi + 1 ) >> 1;
		if ( recs[mid].blockBase <= (int)blockIdx.x ) lo = mid;
		else hi = mid - 1;
	}
	const d_batchRec r = recs[lo];
	Body( *(const Args*)( args + r.args ), (int)blockIdx.x - r.blockBase, r.blocks );
}

static long long d_alignArgs( long long x ) { return ( x + 15 ) & ~15LL; }

/* upload: `src` is copied at once (recorded) or sent from pinned memory (issued) */
static int dev_h2d( b2gDeviceWorld* dw, void* dst, const void* src, size_t bytes )
{
	dw->prefetchValid = 0;
	if ( bytes == 0 ) return 0;
	dw->h2dBytes += (long long)bytes;
	if ( dw->defer )
	{
		d_deferred* d = dw->defer;
		d_deferredOp op;
		memset( &op, 0, sizeof( op ) );
		op.kind = D_OP_H2D;
		op.dev = dst;
		op.bytes = (long long)bytes;
		op.at = (long long)d->up.size();
		d->up.resize( (size_t)d_alignArgs( op.at + op.bytes ) );
		memcpy( d->up.data() + op.at, src, bytes );
		d->ops.push_back( op );
		return 0;
	}
	return (int)cudaMemcpyAsync( dst, src, bytes, cudaMemcpyHostToDevice, dw->stream );
}

/* download into host memory (pinned when issued); valid after the world's next wait */
static int dev_d2h( b2gDeviceWorld* dw, void* dst, const void* src, size_t bytes )
{
	if ( bytes == 0 ) return 0;
	dw->d2hBytes += (long long)bytes;
	if ( dw->defer )
	{
		d_deferredOp op;
		memset( &op, 0, sizeof( op ) );
		op.kind = D_OP_D2H;
		op.dev = (void*)src;
		op.host = dst;
		op.bytes = (long long)bytes;
		dw->defer->ops.push_back( op );
		return 0;
	}
	return (int)cudaMemcpyAsync( dst, src, bytes, cudaMemcpyDeviceToHost, dw->stream );
}

static int dev_memset( b2gDeviceWorld* dw, void* dst, int value, size_t bytes )
{
	dw->prefetchValid = 0;
	if ( dw->defer )
	{
		d_deferredOp op;
		memset( &op, 0, sizeof( op ) );
		op.kind = D_OP_MEMSET;
		op.dev = dst;
		op.bytes = (long long)bytes;
		op.value = value;
		dw->defer->ops.push_back( op );
		return 0;
	}
	return (int)cudaMemsetAsync( dst, value, bytes, dw->stream );
}

template <class Args, void ( *Body )( const Args&, int, int ), int MinBlocks = 1>
static int dev_launch( b2gDeviceWorld* dw, int kernel, int grid, const Args& a )
{
	if ( grid <= 0 ) return 0;
	dw->prefetchValid = 0;
	dw->launches += 1;
	if ( dw->defer )
	{
		d_deferred* d = dw->defer;
		d_deferredOp op;
		memset( &op, 0, sizeof( op ) );
		op.kind = D_OP_KERNEL;
		op.kernel = kernel;
		op.grid = grid;
		op.bytes = (long long)sizeof( Args );
		op.at = (long long)d->args.size();
		d->args.resize( (size_t)d_alignArgs( op.at + op.bytes ) );
		memcpy( d->args.data() + op.at, &a, sizeof( Args ) );
		d->ops.push_back( op );
		return 0;
	}
	k_single<Args, Body, MinBlocks><<<grid, B2G_THREADS, 0, dw->stream>>>( a );
	return (int)cudaGetLastError();
}

/* events only time issued work */
static void dev_event( b2gDeviceWorld* dw, cudaEvent_t ev )
{
	if ( dw->defer == NULL ) cudaEventRecord( ev, dw->stream );
}

/* ---- the device pair set: the host's pair set (broad_phase.c b2PairQueryCallback's
   b2ContainsKey) kept beside the contact slots, so that the query returns new pairs only ---- */
#define D_PAIR_EMPTY 0xffffffffffffffffull
#define D_PAIR_REMOVED 0xfffffffffffffffeull

static __device__ __forceinline__ unsigned long long d_pairKey( int a, int b )
{
	return a < b ? ( (unsigned long long)(unsigned)a << 32 ) | (unsigned)b : ( (unsigned long long)(unsigned)b << 32 ) | (unsigned)a;
}

static __device__ __forceinline__ unsigned long long d_pairMix( unsigned long long k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdull;
	k ^= k >> 33;
	return k;
}

/* probes are bounded by the capacity: the set is at most half full, so a probe meets an
   empty slot long before */
static __device__ void d_pairSetInsert( unsigned long long* set, int cap, unsigned long long key )
{
	if ( cap <= 0 ) return;
	unsigned mask = (unsigned)cap - 1u;
	unsigned i = (unsigned)d_pairMix( key ) & mask;
	for ( int probe = 0; probe < cap; ++probe )
	{
		unsigned long long old = atomicCAS( set + i, D_PAIR_EMPTY, key );
		if ( old == D_PAIR_EMPTY || old == key ) return;
		i = ( i + 1u ) & mask;
	}
}

static __device__ bool d_pairSetContains( const unsigned long long* __restrict__ set, int cap, unsigned long long key )
{
	if ( cap <= 0 ) return false;
	unsigned mask = (unsigned)cap - 1u;
	unsigned i = (unsigned)d_pairMix( key ) & mask;
	for ( int probe = 0; probe < cap; ++probe )
	{
		unsigned long long v = set[i];
		if ( v == key ) return true;
		if ( v == D_PAIR_EMPTY ) return false;
		i = ( i + 1u ) & mask;
	}
	return false;
}

static __device__ void d_pairSetRemove( unsigned long long* set, int cap, unsigned long long key )
{
	if ( cap <= 0 ) return;
	unsigned mask = (unsigned)cap - 1u;
	unsigned i = (unsigned)d_pairMix( key ) & mask;
	for ( int probe = 0; probe < cap; ++probe )
	{
		unsigned long long v = set[i];
		if ( v == key )
		{
			set[i] = D_PAIR_REMOVED;
			return;
		}
		if ( v == D_PAIR_EMPTY ) return;
		i = ( i + 1u ) & mask;
	}
}

/* ======================= broadphase pair query ======================= */
struct d_markMovedArgs
{
	unsigned char *movedDyn, *movedKin, *movedStat;
	const int* keys;
	int n;
	unsigned char value;
	b2gStepCounters* reset; /* zeroed by the first thread (the query's counters), or NULL */
	/* the trees the query walks next: their nodes are prefetched into L2, so that the
	   query's dependent node reads do not each wait on DRAM */
	const b2gTreeNode* trees[3];
	int treeNodes[3];
	const unsigned long long* pairSet; /* the set the query probes, prefetched as well */
	int pairSetCap;
};

static __device__ void b_markMoved( const d_markMovedArgs& a, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i == 0 && a.reset != nullptr )
	{
		int* w = (int*)a.reset;
		for ( int k = 0; k < (int)( sizeof( b2gStepCounters ) / sizeof( int ) ); ++k ) w[k] = 0;
	}
	const int threads = grid * blockDim.x;
	for ( int t = 0; t < 3; ++t )
	{
		const char* base = (const char*)a.trees[t];
		const int lines = ( a.treeNodes[t] * (int)sizeof( b2gTreeNode ) + 127 ) / 128;
		for ( int l = i; l < lines; l += threads ) asm volatile( "prefetch.global.L2 [%0];" ::"l"( base + 128 * (size_t)l ) );
	}
	{
		const char* base = (const char*)a.pairSet;
		const int lines = (int)( ( (long long)a.pairSetCap * 8 + 127 ) / 128 );
		for ( int l = i; l < lines; l += threads ) asm volatile( "prefetch.global.L2 [%0];" ::"l"( base + 128 * (size_t)l ) );
	}
	if ( i >= a.n ) return;
	int key = a.keys[i];
	int type = key & 3, id = key >> 2;
	unsigned char* m = type == b2_dynamicBody ? a.movedDyn : ( type == b2_kinematicBody ? a.movedKin : a.movedStat );
	m[id] = a.value;
}

/* one thread per moved proxy; stack DFS with child1 pushed before child2, as
   b2DynamicTree_Query (dynamic_tree.c:1085-1135); dedupe as b2PairQueryCallback
   (broad_phase.c:172-219). Hits are written in visit order. Both children of a popped
   node are loaded and tested together and only overlapping ones are pushed: the visit
   order of the overlapping nodes is the reference's, with half the dependent loads. A
   stack entry is (child1, child2) of an overlapping internal node, or (~leaf node, shape). */
struct d_findPairsArgs
{
	const b2gTreeNode *tStat, *tKin, *tDyn;
	int rootStat, rootKin, rootDyn;
	const unsigned char* movedDyn;
	const int* keys;
	const float4* boxes;
	const int* queryShapes;
	int n;
	int* pairs;
	int* counts;
	int capPerMove;
	b2gStepCounters* counters;
	int* packed;  /* every move's pairs, one contiguous run per move */
	int* offsets; /* where each move's run starts (in pairs) */
	const unsigned long long* pairSet; /* pairs that have a contact already: dropped */
	int pairSetCap;
};

static __device__ void b_findPairs( const d_findPairsArgs& fa, int block, int grid )
{
	const b2gTreeNode* __restrict__ tStat = fa.tStat;
	const b2gTreeNode* __restrict__ tKin = fa.tKin;
	const b2gTreeNode* __restrict__ tDyn = fa.tDyn;
	const int rootStat = fa.rootStat, rootKin = fa.rootKin, rootDyn = fa.rootDyn;
	const unsigned char* __restrict__ movedDyn = fa.movedDyn;
	const int* __restrict__ keys = fa.keys;
	const float4* __restrict__ boxes = fa.boxes;
	const int* __restrict__ queryShapes = fa.queryShapes;
	const int n = fa.n, capPerMove = fa.capPerMove;
	int* __restrict__ pairs = fa.pairs;
	int* __restrict__ counts = fa.counts;
	b2gStepCounters* counters = fa.counters;
	int i = block * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	int queryKey = keys[i];
	int queryType = queryKey & 3;
	float4 box = boxes[i];
	int queryShape = queryShapes[i];
	int count = 0;
	int2 stack[B2G_PAIR_STACK];
	for ( int pass = 0; pass < 3; ++pass )
	{
		int treeType;
		const b2gTreeNode* nodes;
		int root;
		if ( pass == 0 )
		{
			if ( queryType != b2_dynamicBody ) continue;
			treeType = b2_kinematicBody;
			nodes = tKin;
			root = rootKin;
		}
		else if ( pass == 1 )
		{
			if ( queryType != b2_dynamicBody ) continue;
			treeType = b2_staticBody;
			nodes = tStat;
			root = rootStat;
		}
		else
		{
			treeType = b2_dynamicBody;
			nodes = tDyn;
			root = rootDyn;
		}
		if ( root < 0 ) continue;
		int sp = 0;
		{
			const b2gTreeNode r = nodes[root];
			if ( d_overlaps( r.aabb, box ) == false || r.categoryNonZero == 0 ) continue;
			stack[sp++] = r.isLeaf ? make_int2( ~root, r.child1 ) : make_int2( r.child1, r.child2 );
		}
		bool full = false;
		while ( sp > 0 )
		{
			int2 e = stack[--sp];
			if ( e.x < 0 )
			{
				int nodeId = ~e.x;
				int proxyKey = ( nodeId << 2 ) | treeType;
				if ( proxyKey == queryKey ) continue;
				if ( queryType == b2_dynamicBody )
				{
					if ( treeType == b2_dynamicBody && proxyKey < queryKey && movedDyn[nodeId] ) continue;
				}
				else
				{
					if ( movedDyn[nodeId] ) continue;
				}
				int shapeId = e.y;
				int a = proxyKey < queryKey ? shapeId : queryShape;
				int b = proxyKey < queryKey ? queryShape : shapeId;
				if ( d_pairSetContains( fa.pairSet, fa.pairSetCap, d_pairKey( a, b ) ) ) continue;
				if ( count < capPerMove )
				{
					pairs[2 * ( (size_t)i * capPerMove + count )] = a;
					pairs[2 * ( (size_t)i * capPerMove + count ) + 1] = b;
				}
				count += 1;
				continue;
			}
			const b2gTreeNode c1 = nodes[e.x];
			const b2gTreeNode c2 = nodes[e.y];
			bool hit1 = d_overlaps( c1.aabb, box ) && c1.categoryNonZero != 0;
			bool hit2 = d_overlaps( c2.aabb, box ) && c2.categoryNonZero != 0;
			if ( sp + 2 > d_pairStackLimit )
			{
				full = true;
				break;
			}
			if ( hit1 ) stack[sp++] = c1.isLeaf ? make_int2( ~e.x, c1.child1 ) : make_int2( c1.child1, c1.child2 );
			if ( hit2 ) stack[sp++] = c2.isLeaf ? make_int2( ~e.y, c2.child1 ) : make_int2( c2.child1, c2.child2 );
		}
		if ( full )
		{
			atomicOr( &counters->status, B2G_STATUS_CAPACITY );
			break;
		}
	}
	counts[i] = count;
	if ( count > capPerMove ) atomicMax( &counters->pairOverflow, count );
	/* claim a contiguous run of the packed buffer and copy the move's pairs there: the host
	   reads them back per move through the offsets, so the runs' order does not matter */
	int c = count < capPerMove ? count : capPerMove;
	int o = atomicAdd( &counters->pairCount, c );
	fa.offsets[i] = o;
	const int2* src = (const int2*)pairs + (size_t)i * capPerMove;
	int2* dst = (int2*)fa.packed + o;
	for ( int k = 0; k < c; ++k ) dst[k] = src[k];
}

/* ======================= contacts ======================= */
struct d_pairSetArgs
{
	const b2gContact* contacts;
	int n;
	unsigned long long* set;
	int cap;
};

/* the keys of every live slot, into an emptied set */
static __device__ void b_pairSetRebuild( const d_pairSetArgs& a, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i >= a.n ) return;
	const b2gContact* c = a.contacts + i;
	if ( ( c->simFlags & B2G_S_LIVE ) == 0 ) return;
	d_pairSetInsert( a.set, a.cap, d_pairKey( c->shapeIdA, c->shapeIdB ) );
}

struct d_contactListArgs
{
	b2gContact* contacts;
	const void* list; /* b2gContactInit (init) or contact ids (kill) */
	int n;
	unsigned long long* pairSet;
	int pairSetCap;
};

static __device__ void b_initContacts( const d_contactListArgs& a, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i >= a.n ) return;
	b2gContact* contacts = a.contacts;
	b2gContactInit in = ( (const b2gContactInit*)a.list )[i];
	b2gContact c;
	memset( &c, 0, sizeof( c ) );
	c.shapeIdA = in.shapeIdA;
	c.shapeIdB = in.shapeIdB;
	c.simFlags = in.simFlags | B2G_S_LIVE;
	c.bodySimIndexA = -1;
	c.bodySimIndexB = -1;
	c.friction = in.friction;
	c.restitution = in.restitution;
	contacts[in.contactId] = c;
	d_pairSetInsert( a.pairSet, a.pairSetCap, d_pairKey( in.shapeIdA, in.shapeIdB ) );
}

static __device__ void b_killContacts( const d_contactListArgs& a, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i >= a.n ) return;
	b2gContact* c = a.contacts + ( (const int*)a.list )[i];
	if ( c->simFlags & B2G_S_LIVE ) d_pairSetRemove( a.pairSet, a.pairSetCap, d_pairKey( c->shapeIdA, c->shapeIdB ) );
	c->simFlags = 0;
}

/* ======================= islands and sleeping ======================= */
enum
{
	D_ISLAND_WAKE = 0,	   /* append woken bodies to the awake set */
	D_ISLAND_SLEEP = 1,	   /* bodies that left the awake set */
	D_ISLAND_GATHER = 2,   /* awake slots moved by the swap-removals */
	D_ISLAND_CONTACTS = 3, /* contacts leaving or rejoining the narrowphase */
	D_ISLAND_REFRESH = 4,  /* colored contacts' awake body indices */
};

struct d_islandOpArgs
{
	int mode, n, value;
	const int* list;
	int* awakeBodyId;
	int* awakeIndex;
	float4* sv;
	float4* sd;
	float* params;
	float4* center0;
	float* sleepTime;
	const uint32_t* bodyFlags;
	const float2* center;
	const float4* xf;
	b2gContact* contacts;
	const int* colorIds;
	const b2gShape* shapes;
};

/* solver_set.c:35-76 (a woken body gets the identity state with the body's flags, its sim
   as it fell asleep: center0 = center, rotation0 = q) and :200-250 (b2RemoveBodySim's
   swap-removal); the moved slots' sources all lie at or past the new count, so the gather
   reads nothing it writes */
static __device__ void b_islandOp( const d_islandOpArgs& a, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i >= a.n ) return;
	switch ( a.mode )
	{
		case D_ISLAND_WAKE:
		{
			const int* r = a.list + 10 * i;
			int bodyId = r[0], idx = r[1];
			a.awakeBodyId[idx] = bodyId;
			a.awakeIndex[bodyId] = idx;
			a.sv[idx] = make_float4( 0.0f, 0.0f, 0.0f, __uint_as_float( a.bodyFlags[bodyId] ) );
			a.sd[idx] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
			for ( int k = 0; k < 8; ++k ) a.params[8 * idx + k] = __int_as_float( r[2 + k] );
			float2 c = a.center[bodyId];
			float4 x = a.xf[bodyId];
			a.center0[idx] = make_float4( c.x, c.y, x.z, x.w );
			a.sleepTime[idx] = 0.0f;
			break;
		}
		case D_ISLAND_SLEEP:
			a.awakeIndex[a.list[i]] = -1;
			break;
		case D_ISLAND_GATHER:
		{
			int dst = a.list[2 * i], src = a.list[2 * i + 1];
			int bodyId = a.awakeBodyId[src];
			a.awakeBodyId[dst] = bodyId;
			a.awakeIndex[bodyId] = dst;
			a.sv[dst] = a.sv[src];
			a.sd[dst] = a.sd[src];
			for ( int k = 0; k < 8; ++k ) a.params[8 * dst + k] = a.params[8 * src + k];
			a.center0[dst] = a.center0[src];
			a.sleepTime[dst] = a.sleepTime[src];
			break;
		}
		case D_ISLAND_CONTACTS:
		{
			b2gContact* c = a.contacts + a.list[i];
			if ( a.value ) c->simFlags |= B2G_S_ASLEEP;
			else c->simFlags &= ~(uint32_t)B2G_S_ASLEEP;
			break;
		}
		case D_ISLAND_REFRESH:
		{
			/* constraint_graph.c:143-178: a contact entering the graph takes its bodies'
			   current awake indices */
			b2gContact* c = a.contacts + a.colorIds[i];
			c->bodySimIndexA = a.awakeIndex[a.shapes[c->shapeIdA].bodyId];
			c->bodySimIndexB = a.awakeIndex[a.shapes[c->shapeIdB].bodyId];
			break;
		}
		default:
			break;
	}
}

struct d_collideArgs
{
	b2gContact* contacts;
	int capacity;
	const b2gShape* shapes;
	const float4* fat;
	const float4* xf;
	const float2* center;
	const float2* localCenter;
	const float* invMass;
	const float* invI;
	const float* maxExtent;
	const int* awakeIndex;
	const int* bodyType;
	const uint32_t* bodyFlags;
	int* changes;
	b2gStepCounters* counters;
	float recycleDistance;
};

/* physics_world.c:451-609 and contact.c:519-698, one thread per contact slot */
static __device__ void b_collide( const d_collideArgs& a, int block, int grid )
{
	int contactId = block * blockDim.x + threadIdx.x;
	if ( contactId >= a.capacity ) return;
	b2gContact* cs = a.contacts + contactId;
	uint32_t simFlags = cs->simFlags;
	if ( ( simFlags & B2G_S_LIVE ) == 0 || ( simFlags & B2G_S_ASLEEP ) != 0 ) return;
	simFlags &= ~(uint32_t)B2G_S_RECYCLED;
	float recycleDistance = a.recycleDistance;
	float recycleNonTouching = d_min( recycleDistance, D_SPECULATIVE_DISTANCE );
	int shapeIdA = cs->shapeIdA, shapeIdB = cs->shapeIdB;
	const b2gShape* shapeA = a.shapes + shapeIdA;
	const b2gShape* shapeB = a.shapes + shapeIdB;
	float4 fa = a.fat[shapeIdA], fb = a.fat[shapeIdB];
	bool overlap = !( fb.x > fa.z || fb.y > fa.w || fa.x > fb.z || fa.y > fb.w );
	if ( overlap == false )
	{
		simFlags |= B2G_S_DISJOINT;
		simFlags &= ~B2G_S_TOUCHING;
		cs->simFlags = simFlags;
		int slot = atomicAdd( &a.counters->stateChangeCount, 1 );
		a.changes[2 * slot] = contactId;
		a.changes[2 * slot + 1] = (int)simFlags;
		return;
	}
	bool wasTouching = ( simFlags & B2G_S_TOUCHING ) != 0;
	int bodyIdA = shapeA->bodyId, bodyIdB = shapeB->bodyId;
	float4 xa = a.xf[bodyIdA], xb = a.xf[bodyIdB];
	b2Transform xfA = { { xa.x, xa.y }, { xa.z, xa.w } };
	b2Transform xfB = { { xb.x, xb.y }, { xb.z, xb.w } };
	cs->bodySimIndexA = a.awakeIndex[bodyIdA];
	cs->invMassA = a.invMass[bodyIdA];
	cs->invIA = a.invI[bodyIdA];
	cs->bodySimIndexB = a.awakeIndex[bodyIdB];
	cs->invMassB = a.invMass[bodyIdB];
	cs->invIB = a.invI[bodyIdB];
	bool isFast = ( a.bodyFlags[bodyIdA] & B2G_IS_FAST ) || ( a.bodyFlags[bodyIdB] & B2G_IS_FAST );
	if ( isFast == false && recycleDistance > 0.0f && ( simFlags & B2G_S_RELATIVE_VALID ) && ( simFlags & B2G_C_RECYCLE ) )
	{
		b2Rot cachedQA = cs->cachedRotationA, cachedQB = cs->cachedRotationB;
		b2Transform xfc = cs->cachedRelativePose;
		b2Transform xf = d_invMulTransforms( xfA, xfB );
		float cosA = d_relativeCos( xfA.q, cachedQA );
		float cosB = d_relativeCos( xfB.q, cachedQB );
		float minCos = d_min( cosA, cosB );
		float maxExtentA = a.bodyType[bodyIdA] == b2_staticBody ? 0.0f : a.maxExtent[bodyIdA];
		float maxExtentB = a.bodyType[bodyIdB] == b2_staticBody ? 0.0f : a.maxExtent[bodyIdB];
		float maxExtent = d_max( maxExtentA, maxExtentB );
		float distance = d_distance( xf.p, xfc.p );
		b2Rot qr = d_invMulRot( xf.q, xfc.q );
		float tolerance = wasTouching ? recycleDistance : recycleNonTouching;
		if ( minCos > D_CONTACT_RECYCLE_COS_ANGLE && distance + maxExtent * d_abs( qr.s ) < tolerance )
		{
			b2Rot dqA = d_mulRot( xfA.q, d_invertRot( cachedQA ) );
			b2Rot dqB = d_mulRot( xfB.q, d_invertRot( cachedQB ) );
			b2Vec2 normal = cs->manifold.normal;
			float2 cA = a.center[bodyIdA], cB = a.center[bodyIdB];
			b2Vec2 dc = { cB.x - cA.x, cB.y - cA.y };
			for ( int i = 0; i < cs->manifold.pointCount; ++i )
			{
				b2ManifoldPoint* mp = cs->manifold.points + i;
				b2Vec2 rA = d_rotate( dqA, mp->anchorA );
				b2Vec2 rB = d_rotate( dqB, mp->anchorB );
				b2Vec2 dp = d_add( dc, d_sub( rB, rA ) );
				mp->separation = mp->baseSeparation + d_dot( dp, normal );
				mp->persisted = true;
			}
			/* marks the manifold as carried over for the differentiable tape */
			cs->simFlags = simFlags | B2G_S_RECYCLED;
			atomicAdd( &a.counters->recycledContactCount, 1 );
			return;
		}
	}
	cs->cachedRotationA = xfA.q;
	cs->cachedRotationB = xfB.q;
	cs->cachedRelativePose = d_invMulTransforms( xfA, xfB );
	simFlags |= B2G_S_RELATIVE_VALID;
	float2 lcA = a.localCenter[bodyIdA], lcB = a.localCenter[bodyIdB];
	b2Vec2 centerOffsetA = d_rotate( xfA.q, d_v( lcA.x, lcA.y ) );
	b2Vec2 centerOffsetB = d_rotate( xfB.q, d_v( lcB.x, lcB.y ) );

	/* b2UpdateContact */
	b2Manifold oldManifold = cs->manifold;
	b2Transform rel = d_invMulTransforms( xfA, xfB );
	d_simplexCache cache;
	cache.count = cs->cacheCount;
	for ( int k = 0; k < 3; ++k )
	{
		cache.indexA[k] = cs->cacheA[k];
		cache.indexB[k] = cs->cacheB[k];
	}
	b2LocalManifold local = d_collideShapes( shapeA, shapeB, rel, &cache );
	cs->cacheCount = (uint8_t)cache.count;
	for ( int k = 0; k < 3; ++k )
	{
		cs->cacheA[k] = (uint8_t)cache.indexA[k];
		cs->cacheB[k] = (uint8_t)cache.indexB[k];
	}
	b2Manifold m;
	memset( &m, 0, sizeof( m ) );
	m.normal = d_rotate( xfA.q, local.normal );
	m.pointCount = local.pointCount;
	b2Vec2 originDelta = { xfA.p.x - xfB.p.x, xfA.p.y - xfB.p.y };
	for ( int i = 0; i < local.pointCount; ++i )
	{
		b2ManifoldPoint* mp = m.points + i;
		mp->anchorA = d_rotate( xfA.q, local.points[i].point );
		mp->anchorB = d_add( mp->anchorA, originDelta );
		mp->separation = local.points[i].separation;
		mp->id = local.points[i].id;
	}
	cs->friction = sqrtf( shapeA->friction * shapeB->friction );
	cs->restitution = d_max( shapeA->restitution, shapeB->restitution );
	if ( shapeA->rollingResistance > 0.0f || shapeB->rollingResistance > 0.0f )
	{
		float rA = shapeA->type == b2_segmentShape ? 0.0f : shapeA->radius;
		float rB = shapeB->type == b2_segmentShape ? 0.0f : shapeB->radius;
		float maxRadius = d_max( rA, rB );
		cs->rollingResistance = d_max( shapeA->rollingResistance, shapeB->rollingResistance ) * maxRadius;
	}
	else
	{
		cs->rollingResistance = 0.0f;
	}
	cs->tangentSpeed = shapeA->tangentSpeed + shapeB->tangentSpeed;
	int pointCount = m.pointCount;
	bool touching = pointCount > 0;
	if ( touching && ( shapeA->enableHitEvents || shapeB->enableHitEvents ) ) simFlags |= B2G_S_HIT_EVENT;
	else simFlags &= ~B2G_S_HIT_EVENT;
	if ( pointCount > 0 ) m.rollingImpulse = oldManifold.rollingImpulse;
	for ( int i = 0; i < pointCount; ++i )
	{
		b2ManifoldPoint* mp2 = m.points + i;
		mp2->anchorA = d_sub( mp2->anchorA, centerOffsetA );
		mp2->anchorB = d_sub( mp2->anchorB, centerOffsetB );
		mp2->normalImpulse = 0.0f;
		mp2->tangentImpulse = 0.0f;
		mp2->totalNormalImpulse = 0.0f;
		mp2->normalVelocity = 0.0f;
		mp2->persisted = false;
		uint16_t id2 = mp2->id;
		for ( int j = 0; j < oldManifold.pointCount; ++j )
		{
			b2ManifoldPoint* mp1 = oldManifold.points + j;
			if ( mp1->id == id2 )
			{
				mp2->normalImpulse = mp1->normalImpulse;
				mp2->tangentImpulse = mp1->tangentImpulse;
				mp2->persisted = true;
				mp1->normalImpulse = 0.0f;
				mp1->tangentImpulse = 0.0f;
				break;
			}
		}
	}
	if ( touching ) simFlags |= B2G_S_TOUCHING;
	else simFlags &= ~B2G_S_TOUCHING;
	for ( int i = 0; i < m.pointCount; ++i ) m.points[i].baseSeparation = m.points[i].separation;
	cs->manifold = m;
	bool changed = false;
	if ( touching && wasTouching == false )
	{
		simFlags |= B2G_S_STARTED;
		changed = true;
	}
	else if ( touching == false && wasTouching )
	{
		simFlags |= B2G_S_STOPPED;
		changed = true;
	}
	if ( changed )
	{
		/* the host's state pass clears the started / stopped bits */
		int slot = atomicAdd( &a.counters->stateChangeCount, 1 );
		a.changes[2 * slot] = contactId;
		a.changes[2 * slot + 1] = (int)simFlags;
		simFlags &= ~( B2G_S_STARTED | B2G_S_STOPPED );
	}
	cs->simFlags = simFlags;
}

#include "stages.cuh"

extern "C" int b2gDev_LaunchPersistent( const d_solveArgs* a, const d_finalizeArgs* f, const int* colorRanges,
										 int activeColorCount, const int* overflowRange, int total, int jointTotal,
										 int awakeCount, int substeps, const d_jointBodies* jb, unsigned int* barrier,
										 int* error, int* anyRestitution, cudaStream_t stream );

/* ---- per-stage kernels (one launch per stage and color) ---- */
__global__ void k_prepareContacts( d_solveArgs a, int total, int overflowBegin )
{
	int slot = blockIdx.x * blockDim.x + threadIdx.x;
	if ( slot < total ) d_prepareContactSlot( a, slot, overflowBegin );
}

__global__ void k_prepareJoints( d_solveArgs a, d_jointBodies bodies, int count )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < count ) d_prepareJointItem( a, bodies, i );
}

__global__ void k_integrateVelocities( d_solveArgs a )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < a.awakeCount ) d_integrateVelocitiesItem( a, i );
}

__global__ void k_integratePositions( d_solveArgs a )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < a.awakeCount ) d_integratePositionsItem( a, i );
}

__global__ void k_colorStage( d_solveArgs a, int jointBegin, int jointCount, int laneBegin, int laneCount, int stage )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < jointCount + laneCount ) d_colorStageItem( a, jointBegin, jointCount, laneBegin, laneCount, stage, i );
}

__global__ void k_overflowStage( d_solveArgs a, int jointBegin, int jointCount, int laneBegin, int laneCount, int stage )
{
	if ( blockIdx.x == 0 && threadIdx.x == 0 ) d_overflowStageAll( a, jointBegin, jointCount, laneBegin, laneCount, stage );
}

__global__ void k_storeImpulses( d_solveArgs a, int total, int overflowBegin )
{
	int slot = blockIdx.x * blockDim.x + threadIdx.x;
	if ( slot < total ) d_storeSlot( a, slot, overflowBegin );
}

/* the register cap keeps the common path at full occupancy; the rare continuous sweep of
   a fast body spills instead */
static __device__ void b_finalize( const d_finalizeArgs& f, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i < f.awakeCount ) d_finalizeBody( f, i );
}

__global__ void k_setVelocity( float4* sv, int index, float vx, float vy, float w, int which )
{
	float4 s = sv[index];
	if ( which == 1 )
	{
		s.x = vx;
		s.y = vy;
	}
	else
	{
		s.z = w;
	}
	sv[index] = s;
}

/* ======================= ABI ======================= */
extern "C" const char* b2gDev_ErrorString( int code ) { return cudaGetErrorString( (cudaError_t)code ); }

extern "C" int b2gDev_Create( b2gDeviceWorld** out )
{
	int count = 0;
	cudaError_t e = cudaGetDeviceCount( &count );
	if ( e != cudaSuccess ) return (int)e;
	if ( count == 0 ) return (int)cudaErrorNoDevice;
	b2gDeviceWorld* dw = new b2gDeviceWorld(); /* value-initialized: every field zero */
	CK( cudaGetDevice( &dw->device ) );
	{
		const char* limit = getenv( "B2G_PAIR_STACK_LIMIT" );
		int v = limit != NULL ? atoi( limit ) : 0;
		if ( v >= 2 && v <= B2G_PAIR_STACK ) CK( cudaMemcpyToSymbol( d_pairStackLimit, &v, sizeof( int ) ) );
	}
	/* a blocking stream: buffer growth (cudaMalloc + cudaMemset / cudaMemcpy on the legacy
	   default stream) is then ordered before every kernel of this world */
	CK( cudaStreamCreate( &dw->stream ) );
	for ( int i = 0; i < 10; ++i ) CK( cudaEventCreate( dw->ev + i ) );
	CK( cudaEventCreateWithFlags( &dw->syncEvent, cudaEventBlockingSync | cudaEventDisableTiming ) );
	CK( cudaMalloc( &dw->counters, sizeof( b2gStepCounters ) ) );
	CK( cudaMallocHost( &dw->hCounters, sizeof( b2gStepCounters ) ) );
	for ( int t = 0; t < 3; ++t ) dw->treeRoot[t] = -1;
	dw->pairPerMove = 32;
	{
		const char* mode = getenv( "B2G_SOLVER" );
		dw->solverMode = B2G_SOLVER_COMPONENTS;
		if ( mode != NULL && strcmp( mode, "launches" ) == 0 ) dw->solverMode = B2G_SOLVER_LAUNCHES;
		if ( mode != NULL && strcmp( mode, "persistent" ) == 0 ) dw->solverMode = B2G_SOLVER_PERSISTENT;
	}
	*out = dw;
	return 0;
}

extern "C" void b2gDev_Destroy( b2gDeviceWorld* dw )
{
	if ( dw == NULL ) return;
	cudaStreamSynchronize( dw->stream );
	cudaEventDestroy( dw->syncEvent );
	if ( dw->prefetchEvent ) cudaEventDestroy( dw->prefetchEvent );
	void* dptrs[] = { dw->xf,		  dw->center,	 dw->localCenter, dw->invMass,		dw->invI,		  dw->minExtent,
					  dw->maxExtent,  dw->sleepThreshold, dw->safetyFactor, dw->awakeIndex, dw->bodyType,	dw->bodyFlags,
					  dw->shapeStart, dw->shapeCount, dw->shapeList, dw->awakeBodyId,	dw->stateV,		  dw->stateD,
					  dw->params,	  dw->center0,	 dw->enlargedBody, dw->shapes,		dw->aabb,		  dw->fat,
					  dw->shapeEnlarged, dw->contacts, dw->colorIds,	dw->lanes,		dw->joints,		  dw->tree[0],
					  dw->tree[1],	  dw->tree[2], dw->treeRaw[0], dw->treeRaw[1], dw->treeRaw[2],	 dw->moved[0],	  dw->moved[1],		dw->moved[2],	  
					  dw->moveStage, dw->pairPacked, dw->pairBuf, dw->pairSet,	  dw->pairCounts,	dw->changes,	  dw->enlargedRecs,
					  dw->enlargedBoxes, dw->counters, dw->persistentScratch, dw->partnerOffsets, dw->partnerList,
					  dw->sleepTime, dw->islandLocal, dw->islandInfo, dw->islandBits, dw->sensorIds, dw->sensorPairs,
					  dw->sensorCount, dw->bulletSims, dw->bulletRecs, dw->bulletBoxes, dw->bulletCount, dw->sensorHits };
	b2gDev_CompFree( &dw->comp );
	for ( size_t i = 0; i < sizeof( dptrs ) / sizeof( dptrs[0] ); ++i )
		if ( dptrs[i] ) cudaFree( dptrs[i] );
	if ( dw->upDev ) cudaFree( dw->upDev );
	if ( dw->upHost ) cudaFreeHost( dw->upHost );
	void* hptrs[] = { dw->hCounters, dw->hChanges,	   dw->hRecs,	   dw->hBoxes,	   dw->hPairs,	  dw->hPairCounts,
					  dw->hMoveStage, dw->hPairPacked, dw->hRecsRaw, dw->hBoxesRaw,
					  dw->hXf,		  dw->hCenter,		dw->hFlags,		 dw->hStateV, dw->hSleepTime, dw->hIslandBits,
					  dw->hSensorPairs, dw->hBulletRecs, dw->hBulletBoxes, dw->hSensorHits };
	for ( size_t i = 0; i < sizeof( hptrs ) / sizeof( hptrs[0] ); ++i )
		if ( hptrs[i] ) cudaFreeHost( hptrs[i] );
	free( dw->hSortTmp );
	for ( int i = 0; i < 10; ++i ) cudaEventDestroy( dw->ev[i] );
	if ( dw->treeEvent ) cudaEventDestroy( dw->treeEvent );
	if ( dw->forkEvent ) cudaEventDestroy( dw->forkEvent );
	if ( dw->enlargeEvent ) cudaEventDestroy( dw->enlargeEvent );
	if ( dw->joinEvent ) cudaEventDestroy( dw->joinEvent );
	if ( dw->sideStream ) cudaStreamDestroy( dw->sideStream );
	if ( dw->hClusterStarted ) cudaFreeHost( dw->hClusterStarted );
	cudaStreamDestroy( dw->stream );
	for ( void* r : dw->retired ) cudaFree( r );
	delete dw->defer;
	delete dw;
}

#define GROW( field, capField, need, T ) CK2( grow( dw, (void**)&dw->field, &dw->capField, ( need ), sizeof( T ) ) )
#define CK2( x )                                                                                                               \
	do                                                                                                                           \
	{                                                                                                                            \
		int r_ = ( x );                                                                                                          \
		if ( r_ != 0 ) return r_;                                                                                                \
	} while ( 0 )

extern "C" int b2gDev_UploadShapes( b2gDeviceWorld* dw, const b2gShape* shapes, const float* aabbs, const float* fatAABBs,
									 int count )
{
	int cap = dw->shapeCap;
	CK2( grow( dw, (void**)&dw->shapes, &cap, count, sizeof( b2gShape ) ) );
	cap = dw->shapeCap;
	CK2( grow( dw, (void**)&dw->aabb, &cap, count, sizeof( float4 ) ) );
	cap = dw->shapeCap;
	CK2( grow( dw, (void**)&dw->fat, &cap, count, sizeof( float4 ) ) );
	cap = dw->shapeCap;
	CK2( grow( dw, (void**)&dw->shapeEnlarged, &cap, count, sizeof( int ) ) );
	dw->shapeCap = cap;
	dw->shapeCountTotal = count;
	if ( count > 0 )
	{
		CK( ( dw->h2dBytes += (long long)( (size_t)count * sizeof( b2gShape ) ), cudaMemcpy( dw->shapes, shapes, (size_t)count * sizeof( b2gShape ), cudaMemcpyHostToDevice ) ) );
		CK( ( dw->h2dBytes += (long long)( (size_t)count * sizeof( float4 ) ), cudaMemcpy( dw->aabb, aabbs, (size_t)count * sizeof( float4 ), cudaMemcpyHostToDevice ) ) );
		CK( ( dw->h2dBytes += (long long)( (size_t)count * sizeof( float4 ) ), cudaMemcpy( dw->fat, fatAABBs, (size_t)count * sizeof( float4 ), cudaMemcpyHostToDevice ) ) );
	}
	return 0;
}

template <typename T> static int upload( b2gDeviceWorld* dw, T** dptr, int* cap, const T* src, int n, int* capOut )
{
	dw->prefetchValid = 0;
	int c = *cap;
	CK2( grow( dw, (void**)dptr, &c, n, sizeof( T ) ) );
	*capOut = c;
	if ( n > 0 ) CK( ( dw->h2dBytes += (long long)( (size_t)n * sizeof( T ) ), cudaMemcpy( *dptr, src, (size_t)n * sizeof( T ), cudaMemcpyHostToDevice ) ) );
	return 0;
}

extern "C" int b2gDev_UploadBodies( b2gDeviceWorld* dw, int bodyCount, const float* xf, const float* center,
									 const float* localCenter, const float* invMass, const float* invI, const float* minExtent,
									 const float* maxExtent, const float* sleepThreshold, const float* safetyFactor,
									 const int* awakeIndex, const uint32_t* typeFlags, const int* shapeStart,
									 const int* shapeCount, const int* shapeList, int shapeListCount )
{
	dw->topologyDirty = 1;
	dw->jointEpoch += 1; /* the awake set or the joints changed */
	dw->topologyEpoch += 1;
	int cap0 = dw->bodyCap, capOut = 0;
	CK2( upload( dw, &dw->xf, &cap0, (const float4*)xf, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->center, &cap0, (const float2*)center, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->localCenter, &cap0, (const float2*)localCenter, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->invMass, &cap0, invMass, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->invI, &cap0, invI, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->minExtent, &cap0, minExtent, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->maxExtent, &cap0, maxExtent, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->sleepThreshold, &cap0, sleepThreshold, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->safetyFactor, &cap0, safetyFactor, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->awakeIndex, &cap0, awakeIndex, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->shapeStart, &cap0, shapeStart, bodyCount, &capOut ) );
	cap0 = dw->bodyCap;
	CK2( upload( dw, &dw->shapeCount, &cap0, shapeCount, bodyCount, &capOut ) );
	int* type = (int*)malloc( (size_t)( bodyCount > 0 ? bodyCount : 1 ) * sizeof( int ) );
	uint32_t* flags = (uint32_t*)malloc( (size_t)( bodyCount > 0 ? bodyCount : 1 ) * sizeof( uint32_t ) );
	for ( int i = 0; i < bodyCount; ++i )
	{
		type[i] = (int)( typeFlags[i] & 3 );
		flags[i] = typeFlags[i] >> 2;
	}
	cap0 = dw->bodyCap;
	int rc = upload( dw, &dw->bodyType, &cap0, type, bodyCount, &capOut );
	cap0 = dw->bodyCap;
	if ( rc == 0 ) rc = upload( dw, &dw->bodyFlags, &cap0, flags, bodyCount, &capOut );
	free( type );
	free( flags );
	if ( rc != 0 ) return rc;
	dw->bodyCap = capOut;
	dw->bodyCount = bodyCount;
	CK2( upload( dw, &dw->shapeList, &dw->shapeListCap, shapeList, shapeListCount, &dw->shapeListCap ) );
	return 0;
}

extern "C" int b2gDev_UploadAwake( b2gDeviceWorld* dw, int awakeCount, const int* awakeBodyId, const float* stateV,
									const float* stateD, const float* params, const float* center0, const float* sleepTime )
{
	dw->topologyDirty = 1;
	dw->jointEpoch += 1; /* the awake set or the joints changed */
	dw->topologyEpoch += 1;
	int cap0 = dw->awakeCap, capOut = 0;
	CK2( upload( dw, &dw->awakeBodyId, &cap0, awakeBodyId, awakeCount, &capOut ) );
	cap0 = dw->awakeCap;
	CK2( upload( dw, &dw->stateV, &cap0, (const float4*)stateV, awakeCount, &capOut ) );
	cap0 = dw->awakeCap;
	CK2( upload( dw, &dw->stateD, &cap0, (const float4*)stateD, awakeCount, &capOut ) );
	cap0 = dw->awakeCap;
	CK2( upload( dw, &dw->center0, &cap0, (const float4*)center0, awakeCount, &capOut ) );
	cap0 = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->enlargedBody, &cap0, awakeCount, sizeof( int ) ) );
	cap0 = dw->awakeCap;
	CK2( upload( dw, &dw->sleepTime, &cap0, sleepTime, awakeCount, &capOut ) );
	int pcap = dw->awakeCap * 8;
	CK2( grow( dw, (void**)&dw->params, &pcap, 8 * awakeCount, sizeof( float ) ) );
	if ( awakeCount > 0 ) CK( ( dw->h2dBytes += (long long)( (size_t)awakeCount * 8 * sizeof( float ) ), cudaMemcpy( dw->params, params, (size_t)awakeCount * 8 * sizeof( float ), cudaMemcpyHostToDevice ) ) );
	dw->awakeCap = capOut;
	dw->awakeCount = awakeCount;
	return 0;
}

extern "C" int b2gDev_DownloadAwake( b2gDeviceWorld* dw, int awakeCount, float* stateV, float* stateD, float* params,
									  float* center0 )
{
	if ( awakeCount == 0 ) return 0;
	CK( cudaStreamSynchronize( dw->stream ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)awakeCount * sizeof( float4 ) ), cudaMemcpy( stateV, dw->stateV, (size_t)awakeCount * sizeof( float4 ), cudaMemcpyDeviceToHost ) ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)awakeCount * sizeof( float4 ) ), cudaMemcpy( stateD, dw->stateD, (size_t)awakeCount * sizeof( float4 ), cudaMemcpyDeviceToHost ) ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)awakeCount * 8 * sizeof( float ) ), cudaMemcpy( params, dw->params, (size_t)awakeCount * 8 * sizeof( float ), cudaMemcpyDeviceToHost ) ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)awakeCount * sizeof( float4 ) ), cudaMemcpy( center0, dw->center0, (size_t)awakeCount * sizeof( float4 ), cudaMemcpyDeviceToHost ) ) );
	return 0;
}

static int drain( b2gDeviceWorld* dw );

/* transforms, centers and flags of every body and velocities of the awake bodies, in one
   wait, into page-locked staging that stays valid until the next call */
extern "C" int b2gDev_DownloadState( b2gDeviceWorld* dw, int bodyCount, int awakeCount, const float** xf, const float** center,
									 const uint32_t** flags, const float** stateV, const float** sleepTime )
{
	if ( dw->prefetchValid && dw->prefetchBodies == bodyCount && dw->prefetchAwake == awakeCount )
	{
		/* the step already sent the state down: wait for it (a batched step's flush has
		   delivered it already) */
		dw->prefetchValid = 0;
		if ( dw->prefetchWait )
		{
			if ( dw->prefetchEvent != NULL && dw->blockingSync == 0 ) CK( cudaEventSynchronize( dw->prefetchEvent ) );
			else CK2( drain( dw ) );
		}
		*xf = (const float*)dw->hXf;
		*center = (const float*)dw->hCenter;
		*flags = dw->hFlags;
		*stateV = (const float*)dw->hStateV;
		*sleepTime = dw->hSleepTime;
		return 0;
	}
	int nb = bodyCount > 0 ? bodyCount : 1, na = awakeCount > 0 ? awakeCount : 1;
	CK2( growHost( (void**)&dw->hSleepTime, &dw->hSleepTimeCap, na, sizeof( float ) ) );
	CK2( growHost( (void**)&dw->hXf, &dw->hXfCap, nb, sizeof( float4 ) ) );
	CK2( growHost( (void**)&dw->hCenter, &dw->hCenterCap, nb, sizeof( float2 ) ) );
	CK2( growHost( (void**)&dw->hFlags, &dw->hFlagsCap, nb, sizeof( uint32_t ) ) );
	CK2( growHost( (void**)&dw->hStateV, &dw->hStateVCap, na, sizeof( float4 ) ) );
	if ( bodyCount > 0 )
	{
		CK( cudaMemcpyAsync( dw->hXf, dw->xf, (size_t)bodyCount * sizeof( float4 ), cudaMemcpyDeviceToHost, dw->stream ) );
		CK( cudaMemcpyAsync( dw->hCenter, dw->center, (size_t)bodyCount * sizeof( float2 ), cudaMemcpyDeviceToHost, dw->stream ) );
		CK( cudaMemcpyAsync( dw->hFlags, dw->bodyFlags, (size_t)bodyCount * sizeof( uint32_t ), cudaMemcpyDeviceToHost, dw->stream ) );
	}
	if ( awakeCount > 0 )
	{
		CK( cudaMemcpyAsync( dw->hStateV, dw->stateV, (size_t)awakeCount * sizeof( float4 ), cudaMemcpyDeviceToHost, dw->stream ) );
		CK( cudaMemcpyAsync( dw->hSleepTime, dw->sleepTime, (size_t)awakeCount * sizeof( float ), cudaMemcpyDeviceToHost, dw->stream ) );
	}
	dw->d2hBytes += (long long)bodyCount * 28 + (long long)awakeCount * 20;
	CK2( drain( dw ) );
	*xf = (const float*)dw->hXf;
	*center = (const float*)dw->hCenter;
	*flags = dw->hFlags;
	*stateV = (const float*)dw->hStateV;
	*sleepTime = dw->hSleepTime;
	return 0;
}

/* Send the body state the host mirrors hold (transforms, centers and flags of all bodies,
   velocities and sleep times of the awake set) down behind the step's work without waiting:
   the step's move events and body getters then cost one wait instead of a round trip. In a
   batched step the copies are recorded and land with the last flush. */
extern "C" int b2gDev_PrefetchState( b2gDeviceWorld* dw, int bodyCount, int awakeCount )
{
	int nb = bodyCount > 0 ? bodyCount : 1, na = awakeCount > 0 ? awakeCount : 1;
	CK2( growHost( (void**)&dw->hSleepTime, &dw->hSleepTimeCap, na, sizeof( float ) ) );
	CK2( growHost( (void**)&dw->hXf, &dw->hXfCap, nb, sizeof( float4 ) ) );
	CK2( growHost( (void**)&dw->hCenter, &dw->hCenterCap, nb, sizeof( float2 ) ) );
	CK2( growHost( (void**)&dw->hFlags, &dw->hFlagsCap, nb, sizeof( uint32_t ) ) );
	CK2( growHost( (void**)&dw->hStateV, &dw->hStateVCap, na, sizeof( float4 ) ) );
	if ( bodyCount > 0 )
	{
		CK2( dev_d2h( dw, dw->hXf, dw->xf, (size_t)bodyCount * sizeof( float4 ) ) );
		CK2( dev_d2h( dw, dw->hCenter, dw->center, (size_t)bodyCount * sizeof( float2 ) ) );
		CK2( dev_d2h( dw, dw->hFlags, dw->bodyFlags, (size_t)bodyCount * sizeof( uint32_t ) ) );
	}
	if ( awakeCount > 0 )
	{
		CK2( dev_d2h( dw, dw->hStateV, dw->stateV, (size_t)awakeCount * sizeof( float4 ) ) );
		CK2( dev_d2h( dw, dw->hSleepTime, dw->sleepTime, (size_t)awakeCount * sizeof( float ) ) );
	}
	dw->prefetchValid = 1;
	dw->prefetchWait = dw->defer == NULL;
	if ( dw->defer == NULL )
	{
		if ( dw->prefetchEvent == NULL ) CK( cudaEventCreateWithFlags( &dw->prefetchEvent, cudaEventDisableTiming ) );
		CK( cudaEventRecord( dw->prefetchEvent, dw->stream ) );
	}
	dw->prefetchBodies = bodyCount;
	dw->prefetchAwake = awakeCount;
	return 0;
}

/* device work that changes no body state (the pair query) may follow the prefetch without
   making it stale: the caller reads the flag before and puts it back after */
extern "C" int b2gDev_PrefetchIsValid( b2gDeviceWorld* dw ) { return dw->prefetchValid; }
extern "C" void b2gDev_PrefetchKeep( b2gDeviceWorld* dw, int valid ) { dw->prefetchValid = valid; }

extern "C" int b2gDev_DownloadBodies( b2gDeviceWorld* dw, int bodyCount, float* xf, float* center, uint32_t* flags )
{
	if ( bodyCount == 0 ) return 0;
	CK( cudaStreamSynchronize( dw->stream ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)bodyCount * sizeof( float4 ) ), cudaMemcpy( xf, dw->xf, (size_t)bodyCount * sizeof( float4 ), cudaMemcpyDeviceToHost ) ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)bodyCount * sizeof( float2 ) ), cudaMemcpy( center, dw->center, (size_t)bodyCount * sizeof( float2 ), cudaMemcpyDeviceToHost ) ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)bodyCount * sizeof( uint32_t ) ), cudaMemcpy( flags, dw->bodyFlags, (size_t)bodyCount * sizeof( uint32_t ), cudaMemcpyDeviceToHost ) ) );
	return 0;
}

extern "C" int b2gDev_DownloadShapeBoxes( b2gDeviceWorld* dw, int shapeCount, float* aabbs, float* fatAABBs )
{
	if ( shapeCount == 0 ) return 0;
	CK( cudaStreamSynchronize( dw->stream ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)shapeCount * sizeof( float4 ) ), cudaMemcpy( aabbs, dw->aabb, (size_t)shapeCount * sizeof( float4 ), cudaMemcpyDeviceToHost ) ) );
	CK( ( dw->d2hBytes += (long long)( (size_t)shapeCount * sizeof( float4 ) ), cudaMemcpy( fatAABBs, dw->fat, (size_t)shapeCount * sizeof( float4 ), cudaMemcpyDeviceToHost ) ) );
	return 0;
}

extern "C" int b2gDev_SetBodyVelocity( b2gDeviceWorld* dw, int awakeIndex, float vx, float vy, float w, int which )
{
	dw->prefetchValid = 0;
	k_setVelocity<<<1, 1, 0, dw->stream>>>( dw->stateV, awakeIndex, vx, vy, w, which );
	dw->launches += 1;
	return (int)cudaGetLastError();
}

__global__ void k_setForce( float* params, int index, float fx, float fy, float torque )
{
	float* pr = params + 8 * index;
	pr[0] = fx;
	pr[1] = fy;
	pr[2] = torque;
}

/* the accumulated external force and torque of one awake body (its first three integration
   parameters; the finalize kernel clears them after the step that applies them) */
extern "C" int b2gDev_SetBodyForce( b2gDeviceWorld* dw, int awakeIndex, float fx, float fy, float torque )
{
	k_setForce<<<1, 1, 0, dw->stream>>>( dw->params, awakeIndex, fx, fy, torque );
	dw->launches += 1;
	return (int)cudaGetLastError();
}

/* the pair set sized for every contact slot in use (4x, so that it stays at most half full
   for a quarter of its capacity in further insertions) and filled from the live slots */
static int pairSetRebuild( b2gDeviceWorld* dw, long long pending )
{
	long long slots = dw->contactSlots;
	long long want = 4 * ( slots + pending );
	int cap = dw->pairSetCap > 0 ? dw->pairSetCap : 4096;
	while ( cap < want ) cap *= 2;
	if ( cap != dw->pairSetCap || dw->pairSet == NULL )
	{
		int c = 0;
		unsigned long long* fresh = NULL;
		CK2( grow( dw, (void**)&fresh, &c, cap, sizeof( unsigned long long ) ) );
		if ( dw->pairSet != NULL )
		{
			if ( dw->defer ) dw->retired.push_back( dw->pairSet );
			else CK( cudaFree( dw->pairSet ) );
		}
		dw->pairSet = fresh;
		dw->pairSetCap = cap;
	}
	CK2( dev_memset( dw, dw->pairSet, 0xff, (size_t)cap * sizeof( unsigned long long ) ) );
	int n = dw->contactSlots < dw->contactCap ? dw->contactSlots : dw->contactCap;
	if ( n > 0 )
	{
		d_pairSetArgs a = { dw->contacts, n, dw->pairSet, cap };
		CK2( ( dev_launch<d_pairSetArgs, b_pairSetRebuild>( dw, DK_PAIR_SET, blocks( n ), a ) ) );
	}
	dw->pairSetUsed = slots;
	dw->pairSetStale = 0;
	return 0;
}

/* room for `pending` more keys (a rebuild when the set would pass half full) */
static int pairSetReserve( b2gDeviceWorld* dw, long long pending )
{
	if ( dw->pairSetCap == 0 || dw->pairSetStale || 2 * ( dw->pairSetUsed + pending ) > dw->pairSetCap )
		CK2( pairSetRebuild( dw, pending ) );
	dw->pairSetUsed += pending;
	return 0;
}

extern "C" int b2gDev_ReserveContacts( b2gDeviceWorld* dw, int capacity )
{
	if ( capacity > dw->contactSlots ) dw->contactSlots = capacity;
	CK2( grow( dw, (void**)&dw->contacts, &dw->contactCap, capacity > 0 ? capacity : 1, sizeof( b2gContact ) ) );
	int c = dw->changeCap;
	CK2( grow( dw, (void**)&dw->changes, &c, 2 * ( capacity > 0 ? capacity : 1 ), sizeof( int ) ) );
	dw->changeCap = c;
	return 0;
}

/* every contact slot below `count` (manifolds, impulses, flags, simplex caches) to or from
   the host, for world snapshots; slots the device never held read as zeros */
extern "C" int b2gDev_DownloadContacts( b2gDeviceWorld* dw, b2gContact* out, int count )
{
	if ( count <= 0 ) return 0;
	int held = dw->contacts != NULL ? ( count < dw->contactCap ? count : dw->contactCap ) : 0;
	if ( held < count ) memset( out + held, 0, (size_t)( count - held ) * sizeof( b2gContact ) );
	if ( held == 0 ) return 0;
	dw->d2hBytes += (long long)held * (long long)sizeof( b2gContact );
	CK( cudaMemcpyAsync( out, dw->contacts, (size_t)held * sizeof( b2gContact ), cudaMemcpyDeviceToHost, dw->stream ) );
	CK( cudaStreamSynchronize( dw->stream ) );
	return 0;
}

extern "C" int b2gDev_UploadContacts( b2gDeviceWorld* dw, const b2gContact* in, int count )
{
	CK2( b2gDev_ReserveContacts( dw, count ) );
	dw->prefetchValid = 0;
	/* the slots past the snapshot's held another world state's contacts: cleared, and the
	   pair set is rebuilt from the uploaded slots before its next use */
	dw->pairSetStale = 1;
	dw->contactSlots = count > 0 ? count : 0;
	if ( dw->contactCap > count && dw->contacts != NULL )
		CK( cudaMemsetAsync( dw->contacts + ( count > 0 ? count : 0 ), 0,
							 (size_t)( dw->contactCap - ( count > 0 ? count : 0 ) ) * sizeof( b2gContact ), dw->stream ) );
	if ( count <= 0 ) return 0;
	dw->h2dBytes += (long long)count * (long long)sizeof( b2gContact );
	CK( cudaMemcpyAsync( dw->contacts, in, (size_t)count * sizeof( b2gContact ), cudaMemcpyHostToDevice, dw->stream ) );
	CK( cudaStreamSynchronize( dw->stream ) );
	return 0;
}

/* Upload arena: small per-step uploads are copied into page-locked host memory and sent
   with cudaMemcpyAsync on the world stream, so they need no wait. Arena space is reused
   only after the stream has been drained (every step drains it at its readbacks). */
static int arenaAlloc( b2gDeviceWorld* dw, size_t bytes, size_t* offset )
{
	size_t need = ( bytes + 15 ) & ~(size_t)15;
	if ( dw->upUsed + need > (size_t)dw->upCap )
	{
		if ( dw->defer )
		{
			/* recorded work may still name the old device arena: keep it until the flush */
			int nc = dw->upCap > 0 ? dw->upCap : 1 << 16;
			while ( (size_t)nc < dw->upUsed + need ) nc *= 2;
			void* grown = NULL;
			CK( cudaMalloc( &grown, (size_t)nc ) );
			if ( dw->upDev ) dw->retired.push_back( dw->upDev );
			if ( dw->upHost ) CK( cudaFreeHost( dw->upHost ) );
			CK( cudaMallocHost( &dw->upHost, (size_t)nc ) );
			dw->upDev = grown;
			dw->upCap = nc;
			dw->upUsed = 0;
		}
		else
		{
			/* drain the stream: earlier uploads may still read the arena */
			CK( cudaStreamSynchronize( dw->stream ) );
			dw->upUsed = 0;
			if ( need > (size_t)dw->upCap )
			{
				int nc = dw->upCap > 0 ? dw->upCap : 1 << 16;
				while ( (size_t)nc < need ) nc *= 2;
				if ( dw->upHost ) CK( cudaFreeHost( dw->upHost ) );
				if ( dw->upDev ) CK( cudaFree( dw->upDev ) );
				dw->upHost = NULL;
				dw->upDev = NULL;
				CK( cudaMallocHost( &dw->upHost, (size_t)nc ) );
				CK( cudaMalloc( &dw->upDev, (size_t)nc ) );
				dw->upCap = nc;
			}
		}
	}
	*offset = dw->upUsed;
	dw->upUsed += need;
	return 0;
}

/* send `bytes` from host memory `src` to device address `dst` without waiting */
static int uploadTo( b2gDeviceWorld* dw, void* dst, const void* src, size_t bytes )
{
	if ( bytes == 0 ) return 0;
	if ( dw->defer ) return dev_h2d( dw, dst, src, bytes );
	size_t off = 0;
	CK2( arenaAlloc( dw, bytes, &off ) );
	memcpy( (char*)dw->upHost + off, src, bytes );
	return dev_h2d( dw, dst, (char*)dw->upHost + off, bytes );
}

/* send `bytes` into the device side of the arena; returns the device address */
static int uploadStaged( b2gDeviceWorld* dw, const void* src, size_t bytes, void** devPtr )
{
	size_t off = 0;
	CK2( arenaAlloc( dw, bytes, &off ) );
	*devPtr = (char*)dw->upDev + off;
	if ( dw->defer ) return dev_h2d( dw, *devPtr, src, bytes );
	memcpy( (char*)dw->upHost + off, src, bytes );
	return dev_h2d( dw, *devPtr, (char*)dw->upHost + off, bytes );
}

/* wait for the stream; afterwards the upload arena is free again */
static int drain( b2gDeviceWorld* dw )
{
	if ( dw->blockingSync )
	{
		/* the waiting thread sleeps instead of spinning, so many stepping threads can share
		   the host cores */
		CK( cudaEventRecord( dw->syncEvent, dw->stream ) );
		CK( cudaEventSynchronize( dw->syncEvent ) );
	}
	else
	{
		CK( cudaStreamSynchronize( dw->stream ) );
	}
	dw->upUsed = 0;
	return 0;
}

extern "C" void b2gDev_SetBlockingSync( b2gDeviceWorld* dw, int on ) { dw->blockingSync = on; }

extern "C" int b2gDev_InitContacts( b2gDeviceWorld* dw, const b2gContactInit* inits, int count )
{
	if ( count == 0 ) return 0;
	void* d = NULL;
	CK2( pairSetReserve( dw, count ) );
	CK2( uploadStaged( dw, inits, (size_t)count * sizeof( b2gContactInit ), &d ) );
	d_contactListArgs a = { dw->contacts, d, count, dw->pairSet, dw->pairSetCap };
	return dev_launch<d_contactListArgs, b_initContacts>( dw, DK_INIT_CONTACTS, blocks( count ), a );
}

extern "C" int b2gDev_KillContacts( b2gDeviceWorld* dw, const int* ids, int count )
{
	if ( count == 0 ) return 0;
	void* d = NULL;
	CK2( uploadStaged( dw, ids, (size_t)count * sizeof( int ), &d ) );
	d_contactListArgs a = { dw->contacts, d, count, dw->pairSet, dw->pairSetCap };
	return dev_launch<d_contactListArgs, b_killContacts>( dw, DK_KILL_CONTACTS, blocks( count ), a );
}

static d_islandOpArgs islandArgs( b2gDeviceWorld* dw, int mode, int n, const void* list )
{
	d_islandOpArgs a;
	memset( &a, 0, sizeof( a ) );
	a.mode = mode;
	a.n = n;
	a.list = (const int*)list;
	a.awakeBodyId = dw->awakeBodyId;
	a.awakeIndex = dw->awakeIndex;
	a.sv = dw->stateV;
	a.sd = dw->stateD;
	a.params = dw->params;
	a.center0 = dw->center0;
	a.sleepTime = dw->sleepTime;
	a.bodyFlags = dw->bodyFlags;
	a.center = dw->center;
	a.xf = dw->xf;
	a.contacts = dw->contacts;
	a.colorIds = dw->colorIds;
	a.shapes = dw->shapes;
	return a;
}

/* the awake arrays hold `count` bodies (contents kept) */
static int growAwake( b2gDeviceWorld* dw, int count )
{
	if ( count <= dw->awakeCap && dw->awakeBodyId != NULL ) return 0;
	int capOut = 0, cap = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->awakeBodyId, &cap, count, sizeof( int ) ) );
	capOut = cap;
	cap = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->stateV, &cap, count, sizeof( float4 ) ) );
	cap = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->stateD, &cap, count, sizeof( float4 ) ) );
	cap = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->center0, &cap, count, sizeof( float4 ) ) );
	cap = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->enlargedBody, &cap, count, sizeof( int ) ) );
	cap = dw->awakeCap;
	CK2( grow( dw, (void**)&dw->sleepTime, &cap, count, sizeof( float ) ) );
	int pcap = dw->awakeCap * 8;
	CK2( grow( dw, (void**)&dw->params, &pcap, 8 * count, sizeof( float ) ) );
	dw->awakeCap = capOut;
	return 0;
}

extern "C" int b2gDev_WakeBodies( b2gDeviceWorld* dw, int newAwakeCount, const int* records, int count )
{
	if ( count <= 0 ) return 0;
	CK2( growAwake( dw, newAwakeCount ) );
	void* d = NULL;
	CK2( uploadStaged( dw, records, (size_t)count * 10 * sizeof( int ), &d ) );
	d_islandOpArgs a = islandArgs( dw, D_ISLAND_WAKE, count, d );
	CK2( ( dev_launch<d_islandOpArgs, b_islandOp>( dw, DK_ISLAND_OP, blocks( count ), a ) ) );
	dw->awakeCount = newAwakeCount;
	dw->topologyDirty = 1;
	dw->jointEpoch += 1; /* the awake set or the joints changed */
	dw->topologyEpoch += 1;
	return 0;
}

extern "C" int b2gDev_SleepBodies( b2gDeviceWorld* dw, int newAwakeCount, const int* slept, int sleptCount, const int* pairs,
								   int pairCount )
{
	if ( sleptCount > 0 )
	{
		void* d = NULL;
		CK2( uploadStaged( dw, slept, (size_t)sleptCount * sizeof( int ), &d ) );
		d_islandOpArgs a = islandArgs( dw, D_ISLAND_SLEEP, sleptCount, d );
		CK2( ( dev_launch<d_islandOpArgs, b_islandOp>( dw, DK_ISLAND_OP, blocks( sleptCount ), a ) ) );
	}
	if ( pairCount > 0 )
	{
		void* d = NULL;
		CK2( uploadStaged( dw, pairs, (size_t)pairCount * 2 * sizeof( int ), &d ) );
		d_islandOpArgs a = islandArgs( dw, D_ISLAND_GATHER, pairCount, d );
		CK2( ( dev_launch<d_islandOpArgs, b_islandOp>( dw, DK_ISLAND_OP, blocks( pairCount ), a ) ) );
	}
	dw->awakeCount = newAwakeCount;
	dw->topologyDirty = 1;
	dw->jointEpoch += 1; /* the awake set or the joints changed */
	dw->topologyEpoch += 1;
	return 0;
}

extern "C" int b2gDev_SetContactsAsleep( b2gDeviceWorld* dw, const int* contactIds, int count, int asleep )
{
	if ( count <= 0 ) return 0;
	void* d = NULL;
	CK2( uploadStaged( dw, contactIds, (size_t)count * sizeof( int ), &d ) );
	d_islandOpArgs a = islandArgs( dw, D_ISLAND_CONTACTS, count, d );
	a.value = asleep ? 1 : 0;
	return dev_launch<d_islandOpArgs, b_islandOp>( dw, DK_ISLAND_OP, blocks( count ), a );
}

extern "C" int b2gDev_RefreshContactBodies( b2gDeviceWorld* dw )
{
	int total = dw->colorOffsets[B2_GRAPH_COLOR_COUNT];
	dw->topologyEpoch += 1;
	if ( total <= 0 ) return 0;
	d_islandOpArgs a = islandArgs( dw, D_ISLAND_REFRESH, total, NULL );
	return dev_launch<d_islandOpArgs, b_islandOp>( dw, DK_ISLAND_OP, blocks( total ), a );
}

extern "C" int b2gDev_UploadIslands( b2gDeviceWorld* dw, const int* islandLocal, int awakeCount, const int* islandInfo,
									 int islandCount )
{
	if ( islandCount < 0 )
	{
		dw->islandsOn = 0;
		dw->islandCount = 0;
		return 0;
	}
	CK2( grow( dw, (void**)&dw->islandLocal, &dw->islandLocalCap, awakeCount > 0 ? awakeCount : 1, sizeof( int ) ) );
	CK2( grow( dw, (void**)&dw->islandInfo, &dw->islandInfoCap, islandCount > 0 ? islandCount : 1, sizeof( int2 ) ) );
	if ( awakeCount > 0 ) CK2( uploadTo( dw, dw->islandLocal, islandLocal, (size_t)awakeCount * sizeof( int ) ) );
	if ( islandCount > 0 ) CK2( uploadTo( dw, dw->islandInfo, islandInfo, (size_t)islandCount * sizeof( int2 ) ) );
	dw->islandsOn = 1;
	dw->islandCount = islandCount;
	return 0;
}

extern "C" int b2gDev_IslandResults( b2gDeviceWorld* dw, const uint32_t** awakeIslandBits, int* islandCount,
									  unsigned long long* splitKey )
{
	*awakeIslandBits = dw->pendingIslandWords > 0 ? dw->hIslandBits : NULL;
	*islandCount = dw->pendingIslandWords > 0 ? dw->islandCount : 0;
	*splitKey = dw->hCounters->splitKey;
	return 0;
}

extern "C" int b2gDev_UploadColors( b2gDeviceWorld* dw, const int* ids, const int* offsets, int total )
{
	dw->topologyDirty = 1;
	dw->topologyEpoch += 1;
	CK2( grow( dw, (void**)&dw->colorIds, &dw->colorIdsCap, total > 0 ? total : 1, sizeof( int ) ) );
	CK2( uploadTo( dw, dw->colorIds, ids, (size_t)total * sizeof( int ) ) );
	memcpy( dw->colorOffsets, offsets, sizeof( dw->colorOffsets ) );
	return 0;
}

/* the same from the colors' own lists: gathered straight into the upload arena */
extern "C" int b2gDev_UploadColorLists( b2gDeviceWorld* dw, const int* const* lists, const int* counts, int listCount,
										const int* offsets, int total )
{
	dw->topologyDirty = 1;
	dw->topologyEpoch += 1;
	CK2( grow( dw, (void**)&dw->colorIds, &dw->colorIdsCap, total > 0 ? total : 1, sizeof( int ) ) );
	memcpy( dw->colorOffsets, offsets, sizeof( dw->colorOffsets ) );
	if ( total <= 0 ) return 0;
	size_t bytes = (size_t)total * sizeof( int );
	int* dst = NULL;
	size_t off = 0;
	if ( dw->defer )
	{
		dst = (int*)malloc( bytes ); /* a recorded upload copies its source at once */
		if ( dst == NULL ) return (int)cudaErrorMemoryAllocation;
	}
	else
	{
		CK2( arenaAlloc( dw, bytes, &off ) );
		dst = (int*)( (char*)dw->upHost + off );
	}
	int at = 0;
	for ( int i = 0; i < listCount; ++i )
	{
		if ( counts[i] > 0 ) memcpy( dst + at, lists[i], (size_t)counts[i] * sizeof( int ) );
		at += counts[i];
	}
	int rc = dev_h2d( dw, dw->colorIds, dst, bytes );
	if ( dw->defer ) free( dst );
	return rc;
}

extern "C" void b2gDev_ContactView( b2gDeviceWorld* dw, const b2gContact** contacts, const int** colorIds, int* colorOffsets,
									void** stream, int* device )
{
	*device = dw->device;
	*contacts = dw->contacts;
	*colorIds = dw->colorIds;
	memcpy( colorOffsets, dw->colorOffsets, sizeof( dw->colorOffsets ) );
	*stream = (void*)dw->stream;
}

extern "C" int b2gDev_UploadJoints( b2gDeviceWorld* dw, const b2gJoint* joints, int count, const int* offsets )
{
	dw->topologyDirty = 1;
	dw->jointEpoch += 1; /* the awake set or the joints changed */
	dw->topologyEpoch += 1;
	CK2( grow( dw, (void**)&dw->joints, &dw->jointCap, count > 0 ? count : 1, sizeof( b2gJoint ) ) );
	CK2( uploadTo( dw, dw->joints, joints, (size_t)count * sizeof( b2gJoint ) ) );
	memcpy( dw->jointOffsets, offsets, sizeof( dw->jointOffsets ) );
	dw->jointCount = count;
	return 0;
}

/* ======================= tape capture (differentiable stepping) ======================= */
struct d_colorOffsets
{
	int v[B2_GRAPH_COLOR_COUNT + 1];
};

/* one step record: header, every body's pose and velocity, integration parameters, and the
   colored contacts in slot order as the narrowphase left them */
struct d_captureArgs
{
	unsigned char* rec;
	b2gStepParams params;
	d_colorOffsets offsets;
	int bodyCount, awakeCount, slotCount, jointCount;
	const float4* xf;
	const float2* center;
	const float2* localCenter;
	const int* awakeIndex;
	const int* bodyType;
	const float4* sv;
	const float* bodyParams;
	const int* colorIds;
	const b2gContact* contacts;
};

static __device__ void b_capture( const d_captureArgs& ca, int block, int grid )
{
	unsigned char* rec = ca.rec;
	const b2gStepParams& params = ca.params;
	const d_colorOffsets& offsets = ca.offsets;
	const int bodyCount = ca.bodyCount, awakeCount = ca.awakeCount, slotCount = ca.slotCount, jointCount = ca.jointCount;
	const float4* __restrict__ xf = ca.xf;
	const float2* __restrict__ center = ca.center;
	const float2* __restrict__ localCenter = ca.localCenter;
	const int* __restrict__ awakeIndex = ca.awakeIndex;
	const int* __restrict__ bodyType = ca.bodyType;
	const float4* __restrict__ sv = ca.sv;
	const float* __restrict__ bodyParams = ca.bodyParams;
	const int* __restrict__ colorIds = ca.colorIds;
	const b2gContact* __restrict__ contacts = ca.contacts;
	int t = block * blockDim.x + threadIdx.x;
	int nt = grid * blockDim.x;
	if ( t == 0 )
	{
		b2gTapeStep h;
		memset( &h, 0, sizeof( h ) );
		h.params = params;
		h.bodyCount = bodyCount;
		h.awakeCount = awakeCount;
		h.slotCount = slotCount;
		h.jointCount = jointCount;
		for ( int i = 0; i <= B2_GRAPH_COLOR_COUNT; ++i ) h.colorOffsets[i] = offsets.v[i];
		h.bytes = (int)b2gTapeStepBytes( bodyCount, awakeCount, slotCount );
		*(b2gTapeStep*)rec = h;
	}
	b2gTapeBody* bodies = (b2gTapeBody*)( rec + b2gTapeBodiesOffset() );
	for ( int i = t; i < bodyCount; i += nt )
	{
		b2gTapeBody b;
		float4 x = xf[i];
		float2 c = center[i], lc = localCenter[i];
		b.xf.p = d_v( x.x, x.y );
		b.xf.q = b2Rot{ x.z, x.w };
		b.center = d_v( c.x, c.y );
		b.localCenter = d_v( lc.x, lc.y );
		int ai = awakeIndex[i];
		b.awakeIndex = ai;
		b.type = bodyType[i];
		if ( ai >= 0 )
		{
			float4 v = sv[ai];
			b.vx = v.x;
			b.vy = v.y;
			b.w = v.z;
			b.flags = __float_as_uint( v.w );
		}
		else
		{
			b.vx = 0.0f;
			b.vy = 0.0f;
			b.w = 0.0f;
			b.flags = 0;
		}
		bodies[i] = b;
	}
	float* pr = (float*)( rec + b2gTapeParamsOffset( bodyCount ) );
	for ( int i = t; i < 8 * awakeCount; i += nt ) pr[i] = bodyParams[i];
	float* toi = (float*)( rec + b2gTapeToiOffset( bodyCount, awakeCount ) );
	for ( int i = t; i < awakeCount; i += nt ) toi[i] = 1.0f;
	int* ids = (int*)( rec + b2gTapeIdsOffset( bodyCount, awakeCount ) );
	b2gContact* cs = (b2gContact*)( rec + b2gTapeContactsOffset( bodyCount, awakeCount, slotCount ) );
	for ( int s = t; s < slotCount; s += nt )
	{
		int id = colorIds[s];
		ids[s] = id;
		cs[s] = contacts[id];
	}
}

extern "C" int b2gDev_CaptureTape( b2gDeviceWorld* dw, const b2gStepParams* p, int bodyCount, int awakeCount, int jointCount,
								   void** arena, long long* capacity, long long* used, long long* offset )
{
	int slotCount = dw->colorOffsets[B2_GRAPH_COLOR_COUNT];
	long long bytes = b2gTapeStepBytes( bodyCount, awakeCount, slotCount );
	if ( *used + bytes > *capacity )
	{
		/* room for 128 records of this size at first, then four times as much: growing is
		   an allocation and a copy, which many worlds recording together should rarely pay */
		long long cap = *capacity > 0 ? 4 * *capacity : 128 * bytes;
		if ( cap < ( 1LL << 20 ) ) cap = 1LL << 20;
		while ( cap < *used + bytes ) cap *= 4;
		void* grown = NULL;
		CK( cudaMalloc( &grown, (size_t)cap ) );
		if ( *arena != NULL )
		{
			if ( dw->defer )
			{
				/* recorded captures of earlier steps have run (every flush waits), but this
				   step's records may not: copy in order at the flush */
				d_deferredOp op;
				memset( &op, 0, sizeof( op ) );
				op.kind = D_OP_D2D;
				op.dev = grown;
				op.host = *arena;
				op.bytes = *used;
				if ( *used > 0 ) dw->defer->ops.push_back( op );
				dw->retired.push_back( *arena );
			}
			else
			{
				if ( *used > 0 ) CK( cudaMemcpyAsync( grown, *arena, (size_t)*used, cudaMemcpyDeviceToDevice, dw->stream ) );
				CK( cudaStreamSynchronize( dw->stream ) );
				CK( cudaFree( *arena ) );
			}
		}
		*arena = grown;
		*capacity = cap;
	}
	d_colorOffsets offsets;
	memcpy( offsets.v, dw->colorOffsets, sizeof( offsets.v ) );
	int n = bodyCount > slotCount ? bodyCount : slotCount;
	n = n > 8 * awakeCount ? n : 8 * awakeCount;
	int grid = blocks( n > 0 ? n : 1 );
	d_captureArgs ca;
	ca.rec = (unsigned char*)*arena + *used;
	ca.params = *p;
	ca.offsets = offsets;
	ca.bodyCount = bodyCount;
	ca.awakeCount = awakeCount;
	ca.slotCount = slotCount;
	ca.jointCount = jointCount;
	ca.xf = dw->xf;
	ca.center = dw->center;
	ca.localCenter = dw->localCenter;
	ca.awakeIndex = dw->awakeIndex;
	ca.bodyType = dw->bodyType;
	ca.sv = dw->stateV;
	ca.bodyParams = dw->params;
	ca.colorIds = dw->colorIds;
	ca.contacts = dw->contacts;
	CK2( ( dev_launch<d_captureArgs, b_capture>( dw, DK_CAPTURE, grid, ca ) ) );
	*offset = *used;
	dw->tapeToi = (float*)( (unsigned char*)*arena + *used + b2gTapeToiOffset( bodyCount, awakeCount ) );
	*used += bytes;
	return 0;
}

extern "C" void b2gDev_FreeTapeArena( void* arena )
{
	if ( arena != NULL ) cudaFree( arena );
}

extern "C" const b2gShape* b2gDev_ShapeArray( b2gDeviceWorld* dw, int* count )
{
	*count = dw->shapeCountTotal;
	return dw->shapes;
}

extern "C" int b2gDev_ContactCapacity( b2gDeviceWorld* dw ) { return dw->contactCap; }

extern "C" int b2gDev_LastCounters( b2gDeviceWorld* dw, b2gStepCounters* out )
{
	*out = *dw->hCounters;
	return 0;
}

extern "C" int b2gDev_UploadJointPartners( b2gDeviceWorld* dw, const int* offsets, int bodyCount, const int* list, int listCount )
{
	dw->partnerCount = listCount;
	if ( listCount == 0 ) return 0;
	CK2( grow( dw, (void**)&dw->partnerOffsets, &dw->partnerOffsetsCap, bodyCount + 1, sizeof( int ) ) );
	CK2( grow( dw, (void**)&dw->partnerList, &dw->partnerListCap, listCount, sizeof( int ) ) );
	CK2( uploadTo( dw, dw->partnerOffsets, offsets, (size_t)( bodyCount + 1 ) * sizeof( int ) ) );
	CK2( uploadTo( dw, dw->partnerList, list, (size_t)listCount * sizeof( int ) ) );
	return 0;
}

extern "C" int b2gDev_DownloadJoints( b2gDeviceWorld* dw, b2gJoint* byId, int idCount )
{
	int n = dw->jointCount;
	if ( n == 0 ) return 0;
	b2gJoint* tmp = (b2gJoint*)malloc( (size_t)n * sizeof( b2gJoint ) );
	CK( cudaStreamSynchronize( dw->stream ) );
	cudaError_t e = ( dw->d2hBytes += (long long)( (size_t)n * sizeof( b2gJoint ) ), cudaMemcpy( tmp, dw->joints, (size_t)n * sizeof( b2gJoint ), cudaMemcpyDeviceToHost ) );
	if ( e == cudaSuccess )
	{
		for ( int i = 0; i < n; ++i )
			if ( tmp[i].jointId >= 0 && tmp[i].jointId < idCount ) byId[tmp[i].jointId] = tmp[i];
	}
	free( tmp );
	return (int)e;
}

struct d_convertTreeArgs
{
	const b2gHostTreeNode* raw;
	b2gTreeNode* out;
	int n;
};

static __device__ void b_convertTree( const d_convertTreeArgs& a, int block, int grid )
{
	int i = block * blockDim.x + threadIdx.x;
	if ( i >= a.n ) return;
	b2gTreeNode* __restrict__ out = a.out;
	b2gHostTreeNode h = a.raw[i];
	b2gTreeNode d;
	d.aabb = h.aabb;
	d.isLeaf = ( h.flags & 0x4 ) ? 1 : 0;
	d.categoryNonZero = h.categoryBits != 0;
	d.child1 = d.isLeaf ? (int)h.userData : h.child1;
	d.child2 = d.isLeaf ? -1 : h.child2;
	out[i] = d;
}

static int sideReady( b2gDeviceWorld* dw );

/* order a tree enlargement that ran on the second stream before the world's next use of
   the trees (the pair query, the bullet sweeps, a tree upload); recorded work waits on
   the host, since it replays on another stream */
static int joinEnlarge( b2gDeviceWorld* dw )
{
	if ( dw->enlargeOnSide == 0 ) return 0;
	if ( dw->defer ) CK( cudaEventSynchronize( dw->enlargeEvent ) );
	else CK( cudaStreamWaitEvent( dw->stream, dw->enlargeEvent, 0 ) );
	dw->enlargeOnSide = 0;
	return 0;
}

extern "C" int b2gDev_UploadTree( b2gDeviceWorld* dw, int type, const b2gHostTreeNode* nodes, int nodeCount, int root,
								   int hostPinned )
{
	CK2( joinEnlarge( dw ) );
	int need = nodeCount > 0 ? nodeCount : 1;
	CK2( grow( dw, (void**)&dw->tree[type], &dw->treeCap[type], need, sizeof( b2gTreeNode ) ) );
	CK2( grow( dw, (void**)&dw->treeRaw[type], &dw->treeRawCap[type], need, sizeof( b2gHostTreeNode ) ) );
	if ( nodeCount > 0 )
	{
		if ( hostPinned || dw->defer )
		{
			CK2( dev_h2d( dw, dw->treeRaw[type], nodes, (size_t)nodeCount * sizeof( b2gHostTreeNode ) ) );
		}
		else
		{
			/* small trees live in pageable memory: stage them through the upload arena */
			CK2( uploadTo( dw, dw->treeRaw[type], nodes, (size_t)nodeCount * sizeof( b2gHostTreeNode ) ) );
		}
		d_convertTreeArgs ca = { dw->treeRaw[type], dw->tree[type], nodeCount };
		CK2( ( dev_launch<d_convertTreeArgs, b_convertTree>( dw, DK_CONVERT_TREE, blocks( nodeCount ), ca ) ) );
	}
	int mc = dw->movedCap[type];
	CK2( grow( dw, (void**)&dw->moved[type], &mc, need, 1 ) );
	dw->movedCap[type] = mc;
	dw->treeRoot[type] = root;
	dw->treeNodes[type] = nodeCount;
	return 0;
}

/* grow a device tree node's box by `b` with atomic min / max (the result does not depend on
   the order of the threads); returns whether it changed */
static __device__ bool d_atomicLowerF( float* p, float v )
{
	int* ip = (int*)p;
	int cur = *(volatile int*)ip;
	while ( v < __int_as_float( cur ) )
	{
		int prev = atomicCAS( ip, cur, __float_as_int( v ) );
		if ( prev == cur ) return true;
		cur = prev;
	}
	return false;
}

static __device__ bool d_atomicRaiseF( float* p, float v )
{
	int* ip = (int*)p;
	int cur = *(volatile int*)ip;
	while ( __int_as_float( cur ) < v )
	{
		int prev = atomicCAS( ip, cur, __float_as_int( v ) );
		if ( prev == cur ) return true;
		cur = prev;
	}
	return false;
}

/* dynamic_tree.c:798-837 on the device's query trees: each enlarged proxy's leaf takes its
   fat box and its ancestors grow until one already holds it. Every ancestor ends with its
   old box grown by the new boxes of the enlarged leaves below it, as the host's serial
   enlargement leaves it (the flags the host also sets are of no use to the queries). */
__global__ void k_enlargeTrees( const int* __restrict__ recs, const float4* __restrict__ boxes, int n,
								const b2gShape* __restrict__ shapes, b2gTreeNode* kinematicTree, b2gTreeNode* dynamicTree,
								const b2gHostTreeNode* __restrict__ kinematicRaw, const b2gHostTreeNode* __restrict__ dynamicRaw )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n ) return;
	const int* r = recs + 4 * i;
	if ( r[2] == 0 || r[3] != 0 ) return; /* not enlarged, or a fast bullet (the bullet pass handles it) */
	int key = shapes[r[1]].proxyKey;
	if ( key < 0 ) return;
	int type = key & 3, id = key >> 2;
	if ( type != b2_kinematicBody && type != b2_dynamicBody ) return;
	b2gTreeNode* tree = type == b2_dynamicBody ? dynamicTree : kinematicTree;
	const b2gHostTreeNode* raw = type == b2_dynamicBody ? dynamicRaw : kinematicRaw;
	float4 f = boxes[i];
	tree[id].aabb.lowerBound.x = f.x;
	tree[id].aabb.lowerBound.y = f.y;
	tree[id].aabb.upperBound.x = f.z;
	tree[id].aabb.upperBound.y = f.w;
	for ( int p = raw[id].parent; p >= 0; p = raw[p].parent )
	{
		b2AABB* box = &tree[p].aabb;
		bool changed = d_atomicLowerF( &box->lowerBound.x, f.x );
		changed = d_atomicLowerF( &box->lowerBound.y, f.y ) || changed;
		changed = d_atomicRaiseF( &box->upperBound.x, f.z ) || changed;
		changed = d_atomicRaiseF( &box->upperBound.y, f.w ) || changed;
		if ( changed == false ) break;
	}
}

extern "C" int b2gDev_EnlargeTrees( b2gDeviceWorld* dw, int recordCount )
{
	if ( dw->treeEvent == NULL ) CK( cudaEventCreateWithFlags( &dw->treeEvent, cudaEventDisableTiming ) );
	CK2( joinEnlarge( dw ) );
	CK( cudaEventRecord( dw->treeEvent, dw->stream ) );
	int n = recordCount < dw->enlargedCap / 4 ? recordCount : dw->enlargedCap / 4;
	if ( n <= 0 || dw->tree[b2_dynamicBody] == NULL || dw->treeRaw[b2_dynamicBody] == NULL ) return 0;
	/* on the second stream, so that the step's state download (queued next on the world's
	   stream) does not wait for it; the next use of the trees does */
	cudaStream_t s = dw->stream;
	if ( dw->enlargeEvent == NULL && sideReady( dw ) == 0 )
		CK( cudaEventCreateWithFlags( &dw->enlargeEvent, cudaEventDisableTiming ) );
	if ( dw->enlargeEvent != NULL )
	{
		s = dw->sideStream;
		CK( cudaStreamWaitEvent( s, dw->treeEvent, 0 ) );
	}
	k_enlargeTrees<<<blocks( n ), B2G_THREADS, 0, s>>>( dw->enlargedRecs, dw->enlargedBoxes, n, dw->shapes,
														dw->tree[b2_kinematicBody], dw->tree[b2_dynamicBody],
														dw->treeRaw[b2_kinematicBody], dw->treeRaw[b2_dynamicBody] );
	dw->launches += 1;
	CK( cudaGetLastError() );
	if ( s != dw->stream )
	{
		CK( cudaEventRecord( dw->enlargeEvent, s ) );
		dw->enlargeOnSide = 1;
	}
	return 0;
}

/* create what the tree enlargement uses (events, the second stream) and load its kernel
   ahead of the first step that needs them, so that none of these one-time costs falls in a
   step */
extern "C" int b2gDev_PrepareEnlarge( b2gDeviceWorld* dw )
{
	if ( dw->treeEvent == NULL ) CK( cudaEventCreateWithFlags( &dw->treeEvent, cudaEventDisableTiming ) );
	if ( dw->enlargeEvent == NULL && sideReady( dw ) == 0 )
		CK( cudaEventCreateWithFlags( &dw->enlargeEvent, cudaEventDisableTiming ) );
	cudaFuncAttributes attr;
	CK( cudaFuncGetAttributes( &attr, k_enlargeTrees ) );
	return 0;
}

extern "C" int b2gDev_WaitTreeUploads( b2gDeviceWorld* dw )
{
	if ( dw->treeEvent != NULL ) CK( cudaEventSynchronize( dw->treeEvent ) );
	return 0;
}

extern "C" void* b2gDev_HostAlloc( size_t bytes )
{
	void* p = NULL;
	if ( cudaMallocHost( &p, bytes ) != cudaSuccess ) return NULL;
	return p;
}

extern "C" void b2gDev_HostFree( void* p )
{
	if ( p != NULL ) cudaFreeHost( p );
}

/* the pair query of one step, issued (or recorded); its results arrive with the world's
   next wait: counters, per-move counts and offsets, and the first `window` packed pairs */
static int findPairsIssue( b2gDeviceWorld* dw, int n, bool countersReset )
{
	CK2( joinEnlarge( dw ) );
	CK2( grow( dw, (void**)&dw->pairBuf, &dw->pairBufCap, 2 * n * dw->pairPerMove, sizeof( int ) ) );
	CK2( grow( dw, (void**)&dw->pairPacked, &dw->pairPackedCap, 2 * n * dw->pairPerMove, sizeof( int ) ) );
	/* the window follows the last count; recorded work (a batched flush) reads back twice
	   that, and a world whose count still exceeds it copies the rest alone after the flush */
	if ( dw->defer && dw->pairWindow < n * dw->pairPerMove ) dw->pairWindow = 2 * dw->pairWindow;
	int window = dw->pairWindow < n * dw->pairPerMove ? dw->pairWindow : n * dw->pairPerMove;
	CK2( growHost( (void**)&dw->hPairPacked, &dw->hPairPackedCap, 2 * window, sizeof( int ) ) );
	if ( countersReset == false ) CK2( dev_memset( dw, dw->counters, 0, sizeof( b2gStepCounters ) ) );
	int* offsets = dw->pairCounts + n;
	d_findPairsArgs fa;
	fa.tStat = dw->tree[b2_staticBody];
	fa.tKin = dw->tree[b2_kinematicBody];
	fa.tDyn = dw->tree[b2_dynamicBody];
	fa.rootStat = dw->treeRoot[b2_staticBody];
	fa.rootKin = dw->treeRoot[b2_kinematicBody];
	fa.rootDyn = dw->treeRoot[b2_dynamicBody];
	fa.movedDyn = dw->moved[b2_dynamicBody];
	fa.keys = dw->moveKeys;
	fa.boxes = dw->moveBoxes;
	fa.queryShapes = dw->moveShapes;
	fa.n = n;
	fa.pairs = dw->pairBuf;
	fa.counts = dw->pairCounts;
	fa.capPerMove = dw->pairPerMove;
	fa.counters = dw->counters;
	fa.packed = dw->pairPacked;
	fa.offsets = offsets;
	/* B2G_PAIR_SET=0: every pair back to the host, which drops the existing ones itself */
	static const int s_pairSetOn = getenv( "B2G_PAIR_SET" ) == NULL || atoi( getenv( "B2G_PAIR_SET" ) ) != 0;
	fa.pairSet = dw->pairSet;
	fa.pairSetCap = s_pairSetOn ? dw->pairSetCap : 0;
	CK2( ( dev_launch<d_findPairsArgs, b_findPairs>( dw, DK_FIND_PAIRS, blocks( n ), fa ) ) );
	CK2( dev_d2h( dw, dw->hCounters, dw->counters, sizeof( b2gStepCounters ) ) );
	/* per-move counts and offsets are one array: one copy */
	CK2( dev_d2h( dw, dw->hPairCounts, dw->pairCounts, (size_t)n * 2 * sizeof( int ) ) );
	CK2( dev_d2h( dw, dw->hPairPacked, dw->pairPacked, (size_t)window * 2 * sizeof( int ) ) );
	dw->pendingMoves = n;
	return 0;
}

extern "C" int b2gDev_FindPairsIssue( b2gDeviceWorld* dw, const int* keys, const float* boxes, const int* shapes, int n )
{
	dev_event( dw, dw->ev[0] );
	/* the pair set is current before the query and its prefetch use it */
	if ( dw->pairSetStale ) CK2( pairSetRebuild( dw, 0 ) );
	/* one staged copy of the moved proxies */
	int stageBytes = n * 24;
	CK2( growHost( &dw->hMoveStage, &dw->hMoveStageCap, stageBytes, 1 ) );
	CK2( grow( dw, &dw->moveStage, &dw->moveStageCap, stageBytes, 1 ) );
	{
		float* sb = (float*)dw->hMoveStage;
		memcpy( sb, boxes, (size_t)n * 16 );
		memcpy( sb + 4 * (size_t)n, keys, (size_t)n * 4 );
		memcpy( sb + 5 * (size_t)n, shapes, (size_t)n * 4 );
	}
	CK2( dev_h2d( dw, dw->moveStage, dw->hMoveStage, (size_t)stageBytes ) );
	dw->moveBoxes = (float4*)dw->moveStage;
	dw->moveKeys = (int*)( dw->moveBoxes + n );
	dw->moveShapes = dw->moveKeys + n;
	/* per-move counts at [0, n), offsets at [n, 2n) */
	CK2( grow( dw, (void**)&dw->pairCounts, &dw->moveCap, 2 * n, sizeof( int ) ) );
	CK2( growHost( (void**)&dw->hPairCounts, &dw->hPairCountsCap, 2 * n, sizeof( int ) ) );
	if ( dw->pairWindow < 64 ) dw->pairWindow = 64;
	d_markMovedArgs ma = { dw->moved[b2_dynamicBody], dw->moved[b2_kinematicBody], dw->moved[b2_staticBody], dw->moveKeys, n, 1,
						   dw->counters };
	for ( int t = 0; t < 3; ++t )
	{
		ma.trees[t] = dw->tree[t];
		ma.treeNodes[t] = dw->tree[t] != NULL && dw->treeRoot[t] >= 0 ? dw->treeNodes[t] : 0;
	}
	ma.pairSet = dw->pairSet;
	ma.pairSetCap = dw->pairSet != NULL ? dw->pairSetCap : 0;
	CK2( ( dev_launch<d_markMovedArgs, b_markMoved>( dw, DK_MARK_MOVED, blocks( n ), ma ) ) );
	return findPairsIssue( dw, n, true );
}

/* after the wait: the pairs of every move in move order. A per-move overflow or a window
   too small is redone at once, outside any batch. */
extern "C" int b2gDev_FindPairsCollect( b2gDeviceWorld* dw, int** outPairs, int** outCounts, int* outTotal )
{
	int n = dw->pendingMoves;
	d_deferred* deferred = dw->defer;
	dw->defer = NULL;
	for ( int attempt = 0; attempt < 8; ++attempt )
	{
		if ( dw->hCounters->pairOverflow <= dw->pairPerMove ) break;
		while ( dw->pairPerMove < dw->hCounters->pairOverflow ) dw->pairPerMove *= 2;
		CK2( findPairsIssue( dw, n, false ) );
		CK2( drain( dw ) );
	}
	/* a query that ran out of traversal stack kept the pairs it found; the status goes out
	   with the step's */
	dw->stageStatus |= dw->hCounters->status;
	int total = dw->hCounters->pairCount;
	int window = dw->pairWindow < n * dw->pairPerMove ? dw->pairWindow : n * dw->pairPerMove;
	if ( total > window )
	{
		CK2( growHost( (void**)&dw->hPairPacked, &dw->hPairPackedCap, 2 * total, sizeof( int ) ) );
		CK2( dev_d2h( dw, dw->hPairPacked + 2 * window, dw->pairPacked + 2 * window, (size_t)( total - window ) * 2 * sizeof( int ) ) );
		CK2( drain( dw ) );
	}
	dw->defer = deferred;
	/* clear the moved flags (recorded with the next batch when batching) */
	d_markMovedArgs ma = { dw->moved[b2_dynamicBody], dw->moved[b2_kinematicBody], dw->moved[b2_staticBody], dw->moveKeys, n, 0,
						   nullptr, { nullptr, nullptr, nullptr }, { 0, 0, 0 }, nullptr, 0 };
	CK2( ( dev_launch<d_markMovedArgs, b_markMoved>( dw, DK_MARK_MOVED, blocks( n ), ma ) ) );
	/* next step's window follows this step's count, both ways */
	dw->pairWindow = 2 * total > 64 ? 2 * total : 64;
	/* pairs in move order for the host */
	CK2( growHost( (void**)&dw->hPairs, &dw->hPairsCap, 2 * ( total > 0 ? total : 1 ), sizeof( int ) ) );
	int o = 0;
	for ( int i = 0; i < n; ++i )
	{
		int c = dw->hPairCounts[i];
		memcpy( dw->hPairs + 2 * o, dw->hPairPacked + 2 * (size_t)dw->hPairCounts[n + i], (size_t)c * 2 * sizeof( int ) );
		o += c;
	}
	dev_event( dw, dw->ev[1] );
	dw->pairsTimingPending = dw->defer == NULL;
	*outPairs = dw->hPairs;
	*outCounts = dw->hPairCounts;
	*outTotal = total;
	return 0;
}

/* drop an issued query whose results will not be used: its moved flags are cleared (the
   next query sets its own) */
extern "C" int b2gDev_FindPairsDiscard( b2gDeviceWorld* dw )
{
	int n = dw->pendingMoves;
	dw->pendingMoves = 0;
	dw->pairsTimingPending = 0;
	if ( n <= 0 ) return 0;
	d_markMovedArgs ma = { dw->moved[b2_dynamicBody], dw->moved[b2_kinematicBody], dw->moved[b2_staticBody], dw->moveKeys, n, 0,
						   nullptr, { nullptr, nullptr, nullptr }, { 0, 0, 0 }, nullptr, 0 };
	CK2( ( dev_launch<d_markMovedArgs, b_markMoved>( dw, DK_MARK_MOVED, blocks( n ), ma ) ) );
	return 0;
}

extern "C" int b2gDev_FindPairs( b2gDeviceWorld* dw, const int* keys, const float* boxes, const int* shapes, int n,
								  int** outPairs, int** outCounts, int* outTotal )
{
	CK2( b2gDev_FindPairsIssue( dw, keys, boxes, shapes, n ) );
	CK2( drain( dw ) );
	return b2gDev_FindPairsCollect( dw, outPairs, outCounts, outTotal );
}

static int cmpChange( const void* a, const void* b )
{
	int x = ( (const int*)a )[0], y = ( (const int*)b )[0];
	return ( x > y ) - ( x < y );
}

/* the narrowphase over every live contact slot, issued (or recorded); the counters and the
   first `window` state changes arrive with the world's next wait */
extern "C" int b2gDev_CollideIssue( b2gDeviceWorld* dw, const b2gStepParams* p, int contactIdCapacity )
{
	/* roots from an earlier step's early pass never serve this step's analysis */
	dw->comp.earlyValid = 0;
	dev_event( dw, dw->ev[2] );
	CK2( dev_memset( dw, dw->counters, 0, sizeof( b2gStepCounters ) ) );
	if ( contactIdCapacity > 0 )
	{
		d_collideArgs a;
		a.contacts = dw->contacts;
		a.capacity = contactIdCapacity;
		a.shapes = dw->shapes;
		a.fat = dw->fat;
		a.xf = dw->xf;
		a.center = dw->center;
		a.localCenter = dw->localCenter;
		a.invMass = dw->invMass;
		a.invI = dw->invI;
		a.maxExtent = dw->maxExtent;
		a.awakeIndex = dw->awakeIndex;
		a.bodyType = dw->bodyType;
		a.bodyFlags = dw->bodyFlags;
		a.changes = dw->changes;
		a.counters = dw->counters;
		a.recycleDistance = p->contactRecycleDistance;
		dev_event( dw, dw->ev[9] );
		CK2( ( dev_launch<d_collideArgs, b_collide>( dw, DK_COLLIDE, blocks( contactIdCapacity ), a ) ) );
		dev_event( dw, dw->ev[3] );
	}
	if ( dw->changeWindow < 64 ) dw->changeWindow = 64;
	if ( dw->defer && dw->changeWindow < contactIdCapacity ) dw->changeWindow = 2 * dw->changeWindow;
	int window = dw->changeWindow < contactIdCapacity ? dw->changeWindow : contactIdCapacity;
	CK2( growHost( (void**)&dw->hChanges, &dw->hChangesCap, 2 * ( window > 0 ? window : 1 ), sizeof( int ) ) );
	CK2( dev_d2h( dw, dw->hCounters, dw->counters, sizeof( b2gStepCounters ) ) );
	if ( window > 0 ) CK2( dev_d2h( dw, dw->hChanges, dw->changes, (size_t)window * 2 * sizeof( int ) ) );
	dw->pendingCapacity = contactIdCapacity;
	return 0;
}

/* after the wait: the state changes sorted by contact id */
extern "C" int b2gDev_CollideCollect( b2gDeviceWorld* dw, const int** outChanges, int* outChangeCount, int* outRecycled )
{
	int contactIdCapacity = dw->pendingCapacity;
	int window = dw->changeWindow < contactIdCapacity ? dw->changeWindow : contactIdCapacity;
	if ( dw->defer == NULL )
	{
		if ( contactIdCapacity > 0 )
		{
			float ms = 0.0f;
			cudaEventElapsedTime( &ms, dw->ev[9], dw->ev[3] );
			dw->collideMs += ms;
		}
		if ( dw->pairsTimingPending )
		{
			float ms = 0.0f;
			cudaEventElapsedTime( &ms, dw->ev[0], dw->ev[1] );
			dw->pairsMs += ms;
			dw->pairsTimingPending = 0;
		}
	}
	int n = dw->hCounters->stateChangeCount;
	if ( n > window )
	{
		d_deferred* deferred = dw->defer;
		dw->defer = NULL;
		CK2( growHost( (void**)&dw->hChanges, &dw->hChangesCap, 2 * n, sizeof( int ) ) );
		CK2( dev_d2h( dw, dw->hChanges + 2 * window, dw->changes + 2 * window, (size_t)( n - window ) * 2 * sizeof( int ) ) );
		CK2( drain( dw ) );
		dw->defer = deferred;
	}
	dw->changeWindow = 2 * n > 64 ? 2 * n : 64;
	if ( n > 1 ) qsort( dw->hChanges, (size_t)n, 2 * sizeof( int ), cmpChange );
	*outChanges = dw->hChanges;
	*outChangeCount = n;
	*outRecycled = dw->hCounters->recycledContactCount;
	return 0;
}

extern "C" int b2gDev_Collide( b2gDeviceWorld* dw, const b2gStepParams* p, int contactIdCapacity, const int** outChanges,
								int* outChangeCount, int* outRecycled )
{
	CK2( b2gDev_CollideIssue( dw, p, contactIdCapacity ) );
	CK2( drain( dw ) );
	return b2gDev_CollideCollect( dw, outChanges, outChangeCount, outRecycled );
}

/* the solver and finalize of one step, issued (or recorded: one-CTA worlds only); the
   counters and the first `window` enlarged-proxy records arrive with the world's next wait */
/* the finalize arguments of this world's current state (solver.c b2FinalizeBodiesTask and
   b2SolveContinuous read and write these arrays); trees beyond the static one are off */
static void finalizeArgsFor( b2gDeviceWorld* dw, const b2gStepParams* p, int awakeCount, int shapeTotal, d_finalizeArgs* f )
{
	f->sv = dw->stateV;
	f->sd = dw->stateD;
	f->params = dw->params;
	f->center0 = dw->center0;
	f->awakeBodyId = dw->awakeBodyId;
	f->awakeCount = awakeCount;
	f->xf = dw->xf;
	f->center = dw->center;
	f->localCenter = dw->localCenter;
	f->minExtent = dw->minExtent;
	f->maxExtent = dw->maxExtent;
	f->sleepThreshold = dw->sleepThreshold;
	f->safetyFactor = dw->safetyFactor;
	f->bodyType = dw->bodyType;
	f->bodyFlags = dw->bodyFlags;
	f->shapeStart = dw->shapeStart;
	f->shapeCount = dw->shapeCount;
	f->shapeList = dw->shapeList;
	f->shapes = dw->shapes;
	f->aabb = dw->aabb;
	f->fat = dw->fat;
	f->shapeEnlarged = dw->shapeEnlarged;
	f->enlargedRecs = dw->enlargedRecs;
	f->enlargedBoxes = dw->enlargedBoxes;
	f->enlargedCap = shapeTotal;
	f->counters = dw->counters;
	f->dt = p->dt;
	f->inv_dt = p->inv_dt;
	f->enableSleep = p->enableSleep;
	f->enableContinuous = p->enableContinuous;
	f->ccd.staticTree = dw->tree[b2_staticBody];
	f->ccd.staticRoot = dw->tree[b2_staticBody] != NULL ? dw->treeRoot[b2_staticBody] : -1;
	f->ccd.kinematicTree = NULL;
	f->ccd.kinematicRoot = -1;
	f->ccd.dynamicTree = NULL;
	f->ccd.dynamicRoot = -1;
	f->ccd.shapes = dw->shapes;
	f->ccd.xf = dw->xf;
	f->ccd.center = dw->center;
	f->ccd.localCenter = dw->localCenter;
	f->ccd.bodyFlags = dw->bodyFlags;
	f->ccd.partnerOffsets = dw->partnerCount > 0 ? dw->partnerOffsets : NULL;
	f->ccd.partnerList = dw->partnerCount > 0 ? dw->partnerList : NULL;
	f->ccd.sensorHits = dw->sensorHits;
	f->ccd.sensorHitCap = dw->sensorHitsCap;
	f->ccd.sensorHitCount = &dw->counters->sensorHitCount;
}

/* solver.c:1917-1928 b2BulletBodyTask: each fast bullet body swept against the static,
   kinematic and dynamic trees (the latter two as the host left them after this step's
   broadphase enlargement), moved back to its earliest time of impact, its shapes' boxes
   refreshed; one record (shape id, enlarged) and fat box per bullet shape */
__global__ void k_bullets( d_finalizeArgs f, const int* bulletSims, int count, int* recs, float4* boxes, int* recCount, int recCap )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= count ) return;
	int simIndex = bulletSims[i];
	int bodyId = f.awakeBodyId[simIndex];
	float2 c = f.center[bodyId];
	float4 x = f.xf[bodyId];
	d_solveContinuous( f, simIndex, bodyId, d_v( c.x, c.y ), b2Rot{ x.z, x.w }, true );
	int start = f.shapeStart[bodyId], n = f.shapeCount[bodyId];
	int base = atomicAdd( recCount, n );
	for ( int k = 0; k < n && base + k < recCap; ++k )
	{
		int shapeId = f.shapeList[start + k];
		recs[2 * ( base + k )] = shapeId;
		recs[2 * ( base + k ) + 1] = f.shapeEnlarged[shapeId];
		boxes[base + k] = f.fat[shapeId];
	}
}

extern "C" int b2gDev_SolveBullets( b2gDeviceWorld* dw, const b2gStepParams* p, int awakeCount, const int* bulletSims, int count,
									const int** outRecs, const float** outBoxes, int* outCount )
{
	*outRecs = NULL;
	*outBoxes = NULL;
	*outCount = 0;
	if ( count <= 0 ) return 0;
	CK2( joinEnlarge( dw ) );
	int shapeTotal = dw->shapeCountTotal;
	int cap = shapeTotal > 0 ? shapeTotal : 1;
	CK2( grow( dw, (void**)&dw->bulletSims, &dw->bulletSimsCap, count, sizeof( int ) ) );
	CK2( grow( dw, (void**)&dw->bulletRecs, &dw->bulletRecsCap, 2 * cap, sizeof( int ) ) );
	CK2( grow( dw, (void**)&dw->bulletBoxes, &dw->bulletBoxesCap, cap, sizeof( float4 ) ) );
	if ( dw->bulletCount == NULL ) CK( cudaMalloc( &dw->bulletCount, sizeof( int ) ) );
	CK2( growHost( (void**)&dw->hBulletRecs, &dw->hBulletRecsCap, 2 * cap, sizeof( int ) ) );
	CK2( growHost( (void**)&dw->hBulletBoxes, &dw->hBulletBoxesCap, cap, sizeof( float4 ) ) );
	d_finalizeArgs f;
	memset( &f, 0, sizeof( f ) );
	finalizeArgsFor( dw, p, awakeCount, shapeTotal, &f );
	f.ccd.kinematicTree = dw->tree[b2_kinematicBody];
	f.ccd.kinematicRoot = dw->tree[b2_kinematicBody] != NULL ? dw->treeRoot[b2_kinematicBody] : -1;
	f.ccd.dynamicTree = dw->tree[b2_dynamicBody];
	f.ccd.dynamicRoot = dw->tree[b2_dynamicBody] != NULL ? dw->treeRoot[b2_dynamicBody] : -1;
	f.toi = NULL;
	f.sleepTime = dw->sleepTime;
	CK( cudaMemcpyAsync( dw->bulletSims, bulletSims, (size_t)count * sizeof( int ), cudaMemcpyHostToDevice, dw->stream ) );
	dw->h2dBytes += (long long)count * (long long)sizeof( int );
	CK( cudaMemsetAsync( dw->bulletCount, 0, sizeof( int ), dw->stream ) );
	k_bullets<<<( count + 63 ) / 64, 64, 0, dw->stream>>>( f, dw->bulletSims, count, dw->bulletRecs, dw->bulletBoxes, dw->bulletCount, cap );
	dw->launches += 1;
	CK( cudaGetLastError() );
	int n = 0;
	CK( cudaMemcpyAsync( &n, dw->bulletCount, sizeof( int ), cudaMemcpyDeviceToHost, dw->stream ) );
	CK( cudaStreamSynchronize( dw->stream ) );
	if ( n > cap ) n = cap;
	if ( n > 0 )
	{
		CK( cudaMemcpyAsync( dw->hBulletRecs, dw->bulletRecs, (size_t)n * 2 * sizeof( int ), cudaMemcpyDeviceToHost, dw->stream ) );
		CK( cudaMemcpyAsync( dw->hBulletBoxes, dw->bulletBoxes, (size_t)n * sizeof( float4 ), cudaMemcpyDeviceToHost, dw->stream ) );
		CK( cudaStreamSynchronize( dw->stream ) );
		dw->d2hBytes += (long long)n * (long long)( 2 * sizeof( int ) + sizeof( float4 ) );
	}
	*outRecs = dw->hBulletRecs;
	*outBoxes = (const float*)dw->hBulletBoxes;
	*outCount = n;
	dw->prefetchValid = 0;
	return 0;
}

/* the second stream, its events and the mapped start word, created on first use; 0 when
   ready */
static int sideReady( b2gDeviceWorld* dw )
{
	if ( dw->sideStream != NULL ) return 0;
	cudaStream_t side = NULL;
	cudaEvent_t fork = NULL, join = NULL;
	int* hFlag = NULL;
	int* dFlag = NULL;
	bool ok = cudaStreamCreateWithFlags( &side, cudaStreamNonBlocking ) == cudaSuccess &&
			  cudaEventCreateWithFlags( &fork, cudaEventDisableTiming ) == cudaSuccess &&
			  cudaEventCreateWithFlags( &join, cudaEventDisableTiming ) == cudaSuccess &&
			  cudaHostAlloc( (void**)&hFlag, sizeof( int ), cudaHostAllocMapped ) == cudaSuccess &&
			  cudaHostGetDevicePointer( (void**)&dFlag, hFlag, 0 ) == cudaSuccess;
	if ( ok == false )
	{
		cudaGetLastError();
		if ( hFlag ) cudaFreeHost( hFlag );
		if ( join ) cudaEventDestroy( join );
		if ( fork ) cudaEventDestroy( fork );
		if ( side ) cudaStreamDestroy( side );
		return 1;
	}
	*hFlag = 0;
	dw->sideStream = side;
	dw->forkEvent = fork;
	dw->joinEvent = join;
	dw->hClusterStarted = hFlag;
	dw->dClusterStarted = dFlag;
	return 0;
}

/* The component analysis's union-find, issued right after the narrowphase's results came
   back so that it runs while the host does the contact-state pass and its uploads; the
   solve's analysis starts from its roots unless the awake set or the joints changed in
   between (the state pass woke bodies). Large worlds solved by components only. */
extern "C" int b2gDev_ComponentsEarly( b2gDeviceWorld* dw, int awakeCount )
{
	/* B2G_EARLY_UNION=0: the analysis runs whole at the solve */
	static const int s_on = getenv( "B2G_EARLY_UNION" ) == NULL || atoi( getenv( "B2G_EARLY_UNION" ) ) != 0;
	if ( s_on == 0 || dw->solverMode != B2G_SOLVER_COMPONENTS || dw->defer != NULL || dw->compSkip > 0 || awakeCount < 2048 ||
		 awakeCount >= ( 1 << B2G_CURSOR_BODY_BITS ) )
		return 0;
	/* the pass rewrites the analysis buffers: the last analysis is not reused */
	dw->compValid = 0;
	int jointTotal = dw->jointOffsets[B2_GRAPH_COLOR_COUNT];
	int capacity = dw->contactSlots < dw->contactCap ? dw->contactSlots : dw->contactCap;
	return b2gDev_CompUnionEarly( &dw->comp, dw->contacts, capacity, dw->joints, dw->awakeIndex, awakeCount, jointTotal,
								  dw->jointEpoch, dw->stream, &dw->launches );
}

extern "C" int b2gDev_SolveIssue( b2gDeviceWorld* dw, const b2gStepParams* p, const int* activeColors, int activeColorCount,
								   int awakeCount )
{
	dev_event( dw, dw->ev[4] );
	int total = dw->colorOffsets[B2_GRAPH_COLOR_COUNT];
	int overflowBegin = dw->colorOffsets[B2G_OVERFLOW_INDEX];
	CK2( grow( dw, (void**)&dw->lanes, &dw->laneCap, total > 0 ? total : 1, sizeof( b2gContactLane ) ) );
	CK2( dev_memset( dw, dw->counters, 0, sizeof( b2gStepCounters ) ) );
	d_solveArgs a;
	a.contacts = dw->contacts;
	a.colorIds = dw->colorIds;
	a.lanes = dw->lanes;
	a.joints = dw->joints;
	a.sv = dw->stateV;
	a.sd = dw->stateD;
	a.params = dw->params;
	a.awakeCount = awakeCount;
	a.p = *p;
	memcpy( a.colorOffsets, dw->colorOffsets, sizeof( a.colorOffsets ) );
	int jointTotal = dw->jointOffsets[B2_GRAPH_COLOR_COUNT];
	/* finalize */
	int shapeTotal = dw->shapeCountTotal;
	CK2( grow( dw, (void**)&dw->enlargedRecs, &dw->enlargedCap, 4 * ( shapeTotal > 0 ? shapeTotal : 1 ), sizeof( int ) ) );
	CK2( grow( dw, (void**)&dw->enlargedBoxes, &dw->enlargedBoxesCap, shapeTotal > 0 ? shapeTotal : 1, sizeof( float4 ) ) );
	CK2( grow( dw, (void**)&dw->sensorHits, &dw->sensorHitsCap, 1024, sizeof( int2 ) ) );
	d_finalizeArgs f;
	finalizeArgsFor( dw, p, awakeCount, shapeTotal, &f );
	f.toi = dw->tapeToi;
	dw->tapeToi = NULL;
	f.sleepTime = dw->sleepTime;
	f.islandLocal = NULL;
	f.islandInfo = NULL;
	f.awakeIslandBits = NULL;
	int islandWords = 0;
	if ( dw->islandsOn && dw->islandCount > 0 )
	{
		islandWords = ( dw->islandCount + 31 ) / 32;
		CK2( grow( dw, (void**)&dw->islandBits, &dw->islandBitsCap, islandWords, sizeof( unsigned int ) ) );
		CK2( dev_memset( dw, dw->islandBits, 0, (size_t)islandWords * sizeof( unsigned int ) ) );
		f.islandLocal = dw->islandLocal;
		f.islandInfo = dw->islandInfo;
		f.awakeIslandBits = dw->islandBits;
	}
	int ovJointBegin0 = dw->jointOffsets[B2G_OVERFLOW_INDEX];
	int ovJointCount0 = dw->jointOffsets[B2_GRAPH_COLOR_COUNT] - ovJointBegin0;
	int ovCount0 = total - overflowBegin;
	d_jointBodies jb0 = { dw->xf, dw->center, dw->localCenter, dw->invMass, dw->invI, dw->awakeIndex };
	dev_event( dw, dw->ev[6] );
	bool solved = false;
	long long worldBytes = (long long)B2G_BIN_BODY_BYTES * awakeCount + (long long)B2G_BIN_CONTACT_BYTES * total +
						   (long long)B2G_BIN_JOINT_BYTES * jointTotal;
	if ( dw->solverMode == B2G_SOLVER_COMPONENTS && ovJointCount0 + ovCount0 == 0 && worldBytes <= B2G_WORLD_BIN_MAX_BYTES )
	{
		/* small world: one CTA solves all of it from shared memory */
		if ( dw->defer )
		{
			d_deferred* d = dw->defer;
			int argBytes = 0;
			CK2( b2gDev_SolveWorldBinArgs( &dw->comp, &a, dw->jointOffsets, &jb0, dw->awakeIndex, (int)worldBytes, dw->counters, NULL,
										   &argBytes ) );
			d_deferredOp op;
			memset( &op, 0, sizeof( op ) );
			op.kind = D_OP_KERNEL;
			op.kernel = DK_SOLVE_BIN;
			op.grid = 1;
			op.smem = (int)worldBytes;
			op.bytes = argBytes;
			op.at = (long long)d->args.size();
			d->args.resize( (size_t)d_alignArgs( op.at + op.bytes ) );
			CK2( b2gDev_SolveWorldBinArgs( &dw->comp, &a, dw->jointOffsets, &jb0, dw->awakeIndex, (int)worldBytes, dw->counters,
										   d->args.data() + op.at, &argBytes ) );
			d->ops.push_back( op );
			dw->launches += 1;
		}
		else
		{
			CK2( b2gDev_SolveWorldBin( &dw->comp, &a, dw->jointOffsets, &jb0, dw->awakeIndex, (int)worldBytes, dw->counters,
									   dw->stream, &dw->launches ) );
		}
		dw->compValid = 0;
		solved = true;
	}
	else if ( dw->defer )
	{
		/* batched stepping records one-CTA worlds only */
		return (int)cudaErrorNotSupported;
	}
	else if ( dw->solverMode == B2G_SOLVER_COMPONENTS && dw->compSkip > 0 )
	{
		dw->compSkip -= 1;
		dw->compValid = 0;
	}
	else if ( dw->solverMode == B2G_SOLVER_COMPONENTS && awakeCount < ( 1 << B2G_CURSOR_BODY_BITS ) &&
			  total < ( 1 << B2G_CURSOR_CONTACT_BITS ) && jointTotal < ( 1 << B2G_CURSOR_JOINT_BITS ) )
	{
		/* the components only change with the constraint graph: reuse the last analysis while
		   no color, joint or awake-set upload happened */
		bool reuse = dw->compValid && dw->topologyDirty == 0 && dw->comp.n == awakeCount && dw->comp.total == total &&
					 dw->comp.jointTotal == jointTotal;
		if ( reuse == false )
		{
			int forceBig = ovJointCount0 + ovCount0 > 0;
			CK2( b2gDev_CompAnalyze( &dw->comp, &a, dw->jointOffsets, dw->awakeIndex, total, jointTotal, forceBig, dw->jointEpoch,
									 dw->stream,
									 &dw->launches ) );
			dw->topologyEpoch += 1;
			dw->topologyDirty = 0;
			dw->compValid = 0;
		}
		const b2gCompSummary* hs = dw->comp.hSummary;
		if ( hs->smallComponents > 0 && hs->bigComponents > 0 && sideReady( dw ) == 0 )
		{
			/* The bins of the small components run beside the cluster solve of the big ones
			   (they share no body or contact): the cluster is launched first, and once it is
			   resident (it needs 16 whole SMs, which bins already placed would hold) the bins
			   go to the other SMs from a second stream. */
			dw->compValid = 1;
			CK( cudaEventRecord( dw->forkEvent, dw->stream ) );
			int token = ++dw->clusterToken;
			int rc = b2gDev_ClusterSolve( &dw->comp, &a, dw->jointOffsets, &jb0, activeColors, activeColorCount, 1,
										  hs->bigBodies, &dw->counters->status, dw->topologyEpoch, dw->dClusterStarted, token,
										  dw->stream, &dw->launches );
			if ( rc > 0 ) return rc;
			if ( rc == 0 )
			{
				/* bounded wait for the cluster to start; past it the bins go anyway (they
				   may then delay the cluster, never change a result) */
				uint64_t spins = 0;
				while ( *(volatile int*)dw->hClusterStarted != token && spins < ( 1ull << 17 ) ) ++spins;
				CK( cudaStreamWaitEvent( dw->sideStream, dw->forkEvent, 0 ) );
				CK2( b2gDev_CompSolveBins( &dw->comp, &a, dw->jointOffsets, &jb0, dw->counters, dw->sideStream, &dw->launches ) );
				CK( cudaEventRecord( dw->joinEvent, dw->sideStream ) );
				CK( cudaStreamWaitEvent( dw->stream, dw->joinEvent, 0 ) );
			}
			else
			{
				CK2( b2gDev_CompSolveBins( &dw->comp, &a, dw->jointOffsets, &jb0, dw->counters, dw->stream, &dw->launches ) );
				CK2( b2gDev_CompSolveBig( &dw->comp, &a, dw->jointOffsets, &jb0, activeColors, activeColorCount, total,
										  jointTotal, dw->stream, &dw->launches ) );
			}
			solved = true;
		}
		else if ( hs->smallComponents > 0 )
		{
			dw->compValid = 1;
			CK2( b2gDev_CompSolveBins( &dw->comp, &a, dw->jointOffsets, &jb0, dw->counters, dw->stream, &dw->launches ) );
			if ( hs->bigComponents > 0 )
			{
				int rc = b2gDev_ClusterSolve( &dw->comp, &a, dw->jointOffsets, &jb0, activeColors, activeColorCount, 1,
											  hs->bigBodies, &dw->counters->status, dw->topologyEpoch, NULL, 0, dw->stream,
											  &dw->launches );
				if ( rc > 0 ) return rc;
				if ( rc < 0 )
					CK2( b2gDev_CompSolveBig( &dw->comp, &a, dw->jointOffsets, &jb0, activeColors, activeColorCount, total,
											  jointTotal, dw->stream, &dw->launches ) );
			}
			solved = true;
		}
		/* mostly one big component: skip the analysis for a while */
		if ( 10ll * hs->bigBodies > 9ll * awakeCount || hs->smallComponents == 0 ) dw->compSkip = 15;
	}
	/* one big constraint graph: the cluster solver when it fits */
	if ( solved == false && dw->solverMode == B2G_SOLVER_COMPONENTS && ovJointCount0 + ovCount0 == 0 )
	{
		int rc = b2gDev_ClusterSolve( &dw->comp, &a, dw->jointOffsets, &jb0, activeColors, activeColorCount, 0, awakeCount,
									  &dw->counters->status, dw->topologyEpoch, NULL, 0, dw->stream, &dw->launches );
		if ( rc > 0 ) return rc;
		solved = rc == 0;
	}
	if ( solved )
	{
		dev_event( dw, dw->ev[7] );
		CK2( ( dev_launch<d_finalizeArgs, b_finalize, 8>( dw, DK_FINALIZE, blocks( awakeCount ), f ) ) );
		dev_event( dw, dw->ev[8] );
	}
	else if ( dw->solverMode == B2G_SOLVER_PERSISTENT )
	{
		/* one cooperative launch: solver stages and finalize */
		int ranges[4 * B2_GRAPH_COLOR_COUNT];
		for ( int k = 0; k < activeColorCount; ++k )
		{
			int c = activeColors[k];
			ranges[4 * k] = dw->jointOffsets[c];
			ranges[4 * k + 1] = dw->jointOffsets[c + 1] - dw->jointOffsets[c];
			ranges[4 * k + 2] = dw->colorOffsets[c];
			ranges[4 * k + 3] = dw->colorOffsets[c + 1] - dw->colorOffsets[c];
		}
		int overflowRange[4] = { ovJointBegin0, ovJointCount0, overflowBegin, ovCount0 };
		if ( dw->persistentScratch == NULL )
		{
			CK( cudaMalloc( &dw->persistentScratch, 4 * sizeof( int ) ) );
			CK( cudaMemset( dw->persistentScratch, 0, 4 * sizeof( int ) ) );
		}
		unsigned int* barrier = (unsigned int*)dw->persistentScratch;
		int* error = (int*)dw->persistentScratch + 2;
		int* anyRestitution = (int*)dw->persistentScratch + 3;
		CK2( b2gDev_LaunchPersistent( &a, &f, ranges, activeColorCount, overflowRange, total, jointTotal, awakeCount,
									 p->subStepCount, &jb0, barrier, error, anyRestitution, dw->stream ) );
		dw->launches += 1;
		CK( cudaEventRecord( dw->ev[7], dw->stream ) );
		CK( cudaEventRecord( dw->ev[8], dw->stream ) );
	}
	else
	{
		int jointTotal = dw->jointOffsets[B2_GRAPH_COLOR_COUNT];
		if ( jointTotal > 0 )
		{
			d_jointBodies jb = { dw->xf, dw->center, dw->localCenter, dw->invMass, dw->invI, dw->awakeIndex };
			k_prepareJoints<<<blocks( jointTotal ), B2G_THREADS, 0, dw->stream>>>( a, jb, jointTotal );
			dw->launches += 1;
		}
		if ( total > 0 )
		{
			k_prepareContacts<<<blocks( total ), B2G_THREADS, 0, dw->stream>>>( a, total, overflowBegin );
			dw->launches += 1;
		}
		CK( cudaGetLastError() );
		int ovJointBegin = dw->jointOffsets[B2G_OVERFLOW_INDEX];
		int ovJointCount = dw->jointOffsets[B2_GRAPH_COLOR_COUNT] - ovJointBegin;
		int ovCount = total - overflowBegin;
		bool hasOverflow = ovJointCount + ovCount > 0;
		for ( int sub = 0; sub < p->subStepCount; ++sub )
		{
			k_integrateVelocities<<<blocks( awakeCount ), B2G_THREADS, 0, dw->stream>>>( a );
			dw->launches += 1;
			for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
			{
				if ( stage == STAGE_RELAX )
				{
					k_integratePositions<<<blocks( awakeCount ), B2G_THREADS, 0, dw->stream>>>( a );
					dw->launches += 1;
				}
				if ( hasOverflow )
				{
					k_overflowStage<<<1, 1, 0, dw->stream>>>( a, ovJointBegin, ovJointCount, overflowBegin, ovCount, stage );
					dw->launches += 1;
				}
				for ( int k = 0; k < activeColorCount; ++k )
				{
					int c = activeColors[k];
					int jb = dw->jointOffsets[c], jc = dw->jointOffsets[c + 1] - jb;
					int lb = dw->colorOffsets[c], lc = dw->colorOffsets[c + 1] - lb;
					if ( jc + lc > 0 )
					{
						k_colorStage<<<blocks( jc + lc ), B2G_THREADS, 0, dw->stream>>>( a, jb, jc, lb, lc, stage );
						dw->launches += 1;
					}
				}
			}
		}
		if ( hasOverflow )
		{
			k_overflowStage<<<1, 1, 0, dw->stream>>>( a, ovJointBegin, ovJointCount, overflowBegin, ovCount, STAGE_RESTITUTION );
			dw->launches += 1;
		}
		for ( int k = 0; k < activeColorCount; ++k )
		{
			int c = activeColors[k];
			int lb = dw->colorOffsets[c], lc = dw->colorOffsets[c + 1] - lb;
			if ( lc > 0 )
			{
				k_colorStage<<<blocks( lc ), B2G_THREADS, 0, dw->stream>>>( a, 0, 0, lb, lc, STAGE_RESTITUTION );
				dw->launches += 1;
			}
		}
		if ( total > 0 )
		{
			k_storeImpulses<<<blocks( total ), B2G_THREADS, 0, dw->stream>>>( a, total, overflowBegin );
			dw->launches += 1;
		}
		CK( cudaGetLastError() );


		dev_event( dw, dw->ev[7] );
		CK2( ( dev_launch<d_finalizeArgs, b_finalize, 8>( dw, DK_FINALIZE, blocks( awakeCount ), f ) ) );
		dev_event( dw, dw->ev[8] );
	}
	/* the counters and the first `window` enlarged-proxy records come back in one wait */
	if ( dw->recWindow < 64 ) dw->recWindow = 64;
	if ( dw->defer && dw->recWindow < shapeTotal ) dw->recWindow = 2 * dw->recWindow;
	int recWindow = dw->recWindow < shapeTotal ? dw->recWindow : shapeTotal;
	/* staging for every shape's record, so that a larger count later needs no allocation */
	CK2( growHost( (void**)&dw->hRecsRaw, &dw->hRecsRawCap, 4 * ( shapeTotal > 0 ? shapeTotal : 1 ), sizeof( int ) ) );
	CK2( growHost( (void**)&dw->hBoxesRaw, &dw->hBoxesRawCap, 4 * ( shapeTotal > 0 ? shapeTotal : 1 ), sizeof( float ) ) );
	CK2( dev_d2h( dw, dw->hCounters, dw->counters, sizeof( b2gStepCounters ) ) );
	if ( recWindow > 0 )
	{
		CK2( dev_d2h( dw, dw->hRecsRaw, dw->enlargedRecs, (size_t)recWindow * 4 * sizeof( int ) ) );
		CK2( dev_d2h( dw, dw->hBoxesRaw, dw->enlargedBoxes, (size_t)recWindow * sizeof( float4 ) ) );
	}
	if ( islandWords > 0 )
	{
		CK2( growHost( (void**)&dw->hIslandBits, &dw->hIslandBitsCap, islandWords, sizeof( unsigned int ) ) );
		CK2( dev_d2h( dw, dw->hIslandBits, dw->islandBits, (size_t)islandWords * sizeof( unsigned int ) ) );
	}
	dw->pendingIslandWords = islandWords;
	dw->pendingRecWindow = recWindow;
	dw->pendingShapeTotal = shapeTotal;
	dw->pendingSolved = solved ? 1 : 0;
	return 0;
}

/* after the wait: status and the enlarged-proxy records in ascending awake index */
extern "C" int b2gDev_SolveCollect( b2gDeviceWorld* dw, const int** outRecs, int* outCount, const float** outBoxes,
									 int* outStatus )
{
	int recWindow = dw->pendingRecWindow, shapeTotal = dw->pendingShapeTotal;
	bool solved = dw->pendingSolved != 0;
	d_deferred* deferred = dw->defer;
	dw->defer = NULL;
	if ( deferred == NULL )
	{
		float ms = 0.0f;
		cudaEventElapsedTime( &ms, dw->ev[6], dw->ev[7] );
		dw->solveMs += ms;
		cudaEventElapsedTime( &ms, dw->ev[7], dw->ev[8] );
		dw->finalizeMs += ms;
	}
	if ( solved == false && dw->solverMode == B2G_SOLVER_PERSISTENT )
	{
		int err = 0;
		CK( cudaMemcpy( &err, (int*)dw->persistentScratch + 2, sizeof( int ), cudaMemcpyDeviceToHost ) );
		if ( err != 0 )
		{
			/* a grid barrier gave up: report it and clear the word for the next step */
			dw->hCounters->status |= err;
			CK( cudaMemset( (int*)dw->persistentScratch + 2, 0, sizeof( int ) ) );
		}
	}
	int n = dw->hCounters->enlargedBodyCount;
	if ( n > shapeTotal ) n = shapeTotal;
	CK2( growHost( (void**)&dw->hRecs, &dw->hRecsCap, 4 * ( n > 0 ? n : 1 ), sizeof( int ) ) );
	CK2( growHost( (void**)&dw->hBoxes, &dw->hBoxesCap, 4 * ( n > 0 ? n : 1 ), sizeof( float ) ) );
	if ( n > recWindow )
	{
		CK2( growHost( (void**)&dw->hRecsRaw, &dw->hRecsRawCap, 4 * n, sizeof( int ) ) );
		CK2( growHost( (void**)&dw->hBoxesRaw, &dw->hBoxesRawCap, 4 * n, sizeof( float ) ) );
		CK2( dev_d2h( dw, dw->hRecsRaw + 4 * recWindow, dw->enlargedRecs + 4 * recWindow, (size_t)( n - recWindow ) * 4 * sizeof( int ) ) );
		CK2( dev_d2h( dw, dw->hBoxesRaw + 4 * recWindow, dw->enlargedBoxes + recWindow, (size_t)( n - recWindow ) * sizeof( float4 ) ) );
		CK2( drain( dw ) );
	}
	dw->recWindow = 2 * n > 64 ? 2 * n : 64;
	if ( n > 0 )
	{
		/* records into ascending awake index, keeping the arrival order of a body's shapes
		   (one body's records are contiguous): a counting sort over the awake indices */
		const int* recs = dw->hRecsRaw;
		const float* boxes = dw->hBoxesRaw;
		int top = 0;
		for ( int i = 0; i < n; ++i ) top = recs[4 * i] > top ? recs[4 * i] : top;
		if ( top + 2 > dw->hSortTmpCap )
		{
			int cap = dw->hSortTmpCap > 0 ? dw->hSortTmpCap : 1024;
			while ( cap < top + 2 ) cap *= 2;
			int* grown = (int*)realloc( dw->hSortTmp, (size_t)cap * sizeof( int ) );
			if ( grown == NULL ) return (int)cudaErrorMemoryAllocation;
			dw->hSortTmp = grown;
			dw->hSortTmpCap = cap;
		}
		int* start = dw->hSortTmp;
		memset( start, 0, (size_t)( top + 2 ) * sizeof( int ) );
		for ( int i = 0; i < n; ++i ) start[recs[4 * i] + 1] += 1;
		for ( int s = 1; s <= top + 1; ++s ) start[s] += start[s - 1];
		for ( int i = 0; i < n; ++i )
		{
			int dst = start[recs[4 * i]]++;
			memcpy( dw->hRecs + 4 * dst, recs + 4 * i, 4 * sizeof( int ) );
			memcpy( dw->hBoxes + 4 * dst, boxes + 4 * i, 4 * sizeof( float ) );
		}
	}
	dw->defer = deferred;
	dev_event( dw, dw->ev[5] );
	*outRecs = dw->hRecs;
	*outBoxes = dw->hBoxes;
	*outCount = n;
	*outStatus = dw->hCounters->status | dw->stageStatus;
	dw->stageStatus = 0;
	return 0;
}

extern "C" int b2gDev_Solve( b2gDeviceWorld* dw, const b2gStepParams* p, const int* activeColors, int activeColorCount,
							  const int* colorContactCounts, const int* colorJointCounts, int awakeCount, const int** outRecs,
							  int* outCount, const float** outBoxes, int* outStatus )
{
	(void)colorContactCounts;
	(void)colorJointCounts;
	CK2( b2gDev_SolveIssue( dw, p, activeColors, activeColorCount, awakeCount ) );
	CK2( drain( dw ) );
	return b2gDev_SolveCollect( dw, outRecs, outCount, outBoxes, outStatus );
}

/* whether a world's solve runs as one CTA (and can be batched): the same test as the
   solver's dispatch */
extern "C" int b2gDev_SolveFitsOneBlock( b2gDeviceWorld* dw, int awakeCount )
{
	int total = dw->colorOffsets[B2_GRAPH_COLOR_COUNT];
	int overflow = total - dw->colorOffsets[B2G_OVERFLOW_INDEX];
	int jointTotal = dw->jointOffsets[B2_GRAPH_COLOR_COUNT];
	int jointOverflow = jointTotal - dw->jointOffsets[B2G_OVERFLOW_INDEX];
	long long bytes = (long long)B2G_BIN_BODY_BYTES * awakeCount + (long long)B2G_BIN_CONTACT_BYTES * total +
					  (long long)B2G_BIN_JOINT_BYTES * jointTotal;
	return dw->solverMode == B2G_SOLVER_COMPONENTS && overflow + jointOverflow == 0 && bytes <= B2G_WORLD_BIN_MAX_BYTES;
}

/* the world's wait: its issued work is done and its upload arena free again */
extern "C" int b2gDev_Synchronize( b2gDeviceWorld* dw ) { return drain( dw ); }

/* every stream of the device is idle (before a batch starts recording) */
extern "C" int b2gDev_DeviceSynchronize( void ) { return (int)cudaDeviceSynchronize(); }

/* accumulated device milliseconds per stage since the last reset: pairs (query and
   copies), narrowphase kernel, solver (prepare through store), finalize; and traffic */
extern "C" void b2gDev_Timings( b2gDeviceWorld* dw, float* out, long long* traffic, int reset )
{
	out[0] = dw->pairsMs;
	out[1] = dw->collideMs;
	out[2] = dw->solveMs;
	out[3] = dw->finalizeMs;
	traffic[0] = dw->h2dBytes;
	traffic[1] = dw->d2hBytes;
	traffic[2] = dw->launches;
	if ( reset )
	{
		dw->pairsMs = dw->collideMs = dw->solveMs = dw->finalizeMs = 0.0f;
		dw->h2dBytes = dw->d2hBytes = 0;
		dw->launches = 0;
	}
}

extern "C" void* b2gDev_Stream( b2gDeviceWorld* dw ) { return (void*)dw->stream; }

/* ======================= batched flush of recorded device work ======================= */

/* one copy of a flush: device to device (uploads from the flush's staging, grown buffers,
   downloads into the flush's download area) */
struct d_copyOp
{
	unsigned char* dst;
	const unsigned char* src; /* an offset into the flush's staging when fromStaging */
	long long bytes;
	int value; /* >= 0: fill with this byte instead of copying */
	int fromStaging;
};

__global__ void k_batchCopy( const d_copyOp* __restrict__ ops, int count, const unsigned char* __restrict__ staging )
{
	d_copyOp op = ops[blockIdx.x];
	if ( op.fromStaging ) op.src = staging + (uintptr_t)op.src;
	long long n = op.bytes;
	bool vec = ( ( (uintptr_t)op.dst | (uintptr_t)op.src | (uintptr_t)n ) & 15 ) == 0;
	if ( op.value >= 0 )
	{
		unsigned char v = (unsigned char)op.value;
		for ( long long i = threadIdx.x; i < n; i += blockDim.x ) op.dst[i] = v;
	}
	else if ( vec )
	{
		const uint4* s4 = (const uint4*)op.src;
		uint4* d4 = (uint4*)op.dst;
		for ( long long i = threadIdx.x; i < n / 16; i += blockDim.x ) d4[i] = s4[i];
	}
	else
	{
		for ( long long i = threadIdx.x; i < n; i += blockDim.x ) op.dst[i] = op.src[i];
	}
}

/* A world's part of a flush. Its records split into units -- a run of consecutive uploads,
   a run of consecutive downloads, or one other record -- and unit l of every world runs in
   level l of the replay. `slot` is where unit l sits in its level's table (the first copy,
   the kernel record or the one-CTA solve), `blockBase` a kernel unit's first block. */
struct d_worldFlush
{
	std::vector<int> unitEnd;
	std::vector<long long> downAt; /* per record: download offset within the world's part */
	std::vector<long long> slot;
	std::vector<int> blockBase;
	long long upBase, argBase, downBase, downBytes;
};

struct b2gDevBatch
{
	cudaStream_t stream;
	unsigned char *hBlob, *dBlob, *hDown, *dDown;
	long long blobCap, downCap;
	std::vector<d_worldFlush> plans; /* per world, reused across flushes */
	long long launches;
	double assembleMs, waitMs;
	double partMs[5]; /* plan, layout, stage, issue, deliver */
};

static double d_nowMs( void )
{
	struct timespec ts;
	clock_gettime( CLOCK_MONOTONIC, &ts );
	return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

extern "C" void b2gDev_BatchPartTimes( b2gDevBatch* b, double* out, int reset )
{
	for ( int k = 0; k < 5; ++k )
	{
		out[k] = b->partMs[k];
		if ( reset ) b->partMs[k] = 0.0;
	}
}

extern "C" void b2gDev_BatchTimes( b2gDevBatch* b, double* assembleMs, double* waitMs, int reset )
{
	*assembleMs = b->assembleMs;
	*waitMs = b->waitMs;
	if ( reset )
	{
		b->assembleMs = 0.0;
		b->waitMs = 0.0;
	}
}

extern "C" int b2gDev_BatchCreate( b2gDevBatch** out )
{
	b2gDevBatch* b = new b2gDevBatch();
	/* a blocking stream, ordered after buffer growth on the legacy default stream */
	CK( cudaStreamCreate( &b->stream ) );
	*out = b;
	return 0;
}

extern "C" void b2gDev_BatchDestroy( b2gDevBatch* b )
{
	if ( b == NULL ) return;
	cudaStreamSynchronize( b->stream );
	if ( b->hBlob ) cudaFreeHost( b->hBlob );
	if ( b->dBlob ) cudaFree( b->dBlob );
	if ( b->hDown ) cudaFreeHost( b->hDown );
	if ( b->dDown ) cudaFree( b->dDown );
	cudaStreamDestroy( b->stream );
	delete b;
}

/* switch a world between issuing its device work and recording it for a flush */
extern "C" int b2gDev_BatchRecord( b2gDeviceWorld* dw, int on )
{
	if ( on )
	{
		/* the caller has made the world's stream idle (b2gDev_DeviceSynchronize) */
		if ( dw->defer == NULL ) dw->defer = new d_deferred();
		dw->upUsed = 0;
	}
	else
	{
		delete dw->defer;
		dw->defer = NULL;
	}
	return 0;
}

extern "C" int b2gDev_IsRecording( b2gDeviceWorld* dw ) { return dw->defer != NULL; }

extern "C" int b2gDev_RecordedCount( b2gDeviceWorld* dw ) { return dw->defer != NULL ? (int)dw->defer->ops.size() : 0; }

/* sensor.c:43-120 b2SensorQueryCallback, one block per sensor over every shape: the tree
   query's tests (the shape's fat box meets the sensor's box, its category meets the
   sensor's mask), then the callback's (not the sensor itself, sensor events enabled on the
   shape, another body, the shape filter), then GJK distance with radii in the sensor's
   frame below 10 FLT_EPSILON */
__global__ void k_sensorOverlaps( const int* __restrict__ sensorIds, int sensorCount, const b2gShape* __restrict__ shapes,
								  const float4* __restrict__ aabb, const float4* __restrict__ fat, const float4* __restrict__ xf,
								  int shapeCount, int2* out, int outCap, int* outCount )
{
	int sensorIndex = blockIdx.x;
	if ( sensorIndex >= sensorCount ) return;
	int sensorShapeId = sensorIds[sensorIndex];
	if ( sensorShapeId < 0 ) return;
	const b2gShape* sensor = shapes + sensorShapeId;
	float4 q = aabb[sensorShapeId];
	b2AABB query = { { q.x, q.y }, { q.z, q.w } };
	float4 xs = xf[sensor->bodyId];
	b2Transform sensorXf = { { xs.x, xs.y }, { xs.z, xs.w } };
	d_proxy proxyA = d_shapeProxy( sensor );
	for ( int shapeId = threadIdx.x; shapeId < shapeCount; shapeId += blockDim.x )
	{
		if ( shapeId == sensorShapeId ) continue;
		const b2gShape* other = shapes + shapeId;
		if ( other->type < 0 || ( other->categoryBits & sensor->maskBits ) == 0 ) continue;
		if ( d_overlaps( query, fat[shapeId] ) == false ) continue;
		if ( other->enableSensorEvents == 0 || other->bodyId == sensor->bodyId ) continue;
		if ( d_shouldShapesCollide( sensor, other ) == false ) continue;
		float4 xo = xf[other->bodyId];
		b2Transform otherXf = { { xo.x, xo.y }, { xo.z, xo.w } };
		d_proxy proxyB = d_shapeProxy( other );
		d_simplexCache cache;
		cache.count = 0;
		float distance = d_shapeDistance( &proxyA, &proxyB, d_invMulTransforms( sensorXf, otherXf ), &cache );
		distance = d_max( 0.0f, distance - proxyA.radius - proxyB.radius );
		if ( distance < 10.0f * FLT_EPSILON )
		{
			int k = atomicAdd( outCount, 1 );
			if ( k < outCap ) out[k] = make_int2( sensorIndex, shapeId );
		}
	}
}

extern "C" int b2gDev_SensorHits( b2gDeviceWorld* dw, const int** outPairs, int* outCount )
{
	*outPairs = NULL;
	*outCount = 0;
	if ( dw->sensorHits == NULL ) return 0;
	int count = 0;
	CK( cudaMemcpyAsync( &count, &dw->counters->sensorHitCount, sizeof( int ), cudaMemcpyDeviceToHost, dw->stream ) );
	CK( cudaStreamSynchronize( dw->stream ) );
	if ( count > dw->sensorHitsCap ) count = dw->sensorHitsCap;
	CK2( growHost( (void**)&dw->hSensorHits, &dw->hSensorHitsCap, count > 0 ? count : 1, sizeof( int2 ) ) );
	if ( count > 0 )
	{
		CK( cudaMemcpy( dw->hSensorHits, dw->sensorHits, (size_t)count * sizeof( int2 ), cudaMemcpyDeviceToHost ) );
		dw->d2hBytes += (long long)count * (long long)sizeof( int2 );
	}
	*outPairs = (const int*)dw->hSensorHits;
	*outCount = count;
	return 0;
}

extern "C" int b2gDev_SensorOverlaps( b2gDeviceWorld* dw, const int* sensorShapeIds, int sensorCount, int shapeCount,
									  const int** outPairs, int* outCount )
{
	*outPairs = NULL;
	*outCount = 0;
	if ( sensorCount <= 0 ) return 0;
	CK2( grow( dw, (void**)&dw->sensorIds, &dw->sensorIdsCap, sensorCount, sizeof( int ) ) );
	if ( dw->sensorCount == NULL ) CK( cudaMalloc( &dw->sensorCount, sizeof( int ) ) );
	if ( dw->sensorPairsCap == 0 ) CK2( grow( dw, (void**)&dw->sensorPairs, &dw->sensorPairsCap, 4 * sensorCount + 64, sizeof( int2 ) ) );
	CK( cudaMemcpyAsync( dw->sensorIds, sensorShapeIds, (size_t)sensorCount * sizeof( int ), cudaMemcpyHostToDevice, dw->stream ) );
	dw->h2dBytes += (long long)sensorCount * (long long)sizeof( int );
	int count = 0;
	for ( int attempt = 0; attempt < 2; ++attempt )
	{
		CK( cudaMemsetAsync( dw->sensorCount, 0, sizeof( int ), dw->stream ) );
		k_sensorOverlaps<<<sensorCount, 128, 0, dw->stream>>>( dw->sensorIds, sensorCount, dw->shapes, dw->aabb, dw->fat, dw->xf,
															   shapeCount, dw->sensorPairs, dw->sensorPairsCap, dw->sensorCount );
		dw->launches += 1;
		CK( cudaGetLastError() );
		CK( cudaMemcpyAsync( &count, dw->sensorCount, sizeof( int ), cudaMemcpyDeviceToHost, dw->stream ) );
		CK( cudaStreamSynchronize( dw->stream ) );
		if ( count <= dw->sensorPairsCap ) break;
		/* more overlaps than the output holds: grow it and run the pass again */
		CK2( grow( dw, (void**)&dw->sensorPairs, &dw->sensorPairsCap, count, sizeof( int2 ) ) );
	}
	CK2( growHost( (void**)&dw->hSensorPairs, &dw->hSensorPairsCap, count > 0 ? count : 1, sizeof( int2 ) ) );
	if ( count > 0 )
	{
		CK( cudaMemcpy( dw->hSensorPairs, dw->sensorPairs, (size_t)count * sizeof( int2 ), cudaMemcpyDeviceToHost ) );
		dw->d2hBytes += (long long)count * (long long)sizeof( int2 );
	}
	*outPairs = (const int*)dw->hSensorPairs;
	*outCount = count;
	return 0;
}

static int d_reserve( unsigned char** h, unsigned char** d, long long* cap, long long need )
{
	if ( need <= *cap ) return 0;
	long long nc = *cap > 0 ? *cap : ( 1LL << 20 );
	while ( nc < need ) nc *= 2;
	if ( *h ) CK( cudaFreeHost( *h ) );
	if ( *d ) CK( cudaFree( *d ) );
	*h = NULL;
	*d = NULL;
	CK( cudaMallocHost( (void**)h, (size_t)nc ) );
	CK( cudaMalloc( (void**)d, (size_t)nc ) );
	*cap = nc;
	return 0;
}

/* a level of the replay: at most one unit of every world, run together */
struct d_levelPlan
{
	long long copies, copyCount;						  /* blob offsets of the level's copy table */
	long long recs[DK_COUNT], recCount[DK_COUNT];		  /* record tables per kernel kind */
	int blocks[DK_COUNT];								  /* total blocks per kernel kind */
	int smem;											  /* largest one-CTA world solve */
};

template <class Args, void ( *Body )( const Args&, int, int ), int MinBlocks>
static int d_launchBatched( b2gDevBatch* b, const d_levelPlan& L, int kind )
{
	if ( L.recCount[kind] == 0 ) return 0;
	k_batched<Args, Body, MinBlocks><<<L.blocks[kind], B2G_THREADS, 0, b->stream>>>(
		(const d_batchRec*)( b->dBlob + L.recs[kind] ), (int)L.recCount[kind], b->dBlob );
	b->launches += 1;
	return (int)cudaGetLastError();
}

struct d_flushCtx
{
	b2gDevBatch* b;
	b2gDeviceWorld* const* worlds;
	d_worldFlush* plan;
	d_levelPlan* levels;
	int count;
};

static bool d_isCopy( int kind ) { return kind != D_OP_KERNEL; }

/* pass 1, per world: units and download layout */
static void d_planWorld( void* ctx, int w )
{
	const d_flushCtx* c = (const d_flushCtx*)ctx;
	d_worldFlush& P = c->plan[w];
	P.unitEnd.clear();
	P.downBytes = 0;
	const d_deferred* d = c->worlds[w]->defer;
	if ( d == NULL ) return;
	int count = (int)d->ops.size();
	P.downAt.assign( (size_t)count, -1 );
	for ( int i = 0; i < count; )
	{
		int k = d->ops[i].kind;
		int j = i + 1;
		if ( k == D_OP_H2D || k == D_OP_D2H )
			while ( j < count && d->ops[j].kind == k ) ++j;
		P.unitEnd.push_back( j );
		i = j;
	}
	for ( int i = 0; i < count; ++i )
	{
		if ( d->ops[i].kind != D_OP_D2H ) continue;
		P.downAt[i] = P.downBytes;
		P.downBytes = d_alignArgs( P.downBytes + d->ops[i].bytes );
	}
	P.slot.assign( P.unitEnd.size(), 0 );
	P.blockBase.assign( P.unitEnd.size(), 0 );
}

/* layout, per level: the level's table sizes and every world's slot in them */
static void d_layoutLevel( void* ctx, int l )
{
	const d_flushCtx* c = (const d_flushCtx*)ctx;
	d_levelPlan& L = c->levels[l];
	for ( int w = 0; w < c->count; ++w )
	{
		const d_deferred* d = c->worlds[w]->defer;
		d_worldFlush& P = c->plan[w];
		if ( d == NULL || (size_t)l >= P.unitEnd.size() ) continue;
		int begin = l > 0 ? P.unitEnd[(size_t)l - 1] : 0;
		const d_deferredOp& op = d->ops[(size_t)begin];
		if ( d_isCopy( op.kind ) )
		{
			P.slot[(size_t)l] = L.copyCount;
			L.copyCount += P.unitEnd[(size_t)l] - begin;
		}
		else if ( op.kernel == DK_SOLVE_BIN )
		{
			P.slot[(size_t)l] = L.recCount[DK_SOLVE_BIN]++;
			L.smem = op.smem > L.smem ? op.smem : L.smem;
		}
		else
		{
			P.slot[(size_t)l] = L.recCount[op.kernel]++;
			P.blockBase[(size_t)l] = L.blocks[op.kernel];
			L.blocks[op.kernel] += op.grid;
		}
	}
}

/* pass 2, per world: upload bytes and kernel arguments into the pinned staging, and the
   world's entries of every level's copy and record tables */
static void d_stageWorld( void* ctx, int w )
{
	const d_flushCtx* c = (const d_flushCtx*)ctx;
	const d_worldFlush& P = c->plan[w];
	const d_deferred* d = c->worlds[w]->defer;
	if ( d == NULL ) return;
	unsigned char* h = c->b->hBlob;
	if ( d->up.size() > 0 ) memcpy( h + P.upBase, d->up.data(), d->up.size() );
	if ( d->args.size() > 0 ) memcpy( h + P.argBase, d->args.data(), d->args.size() );
	int begin = 0;
	for ( size_t l = 0; l < P.unitEnd.size(); ++l )
	{
		const d_levelPlan& L = c->levels[l];
		int end = P.unitEnd[l];
		if ( d_isCopy( d->ops[begin].kind ) )
		{
			d_copyOp* table = (d_copyOp*)( h + L.copies ) + P.slot[l];
			for ( int i = begin; i < end; ++i )
			{
				const d_deferredOp& op = d->ops[(size_t)i];
				d_copyOp cp;
				cp.value = -1;
				cp.fromStaging = 0;
				cp.bytes = op.bytes;
				if ( op.kind == D_OP_H2D )
				{
					cp.dst = (unsigned char*)op.dev;
					cp.src = (const unsigned char*)(uintptr_t)( P.upBase + op.at );
					cp.fromStaging = 1;
				}
				else if ( op.kind == D_OP_D2D )
				{
					cp.dst = (unsigned char*)op.dev;
					cp.src = (const unsigned char*)op.host;
				}
				else if ( op.kind == D_OP_D2H )
				{
					cp.dst = c->b->dDown + P.downBase + P.downAt[(size_t)i];
					cp.src = (const unsigned char*)op.dev;
				}
				else
				{
					cp.dst = (unsigned char*)op.dev;
					cp.src = NULL;
					cp.value = op.value & 0xff;
				}
				table[i - begin] = cp;
			}
		}
		else
		{
			const d_deferredOp& op = d->ops[(size_t)begin];
			if ( op.kernel == DK_SOLVE_BIN )
			{
				( (long long*)( h + L.recs[DK_SOLVE_BIN] ) )[P.slot[l]] = P.argBase + op.at;
			}
			else
			{
				d_batchRec r;
				r.args = P.argBase + op.at;
				r.blockBase = P.blockBase[l];
				r.blocks = op.grid;
				( (d_batchRec*)( h + L.recs[op.kernel] ) )[P.slot[l]] = r;
			}
		}
		begin = end;
	}
}

/* world w's downloads to where its records asked, then its records are spent */
static void d_deliverWorld( void* ctx, int w )
{
	const d_flushCtx* c = (const d_flushCtx*)ctx;
	b2gDeviceWorld* dw = c->worlds[w];
	d_deferred* d = dw->defer;
	if ( d == NULL ) return;
	const d_worldFlush& P = c->plan[w];
	for ( size_t i = 0; i < d->ops.size(); ++i )
		if ( d->ops[i].kind == D_OP_D2H )
			memcpy( d->ops[i].host, c->b->hDown + P.downBase + P.downAt[i], (size_t)d->ops[i].bytes );
	d->ops.clear();
	d->up.clear();
	d->args.clear();
	dw->upUsed = 0;
}

static void d_serialFor( void* pool, int count, void ( *fn )( void*, int ), void* ctx )
{
	(void)pool;
	for ( int i = 0; i < count; ++i ) fn( ctx, i );
}

/* replay the recorded work of `n` worlds: every world's records run in order; records of
   different worlds at the same position run in one launch per kind. One upload, one
   download and one wait in all. `pf` runs the per-world planning, staging and delivery on
   the caller's threads (NULL: serially); only the table layout is serial. */
extern "C" int b2gDev_BatchFlush( b2gDevBatch* b, b2gDeviceWorld* const* worlds, int n, b2gParallelFor pf, void* pool )
{
	if ( pf == NULL ) pf = d_serialFor;
	double t0 = d_nowMs();
	if ( b->plans.size() < (size_t)n ) b->plans.resize( (size_t)n );
	d_worldFlush* plan = b->plans.data();
	d_flushCtx fc = { b, worlds, plan, NULL, n };
	pf( pool, n, d_planWorld, &fc );
	double tPlan = d_nowMs();
	b->partMs[0] += tPlan - t0;
	/* staging layout: every world's upload bytes and kernel arguments, then the tables;
	   download layout */
	size_t levels = 0;
	long long at = 0, down = 0;
	for ( int w = 0; w < n; ++w )
	{
		const d_deferred* d = worlds[w]->defer;
		d_worldFlush& P = plan[w];
		P.upBase = P.argBase = P.downBase = 0;
		if ( d == NULL ) continue;
		levels = P.unitEnd.size() > levels ? P.unitEnd.size() : levels;
		P.upBase = at;
		at = d_alignArgs( at + (long long)d->up.size() );
		P.argBase = at;
		at = d_alignArgs( at + (long long)d->args.size() );
		P.downBase = down;
		down += P.downBytes;
	}
	if ( levels == 0 ) return 0;
	const long long tableBase = at;
	CK2( d_reserve( &b->hDown, &b->dDown, &b->downCap, down > 0 ? down : 16 ) );
	/* each world's place in every level's tables, in world order (kernel records stay
	   sorted by their first block); the levels are independent, one task each */
	std::vector<d_levelPlan> plans( levels );
	for ( size_t l = 0; l < levels; ++l ) memset( &plans[l], 0, sizeof( d_levelPlan ) );
	fc.levels = plans.data();
	fc.count = n;
	pf( pool, (int)levels, d_layoutLevel, &fc );
	long long total = tableBase;
	for ( size_t l = 0; l < levels; ++l )
	{
		d_levelPlan& L = plans[l];
		L.copies = total;
		total = d_alignArgs( total + L.copyCount * (long long)sizeof( d_copyOp ) );
		for ( int k = 0; k < DK_COUNT; ++k )
		{
			L.recs[k] = total;
			long long entry = k == DK_SOLVE_BIN ? (long long)sizeof( long long ) : (long long)sizeof( d_batchRec );
			total = d_alignArgs( total + L.recCount[k] * entry );
		}
	}
	CK2( d_reserve( &b->hBlob, &b->dBlob, &b->blobCap, total ) );
	double tLayout = d_nowMs();
	b->partMs[1] += tLayout - tPlan;
	pf( pool, n, d_stageWorld, &fc );
	double t1 = d_nowMs();
	b->partMs[2] += t1 - tLayout;
	b->assembleMs += t1 - t0;
	CK( cudaMemcpyAsync( b->dBlob, b->hBlob, (size_t)total, cudaMemcpyHostToDevice, b->stream ) );
	for ( size_t l = 0; l < levels; ++l )
	{
		const d_levelPlan& L = plans[l];
		if ( L.copyCount > 0 )
		{
			k_batchCopy<<<(int)L.copyCount, 256, 0, b->stream>>>( (const d_copyOp*)( b->dBlob + L.copies ), (int)L.copyCount,
																  b->dBlob );
			b->launches += 1;
			CK( cudaGetLastError() );
		}
		CK2( ( d_launchBatched<d_markMovedArgs, b_markMoved, 1>( b, L, DK_MARK_MOVED ) ) );
		CK2( ( d_launchBatched<d_findPairsArgs, b_findPairs, 1>( b, L, DK_FIND_PAIRS ) ) );
		CK2( ( d_launchBatched<d_pairSetArgs, b_pairSetRebuild, 1>( b, L, DK_PAIR_SET ) ) );
		CK2( ( d_launchBatched<d_convertTreeArgs, b_convertTree, 1>( b, L, DK_CONVERT_TREE ) ) );
		CK2( ( d_launchBatched<d_contactListArgs, b_initContacts, 1>( b, L, DK_INIT_CONTACTS ) ) );
		CK2( ( d_launchBatched<d_contactListArgs, b_killContacts, 1>( b, L, DK_KILL_CONTACTS ) ) );
		CK2( ( d_launchBatched<d_collideArgs, b_collide, 1>( b, L, DK_COLLIDE ) ) );
		CK2( ( d_launchBatched<d_finalizeArgs, b_finalize, 8>( b, L, DK_FINALIZE ) ) );
		CK2( ( d_launchBatched<d_captureArgs, b_capture, 1>( b, L, DK_CAPTURE ) ) );
		CK2( ( d_launchBatched<d_islandOpArgs, b_islandOp, 1>( b, L, DK_ISLAND_OP ) ) );
		if ( L.recCount[DK_SOLVE_BIN] > 0 )
		{
			CK2( b2gDev_SolveWorldBinBatch( (const long long*)( b->dBlob + L.recs[DK_SOLVE_BIN] ), b->dBlob, (int)L.recCount[DK_SOLVE_BIN],
											L.smem, b->stream ) );
			b->launches += 1;
		}
	}
	if ( down > 0 ) CK( cudaMemcpyAsync( b->hDown, b->dDown, (size_t)down, cudaMemcpyDeviceToHost, b->stream ) );
	double tIssue = d_nowMs();
	b->partMs[3] += tIssue - t1;
	CK( cudaStreamSynchronize( b->stream ) );
	double tWait = d_nowMs();
	b->waitMs += tWait - t1;
	pf( pool, n, d_deliverWorld, &fc );
	b->partMs[4] += d_nowMs() - tWait;
	for ( int w = 0; w < n; ++w )
	{
		b2gDeviceWorld* dw = worlds[w];
		for ( void* r : dw->retired ) cudaFree( r );
		dw->retired.clear();
	}
	return 0;
}

extern "C" long long b2gDev_BatchLaunches( b2gDevBatch* b ) { return b->launches; }
