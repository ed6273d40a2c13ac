/*
 * Cluster solver for large components: one thread-block cluster (16 CTAs where the GPU
 * allows it, else 8) runs the whole Soft Step of solver.c:1010-1198 -- prepare, every
 * substep's integrate velocities / warm start / solve / integrate positions / relax per
 * color, restitution, store -- in one launch. Each color's constraints are split evenly
 * over the CTAs; a CTA keeps its contact constraints in its own shared memory for the whole
 * step. The body state lives in the cluster's distributed shared memory: body position p
 * (its index in the solved body list) sits in CTA p % ranks, slot p / ranks, and every
 * constraint reads and writes it there through the cluster's shared-memory window. Colors
 * are separated by the hardware cluster barrier, whose release/acquire semantics order the
 * body-state writes of one color before the reads of the next. Joints stay in global
 * memory; each joint is always processed by the same thread.
 *
 * This file is compiled with -Xptxas -dlcm=cg: global loads bypass L1.
 *
 * Used when the component path leaves constraints in components too big for a bin, no
 * overflow color exists and the constraints fit the cluster's shared memory; the results
 * equal the per-color launch path bit for bit (same stage functions, same order).
 */
#include "components.cuh"

#include <cooperative_groups.h>
#include <pthread.h>
#include <string.h>

namespace cg = cooperative_groups;

#define B2G_CLUSTER_THREADS 512
#define B2G_CLUSTER_SMEM_MAX ( 220 * 1024 )

struct d_clusterPlan
{
	int colorCount;
	int colors[B2_GRAPH_COLOR_COUNT];
	int jointOffsets[B2_GRAPH_COLOR_COUNT + 1];
	int useLists; /* constraints from the big-component lists (counts on the device) */
	const int* slotList;
	const int* jointList;
	const int* bodyList; /* NULL: all awake bodies */
	const int* positionOf; /* awake index -> position in bodyList (lists only) */
	const b2gCompSummary* summary;
	int bodyCount;
	int rankShift; /* ranks = 1 << rankShift */
	int slotsPerRank;
};

/* body state in distributed shared memory: position p -> CTA p & mask, slot p >> shift */
struct d_clusterBodies
{
	float4* sv;
	float4* sd;
	int shift, mask;
	__device__ __forceinline__ float4& v( int i ) const
	{
		return *cg::this_cluster().map_shared_rank( sv + ( i >> shift ), (unsigned)( i & mask ) );
	}
	__device__ __forceinline__ float4& d( int i ) const
	{
		return *cg::this_cluster().map_shared_rank( sd + ( i >> shift ), (unsigned)( i & mask ) );
	}
};

static __device__ __forceinline__ int d_planContactCount( const d_solveArgs& a, const d_clusterPlan& plan, int color )
{
	return plan.useLists ? plan.summary->bigContactCount[color] : a.colorOffsets[color + 1] - a.colorOffsets[color];
}

static __device__ __forceinline__ int d_planJointCount( const d_clusterPlan& plan, int color )
{
	return plan.useLists ? plan.summary->bigJointCount[color] : plan.jointOffsets[color + 1] - plan.jointOffsets[color];
}

__global__ void __launch_bounds__( B2G_CLUSTER_THREADS ) k_solveCluster( d_solveArgs a, d_jointBodies jb, d_clusterPlan plan )
{
	cg::cluster_group cluster = cg::this_cluster();
	const int rank = (int)cluster.block_rank();
	const int ranks = 1 << plan.rankShift;
	const int mask = ranks - 1;
	extern __shared__ float4 s_mem[];
	float4* sv = s_mem;
	float4* sd = sv + plan.slotsPerRank;
	b2gContactLane* lanes = (b2gContactLane*)( sd + plan.slotsPerRank );
	__shared__ int s_cBegin[B2_GRAPH_COLOR_COUNT], s_cCount[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_jBegin[B2_GRAPH_COLOR_COUNT], s_jCount[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_laneOffset[B2_GRAPH_COLOR_COUNT];
	const int tid = threadIdx.x, nt = blockDim.x;
	const b2gStepParams& P = a.p;
	const int overflowBegin = a.colorOffsets[B2G_OVERFLOW_INDEX];
	d_clusterBodies bodies = { sv, sd, plan.rankShift, mask };
	/* this CTA's bodies: positions rank, rank + ranks, ... */
	const int localCount = plan.bodyCount > rank ? ( plan.bodyCount - rank + ranks - 1 ) >> plan.rankShift : 0;

	/* this CTA's share of every color */
	if ( tid == 0 )
	{
		int offset = 0;
		for ( int k = 0; k < plan.colorCount; ++k )
		{
			int color = plan.colors[k];
			int nc = d_planContactCount( a, plan, color ), nj = d_planJointCount( plan, color );
			int cb = (int)( ( (long long)nc * rank ) / ranks ), ce = (int)( ( (long long)nc * ( rank + 1 ) ) / ranks );
			int jb0 = (int)( ( (long long)nj * rank ) / ranks ), je = (int)( ( (long long)nj * ( rank + 1 ) ) / ranks );
			s_cBegin[k] = cb;
			s_cCount[k] = ce - cb;
			s_jBegin[k] = jb0;
			s_jCount[k] = je - jb0;
			s_laneOffset[k] = offset;
			offset += ce - cb;
		}
	}
	for ( int s = tid; s < localCount; s += nt )
	{
		int p = ( s << plan.rankShift ) + rank;
		int ai = plan.bodyList ? plan.bodyList[p] : p;
		sv[s] = a.sv[ai];
		sd[s] = a.sd[ai];
	}
	__syncthreads();

	/* prepare: joints in place (global), contacts into this CTA's shared memory; body
	   references become positions */
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		int color = plan.colors[k];
		for ( int t = tid; t < s_jCount[k]; t += nt )
		{
			int idx = plan.jointOffsets[color] + s_jBegin[k] + t;
			b2gJoint* J = a.joints + ( plan.useLists ? plan.jointList[idx] : idx );
			d_prepareJoint( J, &jb, P.h, P.inv_h, P.enableWarmStarting != 0 );
			if ( plan.positionOf )
			{
				J->indexA = J->indexA >= 0 ? plan.positionOf[J->indexA] : -1;
				J->indexB = J->indexB >= 0 ? plan.positionOf[J->indexB] : -1;
			}
		}
		for ( int t = tid; t < s_cCount[k]; t += nt )
		{
			int idx = a.colorOffsets[color] + s_cBegin[k] + t;
			b2gContactLane* L = lanes + s_laneOffset[k] + t;
			d_prepareContactLane( a, plan.useLists ? plan.slotList[idx] : idx, overflowBegin, L );
			if ( plan.positionOf )
			{
				L->indexA = L->indexA != 0 ? plan.positionOf[L->indexA - 1] + 1 : 0;
				L->indexB = L->indexB != 0 ? plan.positionOf[L->indexB - 1] + 1 : 0;
			}
		}
	}
	cluster.sync();

	for ( int sub = 0; sub < P.subStepCount; ++sub )
	{
		for ( int s = tid; s < localCount; s += nt )
		{
			int p = ( s << plan.rankShift ) + rank;
			int ai = plan.bodyList ? plan.bodyList[p] : p;
			d_integrateVelocitiesState( P, sv, s, a.params + 8 * ai );
		}
		cluster.sync();
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int s = tid; s < localCount; s += nt ) d_integratePositionsState( P, sv, sd, s );
				cluster.sync();
			}
			for ( int k = 0; k < plan.colorCount; ++k )
			{
				int color = plan.colors[k];
				int nj = s_jCount[k], n = nj + s_cCount[k];
				for ( int t = tid; t < n; t += nt )
				{
					if ( t < nj )
					{
						int idx = plan.jointOffsets[color] + s_jBegin[k] + t;
						d_jointStageT( P, a.joints + ( plan.useLists ? plan.jointList[idx] : idx ), bodies, stage );
					}
					else
					{
						d_laneStageT( P, lanes + s_laneOffset[k] + ( t - nj ), bodies, stage );
					}
				}
				cluster.sync();
			}
		}
	}
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		for ( int t = tid; t < s_cCount[k]; t += nt )
			d_laneStageT( P, lanes + s_laneOffset[k] + t, bodies, STAGE_RESTITUTION );
		cluster.sync();
	}

	/* store impulses (contact_solver.c:2238-2331), restore joint body indices, write the
	   bodies back; no CTA touches another's shared memory after the last barrier */
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		int color = plan.colors[k];
		for ( int t = tid; t < s_cCount[k]; t += nt )
		{
			int idx = a.colorOffsets[color] + s_cBegin[k] + t;
			int slot = plan.useLists ? plan.slotList[idx] : idx;
			d_storeLane( lanes + s_laneOffset[k] + t, &a.contacts[a.colorIds[slot]].manifold, false );
		}
		if ( plan.positionOf )
		{
			for ( int t = tid; t < s_jCount[k]; t += nt )
			{
				int idx = plan.jointOffsets[color] + s_jBegin[k] + t;
				b2gJoint* J = a.joints + plan.jointList[idx];
				J->indexA = J->indexA >= 0 ? plan.bodyList[J->indexA] : -1;
				J->indexB = J->indexB >= 0 ? plan.bodyList[J->indexB] : -1;
			}
		}
	}
	for ( int s = tid; s < localCount; s += nt )
	{
		int p = ( s << plan.rankShift ) + rank;
		int ai = plan.bodyList ? plan.bodyList[p] : p;
		a.sv[ai] = sv[s];
		a.sd[ai] = sd[s];
	}
}

/* shared memory one CTA needs for its share of `counts` contacts per color */
static size_t clusterSmem( const int* contactCounts, int colorCount, int ranks )
{
	size_t lanes = 0;
	for ( int k = 0; k < colorCount; ++k ) lanes += (size_t)( contactCounts[k] + ranks - 1 ) / ranks;
	return lanes * sizeof( b2gContactLane );
}

/* Launch the cluster solver over the active colors. useLists selects the big-component
   lists of `b` (and its big body list); otherwise every constraint and awake body. Returns
   0 when launched, -1 when the constraints do not fit a cluster (the caller then uses the
   per-color launches), or a CUDA error code. */
extern "C" int b2gDev_ClusterSolve( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									const int* activeColors, int activeColorCount, int useLists, int bodyCount,
									cudaStream_t stream, long long* launches )
{
	static pthread_mutex_t s_lock = PTHREAD_MUTEX_INITIALIZER;
	static int s_ranks = -1;
	pthread_mutex_lock( &s_lock );
	if ( s_ranks < 0 )
	{
		s_ranks = 0;
		if ( cudaFuncSetAttribute( k_solveCluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 ) != cudaSuccess ||
			 cudaFuncSetAttribute( k_solveCluster, cudaFuncAttributeMaxDynamicSharedMemorySize, B2G_CLUSTER_SMEM_MAX ) !=
				 cudaSuccess )
		{
			cudaGetLastError();
			pthread_mutex_unlock( &s_lock );
			return -1;
		}
		for ( int ranks = 16; ranks >= 8 && s_ranks == 0; ranks /= 2 )
		{
			cudaLaunchConfig_t cfg;
			memset( &cfg, 0, sizeof( cfg ) );
			cudaLaunchAttribute attr;
			attr.id = cudaLaunchAttributeClusterDimension;
			attr.val.clusterDim.x = ranks;
			attr.val.clusterDim.y = 1;
			attr.val.clusterDim.z = 1;
			cfg.gridDim = dim3( ranks );
			cfg.blockDim = dim3( B2G_CLUSTER_THREADS );
			cfg.dynamicSmemBytes = B2G_CLUSTER_SMEM_MAX;
			cfg.attrs = &attr;
			cfg.numAttrs = 1;
			int clusters = 0;
			if ( cudaOccupancyMaxActiveClusters( &clusters, k_solveCluster, &cfg ) == cudaSuccess && clusters > 0 ) s_ranks = ranks;
			cudaGetLastError();
		}
	}
	int ranks = s_ranks;
	pthread_mutex_unlock( &s_lock );
	if ( ranks == 0 ) return -1;
	int counts[B2_GRAPH_COLOR_COUNT];
	for ( int k = 0; k < activeColorCount; ++k )
		counts[k] = useLists ? b->hSummary->bigContactCount[activeColors[k]]
							 : a->colorOffsets[activeColors[k] + 1] - a->colorOffsets[activeColors[k]];
	int rankShift = ranks == 16 ? 4 : 3;
	int slotsPerRank = ( bodyCount + ranks - 1 ) / ranks;
	size_t smem = clusterSmem( counts, activeColorCount, ranks ) + (size_t)slotsPerRank * 2 * sizeof( float4 );
	if ( smem > B2G_CLUSTER_SMEM_MAX ) return -1;
	d_clusterPlan plan;
	memset( &plan, 0, sizeof( plan ) );
	plan.colorCount = activeColorCount;
	for ( int k = 0; k < activeColorCount; ++k ) plan.colors[k] = activeColors[k];
	memcpy( plan.jointOffsets, jointOffsets, sizeof( plan.jointOffsets ) );
	plan.useLists = useLists;
	plan.slotList = useLists ? b->bigSlotList : NULL;
	plan.jointList = useLists ? b->bigJointList : NULL;
	plan.bodyList = useLists ? b->bigBodyList : NULL;
	plan.positionOf = useLists ? b->localIndex : NULL;
	plan.summary = b->summary;
	plan.bodyCount = bodyCount;
	plan.rankShift = rankShift;
	plan.slotsPerRank = slotsPerRank;

	/* threads per CTA: the largest per-CTA share of one color (joints + contacts), rounded to
	   warps, so a color phase is one pass and no more warps than needed meet at each barrier */
	int share = 1;
	for ( int k = 0; k < activeColorCount; ++k )
	{
		int color = activeColors[k];
		int joints = useLists ? b->hSummary->bigJointCount[color] : jointOffsets[color + 1] - jointOffsets[color];
		int items = ( joints + ranks - 1 ) / ranks + ( counts[k] + ranks - 1 ) / ranks;
		if ( items > share ) share = items;
	}
	int threads = ( ( share + 31 ) / 32 ) * 32;
	if ( threads < 128 ) threads = 128;
	if ( threads > B2G_CLUSTER_THREADS ) threads = B2G_CLUSTER_THREADS;

	cudaLaunchConfig_t cfg;
	memset( &cfg, 0, sizeof( cfg ) );
	cudaLaunchAttribute attr;
	attr.id = cudaLaunchAttributeClusterDimension;
	attr.val.clusterDim.x = ranks;
	attr.val.clusterDim.y = 1;
	attr.val.clusterDim.z = 1;
	cfg.gridDim = dim3( ranks );
	cfg.blockDim = dim3( threads );
	cfg.dynamicSmemBytes = smem > 0 ? smem : 16;
	cfg.stream = stream;
	cfg.attrs = &attr;
	cfg.numAttrs = 1;
	cudaError_t e = cudaLaunchKernelEx( &cfg, k_solveCluster, *a, *jb, plan );
	*launches += 1;
	return (int)e;
}
