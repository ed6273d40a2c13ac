/*
 * Cluster solver for large components: one thread-block cluster (16 CTAs where the GPU
 * allows it, else 8) runs the whole Soft Step of solver.c:1010-1198 -- prepare, every
 * substep's integrate velocities / warm start / solve / integrate positions / relax per
 * color, restitution, store -- in one launch. Each color's constraints are split evenly
 * over the CTAs; a CTA keeps its contact constraints in its own shared memory for the whole
 * step; body state stays in global memory (L2). Colors are separated by the hardware
 * cluster barrier, whose release/acquire semantics order the global body-state writes of
 * one color before the reads of the next.
 *
 * This file is compiled with -Xptxas -dlcm=cg: global loads bypass L1, so body state
 * written by one SM is read from L2 by the others after a barrier.
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
	const b2gCompSummary* summary;
	int bodyCount;
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
	const int ranks = (int)cluster.num_blocks();
	extern __shared__ float4 s_mem[];
	b2gContactLane* lanes = (b2gContactLane*)s_mem;
	__shared__ int s_cBegin[B2_GRAPH_COLOR_COUNT], s_cCount[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_jBegin[B2_GRAPH_COLOR_COUNT], s_jCount[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_laneOffset[B2_GRAPH_COLOR_COUNT];
	const int tid = threadIdx.x, nt = blockDim.x;
	const b2gStepParams& P = a.p;
	const int overflowBegin = a.colorOffsets[B2G_OVERFLOW_INDEX];

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
	__syncthreads();

	/* prepare: joints in place (global), contacts into this CTA's shared memory */
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		int color = plan.colors[k];
		for ( int t = tid; t < s_jCount[k]; t += nt )
		{
			int idx = plan.jointOffsets[color] + s_jBegin[k] + t;
			d_prepareJointItem( a, jb, plan.useLists ? plan.jointList[idx] : idx );
		}
		for ( int t = tid; t < s_cCount[k]; t += nt )
		{
			int idx = a.colorOffsets[color] + s_cBegin[k] + t;
			d_prepareContactLane( a, plan.useLists ? plan.slotList[idx] : idx, overflowBegin, lanes + s_laneOffset[k] + t );
		}
	}
	cluster.sync();

	const int gtid = rank * nt + tid, gstride = ranks * nt;
	for ( int sub = 0; sub < P.subStepCount; ++sub )
	{
		for ( int i = gtid; i < plan.bodyCount; i += gstride )
			d_integrateVelocitiesItem( a, plan.bodyList ? plan.bodyList[i] : i );
		cluster.sync();
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int i = gtid; i < plan.bodyCount; i += gstride )
					d_integratePositionsItem( a, plan.bodyList ? plan.bodyList[i] : i );
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
						d_jointStage( P, a.joints + ( plan.useLists ? plan.jointList[idx] : idx ), a.sv, a.sd, stage );
					}
					else
					{
						d_laneStage( P, lanes + s_laneOffset[k] + ( t - nj ), a.sv, a.sd, stage );
					}
				}
				cluster.sync();
			}
		}
	}
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		for ( int t = tid; t < s_cCount[k]; t += nt )
			d_laneStage( P, lanes + s_laneOffset[k] + t, a.sv, a.sd, STAGE_RESTITUTION );
		cluster.sync();
	}

	/* store impulses (contact_solver.c:2238-2331) */
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		int color = plan.colors[k];
		for ( int t = tid; t < s_cCount[k]; t += nt )
		{
			int idx = a.colorOffsets[color] + s_cBegin[k] + t;
			int slot = plan.useLists ? plan.slotList[idx] : idx;
			d_storeLane( lanes + s_laneOffset[k] + t, &a.contacts[a.colorIds[slot]].manifold, false );
		}
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
	size_t smem = clusterSmem( counts, activeColorCount, ranks );
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
	plan.summary = b->summary;
	plan.bodyCount = bodyCount;

	cudaLaunchConfig_t cfg;
	memset( &cfg, 0, sizeof( cfg ) );
	cudaLaunchAttribute attr;
	attr.id = cudaLaunchAttributeClusterDimension;
	attr.val.clusterDim.x = ranks;
	attr.val.clusterDim.y = 1;
	attr.val.clusterDim.z = 1;
	cfg.gridDim = dim3( ranks );
	cfg.blockDim = dim3( B2G_CLUSTER_THREADS );
	cfg.dynamicSmemBytes = smem > 0 ? smem : 16;
	cfg.stream = stream;
	cfg.attrs = &attr;
	cfg.numAttrs = 1;
	cudaError_t e = cudaLaunchKernelEx( &cfg, k_solveCluster, *a, *jb, plan );
	*launches += 1;
	return (int)e;
}
