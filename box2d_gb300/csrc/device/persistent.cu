/*
 * Persistent Soft Step solver: one cooperative launch per step runs every solver stage of
 * the reference's b2SolverTask (solver.c:1010-1198) -- prepare, then per substep integrate
 * velocities, warm start / solve per color, integrate positions, relax per color, then
 * restitution, impulse storage and body finalization -- with a grid-wide barrier between
 * dependent phases instead of a kernel boundary.
 *
 * The grid is sized to the co-resident capacity of the GPU (152 SMs x blocks per SM), so
 * every block is resident and the barrier cannot wait on an unscheduled block. Each
 * barrier spin is bounded: after B2G_BARRIER_SPIN_LIMIT polls the block records
 * B2G_PERSISTENT_TIMEOUT in the error word and the whole grid leaves at the next barrier.
 *
 * This file is compiled with -Xptxas -dlcm=cg: global loads bypass L1, so body states and
 * constraint slots written by one SM are read fresh from L2 by another after a barrier.
 */
#include "stages.cuh"

#include <cuda_runtime.h>

#define B2G_BARRIER_SPIN_LIMIT ( 1u << 22 )

#include <stdlib.h>

struct d_colorRange
{
	int jointBegin, jointCount, laneBegin, laneCount;
};

struct d_persistentPlan
{
	int activeColorCount;
	d_colorRange colors[B2_GRAPH_COLOR_COUNT];
	int ovJointBegin, ovJointCount, ovLaneBegin, ovLaneCount;
	int total, jointTotal, awakeCount, substeps;
	d_jointBodies jb;
	unsigned int* barrier; /* [0] arrivals, [1] generation */
	unsigned int spinLimit; /* polls before a barrier gives up */
	int* error;
	int* anyRestitution;
};

enum
{
	B2G_PERSISTENT_TIMEOUT = 4,
};

/* grid barrier: one arrival per block on an L2 counter, the last arrival bumps the
   generation; the others poll the generation with a bounded spin. Returns false when the
   grid must stop (a timeout anywhere). */
static __device__ bool d_gridBarrier( const d_persistentPlan& plan )
{
	__syncthreads();
	__shared__ int s_stop;
	if ( threadIdx.x == 0 )
	{
		volatile unsigned int* gen = plan.barrier + 1;
		unsigned int myGen = *gen;
		__threadfence();
		unsigned int arrived = atomicAdd( plan.barrier, 1u );
		if ( arrived == gridDim.x - 1 )
		{
			atomicExch( plan.barrier, 0u );
			__threadfence();
			atomicAdd( plan.barrier + 1, 1u );
		}
		else
		{
			unsigned int polls = 0;
			while ( *gen == myGen )
			{
				if ( ++polls > plan.spinLimit )
				{
					atomicOr( plan.error, B2G_PERSISTENT_TIMEOUT );
					break;
				}
				__nanosleep( 32 );
			}
		}
		__threadfence();
		s_stop = *(volatile int*)plan.error != 0;
	}
	__syncthreads();
	return s_stop == 0;
}

__global__ void __launch_bounds__( 256, 2 ) k_solvePersistent( d_solveArgs a, d_finalizeArgs f, d_persistentPlan plan )
{
	const int stride = gridDim.x * blockDim.x;
	const int tid = blockIdx.x * blockDim.x + threadIdx.x;
	const int overflowBegin = plan.ovLaneBegin;

	/* prepare joints and contacts (joint.c:1593-1629, contact_solver.c:1573-1809, :20-160) */
	for ( int i = tid; i < plan.jointTotal; i += stride ) d_prepareJointItem( a, plan.jb, i );
	for ( int s = tid; s < plan.total; s += stride )
	{
		d_prepareContactSlot( a, s, overflowBegin );
		if ( a.contacts[a.colorIds[s]].restitution != 0.0f ) atomicOr( plan.anyRestitution, 1 );
	}
	if ( d_gridBarrier( plan ) == false ) return;
	const bool hasOverflow = plan.ovJointCount + plan.ovLaneCount > 0;
	const bool restitution = *(volatile int*)plan.anyRestitution != 0;

	for ( int sub = 0; sub < plan.substeps; ++sub )
	{
		for ( int i = tid; i < plan.awakeCount; i += stride ) d_integrateVelocitiesItem( a, i );
		if ( d_gridBarrier( plan ) == false ) return;
		for ( int stage = STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int i = tid; i < plan.awakeCount; i += stride ) d_integratePositionsItem( a, i );
				if ( d_gridBarrier( plan ) == false ) return;
			}
			if ( hasOverflow )
			{
				if ( tid == 0 )
					d_overflowStageAll( a, plan.ovJointBegin, plan.ovJointCount, plan.ovLaneBegin, plan.ovLaneCount, stage );
				if ( d_gridBarrier( plan ) == false ) return;
			}
			for ( int k = 0; k < plan.activeColorCount; ++k )
			{
				const d_colorRange r = plan.colors[k];
				const int n = r.jointCount + r.laneCount;
				for ( int i = tid; i < n; i += stride )
					d_colorStageItem( a, r.jointBegin, r.jointCount, r.laneBegin, r.laneCount, stage, i );
				if ( d_gridBarrier( plan ) == false ) return;
			}
		}
	}

	if ( restitution )
	{
		if ( hasOverflow )
		{
			if ( tid == 0 )
				d_overflowStageAll( a, plan.ovJointBegin, plan.ovJointCount, plan.ovLaneBegin, plan.ovLaneCount,
									STAGE_RESTITUTION );
			if ( d_gridBarrier( plan ) == false ) return;
		}
		for ( int k = 0; k < plan.activeColorCount; ++k )
		{
			const d_colorRange r = plan.colors[k];
			for ( int i = tid; i < r.laneCount; i += stride )
				d_colorStageItem( a, 0, 0, r.laneBegin, r.laneCount, STAGE_RESTITUTION, i );
			if ( d_gridBarrier( plan ) == false ) return;
		}
	}

	/* store impulses and finalize bodies touch disjoint data: one phase */
	for ( int s = tid; s < plan.total; s += stride ) d_storeSlot( a, s, overflowBegin );
	for ( int i = tid; i < f.awakeCount; i += stride ) d_finalizeBody( f, i );
}

/* launch one persistent solver pass on `stream`; colors as (jointBegin, jointCount,
   laneBegin, laneCount) per active color. Returns a CUDA error code. */
extern "C" int b2gDev_LaunchPersistent( const d_solveArgs* a, const d_finalizeArgs* f, const int* colorRanges,
										 int activeColorCount, const int* overflowRange, int total, int jointTotal,
										 int awakeCount, int substeps, const d_jointBodies* jb, unsigned int* barrier,
										 int* error, int* anyRestitution, cudaStream_t stream )
{
	static int s_blocksPerSM = -1, s_numSMs = 0;
	if ( s_blocksPerSM < 0 )
	{
		int dev = 0;
		cudaGetDevice( &dev );
		cudaDeviceGetAttribute( &s_numSMs, cudaDevAttrMultiProcessorCount, dev );
		cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor( &s_blocksPerSM, k_solvePersistent, 256, 0 );
		if ( e != cudaSuccess ) return (int)e;
		if ( s_blocksPerSM > 2 ) s_blocksPerSM = 2;
	}
	d_persistentPlan plan;
	memset( &plan, 0, sizeof( plan ) );
	plan.activeColorCount = activeColorCount;
	for ( int k = 0; k < activeColorCount; ++k )
	{
		plan.colors[k].jointBegin = colorRanges[4 * k];
		plan.colors[k].jointCount = colorRanges[4 * k + 1];
		plan.colors[k].laneBegin = colorRanges[4 * k + 2];
		plan.colors[k].laneCount = colorRanges[4 * k + 3];
	}
	plan.ovJointBegin = overflowRange[0];
	plan.ovJointCount = overflowRange[1];
	plan.ovLaneBegin = overflowRange[2];
	plan.ovLaneCount = overflowRange[3];
	plan.total = total;
	plan.jointTotal = jointTotal;
	plan.awakeCount = awakeCount;
	plan.substeps = substeps;
	plan.jb = *jb;
	plan.barrier = barrier;
	/* B2G_PERSISTENT_SPIN_LIMIT shortens the barrier's patience, so that a test can make a
	   barrier give up and check the reported status */
	plan.spinLimit = B2G_BARRIER_SPIN_LIMIT;
	{
		const char* limit = getenv( "B2G_PERSISTENT_SPIN_LIMIT" );
		if ( limit != NULL && atoi( limit ) > 0 ) plan.spinLimit = (unsigned int)atoi( limit );
	}
	plan.error = error;
	plan.anyRestitution = anyRestitution;
	int maxWork = total > awakeCount ? total : awakeCount;
	if ( jointTotal > maxWork ) maxWork = jointTotal;
	int wanted = ( maxWork + 255 ) / 256;
	int grid = s_numSMs * s_blocksPerSM;
	if ( wanted < grid ) grid = wanted > 0 ? wanted : 1;
	d_solveArgs aa = *a;
	d_finalizeArgs ff = *f;
	void* args[] = { &aa, &ff, &plan };
	cudaError_t e = cudaMemsetAsync( barrier, 0, 2 * sizeof( unsigned int ), stream );
	if ( e == cudaSuccess ) e = cudaMemsetAsync( anyRestitution, 0, sizeof( int ), stream );
	if ( e == cudaSuccess ) e = cudaLaunchCooperativeKernel( (void*)k_solvePersistent, dim3( grid ), dim3( 256 ), args, 0, stream );
	return (int)e;
}
