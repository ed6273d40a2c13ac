/*
 * Cluster solver for large components: one thread-block cluster (16 CTAs where the GPU
 * allows it, else 8) runs the whole Soft Step of solver.c:1010-1198 -- prepare, every
 * substep's integrate velocities / warm start / solve / integrate positions / relax per
 * color, restitution, store -- in one launch. Each color's constraints are split evenly
 * over the CTAs; a CTA keeps its contact constraints in its own shared memory for the whole
 * step. The body state lives in the cluster's distributed shared memory: body position p
 * (its index in the solved body list) sits in CTA p / slotsPerRank, slot p % slotsPerRank,
 * and every constraint reads and writes it there through the cluster's shared-memory window.
 * Colors are separated by the hardware cluster barrier, whose release/acquire semantics
 * order the body-state writes of one color before the reads of the next. Joints stay in
 * global memory; each joint is always processed by the same thread. In a cluster without
 * joints the warm start runs per body, right after the body's integrate velocities, which
 * takes the warm-start colors' barriers out of every substep.
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
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

namespace cg = cooperative_groups;

#define B2G_CLUSTER_THREADS 512
#define B2G_CLUSTER_SMEM_MAX ( 220 * 1024 )
#define B2G_CLUSTER_MAX_RANKS 16
/* clusterCounts, by [k * 16 + rank] for active color k: the contact lanes claimed from a
   CTA and given to it, the joints claimed and given; then per CTA the lanes claimed over all
   colors */
#define B2G_CLUSTER_CLAIMS 0
#define B2G_CLUSTER_FILLS ( B2_GRAPH_COLOR_COUNT * B2G_CLUSTER_MAX_RANKS )
#define B2G_CLUSTER_JCLAIMS ( 2 * B2_GRAPH_COLOR_COUNT * B2G_CLUSTER_MAX_RANKS )
#define B2G_CLUSTER_JFILLS ( 3 * B2_GRAPH_COLOR_COUNT * B2G_CLUSTER_MAX_RANKS )
#define B2G_CLUSTER_TOTALS ( 4 * B2_GRAPH_COLOR_COUNT * B2G_CLUSTER_MAX_RANKS )
#define B2G_CLUSTER_COUNT_WORDS ( ( 4 * B2_GRAPH_COLOR_COUNT + 1 ) * B2G_CLUSTER_MAX_RANKS )

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
	int ranks;
	int slotsPerRank; /* bodies per CTA: position p lives in CTA p / slotsPerRank */
	int laneCap;	  /* contact lanes one CTA's shared memory holds */
	int jointSlotCap; /* joints whose accumulated impulses (s[]) a CTA keeps in shared memory */
	int colorCap[B2_GRAPH_COLOR_COUNT]; /* lanes of an active color a CTA takes in one pass */
	int bodyWarm;	/* warm start per body, fused with integrate velocities (contact-only clusters) */
	int entryBytes; /* bytes of the per-body warm-start entries in each CTA's shared memory */
	int jointConstants; /* plain revolute joints in slots read their constants from the slot */
	int jointCap[B2_GRAPH_COLOR_COUNT]; /* joints of an active color a CTA takes in one pass */
	int* assignedJoints;				/* color c, CTA r: joints at [jointOffset(c) * ranks + r * count(c)] */
	int* assigned;	  /* color c, CTA r: slots at assigned[offset(c) * ranks + r * count(c)] */
	int* counts;	  /* B2G_CLUSTER_COUNT_WORDS assignment counters */
	int* status;	  /* B2G_STATUS_CAPACITY if a CTA was given more lanes than it holds */
	int* startFlag;	  /* host-visible word set to startToken once the cluster runs (or NULL) */
	int startToken;
};

/* A body reference inside the cluster is (owning CTA << 16 | slot in that CTA). Positions
   are split in contiguous blocks, so bodies that touch each other -- neighbours in the
   awake order -- mostly share a CTA, and a contact is solved by the CTA that owns its first
   dynamic body: most body accesses stay in the CTA's own shared memory. */
static __device__ __forceinline__ int d_clusterKey( const d_clusterPlan& plan, int p )
{
	int r = p / plan.slotsPerRank;
	return ( r << 16 ) | ( p - r * plan.slotsPerRank );
}

static __device__ __forceinline__ int d_clusterPosition( const d_clusterPlan& plan, int key )
{
	return ( key >> 16 ) * plan.slotsPerRank + ( key & 0xffff );
}

/* body state in distributed shared memory, addressed by cluster key */
struct d_clusterBodies
{
	float4* sv;
	float4* sd;
	__device__ __forceinline__ float4& v( int key ) const
	{
		return *cg::this_cluster().map_shared_rank( sv + ( key & 0xffff ), (unsigned)( key >> 16 ) );
	}
	__device__ __forceinline__ float4& d( int key ) const
	{
		return *cg::this_cluster().map_shared_rank( sd + ( key & 0xffff ), (unsigned)( key >> 16 ) );
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

/* one claim on CTA r for active color k: a lane slot within the color's one-pass share
   (unless `anyShare`) and within the CTA's shared memory */
static __device__ __forceinline__ bool d_clusterClaim( const d_clusterPlan& plan, int k, int r, bool anyShare )
{
	if ( anyShare == false && atomicAdd( plan.counts + B2G_CLUSTER_CLAIMS + k * B2G_CLUSTER_MAX_RANKS + r, 1 ) >= plan.colorCap[k] )
		return false;
	return atomicAdd( plan.counts + B2G_CLUSTER_TOTALS + r, 1 ) < plan.laneCap;
}

/* Give each contact of the solve to the CTA owning its first dynamic body, else to the
   owner of the other body, else to the next CTA with room: a CTA takes at most one pass of
   lanes per color while another has room, and never more lanes than its shared memory
   holds (the host checks that all lanes fit the cluster). Grid: x over a color's contacts,
   y over the active colors. Within a color the order of the lanes does not matter: they
   touch disjoint bodies. */
static __device__ void d_clusterAssignJoint( const d_clusterPlan& plan, const b2gJoint* joints, int k, int i );

__global__ void k_clusterAssign( d_solveArgs a, d_clusterPlan plan )
{
	const int k = blockIdx.y;
	const int color = plan.colors[k];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( blockIdx.z == 1 )
	{
		if ( i < d_planJointCount( plan, color ) ) d_clusterAssignJoint( plan, a.joints, k, i );
		return;
	}
	if ( i >= d_planContactCount( a, plan, color ) ) return;
	const int begin = a.colorOffsets[color], colorSize = a.colorOffsets[color + 1] - begin;
	const int slot = plan.useLists ? plan.slotList[begin + i] : begin + i;
	const b2gContact* cs = a.contacts + a.colorIds[slot];
	int owners[2] = { -1, -1 };
	int bodies[2] = { cs->bodySimIndexA, cs->bodySimIndexB };
	for ( int j = 0; j < 2; ++j )
	{
		if ( bodies[j] < 0 ) continue;
		int p = plan.positionOf ? plan.positionOf[bodies[j]] : bodies[j];
		owners[j] = min( p / plan.slotsPerRank, plan.ranks - 1 );
	}
	if ( owners[0] < 0 ) owners[0] = owners[1] >= 0 ? owners[1] : 0;
	int r = -1;
	if ( d_clusterClaim( plan, k, owners[0], false ) ) r = owners[0];
	else if ( owners[1] >= 0 && owners[1] != owners[0] && d_clusterClaim( plan, k, owners[1], false ) ) r = owners[1];
	for ( int pass = 0; pass < 2 && r < 0; ++pass )
	{
		for ( int j = 1; j <= plan.ranks && r < 0; ++j )
		{
			int c = owners[0] + j < plan.ranks ? owners[0] + j : owners[0] + j - plan.ranks;
			if ( d_clusterClaim( plan, k, c, pass == 1 ) ) r = c;
		}
	}
	if ( r < 0 )
	{
		atomicExch( plan.status, B2G_STATUS_CAPACITY );
		return;
	}
	int idx = atomicAdd( plan.counts + B2G_CLUSTER_FILLS + k * B2G_CLUSTER_MAX_RANKS + r, 1 );
	plan.assigned[(long long)begin * plan.ranks + (long long)r * colorSize + idx] = slot;
}

/* joints likewise, without a shared-memory limit (joints stay in global memory) */
static __device__ void d_clusterAssignJoint( const d_clusterPlan& plan, const b2gJoint* joints, int k, int i )
{
	const int color = plan.colors[k];
	const int begin = plan.jointOffsets[color], colorSize = plan.jointOffsets[color + 1] - begin;
	const int index = plan.useLists ? plan.jointList[begin + i] : begin + i;
	const b2gJoint* J = joints + index;
	int bodies[2] = { J->indexA, J->indexB };
	int owners[2] = { -1, -1 };
	for ( int j = 0; j < 2; ++j )
	{
		if ( bodies[j] < 0 ) continue;
		int p = plan.positionOf ? plan.positionOf[bodies[j]] : bodies[j];
		owners[j] = min( p / plan.slotsPerRank, plan.ranks - 1 );
	}
	if ( owners[0] < 0 ) owners[0] = owners[1] >= 0 ? owners[1] : 0;
	int* claims = plan.counts + B2G_CLUSTER_JCLAIMS + k * B2G_CLUSTER_MAX_RANKS;
	int r = -1;
	if ( atomicAdd( claims + owners[0], 1 ) < plan.jointCap[k] ) r = owners[0];
	else if ( owners[1] >= 0 && owners[1] != owners[0] && atomicAdd( claims + owners[1], 1 ) < plan.jointCap[k] ) r = owners[1];
	for ( int j = 1; j <= plan.ranks && r < 0; ++j )
	{
		int c = owners[0] + j < plan.ranks ? owners[0] + j : owners[0] + j - plan.ranks;
		if ( atomicAdd( claims + c, 1 ) < plan.jointCap[k] ) r = c;
	}
	if ( r < 0 ) r = owners[0]; /* every CTA has its one-pass share: the owner loops */
	int idx = atomicAdd( plan.counts + B2G_CLUSTER_JFILLS + k * B2G_CLUSTER_MAX_RANKS + r, 1 );
	plan.assignedJoints[(long long)begin * plan.ranks + (long long)r * colorSize + idx] = index;
}

/* A joint record held in registers between its load and its stage. */
union d_jointCopy
{
	b2gJoint j;
	float4 w[sizeof( b2gJoint ) / 16];
};

/* A joint slot in a CTA's shared memory is 8 float4: the joint's s[] (accumulated impulses
   and solver constants), then the constants a plain revolute joint (no spring, motor or
   limit) reads in its warm start and solve, written at prepare:
     [4] indexA, indexB (cluster keys, as int bits), invMassA, invMassB
     [5] invIA, invIB, frameA.p
     [6] frameB.p, deltaCenter
     [7] softBias, softMass, softImpulse, 1 (plain revolute) or 0 (any other joint) */
#define B2G_JOINT_SLOT_FLOAT4 8

static __device__ __forceinline__ void d_clusterJointConstants( const b2gJoint* J, float4* slot, bool allow )
{
	bool plain = allow && J->type == b2_revoluteJoint && J->enableSpring == 0 && J->enableMotor == 0 && J->enableLimit == 0;
	slot[4] = make_float4( __int_as_float( J->indexA ), __int_as_float( J->indexB ), J->invMassA, J->invMassB );
	slot[5] = make_float4( J->invIA, J->invIB, J->frameA.p.x, J->frameA.p.y );
	slot[6] = make_float4( J->frameB.p.x, J->frameB.p.y, J->deltaCenter.x, J->deltaCenter.y );
	slot[7] = make_float4( J->softBias, J->softMass, J->softImpulse, __int_as_float( plain ? 1 : 0 ) );
}

/* Load a joint for a stage: the accumulated impulses and solver constants (s[]) from the
   CTA's shared-memory slot when it has one, else from the record; a plain revolute joint's
   constants from the slot too (revolute_joint.c:283-500 read nothing else with spring,
   motor and limit off: the frames' rotations only feed the spring and the limit), any
   other joint's constant part from global memory. */
static __device__ __forceinline__ void d_clusterJointLoad( const b2gJoint* J, const float4* slot, d_jointCopy& copy )
{
	const float4* src = (const float4*)J;
	const int sBegin = (int)( offsetof( b2gJoint, s ) / 16 );
	if ( slot != nullptr && __float_as_int( slot[7].w ) == 1 )
	{
		const float4 c0 = slot[4], c1 = slot[5], c2 = slot[6], c3 = slot[7];
		b2gJoint& j = copy.j;
		j.type = b2_revoluteJoint;
		j.indexA = __float_as_int( c0.x );
		j.indexB = __float_as_int( c0.y );
		j.invMassA = c0.z;
		j.invMassB = c0.w;
		j.invIA = c1.x;
		j.invIB = c1.y;
		j.frameA.p = b2Vec2{ c1.z, c1.w };
		j.frameA.q = b2Rot{ 1.0f, 0.0f };
		j.frameB.p = b2Vec2{ c2.x, c2.y };
		j.frameB.q = b2Rot{ 1.0f, 0.0f };
		j.deltaCenter = b2Vec2{ c2.z, c2.w };
		j.softBias = c3.x;
		j.softMass = c3.y;
		j.softImpulse = c3.z;
		j.enableSpring = 0;
		j.enableMotor = 0;
		j.enableLimit = 0;
#pragma unroll
		for ( int i = 0; i < 4; ++i ) copy.w[sBegin + i] = slot[i];
		return;
	}
#pragma unroll
	for ( int i = 0; i < (int)( sizeof( b2gJoint ) / 16 ); ++i )
		if ( slot == nullptr || i < sBegin || i >= sBegin + 4 ) copy.w[i] = __ldcg( src + i );
	if ( slot != nullptr )
	{
#pragma unroll
		for ( int i = 0; i < 4; ++i ) copy.w[sBegin + i] = slot[i];
	}
}

/* Run a stage on a loaded joint and keep its s[]: in the shared-memory slot (no global store
   in the phase, so the cluster barrier that ends it waits for no store to reach L2), or
   back in the record. */
static __device__ __forceinline__ void d_clusterJointRun( const b2gStepParams& P, b2gJoint* J, float4* slot, d_jointCopy& copy,
														  d_clusterBodies& bodies, int stage )
{
	const int sBegin = (int)( offsetof( b2gJoint, s ) / 16 );
	d_jointStageT( P, &copy.j, bodies, stage );
	float4* dst = slot != nullptr ? slot : (float4*)J->s;
#pragma unroll
	for ( int i = 0; i < 4; ++i ) dst[i] = copy.w[sBegin + i];
}

/* Warm start as seen by one body (contact_solver.c:1811-1871 read per body): a dynamic
   body is in at most one constraint per graph color (constraint_graph.c:84-130), and a
   lane's warm start changes each of its bodies from that body's own velocity and the
   lane's stored impulses only. So applying the body's lanes in color order, with the
   operations of d_warmStartLane for its side, gives its velocity after the warm-start
   colors bit for bit, with no barrier between colors. ent[k] is the body's lane of active
   color k: (lane index in its CTA << 6) | (32 if the body is side B) | CTA rank, or -1. */
static __device__ __forceinline__ void d_clusterWarmBody( float4* sv, int s, const int* ent, int colorCount,
														  const b2gContactLane* lanes )
{
	float4 v = sv[s];
	if ( ( __float_as_uint( v.w ) & B2G_DYNAMIC_FLAG ) == 0 ) return;
	float vx = v.x, vy = v.y, w = v.z;
	for ( int k = 0; k < colorCount; ++k )
	{
		const int e = ent[k];
		if ( e < 0 ) continue;
		const b2gContactLane* c = cg::this_cluster().map_shared_rank( lanes + ( e >> 6 ), (unsigned)( e & 31 ) );
		const float nx = c->normal.x, ny = c->normal.y;
		const float tangentX = ny;
		const float tangentY = 0.0f - nx;
		const float ni1 = c->normalImpulse1, ti1 = c->tangentImpulse1;
		const float ni2 = c->normalImpulse2, ti2 = c->tangentImpulse2;
		const float roll = c->rollingImpulse;
		const float Px1 = ni1 * nx + ti1 * tangentX, Py1 = ni1 * ny + ti1 * tangentY;
		const float Px2 = ni2 * nx + ti2 * tangentX, Py2 = ni2 * ny + ti2 * tangentY;
		if ( ( e & 32 ) == 0 )
		{
			const float invM = c->invMassA, invI = c->invIA;
			const b2Vec2 r1 = c->anchorA1, r2 = c->anchorA2;
			w = w - invI * ( r1.x * Py1 - r1.y * Px1 );
			vx = vx - invM * Px1;
			vy = vy - invM * Py1;
			w = w - invI * ( r2.x * Py2 - r2.y * Px2 );
			vx = vx - invM * Px2;
			vy = vy - invM * Py2;
			w = w - invI * roll;
		}
		else
		{
			const float invM = c->invMassB, invI = c->invIB;
			const b2Vec2 r1 = c->anchorB1, r2 = c->anchorB2;
			w = w + invI * ( r1.x * Py1 - r1.y * Px1 );
			vx = vx + invM * Px1;
			vy = vy + invM * Py1;
			w = w + invI * ( r2.x * Py2 - r2.y * Px2 );
			vx = vx + invM * Px2;
			vy = vy + invM * Py2;
			w = w + invI * roll;
		}
	}
	sv[s] = make_float4( vx, vy, w, v.w );
}

__global__ void __maxnreg__( 128 ) k_solveCluster( d_solveArgs a, d_jointBodies jb, d_clusterPlan plan )
{
	cg::cluster_group cluster = cg::this_cluster();
	const int rank = (int)cluster.block_rank();
	const int ranks = plan.ranks;
	extern __shared__ float4 s_mem[];
	float4* sv = s_mem;
	float4* sd = sv + plan.slotsPerRank;
	float4* jimp = sd + plan.slotsPerRank; /* B2G_JOINT_SLOT_FLOAT4 per joint slot */
	int* entries = (int*)( jimp + B2G_JOINT_SLOT_FLOAT4 * plan.jointSlotCap ); /* [slot * colorCount + k] when bodyWarm */
	b2gContactLane* lanes = (b2gContactLane*)( (char*)entries + plan.entryBytes );
	__shared__ int s_cCount[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_jBegin[B2_GRAPH_COLOR_COUNT], s_jCount[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_jSlot[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_laneOffset[B2_GRAPH_COLOR_COUNT];
	__shared__ int s_restitution;
	const int tid = threadIdx.x, nt = blockDim.x;
	const b2gStepParams& P = a.p;
	/* the cluster is resident: the host may now start other work beside it on the GPU */
	if ( plan.startFlag != nullptr && rank == 0 && tid == 0 )
	{
		*(volatile int*)plan.startFlag = plan.startToken;
		__threadfence_system();
	}
	const int overflowBegin = a.colorOffsets[B2G_OVERFLOW_INDEX];
	d_clusterBodies bodies = { sv, sd };
	/* this CTA's bodies: positions [base, base + localCount) */
	const int base = rank * plan.slotsPerRank;
	const int localCount = max( 0, min( plan.slotsPerRank, plan.bodyCount - base ) );

	/* this CTA's lanes and joints of every color; s_jBegin is where the CTA's joint list of
	   the color starts */
	if ( tid == 0 )
	{
		int offset = 0, jslot = 0;
		for ( int k = 0; k < plan.colorCount; ++k )
		{
			int color = plan.colors[k];
			int nc = plan.counts[B2G_CLUSTER_FILLS + k * B2G_CLUSTER_MAX_RANKS + rank];
			if ( offset + nc > plan.laneCap )
			{
				atomicExch( plan.status, B2G_STATUS_CAPACITY );
				nc = max( 0, plan.laneCap - offset );
			}
			int nj = plan.counts[B2G_CLUSTER_JFILLS + k * B2G_CLUSTER_MAX_RANKS + rank];
			int jbegin = plan.jointOffsets[color];
			s_cCount[k] = nc;
			s_jBegin[k] = jbegin * ranks + rank * ( plan.jointOffsets[color + 1] - jbegin );
			s_jCount[k] = nj;
			s_jSlot[k] = jslot;
			jslot += nj;
			s_laneOffset[k] = offset;
			offset += nc;
		}
		s_restitution = 0;
	}
	for ( int s = tid; s < localCount; s += nt )
	{
		int p = base + s;
		int ai = plan.bodyList ? plan.bodyList[p] : p;
		sv[s] = a.sv[ai];
		sd[s] = a.sd[ai];
	}
	if ( plan.bodyWarm )
	{
		/* every CTA's entries are empty before any lane registers with its bodies */
		for ( int i = tid; i < plan.slotsPerRank * plan.colorCount; i += nt ) entries[i] = -1;
		cluster.sync();
	}
	else
	{
		__syncthreads();
	}

	/* prepare: joints in place (global), contacts into this CTA's shared memory; body
	   references become cluster keys */
	int restitution = 0;
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		int color = plan.colors[k];
		for ( int t = tid; t < s_jCount[k]; t += nt )
		{
			b2gJoint* J = a.joints + plan.assignedJoints[s_jBegin[k] + t];
			d_prepareJoint( J, &jb, P.h, P.inv_h, P.enableWarmStarting != 0 );
			int pa = J->indexA >= 0 ? ( plan.positionOf ? plan.positionOf[J->indexA] : J->indexA ) : -1;
			int pb = J->indexB >= 0 ? ( plan.positionOf ? plan.positionOf[J->indexB] : J->indexB ) : -1;
			J->indexA = pa >= 0 ? d_clusterKey( plan, pa ) : -1;
			J->indexB = pb >= 0 ? d_clusterKey( plan, pb ) : -1;
			int slot = s_jSlot[k] + t;
			if ( slot < plan.jointSlotCap )
			{
				const float4* s4 = (const float4*)J->s;
				float4* js = jimp + B2G_JOINT_SLOT_FLOAT4 * slot;
#pragma unroll
				for ( int i = 0; i < 4; ++i ) js[i] = s4[i];
				d_clusterJointConstants( J, js, plan.jointConstants != 0 );
			}
		}
		const int begin = a.colorOffsets[color];
		const int* mine = plan.assigned + (long long)begin * ranks + (long long)rank * ( a.colorOffsets[color + 1] - begin );
		for ( int t = tid; t < s_cCount[k]; t += nt )
		{
			b2gContactLane* L = lanes + s_laneOffset[k] + t;
			d_prepareContactLane( a, mine[t], overflowBegin, L );
			int pa = L->indexA != 0 ? ( plan.positionOf ? plan.positionOf[L->indexA - 1] : L->indexA - 1 ) : -1;
			int pb = L->indexB != 0 ? ( plan.positionOf ? plan.positionOf[L->indexB - 1] : L->indexB - 1 ) : -1;
			L->indexA = pa >= 0 ? d_clusterKey( plan, pa ) + 1 : 0;
			L->indexB = pb >= 0 ? d_clusterKey( plan, pb ) + 1 : 0;
			restitution |= L->groupFlags & 2;
			if ( plan.bodyWarm )
			{
				/* register the lane with its bodies (kinematic bodies may take several lanes of
				   a color; their entries are never read) */
				const int ref = ( ( s_laneOffset[k] + t ) << 6 ) | rank;
				if ( pa >= 0 )
				{
					int key = L->indexA - 1;
					*cluster.map_shared_rank( entries + ( key & 0xffff ) * plan.colorCount + k, (unsigned)( key >> 16 ) ) = ref;
				}
				if ( pb >= 0 )
				{
					int key = L->indexB - 1;
					*cluster.map_shared_rank( entries + ( key & 0xffff ) * plan.colorCount + k, (unsigned)( key >> 16 ) ) = ref | 32;
				}
			}
		}
	}
	if ( restitution ) s_restitution = 1;
	cluster.sync();
	/* the restitution stage only changes lanes whose 4-wide group has restitution
	   (contact_solver.c:2131); without any in the cluster its color phases are skipped */
	{
		int any = tid < ranks ? *cluster.map_shared_rank( &s_restitution, (unsigned)tid ) : 0;
		restitution = __syncthreads_or( any );
	}

	for ( int sub = 0; sub < P.subStepCount; ++sub )
	{
		for ( int s = tid; s < localCount; s += nt )
		{
			int p = base + s;
			int ai = plan.bodyList ? plan.bodyList[p] : p;
			d_integrateVelocitiesState( P, sv, s, a.params + 8 * ai );
			if ( plan.bodyWarm ) d_clusterWarmBody( sv, s, entries + s * plan.colorCount, plan.colorCount, lanes );
		}
		if ( plan.bodyWarm && plan.colorCount > 0 )
		{
			/* the lanes' own part of the warm start (contact_solver.c:1846,1858) */
			const int laneCount = s_laneOffset[plan.colorCount - 1] + s_cCount[plan.colorCount - 1];
			for ( int i = tid; i < laneCount; i += nt )
			{
				b2gContactLane* c = lanes + i;
				c->totalNormalImpulse1 = c->totalNormalImpulse1 + c->normalImpulse1;
				c->totalNormalImpulse2 = c->totalNormalImpulse2 + c->normalImpulse2;
			}
		}
		cluster.sync();
		for ( int stage = plan.bodyWarm ? STAGE_SOLVE : STAGE_WARM; stage <= STAGE_RELAX; ++stage )
		{
			if ( stage == STAGE_RELAX )
			{
				for ( int s = tid; s < localCount; s += nt ) d_integratePositionsState( P, sv, sd, s );
				cluster.sync();
			}
			/* a thread's first joint of the next color is loaded while the cluster barrier
			   ending the current color completes: arrive, load, wait. Safe because a color's
			   records change only in that color's phases, all before earlier barriers. */
			d_jointCopy next;
			bool haveNext = false;
			for ( int k = 0; k < plan.colorCount; ++k )
			{
				int nj = s_jCount[k], n = nj + s_cCount[k];
				for ( int t = tid; t < n; t += nt )
				{
					if ( t < nj )
					{
						int slot = s_jSlot[k] + t;
						b2gJoint* J = a.joints + plan.assignedJoints[s_jBegin[k] + t];
						float4* sp = slot < plan.jointSlotCap ? jimp + B2G_JOINT_SLOT_FLOAT4 * slot : nullptr;
						if ( t != tid || haveNext == false ) d_clusterJointLoad( J, sp, next );
						d_clusterJointRun( P, J, sp, next, bodies, stage );
					}
					else
					{
						d_laneStageT( P, lanes + s_laneOffset[k] + ( t - nj ), bodies, stage );
					}
				}
				auto token = cluster.barrier_arrive();
				haveNext = k + 1 < plan.colorCount && tid < s_jCount[k + 1];
				if ( haveNext )
				{
					int slot = s_jSlot[k + 1] + tid;
					const b2gJoint* J = a.joints + plan.assignedJoints[s_jBegin[k + 1] + tid];
					d_clusterJointLoad( J, slot < plan.jointSlotCap ? jimp + B2G_JOINT_SLOT_FLOAT4 * slot : nullptr, next );
				}
				cluster.barrier_wait( std::move( token ) );
			}
		}
	}
	if ( restitution )
	{
		for ( int k = 0; k < plan.colorCount; ++k )
		{
			for ( int t = tid; t < s_cCount[k]; t += nt )
				d_laneStageT( P, lanes + s_laneOffset[k] + t, bodies, STAGE_RESTITUTION );
			cluster.sync();
		}
	}

	/* store impulses (contact_solver.c:2238-2331), restore joint body indices, write the
	   bodies back; no CTA touches another's shared memory after the last barrier */
	for ( int k = 0; k < plan.colorCount; ++k )
	{
		int color = plan.colors[k];
		const int begin = a.colorOffsets[color];
		const int* mine = plan.assigned + (long long)begin * ranks + (long long)rank * ( a.colorOffsets[color + 1] - begin );
		for ( int t = tid; t < s_cCount[k]; t += nt )
			d_storeLane( lanes + s_laneOffset[k] + t, &a.contacts[a.colorIds[mine[t]]].manifold, false );
		for ( int t = tid; t < s_jCount[k]; t += nt )
		{
			b2gJoint* J = a.joints + plan.assignedJoints[s_jBegin[k] + t];
			int slot = s_jSlot[k] + t;
			if ( slot < plan.jointSlotCap )
			{
				float4* d4 = (float4*)J->s;
#pragma unroll
				for ( int i = 0; i < 4; ++i ) d4[i] = jimp[B2G_JOINT_SLOT_FLOAT4 * slot + i];
			}
			int pa = J->indexA >= 0 ? d_clusterPosition( plan, J->indexA ) : -1;
			int pb = J->indexB >= 0 ? d_clusterPosition( plan, J->indexB ) : -1;
			J->indexA = pa >= 0 ? ( plan.bodyList ? plan.bodyList[pa] : pa ) : -1;
			J->indexB = pb >= 0 ? ( plan.bodyList ? plan.bodyList[pb] : pb ) : -1;
		}
	}
	for ( int s = tid; s < localCount; s += nt )
	{
		int p = base + s;
		int ai = plan.bodyList ? plan.bodyList[p] : p;
		a.sv[ai] = sv[s];
		a.sd[ai] = sd[s];
	}
}

/* Launch the cluster solver over the active colors. useLists selects the big-component
   lists of `b` (and its big body list); otherwise every constraint and awake body. Returns
   0 when launched, -1 when the constraints do not fit a cluster (the caller then uses the
   per-color launches), or a CUDA error code. A CTA given more lanes than it holds (never
   expected: the host checks the total) sets B2G_STATUS_CAPACITY in *status. */
extern "C" int b2gDev_ClusterSolve( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									const int* activeColors, int activeColorCount, int useLists, int bodyCount, int* status,
									long long epoch, int* startFlag, int startToken, cudaStream_t stream, long long* launches )
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
		for ( int ranks = B2G_CLUSTER_MAX_RANKS; ranks >= 8 && s_ranks == 0; ranks /= 2 )
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
	if ( ranks == 0 || bodyCount <= 0 ) return -1;
	int counts[B2_GRAPH_COLOR_COUNT];
	long long lanesTotal = 0;
	for ( int k = 0; k < activeColorCount; ++k )
	{
		counts[k] = useLists ? b->hSummary->bigContactCount[activeColors[k]]
							 : a->colorOffsets[activeColors[k] + 1] - a->colorOffsets[activeColors[k]];
		lanesTotal += counts[k];
	}
	int slotsPerRank = ( bodyCount + ranks - 1 ) / ranks;
	long long bodyBytes = (long long)slotsPerRank * 2 * sizeof( float4 );
	if ( slotsPerRank > 0xffff || bodyBytes >= (long long)B2G_CLUSTER_SMEM_MAX ) return -1;
	/* joint impulses in shared memory: a CTA's even share of the joints with a quarter more,
	   as long as the contact lanes still fit; joints past the slots keep theirs in global */
	long long jointsTotal = 0;
	for ( int k = 0; k < activeColorCount; ++k )
	{
		int color = activeColors[k];
		jointsTotal += useLists ? b->hSummary->bigJointCount[color] : jointOffsets[color + 1] - jointOffsets[color];
	}
	const long long jointSlotBytes = B2G_JOINT_SLOT_FLOAT4 * (long long)sizeof( float4 );
	long long evenJoints = ( jointsTotal + ranks - 1 ) / ranks;
	int jointSlotCap = jointsTotal > 0 ? (int)( evenJoints + evenJoints / 4 + 32 ) : 0;
	/* without joints, the warm start runs per body with integrate velocities when the body
	   entries fit beside the lanes (B2G_CLUSTER_BODY_WARM=0 keeps the per-color warm start) */
	const char* bodyWarmEnv = getenv( "B2G_CLUSTER_BODY_WARM" );
	int bodyWarm = jointsTotal == 0 && activeColorCount > 0 && ( bodyWarmEnv == NULL || atoi( bodyWarmEnv ) != 0 );
	long long entryBytes = bodyWarm ? ( ( (long long)slotsPerRank * activeColorCount * (long long)sizeof( int ) + 15 ) / 16 ) * 16 : 0;
	/* joint slots take what the lanes leave: an even share of the lanes with an eighth more
	   stays for them, the rest of the shared memory holds as many joints as it can */
	if ( jointSlotCap > 0 )
	{
		long long laneNeed = ( lanesTotal + ranks - 1 ) / ranks;
		laneNeed += laneNeed / 8 + 8;
		long long room = (long long)B2G_CLUSTER_SMEM_MAX - bodyBytes - entryBytes - laneNeed * (long long)sizeof( b2gContactLane );
		long long fit = room > 0 ? room / jointSlotBytes : 0;
		if ( fit < jointSlotCap ) jointSlotCap = (int)fit;
	}
	int laneCap = 0;
	for ( ;; )
	{
		long long laneBytes = (long long)B2G_CLUSTER_SMEM_MAX - bodyBytes - (long long)jointSlotCap * jointSlotBytes - entryBytes;
		laneCap = laneBytes > 0 ? (int)( laneBytes / sizeof( b2gContactLane ) ) : 0;
		if ( lanesTotal <= (long long)laneCap * ranks ) break;
		if ( jointSlotCap > 0 )
			jointSlotCap = jointSlotCap > 64 ? jointSlotCap / 2 : 0;
		else if ( entryBytes > 0 )
			entryBytes = 0, bodyWarm = 0;
		else
			break;
	}
	if ( lanesTotal > (long long)laneCap * ranks ) return -1;

	/* assignment lists: 16 entries per colored slot and colored joint */
	long long need = (long long)B2G_CLUSTER_MAX_RANKS * ( a->colorOffsets[B2G_OVERFLOW_INDEX] > 0 ? a->colorOffsets[B2G_OVERFLOW_INDEX] : 1 );
	if ( need > b->clusterCap || b->clusterAssigned == NULL )
	{
		long long cap = b->clusterCap > 0 ? b->clusterCap : 1024;
		while ( cap < need ) cap *= 2;
		if ( b->clusterAssigned ) cudaFree( b->clusterAssigned );
		b->clusterAssigned = NULL;
		b->clusterEpoch = -1;
		b->clusterCap = 0;
		cudaError_t e = cudaMalloc( (void**)&b->clusterAssigned, (size_t)cap * sizeof( int ) );
		if ( e != cudaSuccess ) return (int)e;
		b->clusterCap = cap;
	}
	long long needJ = (long long)B2G_CLUSTER_MAX_RANKS * ( jointOffsets[B2G_OVERFLOW_INDEX] > 0 ? jointOffsets[B2G_OVERFLOW_INDEX] : 1 );
	if ( needJ > b->clusterJointCap || b->clusterJoints == NULL )
	{
		long long cap = b->clusterJointCap > 0 ? b->clusterJointCap : 1024;
		while ( cap < needJ ) cap *= 2;
		if ( b->clusterJoints ) cudaFree( b->clusterJoints );
		b->clusterJoints = NULL;
		b->clusterEpoch = -1;
		b->clusterJointCap = 0;
		cudaError_t e = cudaMalloc( (void**)&b->clusterJoints, (size_t)cap * sizeof( int ) );
		if ( e != cudaSuccess ) return (int)e;
		b->clusterJointCap = cap;
	}
	if ( b->clusterCounts == NULL )
	{
		cudaError_t e = cudaMalloc( (void**)&b->clusterCounts, B2G_CLUSTER_COUNT_WORDS * sizeof( int ) );
		if ( e != cudaSuccess ) return (int)e;
		b->clusterEpoch = -1;
	}

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
	plan.ranks = ranks;
	plan.slotsPerRank = slotsPerRank;
	plan.laneCap = laneCap;
	plan.jointSlotCap = jointSlotCap;
	plan.bodyWarm = bodyWarm;
	{
		/* B2G_CLUSTER_JOINT_CONSTANTS=0: every joint's constant part from global memory */
		const char* e = getenv( "B2G_CLUSTER_JOINT_CONSTANTS" );
		plan.jointConstants = e == NULL || atoi( e ) != 0;
	}
	plan.entryBytes = (int)entryBytes;
	plan.assigned = b->clusterAssigned;
	plan.counts = b->clusterCounts;
	plan.status = status;
	plan.startFlag = startFlag;
	plan.startToken = startToken;
	plan.assignedJoints = b->clusterJoints;

	/* threads per CTA: the even share of the largest color (joints + contacts) with a
	   quarter more for locality, rounded to warps; a color's constraints go to a CTA past its
	   one-pass share only when every CTA has its share */
	int share = 1, maxCount = 1;
	int jointCounts[B2_GRAPH_COLOR_COUNT];
	for ( int k = 0; k < activeColorCount; ++k )
	{
		int color = activeColors[k];
		jointCounts[k] = useLists ? b->hSummary->bigJointCount[color] : jointOffsets[color + 1] - jointOffsets[color];
		int evenC = ( counts[k] + ranks - 1 ) / ranks, evenJ = ( jointCounts[k] + ranks - 1 ) / ranks;
		int items = evenC + evenC / 4 + evenJ + evenJ / 4;
		if ( items > share ) share = items;
		int range = a->colorOffsets[color + 1] - a->colorOffsets[color];
		if ( range > maxCount ) maxCount = range;
		range = jointOffsets[color + 1] - jointOffsets[color];
		if ( range > maxCount ) maxCount = range;
	}
	int threads = ( ( share + 31 ) / 32 ) * 32;
	if ( threads < 128 ) threads = 128;
	if ( threads > B2G_CLUSTER_THREADS ) threads = B2G_CLUSTER_THREADS;
	for ( int k = 0; k < activeColorCount; ++k )
	{
		int evenC = ( counts[k] + ranks - 1 ) / ranks, evenJ = ( jointCounts[k] + ranks - 1 ) / ranks;
		plan.jointCap[k] = evenJ + evenJ / 4;
		plan.colorCap[k] = threads - plan.jointCap[k] > evenC + evenC / 4 ? threads - plan.jointCap[k] : evenC + evenC / 4;
		if ( evenC + evenJ > 0 && plan.colorCap[k] + plan.jointCap[k] > threads )
		{
			/* the color needs more than one pass anyway: shares in proportion */
			plan.colorCap[k] = evenC + (int)( (long long)( threads > evenC + evenJ ? threads - evenC - evenJ : 0 ) * evenC / ( evenC + evenJ ) );
			plan.jointCap[k] = evenJ + ( threads > evenC + evenJ ? threads - evenC - evenJ : 0 ) - ( plan.colorCap[k] - evenC );
		}
	}

	/* the assignment holds while the constraint graph, the awake set and the solved body
	   list are unchanged (the caller's epoch) and the launch shape is the same */
	bool reuse = epoch >= 0 && b->clusterEpoch == epoch && b->clusterUseLists == useLists && b->clusterBodyCount == bodyCount &&
				 b->clusterThreads == threads && b->clusterRanks == ranks;
	if ( reuse == false )
	{
		cudaError_t e = cudaMemsetAsync( b->clusterCounts, 0, B2G_CLUSTER_COUNT_WORDS * sizeof( int ), stream );
		if ( e != cudaSuccess ) return (int)e;
		dim3 grid( (unsigned)( ( maxCount + 255 ) / 256 ), (unsigned)activeColorCount, 2 );
		k_clusterAssign<<<grid, 256, 0, stream>>>( *a, plan );
		*launches += 1;
		e = cudaGetLastError();
		if ( e != cudaSuccess ) return (int)e;
		b->clusterEpoch = epoch;
		b->clusterUseLists = useLists;
		b->clusterBodyCount = bodyCount;
		b->clusterThreads = threads;
		b->clusterRanks = ranks;
	}

	cudaLaunchConfig_t cfg;
	memset( &cfg, 0, sizeof( cfg ) );
	cudaLaunchAttribute attr;
	attr.id = cudaLaunchAttributeClusterDimension;
	attr.val.clusterDim.x = ranks;
	attr.val.clusterDim.y = 1;
	attr.val.clusterDim.z = 1;
	cfg.gridDim = dim3( ranks );
	cfg.blockDim = dim3( threads );
	cfg.dynamicSmemBytes = B2G_CLUSTER_SMEM_MAX;
	cfg.stream = stream;
	cfg.attrs = &attr;
	cfg.numAttrs = 1;
	cudaError_t e = cudaLaunchKernelEx( &cfg, k_solveCluster, *a, *jb, plan );
	*launches += 1;
	return (int)e;
}
