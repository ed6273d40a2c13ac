/*
 * Component solver interface between world.cu and components.cu.
 *
 * The awake constraint graph splits into connected components over non-static bodies
 * (two bodies are connected when a colored contact or joint links them). Components share
 * no body that the solver writes, so each can run the whole Soft Step -- prepare, every
 * substep's integrate / warm start / solve / relax per color, restitution, store -- on its
 * own, in the reference's color order restricted to its constraints. Because the
 * constraints of one color touch disjoint bodies, the results are bit-identical to the
 * global color sweep of solver.c:1010-1198.
 *
 * Small components are packed into bins; one CTA solves a bin out of shared memory with
 * __syncthreads between colors. Components too large for a bin keep the global per-color
 * path, driven by per-color lists of their constraints.
 */
#pragma once

#include "stages.cuh"

#include <cuda_runtime.h>

/* shared-memory bytes a body, a contact and a joint occupy in a bin */
#define B2G_BIN_BODY_BYTES 32
#define B2G_BIN_CONTACT_BYTES ( (int)sizeof( b2gContactLane ) + 4 )
#define B2G_BIN_JOINT_BYTES ( (int)sizeof( b2gJoint ) + 4 )
/* a component heavier than the bin cap is solved on the global path; a bin holds less than
   twice it. The cap is B2G_BIN_CAP_BYTES unless B2G_BIN_CAP_KB (16 to 100) overrides it. */
#define B2G_BIN_CAP_BYTES ( 40 * 1024 )
extern "C" int b2gBinCapBytes( void );
/* a whole world up to this weight is solved by one CTA without component analysis */
#define B2G_WORLD_BIN_MAX_BYTES ( 200 * 1024 )
/* field widths of the packed (bodies, contacts, joints) allocation cursor */
#define B2G_CURSOR_BODY_BITS 21
#define B2G_CURSOR_CONTACT_BITS 22
#define B2G_CURSOR_JOINT_BITS 21

/* device-written summary of one component analysis, read by the host */
struct b2gCompSummary
{
	unsigned long long cursor; /* packed totals of the small components */
	int bigBodies;			   /* bodies in big components */
	int bigBodyCount;		   /* fill counters of the big lists (written after the analysis) */
	int smallComponents, bigComponents;
	int bigContactCount[B2_GRAPH_COLOR_COUNT];
	int bigJointCount[B2_GRAPH_COLOR_COUNT];
};

/* scratch buffers, grown on demand; sized by awake bodies, contact slots, joints, bins */
struct b2gCompBuffers
{
	int awakeCap, slotCap, jointCap, binCap;
	int* parent;	 /* union-find forest, then the root of each awake body */
	int* compData;	 /* per root: counts (3), offsets (3), fill (3), bin */
	int* bodyList;	 /* small components' bodies, component-contiguous */
	int* localIndex; /* awake index -> index within its bin */
	int* slotList;	 /* small components' contact slots */
	int* jointList;	 /* small components' joint indices */
	int* binRange;	 /* per bin: begin bodies/contacts/joints (min), end (max) */
	int* bigBodyList;
	int* bigSlotList;  /* per color, at the color's slot offset */
	int* bigJointList; /* per color, at the color's joint offset */
	b2gCompSummary* summary;
	b2gCompSummary* hSummary; /* pinned */
	/* sizes of the last analysis */
	int n, total, jointTotal;
	const int* awakeIndex;
	/* cluster solver: per color and CTA, the contact slots the CTA solves (16 times the
	   colored slots), the counters that assign them, an error word */
	int* clusterAssigned;
	long long clusterCap;
	int* clusterJoints; /* the same for joints (16 times the colored joints) */
	long long clusterJointCap;
	/* what the lists were assigned for: the caller's epoch and the launch shape */
	long long clusterEpoch;
	int clusterUseLists, clusterBodyCount, clusterThreads, clusterRanks;
	int* clusterCounts;
	/* the roots of the awake bodies over joints alone (every body points at its root), kept
	   while the joints and the awake set are unchanged (jointEpoch) */
	int* jointForest;
	int jointForestCap, jointForestN, jointForestJoints;
	long long jointForestEpoch;
	/* roots computed right after the narrowphase from the contacts it left touching, for
	   the next analysis when the awake set and the joints are still those (earlyEpoch) */
	int earlyValid, earlyN, earlyJoints;
	long long earlyEpoch;
};

extern "C" int b2gDev_CompReserve( b2gCompBuffers* b, int awake, int slots, int joints );
extern "C" void b2gDev_CompFree( b2gCompBuffers* b );

/* find components, pack the small ones into bins and build the component-contiguous and
   big-component lists; waits for the summary. forceBig puts every component on the
   global path (an overflow color exists). `jointEpoch` changes whenever the joints or the
   awake set change (-1: unknown): the joints' part of the union-find is kept while it
   stays the same. */
extern "C" int b2gDev_CompAnalyze( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const int* awakeIndex,
								   int total, int jointTotal, int forceBig, long long jointEpoch, cudaStream_t stream,
								   long long* launches );

/* the union-find and roots of the next analysis, issued straight after the narrowphase:
   the unions of every live, awake contact the narrowphase left touching (a superset of the
   colored contacts the solver will see, unless the contact-state pass wakes bodies, which
   changes jointEpoch) over the kept joint forest; the analysis then starts from these
   roots when n, jointTotal and jointEpoch match */
extern "C" int b2gDev_CompUnionEarly( b2gCompBuffers* b, const b2gContact* contacts, int capacity, const b2gJoint* joints,
									  const int* awakeIndex, int n, int jointTotal, long long jointEpoch, cudaStream_t stream,
									  long long* launches );

/* solve every bin (small components) */
extern "C" int b2gDev_CompSolveBins( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets,
									 const d_jointBodies* jb, b2gStepCounters* counters, cudaStream_t stream,
									 long long* launches );

/* global per-color path over the big components' constraints */
extern "C" int b2gDev_CompSolveBig( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									const int* activeColors, int activeColorCount, int total, int jointTotal,
									cudaStream_t stream, long long* launches );

/* cluster solver (cluster.cu) over every constraint (useLists = 0) or the big-component
   lists; 0 = launched, -1 = does not fit a cluster, else a CUDA error. `epoch` changes
   whenever colors, joints, the awake set or the component lists change (-1: unknown); the
   assignment of constraints to the cluster's CTAs is reused while it stays the same.
   startFlag (a word of mapped host memory, or NULL) is set to startToken once the cluster
   is resident on the GPU. */
extern "C" int b2gDev_ClusterSolve( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									const int* activeColors, int activeColorCount, int useLists, int bodyCount, int* status,
									long long epoch, int* startFlag, int startToken, cudaStream_t stream,
									long long* launches );

/* the arguments of the one-CTA world solve, for a batched launch (out may be NULL to get
   the size), and the batched launch itself: CTA r solves the world whose arguments are at
   args + offsets[r] */
extern "C" int b2gDev_SolveWorldBinArgs( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
										 const int* awakeIndex, int bytes, b2gStepCounters* counters, void* out, int* outBytes );
extern "C" int b2gDev_SolveWorldBinBatch( const long long* offsets, const unsigned char* args, int count, int smemBytes,
										  cudaStream_t stream );

/* one CTA solves the whole world (bytes = its shared-memory weight, at most
   B2G_WORLD_BIN_MAX_BYTES); no analysis, no lists */
extern "C" int b2gDev_SolveWorldBin( b2gCompBuffers* b, const d_solveArgs* a, const int* jointOffsets, const d_jointBodies* jb,
									 const int* awakeIndex, int bytes, b2gStepCounters* counters, cudaStream_t stream,
									 long long* launches );
