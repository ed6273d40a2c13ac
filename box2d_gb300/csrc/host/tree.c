/*
 * Host broadphase tree of the GB300 step library. Its topology decides the order in
 * which the device pair query reports overlaps, so insertion with rotations
 * (dynamic_tree.c:149-643), enlarge (:798-837), the median-split partial rebuild
 * (:1430-1520, :1723-1996) and the node free list (:95-147) follow the reference exactly.
 * The nodes are mirrored to device memory for the pair query (pairs.cu).
 */
#include "b2g_host.h"

h_tree h_treeCreate( int proxyCapacity )
{
	int capacity = h_maxi( proxyCapacity, 16 );
	h_tree t;
	memset( &t, 0, sizeof( t ) );
	t.root = B2_NULL_INDEX;
	t.nodeCapacity = 2 * capacity - 1;
	t.nodes = h_nodeAlloc( (size_t)t.nodeCapacity * sizeof( h_treeNode ), &t.pinned );
	memset( t.nodes, 0, (size_t)t.nodeCapacity * sizeof( h_treeNode ) );
	for ( int i = 0; i < t.nodeCapacity - 1; ++i ) t.nodes[i].parent = i + 1;
	t.nodes[t.nodeCapacity - 1].parent = B2_NULL_INDEX;
	t.freeList = 0;
	return t;
}

void h_treeDestroy( h_tree* t )
{
	h_nodeFree( t->nodes, t->pinned );
	free( t->leafIndices );
	free( t->leafCenters );
	memset( t, 0, sizeof( *t ) );
}

static int h_allocNode( h_tree* t )
{
	if ( t->freeList == B2_NULL_INDEX )
	{
		int oldCapacity = t->nodeCapacity;
		t->nodeCapacity += oldCapacity >> 1;
		int pinned = 0;
		h_treeNode* grown = h_nodeAlloc( (size_t)t->nodeCapacity * sizeof( h_treeNode ), &pinned );
		memcpy( grown, t->nodes, (size_t)oldCapacity * sizeof( h_treeNode ) );
		h_nodeFree( t->nodes, t->pinned );
		t->nodes = grown;
		t->pinned = pinned;
		memset( t->nodes + t->nodeCount, 0, (size_t)( t->nodeCapacity - t->nodeCount ) * sizeof( h_treeNode ) );
		for ( int i = t->nodeCount; i < t->nodeCapacity - 1; ++i ) t->nodes[i].parent = i + 1;
		t->nodes[t->nodeCapacity - 1].parent = B2_NULL_INDEX;
		t->freeList = t->nodeCount;
	}
	int idx = t->freeList;
	h_treeNode* n = t->nodes + idx;
	t->version += 1;
	t->freeList = n->parent;
	memset( n, 0, sizeof( *n ) );
	n->categoryBits = B2_DEFAULT_CATEGORY_BITS;
	n->child1 = B2_NULL_INDEX;
	n->child2 = B2_NULL_INDEX;
	n->parent = B2_NULL_INDEX;
	n->flags = H_NODE_ALLOCATED;
	++t->nodeCount;
	return idx;
}

static void h_freeNode( h_tree* t, int id )
{
	t->version += 1;
	t->nodes[id].parent = t->freeList;
	t->nodes[id].flags = 0;
	t->freeList = id;
	--t->nodeCount;
}

static uint16_t h_maxu16( uint16_t a, uint16_t b ) { return a > b ? a : b; }

/* dynamic_tree.c:149-247 */
static int h_findBestSibling( const h_tree* t, b2AABB boxD )
{
	b2Vec2 centerD = h_aabbCenter( boxD );
	float areaD = h_perimeter( boxD );
	const h_treeNode* nodes = t->nodes;
	int rootIndex = t->root;
	b2AABB rootBox = nodes[rootIndex].aabb;
	float areaBase = h_perimeter( rootBox );
	float directCost = h_perimeter( h_aabbUnion( rootBox, boxD ) );
	float inheritedCost = 0.0f;
	int bestSibling = rootIndex;
	float bestCost = directCost;
	int index = rootIndex;
	while ( nodes[index].height > 0 )
	{
		int child1 = nodes[index].child1, child2 = nodes[index].child2;
		float cost = directCost + inheritedCost;
		if ( cost < bestCost )
		{
			bestSibling = index;
			bestCost = cost;
		}
		inheritedCost += directCost - areaBase;
		int leaf1 = nodes[child1].height == 0, leaf2 = nodes[child2].height == 0;
		float lowerCost1 = FLT_MAX;
		b2AABB box1 = nodes[child1].aabb;
		float directCost1 = h_perimeter( h_aabbUnion( box1, boxD ) );
		float area1 = 0.0f;
		if ( leaf1 )
		{
			float cost1 = directCost1 + inheritedCost;
			if ( cost1 < bestCost )
			{
				bestSibling = child1;
				bestCost = cost1;
			}
		}
		else
		{
			area1 = h_perimeter( box1 );
			lowerCost1 = inheritedCost + directCost1 + h_min( areaD - area1, 0.0f );
		}
		float lowerCost2 = FLT_MAX;
		b2AABB box2 = nodes[child2].aabb;
		float directCost2 = h_perimeter( h_aabbUnion( box2, boxD ) );
		float area2 = 0.0f;
		if ( leaf2 )
		{
			float cost2 = directCost2 + inheritedCost;
			if ( cost2 < bestCost )
			{
				bestSibling = child2;
				bestCost = cost2;
			}
		}
		else
		{
			area2 = h_perimeter( box2 );
			lowerCost2 = inheritedCost + directCost2 + h_min( areaD - area2, 0.0f );
		}
		if ( leaf1 && leaf2 ) break;
		if ( bestCost <= lowerCost1 && bestCost <= lowerCost2 ) break;
		if ( lowerCost1 == lowerCost2 && leaf1 == 0 )
		{
			b2Vec2 d1 = h_sub( h_aabbCenter( box1 ), centerD );
			b2Vec2 d2 = h_sub( h_aabbCenter( box2 ), centerD );
			lowerCost1 = h_lengthSq( d1 );
			lowerCost2 = h_lengthSq( d2 );
		}
		if ( lowerCost1 < lowerCost2 && leaf1 == 0 )
		{
			index = child1;
			areaBase = area1;
			directCost = directCost1;
		}
		else
		{
			index = child2;
			areaBase = area2;
			directCost = directCost2;
		}
	}
	return bestSibling;
}

/* apply one of the four rotations: child slot 'slotA' of A gets X, and Y (a child of the
   other child of A) is replaced by the node 'moved' */
static void h_rotateNodes( h_tree* t, int iA )
{
	h_treeNode* nodes = t->nodes;
	h_treeNode* A = nodes + iA;
	if ( A->height < 2 ) return;
	int iB = A->child1, iC = A->child2;
	h_treeNode *B = nodes + iB, *C = nodes + iC;
	if ( B->height == 0 )
	{
		int iF = C->child1, iG = C->child2;
		h_treeNode *F = nodes + iF, *G = nodes + iG;
		float costBase = h_perimeter( C->aabb );
		b2AABB aabbBG = h_aabbUnion( B->aabb, G->aabb );
		float costBF = h_perimeter( aabbBG );
		b2AABB aabbBF = h_aabbUnion( B->aabb, F->aabb );
		float costBG = h_perimeter( aabbBF );
		if ( costBase < costBF && costBase < costBG ) return;
		if ( costBF < costBG )
		{
			A->child1 = iF;
			C->child1 = iB;
			B->parent = iC;
			F->parent = iA;
			C->aabb = aabbBG;
			C->height = 1 + h_maxu16( B->height, G->height );
			A->height = 1 + h_maxu16( C->height, F->height );
			C->categoryBits = B->categoryBits | G->categoryBits;
			A->categoryBits = C->categoryBits | F->categoryBits;
			C->flags |= ( B->flags | G->flags ) & H_NODE_ENLARGED;
			A->flags |= ( C->flags | F->flags ) & H_NODE_ENLARGED;
		}
		else
		{
			A->child1 = iG;
			C->child2 = iB;
			B->parent = iC;
			G->parent = iA;
			C->aabb = aabbBF;
			C->height = 1 + h_maxu16( B->height, F->height );
			A->height = 1 + h_maxu16( C->height, G->height );
			C->categoryBits = B->categoryBits | F->categoryBits;
			A->categoryBits = C->categoryBits | G->categoryBits;
			C->flags |= ( B->flags | F->flags ) & H_NODE_ENLARGED;
			A->flags |= ( C->flags | G->flags ) & H_NODE_ENLARGED;
		}
	}
	else if ( C->height == 0 )
	{
		int iD = B->child1, iE = B->child2;
		h_treeNode *D = nodes + iD, *E = nodes + iE;
		float costBase = h_perimeter( B->aabb );
		b2AABB aabbCE = h_aabbUnion( C->aabb, E->aabb );
		float costCD = h_perimeter( aabbCE );
		b2AABB aabbCD = h_aabbUnion( C->aabb, D->aabb );
		float costCE = h_perimeter( aabbCD );
		if ( costBase < costCD && costBase < costCE ) return;
		if ( costCD < costCE )
		{
			A->child2 = iD;
			B->child1 = iC;
			C->parent = iB;
			D->parent = iA;
			B->aabb = aabbCE;
			B->height = 1 + h_maxu16( C->height, E->height );
			A->height = 1 + h_maxu16( B->height, D->height );
			B->categoryBits = C->categoryBits | E->categoryBits;
			A->categoryBits = B->categoryBits | D->categoryBits;
			B->flags |= ( C->flags | E->flags ) & H_NODE_ENLARGED;
			A->flags |= ( B->flags | D->flags ) & H_NODE_ENLARGED;
		}
		else
		{
			A->child2 = iE;
			B->child2 = iC;
			C->parent = iB;
			E->parent = iA;
			B->aabb = aabbCD;
			B->height = 1 + h_maxu16( C->height, D->height );
			A->height = 1 + h_maxu16( B->height, E->height );
			B->categoryBits = C->categoryBits | D->categoryBits;
			A->categoryBits = B->categoryBits | E->categoryBits;
			B->flags |= ( C->flags | D->flags ) & H_NODE_ENLARGED;
			A->flags |= ( B->flags | E->flags ) & H_NODE_ENLARGED;
		}
	}
	else
	{
		int iD = B->child1, iE = B->child2, iF = C->child1, iG = C->child2;
		h_treeNode *D = nodes + iD, *E = nodes + iE, *F = nodes + iF, *G = nodes + iG;
		float areaB = h_perimeter( B->aabb ), areaC = h_perimeter( C->aabb );
		float costBase = areaB + areaC;
		int best = 0;
		float bestCost = costBase;
		b2AABB aabbBG = h_aabbUnion( B->aabb, G->aabb );
		float costBF = areaB + h_perimeter( aabbBG );
		if ( costBF < bestCost )
		{
			best = 1;
			bestCost = costBF;
		}
		b2AABB aabbBF = h_aabbUnion( B->aabb, F->aabb );
		float costBG = areaB + h_perimeter( aabbBF );
		if ( costBG < bestCost )
		{
			best = 2;
			bestCost = costBG;
		}
		b2AABB aabbCE = h_aabbUnion( C->aabb, E->aabb );
		float costCD = areaC + h_perimeter( aabbCE );
		if ( costCD < bestCost )
		{
			best = 3;
			bestCost = costCD;
		}
		b2AABB aabbCD = h_aabbUnion( C->aabb, D->aabb );
		float costCE = areaC + h_perimeter( aabbCD );
		if ( costCE < bestCost ) best = 4;
		switch ( best )
		{
			case 1:
				A->child1 = iF;
				C->child1 = iB;
				B->parent = iC;
				F->parent = iA;
				C->aabb = aabbBG;
				C->height = 1 + h_maxu16( B->height, G->height );
				A->height = 1 + h_maxu16( C->height, F->height );
				C->categoryBits = B->categoryBits | G->categoryBits;
				A->categoryBits = C->categoryBits | F->categoryBits;
				C->flags |= ( B->flags | G->flags ) & H_NODE_ENLARGED;
				A->flags |= ( C->flags | F->flags ) & H_NODE_ENLARGED;
				break;
			case 2:
				A->child1 = iG;
				C->child2 = iB;
				B->parent = iC;
				G->parent = iA;
				C->aabb = aabbBF;
				C->height = 1 + h_maxu16( B->height, F->height );
				A->height = 1 + h_maxu16( C->height, G->height );
				C->categoryBits = B->categoryBits | F->categoryBits;
				A->categoryBits = C->categoryBits | G->categoryBits;
				C->flags |= ( B->flags | F->flags ) & H_NODE_ENLARGED;
				A->flags |= ( C->flags | G->flags ) & H_NODE_ENLARGED;
				break;
			case 3:
				A->child2 = iD;
				B->child1 = iC;
				C->parent = iB;
				D->parent = iA;
				B->aabb = aabbCE;
				B->height = 1 + h_maxu16( C->height, E->height );
				A->height = 1 + h_maxu16( B->height, D->height );
				B->categoryBits = C->categoryBits | E->categoryBits;
				A->categoryBits = B->categoryBits | D->categoryBits;
				B->flags |= ( C->flags | E->flags ) & H_NODE_ENLARGED;
				A->flags |= ( B->flags | D->flags ) & H_NODE_ENLARGED;
				break;
			case 4:
				A->child2 = iE;
				B->child2 = iC;
				C->parent = iB;
				E->parent = iA;
				B->aabb = aabbCD;
				B->height = 1 + h_maxu16( C->height, D->height );
				A->height = 1 + h_maxu16( B->height, E->height );
				B->categoryBits = C->categoryBits | D->categoryBits;
				A->categoryBits = B->categoryBits | E->categoryBits;
				B->flags |= ( C->flags | D->flags ) & H_NODE_ENLARGED;
				A->flags |= ( B->flags | E->flags ) & H_NODE_ENLARGED;
				break;
			default:
				break;
		}
	}
}

/* dynamic_tree.c:520-588 */
static void h_insertLeaf( h_tree* t, int leaf, int shouldRotate )
{
	if ( t->root == B2_NULL_INDEX )
	{
		t->root = leaf;
		t->nodes[leaf].parent = B2_NULL_INDEX;
		return;
	}
	b2AABB leafAABB = t->nodes[leaf].aabb;
	int sibling = h_findBestSibling( t, leafAABB );
	int oldParent = t->nodes[sibling].parent;
	int newParent = h_allocNode( t );
	h_treeNode* nodes = t->nodes;
	nodes[newParent].parent = oldParent;
	nodes[newParent].userData = UINT64_MAX;
	nodes[newParent].aabb = h_aabbUnion( leafAABB, nodes[sibling].aabb );
	nodes[newParent].categoryBits = nodes[leaf].categoryBits | nodes[sibling].categoryBits;
	nodes[newParent].height = nodes[sibling].height + 1;
	nodes[newParent].child1 = sibling;
	nodes[newParent].child2 = leaf;
	nodes[sibling].parent = newParent;
	nodes[leaf].parent = newParent;
	if ( oldParent != B2_NULL_INDEX )
	{
		if ( nodes[oldParent].child1 == sibling ) nodes[oldParent].child1 = newParent;
		else nodes[oldParent].child2 = newParent;
	}
	else
	{
		t->root = newParent;
	}
	int index = nodes[leaf].parent;
	while ( index != B2_NULL_INDEX )
	{
		int c1 = nodes[index].child1, c2 = nodes[index].child2;
		nodes[index].aabb = h_aabbUnion( nodes[c1].aabb, nodes[c2].aabb );
		nodes[index].categoryBits = nodes[c1].categoryBits | nodes[c2].categoryBits;
		nodes[index].height = 1 + h_maxu16( nodes[c1].height, nodes[c2].height );
		nodes[index].flags |= ( nodes[c1].flags | nodes[c2].flags ) & H_NODE_ENLARGED;
		if ( shouldRotate ) h_rotateNodes( t, index );
		index = nodes[index].parent;
	}
}

/* dynamic_tree.c:590-643 */
static void h_removeLeaf( h_tree* t, int leaf )
{
	if ( leaf == t->root )
	{
		t->root = B2_NULL_INDEX;
		return;
	}
	h_treeNode* nodes = t->nodes;
	int parent = nodes[leaf].parent;
	int grandParent = nodes[parent].parent;
	int sibling = nodes[parent].child1 == leaf ? nodes[parent].child2 : nodes[parent].child1;
	if ( grandParent != B2_NULL_INDEX )
	{
		if ( nodes[grandParent].child1 == parent ) nodes[grandParent].child1 = sibling;
		else nodes[grandParent].child2 = sibling;
		nodes[sibling].parent = grandParent;
		h_freeNode( t, parent );
		int index = grandParent;
		while ( index != B2_NULL_INDEX )
		{
			h_treeNode* n = nodes + index;
			h_treeNode* c1 = nodes + n->child1;
			h_treeNode* c2 = nodes + n->child2;
			n->aabb = h_aabbUnion( c1->aabb, c2->aabb );
			n->categoryBits = c1->categoryBits | c2->categoryBits;
			n->height = 1 + h_maxu16( c1->height, c2->height );
			index = n->parent;
		}
	}
	else
	{
		t->root = sibling;
		t->nodes[sibling].parent = B2_NULL_INDEX;
		h_freeNode( t, parent );
	}
}

int h_treeCreateProxy( h_tree* t, b2AABB aabb, uint64_t categoryBits, uint64_t userData )
{
	int id = h_allocNode( t );
	h_treeNode* n = t->nodes + id;
	n->aabb = aabb;
	n->userData = userData;
	n->categoryBits = categoryBits;
	n->height = 0;
	n->flags = H_NODE_ALLOCATED | H_NODE_LEAF;
	h_insertLeaf( t, id, 1 );
	t->proxyCount += 1;
	return id;
}

void h_treeDestroyProxy( h_tree* t, int proxyId )
{
	h_removeLeaf( t, proxyId );
	h_freeNode( t, proxyId );
	t->proxyCount -= 1;
}

void h_treeMoveProxy( h_tree* t, int proxyId, b2AABB aabb )
{
	h_removeLeaf( t, proxyId );
	t->nodes[proxyId].aabb = aabb;
	h_insertLeaf( t, proxyId, 0 );
}

/* dynamic_tree.c:798-837 */
static void h_treeEnlargeOne( h_tree* t, int proxyId, b2AABB aabb );

void h_treeEnlargeProxy( h_tree* t, int proxyId, b2AABB aabb )
{
	t->version += 1;
	h_treeEnlargeOne( t, proxyId, aabb );
}

void h_treeEnlargeProxies( h_tree* t, const int* proxyIds, const b2AABB* boxes, int count )
{
	for ( int i = 0; i < count; ++i ) h_treeEnlargeOne( t, proxyIds[i], boxes[i] );
}

static void h_treeEnlargeOne( h_tree* t, int proxyId, b2AABB aabb )
{
	h_treeNode* nodes = t->nodes;
	nodes[proxyId].aabb = aabb;
	int parentIndex = nodes[proxyId].parent;
	while ( parentIndex != B2_NULL_INDEX )
	{
		int changed = h_enlargeAABB( &nodes[parentIndex].aabb, aabb );
		nodes[parentIndex].flags |= H_NODE_ENLARGED;
		parentIndex = nodes[parentIndex].parent;
		if ( changed == 0 ) break;
	}
	while ( parentIndex != B2_NULL_INDEX )
	{
		if ( nodes[parentIndex].flags & H_NODE_ENLARGED ) break;
		nodes[parentIndex].flags |= H_NODE_ENLARGED;
		parentIndex = nodes[parentIndex].parent;
	}
}

/* h_treeEnlargeProxy for threads enlarging different proxies of one tree at once: box
   growth and flags are atomic. Every ancestor ends up with its old box grown by the new
   boxes of the enlarged leaves below it and flagged enlarged, whatever the order in which
   the threads reach it, so the tree is bit for bit what the enlargements one after another
   give. A walk may stop at an ancestor that already holds the box, since that ancestor's
   own ancestors hold it too or are being grown by the thread that grew it. The caller bumps
   the tree's version. */
static int h_atomicLower( float* p, float v )
{
	float cur;
	__atomic_load( p, &cur, __ATOMIC_RELAXED );
	while ( v < cur )
		if ( __atomic_compare_exchange( p, &cur, &v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED ) ) return 1;
	return 0;
}

static int h_atomicRaise( float* p, float v )
{
	float cur;
	__atomic_load( p, &cur, __ATOMIC_RELAXED );
	while ( cur < v )
		if ( __atomic_compare_exchange( p, &cur, &v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED ) ) return 1;
	return 0;
}

void h_treeEnlargeProxyShared( h_tree* t, int proxyId, b2AABB aabb )
{
	h_treeNode* nodes = t->nodes;
	nodes[proxyId].aabb = aabb;
	int parentIndex = nodes[proxyId].parent;
	while ( parentIndex != B2_NULL_INDEX )
	{
		b2AABB* box = &nodes[parentIndex].aabb;
		int changed = h_atomicLower( &box->lowerBound.x, aabb.lowerBound.x );
		changed |= h_atomicLower( &box->lowerBound.y, aabb.lowerBound.y );
		changed |= h_atomicRaise( &box->upperBound.x, aabb.upperBound.x );
		changed |= h_atomicRaise( &box->upperBound.y, aabb.upperBound.y );
		if ( ( __atomic_load_n( &nodes[parentIndex].flags, __ATOMIC_RELAXED ) & H_NODE_ENLARGED ) == 0 )
			__atomic_fetch_or( &nodes[parentIndex].flags, (uint16_t)H_NODE_ENLARGED, __ATOMIC_RELAXED );
		parentIndex = nodes[parentIndex].parent;
		if ( changed == 0 ) break;
	}
	while ( parentIndex != B2_NULL_INDEX )
	{
		if ( __atomic_load_n( &nodes[parentIndex].flags, __ATOMIC_RELAXED ) & H_NODE_ENLARGED ) break;
		__atomic_fetch_or( &nodes[parentIndex].flags, (uint16_t)H_NODE_ENLARGED, __ATOMIC_RELAXED );
		parentIndex = nodes[parentIndex].parent;
	}
}

int h_treeHeight( const h_tree* t )
{
	return t->root == B2_NULL_INDEX ? 0 : t->nodes[t->root].height;
}

/* dynamic_tree.c:1085-1135: child1 pushed before child2, so child2 is visited first */
void h_treeQuery( const h_tree* t, b2AABB aabb, uint64_t maskBits, h_treeQueryFcn* fcn, void* ctx )
{
	if ( t->nodeCount == 0 ) return;
	int stack[1024];
	int stackCount = 0;
	stack[stackCount++] = t->root;
	while ( stackCount > 0 )
	{
		int nodeId = stack[--stackCount];
		const h_treeNode* n = t->nodes + nodeId;
		if ( h_aabbOverlaps( n->aabb, aabb ) && ( n->categoryBits & maskBits ) != 0 )
		{
			if ( n->flags & H_NODE_LEAF )
			{
				if ( fcn( nodeId, n->userData, ctx ) == 0 ) return;
			}
			else if ( stackCount < 1024 - 1 )
			{
				stack[stackCount++] = n->child1;
				stack[stackCount++] = n->child2;
			}
		}
	}
}

/* dynamic_tree.c:1433-1520 median split */
static int h_partitionMid( int* indices, b2Vec2* centers, int count )
{
	if ( count <= 2 ) return count / 2;
	b2Vec2 lower = centers[0], upper = centers[0];
	for ( int i = 1; i < count; ++i )
	{
		lower = h_vmin( lower, centers[i] );
		upper = h_vmax( upper, centers[i] );
	}
	b2Vec2 d = h_sub( upper, lower );
	b2Vec2 c = { 0.5f * ( lower.x + upper.x ), 0.5f * ( lower.y + upper.y ) };
	int i1 = 0, i2 = count;
	int axisX = d.x > d.y;
	float pivot = axisX ? c.x : c.y;
	while ( i1 < i2 )
	{
		while ( i1 < i2 && ( axisX ? centers[i1].x : centers[i1].y ) < pivot ) i1 += 1;
		while ( i1 < i2 && ( axisX ? centers[i2 - 1].x : centers[i2 - 1].y ) >= pivot ) i2 -= 1;
		if ( i1 < i2 )
		{
			int ti = indices[i1];
			indices[i1] = indices[i2 - 1];
			indices[i2 - 1] = ti;
			b2Vec2 tc = centers[i1];
			centers[i1] = centers[i2 - 1];
			centers[i2 - 1] = tc;
			i1 += 1;
			i2 -= 1;
		}
	}
	if ( i1 > 0 && i1 < count ) return i1;
	return count / 2;
}

typedef struct h_rebuildItem
{
	int nodeIndex, childCount, startIndex, splitIndex, endIndex;
} h_rebuildItem;

/* dynamic_tree.c:1723-1877 */
static int h_buildTree( h_tree* t, int leafCount )
{
	int* leafIndices = t->leafIndices;
	if ( leafCount == 1 )
	{
		t->nodes[leafIndices[0]].parent = B2_NULL_INDEX;
		return leafIndices[0];
	}
	b2Vec2* leafCenters = t->leafCenters;
	h_rebuildItem stack[1024];
	int top = 0;
	stack[0].nodeIndex = h_allocNode( t );
	stack[0].childCount = -1;
	stack[0].startIndex = 0;
	stack[0].endIndex = leafCount;
	stack[0].splitIndex = h_partitionMid( leafIndices, leafCenters, leafCount );
	while ( 1 )
	{
		h_rebuildItem* item = stack + top;
		item->childCount += 1;
		if ( item->childCount == 2 )
		{
			if ( top == 0 ) break;
			h_rebuildItem* parentItem = stack + ( top - 1 );
			h_treeNode* parentNode = t->nodes + parentItem->nodeIndex;
			if ( parentItem->childCount == 0 ) parentNode->child1 = item->nodeIndex;
			else parentNode->child2 = item->nodeIndex;
			h_treeNode* node = t->nodes + item->nodeIndex;
			node->parent = parentItem->nodeIndex;
			h_treeNode* c1 = t->nodes + node->child1;
			h_treeNode* c2 = t->nodes + node->child2;
			node->aabb = h_aabbUnion( c1->aabb, c2->aabb );
			node->height = 1 + h_maxu16( c1->height, c2->height );
			node->categoryBits = c1->categoryBits | c2->categoryBits;
			top -= 1;
		}
		else
		{
			int startIndex, endIndex;
			if ( item->childCount == 0 )
			{
				startIndex = item->startIndex;
				endIndex = item->splitIndex;
			}
			else
			{
				startIndex = item->splitIndex;
				endIndex = item->endIndex;
			}
			int count = endIndex - startIndex;
			if ( count == 1 )
			{
				int childIndex = leafIndices[startIndex];
				h_treeNode* node = t->nodes + item->nodeIndex;
				if ( item->childCount == 0 ) node->child1 = childIndex;
				else node->child2 = childIndex;
				t->nodes[childIndex].parent = item->nodeIndex;
			}
			else
			{
				top += 1;
				h_rebuildItem* newItem = stack + top;
				newItem->nodeIndex = h_allocNode( t );
				newItem->childCount = -1;
				newItem->startIndex = startIndex;
				newItem->endIndex = endIndex;
				newItem->splitIndex = h_partitionMid( leafIndices + startIndex, leafCenters + startIndex, count ) + startIndex;
			}
		}
	}
	h_treeNode* rootNode = t->nodes + stack[0].nodeIndex;
	h_treeNode* c1 = t->nodes + rootNode->child1;
	h_treeNode* c2 = t->nodes + rootNode->child2;
	rootNode->aabb = h_aabbUnion( c1->aabb, c2->aabb );
	rootNode->height = 1 + h_maxu16( c1->height, c2->height );
	rootNode->categoryBits = c1->categoryBits | c2->categoryBits;
	return stack[0].nodeIndex;
}

/* dynamic_tree.c:1879-1996 */
int h_treeRebuild( h_tree* t, int fullBuild )
{
	int proxyCount = t->proxyCount;
	if ( proxyCount == 0 ) return 0;
	t->version += 1;
	if ( proxyCount > t->rebuildCapacity )
	{
		int nc = proxyCount + proxyCount / 2;
		free( t->leafIndices );
		free( t->leafCenters );
		t->leafIndices = malloc( (size_t)nc * sizeof( int ) );
		t->leafCenters = malloc( (size_t)nc * sizeof( b2Vec2 ) );
		t->rebuildCapacity = nc;
	}
	int leafCount = 0;
	int stack[1024];
	int stackCount = 0;
	int nodeIndex = t->root;
	h_treeNode* node = t->nodes + nodeIndex;
	while ( 1 )
	{
		if ( node->height == 0 || ( ( node->flags & H_NODE_ENLARGED ) == 0 && fullBuild == 0 ) )
		{
			t->leafIndices[leafCount] = nodeIndex;
			t->leafCenters[leafCount] = h_aabbCenter( node->aabb );
			leafCount += 1;
			node->parent = B2_NULL_INDEX;
		}
		else
		{
			int doomed = nodeIndex;
			nodeIndex = node->child1;
			if ( stackCount < 1024 ) stack[stackCount++] = node->child2;
			node = t->nodes + nodeIndex;
			h_freeNode( t, doomed );
			continue;
		}
		if ( stackCount == 0 ) break;
		nodeIndex = stack[--stackCount];
		node = t->nodes + nodeIndex;
	}
	t->root = h_buildTree( t, leafCount );
	return leafCount;
}
