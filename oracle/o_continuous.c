/*
 * Oracle (test checker only): continuous collision of fast bodies against static shapes
 * (b2SolveContinuous, solver.c:384-550). Placeholder until the time-of-impact solver is
 * restated: it advances the body like a slow one and counts the occurrence so tests can
 * refuse to compare a run that needed it.
 */
#include "o_core.h"

int o_continuousSkipped = 0;

void o_solveContinuous( o_world* w, int simIndex )
{
	o_bodySim* sim = w->awakeSims.data + simIndex;
	sim->center0 = sim->center;
	sim->rotation0 = sim->transform.q;
	__atomic_fetch_add( &o_continuousSkipped, 1, __ATOMIC_RELAXED );
}
