/*
 * Forwarding header: sources that include the reference's public header path
 * ("box2d/box2d.h", which in the reference also pulls in base.h, collision.h, id.h,
 * math_functions.h and types.h) compile unchanged against the GB300 step library.
 */
#ifndef BOX2D_GB300_FORWARD_BOX2D_H
#define BOX2D_GB300_FORWARD_BOX2D_H

#include "../box2d_gb300.h"

#endif
