/*
 * Forwarding header: the reference's public header path "box2d/types.h" resolves to the
 * GB300 step library's single public header, which declares the same types and functions.
 */
#ifndef BOX2D_GB300_FORWARD_TYPES_H
#define BOX2D_GB300_FORWARD_TYPES_H

#include "../box2d_gb300.h"

#endif
