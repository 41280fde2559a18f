/* Case-correcting forwarder: Source/plane.h:21 includes "Intersection.h" but the file is intersection.h. */
#include "intersection.h"
