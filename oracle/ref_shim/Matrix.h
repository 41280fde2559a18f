/* Case-correcting forwarder: Source/shape.h:22 includes "Matrix.h" but the file is matrix.h. */
#include "matrix.h"
