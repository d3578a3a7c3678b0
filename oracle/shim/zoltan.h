/* Stand-in for <zoltan.h>: the reference headers only need the includes below. */
#include <stdint.h>
#include <stdlib.h>
#include "mpi.h"
