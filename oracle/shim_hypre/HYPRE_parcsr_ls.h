/* Stand-in header: see hypre_standin.h. */
#include "hypre_standin.h"
