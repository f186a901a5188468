/* Empty: every HYPRE name the oracle build needs is declared in _hypre_utilities.h. */
#include "_hypre_utilities.h"
