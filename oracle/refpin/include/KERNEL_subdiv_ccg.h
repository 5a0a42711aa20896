/* Stand-in for a header the reference does not ship: everything it must
 * declare is in refpin_prelude.h. */
#include "refpin_prelude.h"
