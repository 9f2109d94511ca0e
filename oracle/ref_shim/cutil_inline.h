/* Project-written stand-in for the SDK's cutil_inline.h; everything the
   reference needs is in the sibling cutil.h. */
#include "cutil.h"
