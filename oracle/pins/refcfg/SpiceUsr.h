// The SPICE toolkit is absent: the reference's own empty SPICE definitions.
#include "SpiceEmptyDefinitions.h"
