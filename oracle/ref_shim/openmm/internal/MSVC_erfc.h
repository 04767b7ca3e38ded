/* Oracle build shim (test infrastructure only): erf/erfc come from <cmath> here. */
#include <cmath>
