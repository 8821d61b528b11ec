// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT. See x86intrin.h beside it.
#include "x86intrin.h"
