/* Standard headers some reference sources use without including them. */
#include <cstring>
#include <cmath>
#include <algorithm>
#include "parmetis.h"
