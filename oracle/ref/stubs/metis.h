/* See parmetis.h: declarations-only stand-in for the oracle build. */
#include "parmetis.h"
