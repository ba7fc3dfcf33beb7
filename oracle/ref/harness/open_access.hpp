/* Force-included into the dump harness translation units only: pulls in the
 * standard headers first, then opens every class of the reference so the
 * harness can read its internal state (bulk arrays, connection arrays, PVT
 * tables, flash counters) without modifying the reference sources. */
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>
#define private public
#define protected public
