/* Standard headers the reference sources expect from its precompiled header
 * (src/headers.hpp).  Test infrastructure for building the reference oracle. */
#pragma once
#include <stdlib.h>
#include <math.h>
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>
