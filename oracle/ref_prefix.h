/* Oracle test infrastructure.  Pre-included ahead of every reference
 * translation unit (after the per-case configuration header).  It pulls in
 * every standard header the reference uses, then opens class access so the
 * oracle harness can inject fields and markers into GridObj/ObjectManager
 * state.  All reference TUs and the harness see the same definitions, so the
 * one-definition rule holds across the oracle build. */
#ifndef LUMA_ORACLE_REF_PREFIX_H
#define LUMA_ORACLE_REF_PREFIX_H
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <numeric>
#include <sstream>
#include <string>
#include <valarray>
#include <vector>
#include <memory>
#include <map>
#include <set>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#define private public
#define protected public
#endif
