/* Forced include for compiling the reference's multicore engine headers as one
 * translation unit: the standard headers and names those headers use without
 * including them.  TEST INFRASTRUCTURE ONLY (oracle/_ref). */
#ifndef ACDC_REF_PRE_H_
#define ACDC_REF_PRE_H_
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
using namespace std;
#endif
