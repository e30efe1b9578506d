/*
 * ORACLE — test infrastructure only.  Stand-in for the reference's cut/timing.cpp, which needs HDF5 for its
 * log writer: the timer methods do nothing, so the reference's SCOPED_*_QUERY macros compile to no-ops.
 */
#include "cut/timing.h"

TimeLogger g_TimeLogger;

void TimeLogger::release() {}
void TimeLogger::startCUDA(const string &) {}
void TimeLogger::endCUDA(const string &) {}
void TimeLogger::startCPU(const string &) {}
void TimeLogger::endCPU(const string &) {}
void TimeLogger::syncAndReport() {}
