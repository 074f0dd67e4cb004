/* ORACLE shim: Definitions.cpp:75-80 reads FFTW_MEASURE as a default planner
 * flag; no FFT is on the hot path, so only the flag is defined. */
#pragma once
#define FFTW_MEASURE 0u
