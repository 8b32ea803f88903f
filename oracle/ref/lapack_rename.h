// FRICO calls zgetrf_/zgetrs_/zsytrf_/zsytrs_; scipy's bundled OpenBLAS
// exports the same routines with a scipy_ prefix.
#pragma once
#define zgetrf_ scipy_zgetrf_
#define zgetrs_ scipy_zgetrs_
#define zsytrf_ scipy_zsytrf_
#define zsytrs_ scipy_zsytrs_
