// Type-only stand-in for the SILO header (visualisation output is not built).
#pragma once
typedef struct DBfile DBfile;
