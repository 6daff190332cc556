// Learned strategy picker (placeholder).
#include "vs_internal.cuh"
