// TEST INFRASTRUCTURE ONLY: the reference's shader math compiled as the bidirectional
// integrator compiles it, with RECIPROCAL_MULTISCATTER (the Kulla-Conty energy compensation,
// BDPTCommon.hlsl:6), behind the refcheck.h functions with the prefix refK_.
#define RECIPROCAL_MULTISCATTER
#define REFCHECK_NS hlsl_kulla
#define REFCHECK_PREFIX refK_
#include "hlsl_side.cpp"
