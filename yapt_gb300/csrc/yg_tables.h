// Host-side generation of the tables the tracer kernels read (see yg_tables.cpp).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "yg_types.h"

namespace yg
{

struct MsLuts
{
    std::vector<float> ss, ssAvg, ssms, ssmsAvg, transDenser, transLighter, transAvgDenser, transAvgLighter, sheen;
};

bool buildSobolMatrices(const std::string& joeKuoPath, std::vector<uint32_t>& out, std::string& err);
uint32_t sobolUint(const uint32_t* matrices, uint32_t index, uint32_t dim);
bool loadCie(const std::string& path, std::vector<double>& cie471x4, std::string& err);
bool cieForRange(const std::vector<double>& cie, int lmin, int lmax, std::vector<float>& out4, float& ySumInv,
                 float& d65SumInv);
void buildMsLuts(MsLuts& luts);
void buildRgbToSpd(const std::vector<double>& cie, int lmin, int lmax, std::vector<float>& out);

} // namespace yg
