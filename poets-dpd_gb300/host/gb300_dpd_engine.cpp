// Registration stub: link this file into a poets-dpd tool (with libpdpd_gb300.so) and the
// GB300 engines become available by name through DPDEngineFactory::create, like the
// reference's own engines (src/engines/naive_dpd_engine_half_step.cpp).
#include "gb300_dpd_engine.hpp"

#include <memory>

bool gb300_dpd_engine_fp32_registered = DPDEngineFactory::RegisterFactory(
    "gb300_dpd_engine_fp32", []() { return std::make_shared<GB300DPDEngine>(PDPD_FP32); });

bool gb300_dpd_engine_fp64_registered = DPDEngineFactory::RegisterFactory(
    "gb300_dpd_engine_fp64", []() { return std::make_shared<GB300DPDEngine>(PDPD_FP64); });
