// Oracle recipe support (test infrastructure): C entry point over the reference's own
// AliasMap::build (AliasMap.cpp:71-166), compiled in place from the reference tree by
// oracle/build_oracle.py into oracle/_ref/.  Used only to pin the oracle's restatement.
#include "pch.h"

#include "AliasMap.h"

extern "C" __attribute__((visibility("default"))) void ref_alias_build(const float* rgb,
    unsigned int width, unsigned int height, void* out, float* integral)
{
    uvec2 dims{ width, height };
    Aurora::AliasMap::build(rgb, dims, static_cast<Aurora::AliasMap::Entry*>(out),
        size_t(width) * height * sizeof(Aurora::AliasMap::Entry), *integral);
}
