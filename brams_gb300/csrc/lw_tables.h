// Host-side construction of the device table blob (see lw_tables.cpp).
#pragma once
#include <string>
#include <vector>

#include "lw_common.h"

bool gb_build_tables(const char* ref_path, const char* k_path, double cpdair, GbTables& T,
                     std::vector<float>& blob, std::string& err);
