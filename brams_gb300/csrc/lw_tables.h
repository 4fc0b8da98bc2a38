// Host-side construction of the device table blob (see lw_tables.cpp).
#pragma once
#include <string>
#include <vector>

#include "lw_common.h"

// cloud64 (optional): the cloud optics tables in fp64, offsets in T.c64_*
bool gb_build_tables(const char* ref_path, const char* k_path, double cpdair, GbTables& T,
                     std::vector<float>& blob, std::string& err, std::vector<double>* cloud64 = nullptr);

// one float64 array of a table container (Fortran element order)
bool gb_read_table_f64(const char* path, const char* name, std::vector<double>& out, std::string& err);

// every array of a table container file (format: brams_gb300/tables_io.py)
#include <map>
struct GbTableEntry {
  std::vector<double> d;  // float64 arrays
  std::vector<int> i;     // int32 arrays
  int dims[4] = {1, 1, 1, 1};
  int ndim = 0;
  bool is_int = false;
  size_t size() const { return is_int ? i.size() : d.size(); }
};
bool gb_read_container(const char* path, std::map<std::string, GbTableEntry>& out, std::string& err);
