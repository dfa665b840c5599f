// netcdf3.h -- reader for NetCDF-3 files (classic CDF-1 and 64-bit-offset
// CDF-2), written from the published NetCDF classic format specification.
//
// Replaces the netcdf3 0.5.2 crate the reference reads its grids with
// (src/bathymetry/cartesian_netcdf3.rs:167-256,
// src/current/cartesian_current.rs:58-213).  Only what those readers use:
// the header, and whole-variable reads of byte/char/short/int/float/double
// variables (fixed-size or record).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace mr {
namespace nc3 {

enum Type : int { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };

struct Variable {
  std::string name;
  std::vector<uint32_t> dimids;
  int type = 0;
  uint64_t vsize = 0;
  uint64_t begin = 0;
  bool is_record = false;
};

struct Header {
  int version = 0;  // 1 classic, 2 64-bit offset
  uint64_t numrecs = 0;
  std::vector<std::string> dim_names;
  std::vector<uint64_t> dim_lengths;  // 0 = the record dimension
  std::vector<Variable> vars;
  uint64_t record_size = 0;           // bytes per record, all record variables
};

// Status: 0 ok, -3 io error, -4 format/variable error (MR_ERR_* values).
struct Result {
  int code = 0;
  std::string message;
};

// Reads variable `name` of `path`.  Values are converted to double
// (`as f64` in the reference: exact for every NetCDF-3 type).  `type`
// receives the NetCDF type code; `raw_f32` (optional) receives the values
// as the reference's bathymetry axes convert them (`as f32`): integers and
// doubles rounded to nearest f32, floats unchanged.
Result read_variable(const std::string &path, const std::string &name, std::vector<double> *values,
                     int *type, std::vector<float> *raw_f32 = nullptr);

}  // namespace nc3
}  // namespace mr
