// dbd_io.h -- internal file-format and output-writer declarations.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/dbd.h"

namespace dbd {

int read_csr_file(const std::string &path, dbd_csr_host *out, std::string *err);
int write_csr_file(const std::string &path, const dbd_csr_view *m, int fp64, std::string *err);

}  // namespace dbd
