// dbd_io.h -- internal file-format and output-writer declarations.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/dbd.h"

namespace dbd {

int read_csr_file(const std::string &path, dbd_csr_host *out, std::string *err);
// read_csr_file with the Matrix Market / .dat conversion on GPU `device`.
int read_csr_file_gpu(const std::string &path, int device, dbd_csr_host *out, std::string *err);
// The conversion itself (k_mtx.cu): the same CSR and <path>.csr cache as the host's.
int convert_matrix_file_gpu(const std::string &path, int device, dbd_csr_host *m, std::string *err);
int write_csr_file(const std::string &path, const dbd_csr_view *m, int fp64, std::string *err);

}  // namespace dbd
