// fftz: command-line driver with the flags and output lines of
// projection_example.cu:1-279, running the GB300 solver and encoder.
//
//   fftz -i x.bin -e x'.bin [-z out] [-o out] (-1 n | -2 ny nz | -3 nx ny nz)
//        [-f|-d] -M ABS|REL eps -F ABS|REL delta
//
// As in the reference: bounds are absolute whatever ABS/REL says
// (:124-137), eps/delta are parsed as float (:129, :136), -1/-2/-3 must be
// followed by another argument (:111-114), -z/-o are accepted but nothing is
// written (:255-256), max_iterations = 100 and tolerance = 1e-7 (:199-200),
// the four streams are Huffman+ZSTD coded at level 20 (:233-246), and the
// printed "Compression time" is 3*(getter time) + solve time (:250).
#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "HuffmanZSTDCoder.cuh"
#include "fileIO.h"
#include "projection_algorithm.cuh"

namespace {

std::string originalFile, baseDecompFile, compressedFile, decompressedFile;
size_t Nx = 0, Ny = 0, Nz = 1, spatial_size = 0;
bool isDouble = false, isSpatialABS = false, isFreqABS = false;
float spatial_epsilon = 0.f, freq_delta = 0.f;

[[noreturn]] void parseError(const char *error) {
  std::cout << error << std::endl;
  std::cout << "Usage:\n";
  std::cout << "  -i <file_path>  : Specify the file of original data\n";
  std::cout << "  -e <file_path>  : Specify the reconstructed file of base compressor\n";
  std::cout << "  -z <file_path>  : Specify the compressed file\n";
  std::cout << "  -o <file_path>  : Specify the decompressed file (optional)\n";
  std::cout << "  -1 <nx>                : 1D data with <nx> values\n";
  std::cout << "  -2 <nx> <ny>           : 2D data with <nx> * <ny> values\n";
  std::cout << "  -3 <nx> <ny> <nz>      : 3D data with <nx> * <ny> * <nz> values\n";
  std::cout << "  -f              : Use float data type\n";
  std::cout << "  -d              : Use double data type\n";
  std::cout << "  -M ABS <xi>     : Specify the absolute error bound in spatial domain\n";
  std::cout << "  -M REL <xi>     : Specify the relative error bound in spatial domain\n";
  std::cout << "  -F ABS <xi>     : Specify the absolute error bound in frequency domain\n";
  std::cout << "  -F REL <xi>     : Specify the relative error bound in frequency domain\n";
  exit(EXIT_FAILURE);
}

void Parsing(int argc, char *argv[]) {
  bool haveOrig = false, haveBase = false;
  for (int i = 1; i < argc; ++i) {
    const std::string arg = argv[i];
    auto need = [&](const char *msg) {
      if (i + 1 >= argc) parseError(msg);
      return argv[++i];
    };
    if (arg == "-i") {
      originalFile = need("Missing input file path");
      haveOrig = true;
    } else if (arg == "-e") {
      baseDecompFile = need("Missing base reconstructed file path");
      haveBase = true;
    } else if (arg == "-z") {
      compressedFile = need("Missing compressed file path");
    } else if (arg == "-o") {
      decompressedFile = need("Missing decompressed file path");
    } else if (arg == "-1" || arg == "-2" || arg == "-3") {
      const int nd = arg[1] - '0';
      if (i + nd >= argc) parseError("Missing size for 1D data");
      if (nd == 1) {
        Nx = 1;
        Ny = 1;
        Nz = std::stoi(argv[++i]);
      } else if (nd == 2) {
        Nx = 1;
        Ny = std::stoi(argv[++i]);
        Nz = std::stoi(argv[++i]);
      } else {
        Nx = std::stoi(argv[++i]);
        Ny = std::stoi(argv[++i]);
        Nz = std::stoi(argv[++i]);
      }
      spatial_size = Nx * Ny * Nz;
      if (i + 1 >= argc) parseError("Missing size for 1D data");
    } else if (arg == "-f") {
      isDouble = false;
    } else if (arg == "-d") {
      isDouble = true;
    } else if (arg == "-M") {
      isSpatialABS = std::strcmp(need("Missing spatial error bound"), "ABS") == 0;
      spatial_epsilon = std::stof(need("Missing spatial error bound"));
    } else if (arg == "-F") {
      isFreqABS = std::strcmp(need("Missing frequency error bound"), "ABS") == 0;
      freq_delta = std::stof(need("Missing frequency error bound"));
    } else {
      parseError("Unknown argument");
    }
  }
  if (!haveOrig && !haveBase)
    parseError("Input files of original data (-i) and base decompressed data (-e) are mandatory");
}

template <typename T>
void Run() {
  std::vector<T> x(spatial_size), err(spatial_size);
  const DataType dt = sizeof(T) == 4 ? DataType::FLOAT : DataType::DOUBLE;
  readRawArrayBinary(originalFile, x.data(), spatial_size, dt);
  readRawArrayBinary(baseDecompFile, err.data(), spatial_size, dt);
  for (size_t i = 0; i < spatial_size; ++i) err[i] -= x[i];

  ProjectionSolver<T> solver(Nx, Ny, Nz);
  solver.initialize_all_abs(x.data(), spatial_epsilon, freq_delta);
  const int max_iterations = 100;
  const T tolerance = 1e-7f;

  const auto t0 = std::chrono::high_resolution_clock::now();
  solver.solve_all_abs(err.data(), max_iterations, tolerance);
  const auto t1 = std::chrono::high_resolution_clock::now();
  std::vector<uint16_t> fq = solver.get_active_freq_quant_edit_distances();
  std::vector<uint16_t> sq = solver.get_active_spatial_quant_edit_distances();
  std::vector<uint8_t> fp = solver.get_freq_flags_pack();
  std::vector<uint8_t> sp = solver.get_spatial_flags_pack();
  const auto t2 = std::chrono::high_resolution_clock::now();

  size_t extra_storage = 0;
  if (!fq.empty()) {
    extra_storage += cudaHuffmanZstdCompress(fq, 20).compressed_data.size();
    extra_storage += cudaHuffmanZstdCompress(fp, 20).compressed_data.size();
  }
  if (!sq.empty()) {
    extra_storage += cudaHuffmanZstdCompress(sq, 20).compressed_data.size();
    extra_storage += cudaHuffmanZstdCompress(sp, 20).compressed_data.size();
  }
  (void)extra_storage;
  printf("# Active frequency edits: %zu\n", fq.size());
  printf("# Active spatial edits: %zu\n", sq.size());
  using ms = std::chrono::milliseconds;
  const auto ct = std::chrono::duration_cast<ms>((t2 - t1) * 3 + t1 - t0);
  const auto dt2 = std::chrono::duration_cast<ms>((t2 - t1) * 2);
  std::cout << "Compression time: " << ct.count() << " ms" << std::endl;
  std::cout << "Decompression time: " << dt2.count() << " ms" << std::endl;
}

}  // namespace

int main(int argc, char *argv[]) {
  Parsing(argc, argv);
  try {
    if (isDouble) Run<double>();
    else Run<float>();
  } catch (const std::exception &e) {
    std::cerr << "terminate called after throwing an instance of 'std::runtime_error'\n  what():  " << e.what()
              << std::endl;
    return 134;
  }
  return 0;
}
