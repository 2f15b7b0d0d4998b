// Grayscale TIFF images for the `tiff` parser-context type.
//
// The reference opens the file with libtiff and reads one scanline at a time
// (src/dune/copasi/common/tiff_file.cc:15-45, tiff_grayscale.cc:21-80); libtiff is not a
// dependency here, so this is a reader of baseline TIFF written from the TIFF 6.0
// specification: the first image of the file, little- or big-endian, strips,
// uncompressed, PackBits or LZW data (LZW with or without the horizontal-differencing
// predictor), one sample per pixel of 8, 16, 32 or 64 bits.  Pixel values are scaled as
// the reference scales them (TIFFGrayscaleRow::operator[]): v / 2^bits, inverted
// (2^bits - v) for WhiteIsZero images.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dcgpu {

struct TiffGray {
  uint32_t rows = 0, cols = 0;   // ImageLength (scanlines), ImageWidth (pixels per scanline)
  uint16_t bits = 0;
  bool black_is_zero = false;    // PhotometricInterpretation 1 (0: WhiteIsZero)
  float x_res = 0.f, y_res = 0.f, x_off = 0.f, y_off = 0.f;
  std::vector<double> px;        // rows * cols scaled values, scanline-major
};

// Throws ConfigError with the reference's messages for a missing file, a non-grayscale
// image, a non-positive resolution and an unsupported sample size; other layouts the
// reader does not handle (tiles, several samples per pixel, other compressions) are
// reported the same way.
TiffGray read_tiff_gray(const std::string& path);

}  // namespace dcgpu
