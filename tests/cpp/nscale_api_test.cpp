// Exercises the C++ mirror of the nscale / nscale::gpu API (include/nscale_gpu.hpp) the way
// the reference's call sites do, on a synthetic tile, and writes every result as a raw file
// into the directory given as argv[1] (compared against the oracle by the Python test).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "nscale_gpu.hpp"
#include "nsgb_synth.h"

static void save(const std::string& dir, const char* name, const cv::Mat& m) {
  FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
  if (!f) std::exit(2);
  for (int y = 0; y < m.rows; ++y) std::fwrite(m.ptr<unsigned char>(y), m.elemSize(), (size_t)m.cols, f);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  const int H = 300, W = 400;
  cv::Mat mask(H, W, CV_8UC1), marker(H, W, CV_8UC1);
  if (nsgb_synth_tile_u8(mask.data, marker.data, H, W, W, 40, 5) != 0) return 3;
  save(dir, "mask.u8", mask);
  save(dir, "marker.u8", marker);

  // host signatures (MorphologicOperations.h:21-94), computed on the GPU
  cv::Mat recon = nscale::imreconstruct<unsigned char>(marker, mask, 8);
  save(dir, "recon8.u8", recon);
  cv::Mat bin(H, W, CV_8UC1);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) bin.ptr<unsigned char>(y)[x] = recon.ptr<unsigned char>(y)[x] > 128 ? 255 : 0;
  cv::Mat filled = nscale::imfillHoles<unsigned char>(bin, true, 4);
  save(dir, "fill4.u8", filled);
  cv::Mat labels = nscale::bwlabel2(filled, 8, true);
  save(dir, "labels8.i32", labels);
  int count = -1;
  cv::Mat kept = nscale::bwareaopen2(filled, false, true, 11, 1000, 8, count);
  save(dir, "area.u8", kept);
  cv::Mat hmin = nscale::imhmin<unsigned char>(mask, (unsigned char)10, 8);
  save(dir, "hmin8.u8", hmin);
  cv::Mat cross(3, 3, CV_8UC1);  // getStructuringElement(MORPH_ELLIPSE, Size(3, 3))
  for (int i = 0; i < 9; ++i) cross.data[i] = (i % 2) ? 1 : (i == 4 ? 1 : 0);
  cv::Mat opened = nscale::morphOpen<unsigned char>(mask, cross);
  save(dir, "open3.u8", opened);
  cv::Mat bin_mask(H, W, CV_8UC1);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) bin_mask.ptr<unsigned char>(y)[x] = mask.ptr<unsigned char>(y)[x] < 128 ? 255 : 0;
  cv::Mat dist = nscale::distanceTransform(bin_mask);
  save(dir, "dist.f32", dist);

  // device signatures (MorphologicOperations.h:96-190)
  cv::gpu::Stream stream;
  cv::gpu::GpuMat gmask(mask), gmarker(marker);
  unsigned int iter = 0;
  cv::gpu::GpuMat grecon = nscale::gpu::imreconstruct<unsigned char>(gmarker, gmask, 4, stream, iter);
  cv::Mat recon4;
  grecon.download(recon4);
  save(dir, "recon4.u8", recon4);
  std::vector<cv::gpu::GpuMat> seeds{gmarker, gmarker}, images{gmask, gmask};
  std::vector<cv::gpu::GpuMat> batch = nscale::gpu::imreconstructQueueThroughput<unsigned char>(seeds, images, 8, 0, stream);
  cv::Mat b0, b1;
  batch[0].download(b0);
  batch[1].download(b1);
  save(dir, "batch0.u8", b0);
  save(dir, "batch1.u8", b1);
  // the queue variant (MorphologicOperations.h:105-116): grayscale, and binary (the binary
  // reconstruction of the dark objects from a few seed pixels)
  cv::gpu::GpuMat gsp = nscale::gpu::imreconstructQueueSpeedup<unsigned char>(gmarker, gmask, 8, 1, stream);
  cv::Mat sp;
  gsp.download(sp);
  save(dir, "speedup8.u8", sp);
  cv::Mat bseed(H, W, CV_8UC1);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) bseed.ptr<unsigned char>(y)[x] = ((x * 7 + y * 13) % 97 == 0) ? 255 : 0;
  cv::gpu::GpuMat gbseed(bseed), gbin(bin_mask);
  cv::gpu::GpuMat gspb = nscale::gpu::imreconstructQueueSpeedup<unsigned char>(gbseed, gbin, 8, 1, stream, 14, true);
  cv::Mat spb;
  gspb.download(spb);
  save(dir, "speedup_bin8.u8", spb);
  save(dir, "bseed.u8", bseed);

  // per-label bounding boxes of the raster labels (cuda/ccl_uf.cuh:16), device in / device out
  int* d_lab = nullptr;
  if (cudaMalloc(&d_lab, sizeof(int) * (size_t)H * W) != cudaSuccess) return 5;
  for (int y = 0; y < H; ++y)
    cudaMemcpy(d_lab + (size_t)y * W, labels.ptr<int>(y), sizeof(int) * W, cudaMemcpyHostToDevice);
  int compcount = -1;
  int* d_box = nscale::gpu::boundingBox2(W, H, d_lab, 0, compcount, (cudaStream_t)stream.raw());
  std::vector<int> box(5 * (size_t)(compcount > 0 ? compcount : 1));
  cudaMemcpy(box.data(), d_box, sizeof(int) * 5 * (size_t)compcount, cudaMemcpyDeviceToHost);
  cudaFree(d_box);
  cudaFree(d_lab);
  {
    FILE* f = std::fopen((dir + "/bbox.i32").c_str(), "wb");
    if (!f) return 2;
    std::fwrite(box.data(), sizeof(int), 5 * (size_t)compcount, f);
    std::fclose(f);
  }

  // error convention: a type mismatch raises cv::Exception, as CV_Assert does
  bool threw = false;
  try {
    cv::gpu::GpuMat wrong(H, W, CV_32SC1);
    nscale::gpu::imreconstruct<unsigned char>(wrong, gmask, 8, stream);
  } catch (const cv::Exception&) {
    threw = true;
  }
  std::printf("count %d iter %u threw %d boxes %d\n", count, iter, threw ? 1 : 0, compcount);
  return threw ? 0 : 4;
}
