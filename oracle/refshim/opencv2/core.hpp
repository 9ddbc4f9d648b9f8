// Minimal stand-in for OpenCV's cv::Mat, enough for the reference CUDA file
// to compile: its launchers only read Mat::data (PatchMatchCuda.cu:701-703).
#pragma once
namespace cv {
struct Mat {
    unsigned char *data;
    int rows, cols;
};
}  // namespace cv
