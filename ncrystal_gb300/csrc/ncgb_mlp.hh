// The learned beta proposal's network (kernels in ncgb_mlp.cu).
#ifndef NCGB_MLP_HH
#define NCGB_MLP_HH

#include <cuda_runtime.h>

#include <cstdint>

namespace ncgb_mlp {

  constexpr int kIn = 32;        // padded feature count
  constexpr int kInUsed = 19;    // x0, x1, x0*x1, sin/cos(k pi x0) k=1..8
  constexpr int kHidden = 128;
  constexpr int kOut = 62;       // interior quantile knots
  constexpr int kOutPad = 64;
  constexpr int kLayers = 5;     // four hidden layers + output layer

  // Parameter layout in one flat FP32 array: W_l [din][dout] row-major, then b_l.
  struct Layout {
    int din[kLayers], dout[kLayers];
    long w[kLayers], b[kLayers];
    long total;
  };
  Layout layout();

  // Input ranges the features are normalised over (the trained range).
  struct Ranges {
    float loge_min, loge_max, t_min, t_max;
  };

  // Opaque network object (FP32 master weights, Adam state, BF16 copies and
  // activation buffers on one device).
  struct Net;
  Net* create( int device, uint64_t seed );
  void destroy( Net* );
  long nparams();
  int device( const Net* );
  void setParams( Net*, const float* host );
  void getParams( const Net*, float* host );
  void setRanges( Net*, const Ranges& );
  Ranges getRanges( const Net* );
  // Loss and gradients (flat layout, written to h_grad) on the first n
  // samples; returns the mean pinball loss.
  float gradients( Net*, const float* d_loge, const float* d_temp, const float* d_target, int n, float* h_grad,
                   cudaStream_t s );
  // Adam steps on batches drawn with replacement from n samples; the mean
  // loss of every 'trace_every' steps goes to h_trace.
  void train( Net*, const float* d_loge, const float* d_temp, const float* d_target, uint64_t n, uint64_t steps,
              int batch, float lr, uint64_t seed, float* h_trace, uint64_t trace_every, cudaStream_t s );
  // Knots (asinh(beta) quantiles, kOut per point) at n points.
  void knots( Net*, const float* d_loge, const float* d_temp, int n, float* d_knots, cudaStream_t s );
}

#endif
