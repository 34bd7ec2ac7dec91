// Element field output on the GPU: fn_get_field_output.m:1-135 for the frames
// a load step produces (fn_BristolFE_v2.m:145).
//
// One thread per element gathers, for each used node column, the node's
// values through gl_lookup and reduces them in the reference's order:
//  sqrt(KE)   KE_g = |v^2 m_g| / 2, summed over the node's DOF columns
//             (:66-75), averaged over the element's used nodes (:121-132),
//             square root (:78);
//  mean(.k)   component k averaged over the used nodes (:35-37);
//  div, curl  sum over node columns of (nodal vector . unit vector) (:55-58),
//             the unit vectors from the element centre to its nodes
//             (:85-99, rotated by 90 degrees for curl, :101-105) precomputed
//             on the host in FP64.
// The frame is either a stored n-vector or, fused into the time march, the
// difference of two state vectors divided by dt, so a run never materialises
// the n x n_frames field.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

#include "../../include/bfe_gb300.h"
#include "bfe_internal.h"

namespace bfe {

template <typename T>
__device__ __forceinline__ double frame_value(const T* un, const T* uo, int is_vel, double dt, int g) {
  const double x = (double)un[g];
  return is_vel ? (x - (double)uo[g]) / dt : x;
}

template <typename T>
__global__ void __launch_bounds__(256) field_kernel(FieldArgs f, const T* __restrict__ un,
                                                    const T* __restrict__ uo, int is_vel, double dt,
                                                    double* __restrict__ out, const int64_t* ti_dev,
                                                    int64_t ti, int64_t every) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= f.n_el) return;
  if (every > 0) {                             // inside a march: frame steps only
    const int64_t step = ti_dev ? *ti_dev + ti : ti;
    if (step % every) return;
    out += f.n_el * (step / every);
  }
  const int32_t* en = f.els + e * f.el_cols;
  double acc = 0.0;
  int used = 0;
  if (f.type == BFE_FIELD_SQRT_KE || f.type == BFE_FIELD_MEAN) {
    for (int i = 0; i < f.el_cols; ++i) {
      const int nd = __ldg(en + i);
      if (nd < 0) continue;
      ++used;
      const int32_t* gn = f.gl + (int64_t)nd * f.max_df;
      if (f.type == BFE_FIELD_MEAN) {
        const int g = __ldg(gn + f.comp);
        if (g >= 0) acc += frame_value(un, uo, is_vel, dt, g);
      } else {
        double ke = 0.0;
        for (int d = 0; d < f.max_df; ++d) {
          const int g = __ldg(gn + d);
          if (g < 0) continue;
          const double v = frame_value(un, uo, is_vel, dt, g);
          ke += fabs(v * v * __ldg(f.m_diag + g)) / 2;
        }
        acc += ke;
      }
    }
    acc /= (double)used;                       // 0 / 0 = NaN for an element without nodes
    out[e] = f.type == BFE_FIELD_SQRT_KE ? sqrt(acc) : acc;
    return;
  }
  const double* uv = f.uv + e * f.el_cols * f.dims;
  for (int i = 0; i < f.el_cols; ++i) {
    const int nd = __ldg(en + i);
    if (nd < 0) continue;                      // unit vectors are zero there
    const int32_t* gn = f.gl + (int64_t)nd * f.max_df;
    double s = 0.0;
    for (int c = 0; c < f.dims && c < f.max_df; ++c) {
      const int g = __ldg(gn + c);
      if (g >= 0) s += frame_value(un, uo, is_vel, dt, g) * __ldg(uv + i * f.dims + c);
    }
    acc += s;
  }
  out[e] = acc;
}

cudaError_t launch_field_step(const FieldArgs& f, const void* u_new, const void* u_old, int precision,
                              int is_vel, double dt, double* out, const int64_t* ti_dev, int64_t ti,
                              int64_t every, cudaStream_t st) {
  if (f.n_el == 0) return cudaSuccess;
  const int threads = 256;
  const unsigned blocks = (unsigned)((f.n_el + threads - 1) / threads);
  if (precision == 0)
    field_kernel<double><<<blocks, threads, 0, st>>>(f, static_cast<const double*>(u_new),
                                                     static_cast<const double*>(u_old), is_vel, dt, out,
                                                     ti_dev, ti, every);
  else
    field_kernel<float><<<blocks, threads, 0, st>>>(f, static_cast<const float*>(u_new),
                                                    static_cast<const float*>(u_old), is_vel, dt, out,
                                                    ti_dev, ti, every);
  return cudaGetLastError();
}

cudaError_t launch_field(const FieldArgs& f, const void* u_new, const void* u_old, int precision,
                         int is_vel, double dt, double* out, cudaStream_t st) {
  return launch_field_step(f, u_new, u_old, precision, is_vel, dt, out, nullptr, 0, 0, st);
}

}  // namespace bfe

namespace {

template <typename T>
struct DArr {
  T* p = nullptr;
  ~DArr() { if (p) cudaFree(p); }
  cudaError_t upload(const std::vector<T>& h) {
    if (h.empty()) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, h.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
};

int ffail(int code, const char* msg) {
  bfe::set_last_error(msg);
  return code;
}

}  // namespace

struct bfe_field {
  int device = 0;
  int64_t n = 0;
  cudaStream_t stream = nullptr;
  DArr<int32_t> els, gl;
  DArr<double> m_diag, uv;
  bfe::FieldArgs args{};
  ~bfe_field() { if (stream) cudaStreamDestroy(stream); }
};

namespace bfe {
const FieldArgs& field_args(const bfe_field* f) { return f->args; }
int64_t field_ndof(const bfe_field* f) { return f->n; }
int field_device(const bfe_field* f) { return f->device; }
}  // namespace bfe

extern "C" {

int bfe_field_create(int32_t type, int32_t component, int64_t n, int64_t n_nodes, int32_t n_dims,
                     const double* nds, int32_t max_df, const int64_t* gl_lookup, int64_t n_el,
                     int32_t el_cols, const int64_t* els, const double* m_diag, bfe_field** out) try {
  bfe::set_last_error("");
  if (!out) return ffail(BFE_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (type < BFE_FIELD_SQRT_KE || type > BFE_FIELD_CURL) return ffail(BFE_ERR_ARG, "unknown field output type");
  if (n <= 0 || n_nodes <= 0 || n_el < 0 || max_df <= 0 || el_cols <= 0)
    return ffail(BFE_ERR_ARG, "invalid sizes");
  if (n > INT32_MAX || n_nodes > INT32_MAX) return ffail(BFE_ERR_UNSUPPORTED, "too many DOFs or nodes");
  if (!gl_lookup || (n_el > 0 && !els)) return ffail(BFE_ERR_ARG, "gl_lookup/els is NULL");
  if (type == BFE_FIELD_MEAN && (component < 1 || component > max_df))
    return ffail(BFE_ERR_ARG, "field component out of range");
  if (type == BFE_FIELD_SQRT_KE && !m_diag) return ffail(BFE_ERR_ARG, "m_diag is NULL");
  if ((type == BFE_FIELD_DIV || type == BFE_FIELD_CURL) && (!nds || n_dims < 1))
    return ffail(BFE_ERR_ARG, "node coordinates are needed for div/curl");
  if (type == BFE_FIELD_CURL && n_dims > 2)
    return ffail(BFE_ERR_UNSUPPORTED, "Cannot output curl for 3D models");   // fn_get_field_output.m:47-49
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return ffail(BFE_ERR_NO_DEVICE, "no CUDA device available");
  std::vector<int32_t> hgl((size_t)n_nodes * max_df), hel((size_t)n_el * el_cols);
  for (int64_t a = 0; a < n_nodes; ++a)
    for (int32_t d = 0; d < max_df; ++d) {
      const int64_t g = gl_lookup[a + n_nodes * d];
      if (g < 0 || g > n) return ffail(BFE_ERR_ARG, "gl_lookup entry out of range");
      hgl[(size_t)a * max_df + d] = (int32_t)(g - 1);
    }
  for (int64_t e = 0; e < n_el; ++e)
    for (int32_t i = 0; i < el_cols; ++i) {
      const int64_t nd = els[e + n_el * i];
      if (nd < 0 || nd > n_nodes) return ffail(BFE_ERR_ARG, "element node out of range");
      hel[(size_t)e * el_cols + i] = (int32_t)(nd - 1);
    }
  bfe_field* f = new bfe_field();
  std::unique_ptr<bfe_field> guard(f);
  f->n = n;
  cudaGetDevice(&f->device);
  bfe::FieldArgs& a = f->args;
  a.type = type;
  a.comp = component - 1;
  a.n_el = n_el;
  a.el_cols = el_cols;
  a.max_df = max_df;
  a.dims = n_dims;
  cudaError_t ce;
  if ((ce = f->els.upload(hel)) != cudaSuccess || (ce = f->gl.upload(hgl)) != cudaSuccess)
    return ffail(BFE_ERR_CUDA, cudaGetErrorString(ce));
  if (type == BFE_FIELD_SQRT_KE) {
    if ((ce = f->m_diag.upload(std::vector<double>(m_diag, m_diag + n))) != cudaSuccess)
      return ffail(BFE_ERR_CUDA, cudaGetErrorString(ce));
  }
  if (type == BFE_FIELD_DIV || type == BFE_FIELD_CURL) {
    // unit vectors from each element's centre (mean of its used nodes,
    // code/fn_calc_element_centres.m) to its nodes; zero for every column of
    // an element with an unused column (fn_get_field_output.m:85-99)
    std::vector<double> uv((size_t)n_el * el_cols * n_dims, 0.0), ctr(n_dims);
    for (int64_t e = 0; e < n_el; ++e) {
      bool valid = true;
      int used = 0;
      for (int c = 0; c < n_dims; ++c) ctr[c] = 0.0;
      for (int32_t i = 0; i < el_cols; ++i) {
        const int32_t nd = hel[(size_t)e * el_cols + i];
        if (nd < 0) { valid = false; continue; }
        ++used;
        for (int c = 0; c < n_dims; ++c) ctr[c] += nds[nd + n_nodes * c];
      }
      if (!valid) continue;
      for (int c = 0; c < n_dims; ++c) ctr[c] /= used;
      for (int32_t i = 0; i < el_cols; ++i) {
        const int32_t nd = hel[(size_t)e * el_cols + i];
        double* w = uv.data() + ((size_t)e * el_cols + i) * n_dims;
        double len2 = 0.0;
        for (int c = 0; c < n_dims; ++c) {
          w[c] = nds[nd + n_nodes * c] - ctr[c];
          len2 += w[c] * w[c];
        }
        const double len = std::sqrt(len2);
        for (int c = 0; c < n_dims; ++c) w[c] /= len;
        if (type == BFE_FIELD_CURL && n_dims == 2) {
          const double x = w[0];
          w[0] = w[1];
          w[1] = -x;
        }
      }
    }
    if ((ce = f->uv.upload(uv)) != cudaSuccess) return ffail(BFE_ERR_CUDA, cudaGetErrorString(ce));
  }
  a.els = f->els.p;
  a.gl = f->gl.p;
  a.m_diag = f->m_diag.p;
  a.uv = f->uv.p;
  if ((ce = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return ffail(BFE_ERR_CUDA, cudaGetErrorString(ce));
  *out = guard.release();
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_field_destroy(bfe_field* field) {
  delete field;
  return BFE_OK;
}

int bfe_field_apply(bfe_field* f, int64_t n_frames, const double* fld, double* out) try {
  bfe::set_last_error("");
  if (!f) return ffail(BFE_ERR_ARG, "field is NULL");
  if (n_frames < 0) return ffail(BFE_ERR_ARG, "invalid sizes");
  if (n_frames == 0) return BFE_OK;
  if (!fld || !out) return ffail(BFE_ERR_ARG, "fld/out is NULL");
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != f->device) cudaSetDevice(f->device);
  const int64_t n = f->n, ne = f->args.n_el;
  double *d_in = nullptr, *d_out = nullptr;
  cudaError_t ce = cudaMalloc(&d_in, sizeof(double) * n * n_frames);
  if (ce == cudaSuccess && ne) ce = cudaMalloc(&d_out, sizeof(double) * ne * n_frames);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(d_in, fld, sizeof(double) * n * n_frames, cudaMemcpyHostToDevice, f->stream);
  for (int64_t k = 0; k < n_frames && ce == cudaSuccess && ne; ++k)
    ce = bfe::launch_field(f->args, d_in + n * k, nullptr, 0, 0, 1.0, d_out + ne * k, f->stream);
  if (ce == cudaSuccess && ne)
    ce = cudaMemcpyAsync(out, d_out, sizeof(double) * ne * n_frames, cudaMemcpyDeviceToHost, f->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(f->stream);
  cudaFree(d_in);
  if (d_out) cudaFree(d_out);
  if (dev != f->device) cudaSetDevice(dev);
  if (ce != cudaSuccess) return ffail(BFE_ERR_CUDA, cudaGetErrorString(ce));
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

}  // extern "C"
