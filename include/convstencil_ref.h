/*
 * convstencil_ref.h — link-compatible drop-in for the reference's host
 * wrappers (C++ linkage, identical signatures).
 *
 * A program written against microsoft/ConvStencil's headers
 * (src/1d/1d_utils.h:75-87, src/2d/2d_utils.h:77-87, src/3d/3d_utils.h:75-85)
 * links against libconvstencil_gb300.so unchanged. Behaviour matches the
 * reference: host buffers in the reference's padded layouts, timing lines on
 * stdout, and on a CUDA failure an error report and exit(1) (the reference's
 * CUDA_CHECK, src/2d/2d_utils.h:51-65). Unlike the reference, device memory
 * is released before returning. The breakdown entry points run the same
 * (final) kernels: they exist for link compatibility with the reference's
 * ablation CLI mode.
 *
 * New code should call the C ABI in convstencil.h, which reports errors as
 * status codes instead.
 */
#ifndef CONVSTENCIL_REF_H
#define CONVSTENCIL_REF_H

/* src/1d/1d_utils.h:75-87 */
void gpu_1d1r(const double *__restrict__ in, double *__restrict__ out,
              const double *__restrict__ params, const int time, const int input_n);
void gpu_1d1r_breakdown4(const double *__restrict__ in, double *__restrict__ out,
                         const double *__restrict__ params, const int time, const int input_n);
void gpu_1d1r_breakdown3(const double *__restrict__ in, double *__restrict__ out,
                         const double *__restrict__ params, const int time, const int input_n);
void gpu_1d1r_breakdown2(const double *__restrict__ in, double *__restrict__ out,
                         const double *__restrict__ params, const int time, const int input_n);
void gpu_1d1r_breakdown1(const double *__restrict__ in, double *__restrict__ out,
                         const double *__restrict__ params, const int time, const int input_n);
void gpu_star_1d2r_step2(const double *__restrict__ in, double *__restrict__ out,
                         const double *__restrict__ params, const int time, const int input_n);

/* src/2d/2d_utils.h:77-87 */
void gpu_box_2d1r(const double *__restrict__ in, double *__restrict__ out,
                  const double *__restrict__ params, const int time, const int input_m,
                  const int input_n);
void gpu_box_2d3r(const double *__restrict__ in, double *__restrict__ out,
                  const double *__restrict__ params, const int time, const int input_m,
                  const int input_n);
void gpu_box_2d1r_breakdown4(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int time,
                             const int input_m, const int input_n);
void gpu_box_2d1r_breakdown3(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int time,
                             const int input_m, const int input_n);
void gpu_box_2d1r_breakdown2(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int time,
                             const int input_m, const int input_n);
void gpu_box_2d1r_breakdown1(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int time,
                             const int input_m, const int input_n);

/* src/3d/3d_utils.h:75-85 */
void gpu_box_3d1r(const double *__restrict__ in, double *__restrict__ out,
                  const double *__restrict__ params, const int times, const int input_h,
                  const int input_m, const int input_n);
void gpu_box_3d1r_breakdown4(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int times,
                             const int input_h, const int input_m, const int input_n);
void gpu_box_3d1r_breakdown3(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int times,
                             const int input_h, const int input_m, const int input_n);
void gpu_box_3d1r_breakdown2(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int times,
                             const int input_h, const int input_m, const int input_n);
void gpu_box_3d1r_breakdown1(const double *__restrict__ in, double *__restrict__ out,
                             const double *__restrict__ params, const int times,
                             const int input_h, const int input_m, const int input_n);
void gpu_star_3d1r(const double *__restrict__ in, double *__restrict__ out,
                   const double *__restrict__ params, const int times, const int input_h,
                   const int input_m, const int input_n);

#endif
