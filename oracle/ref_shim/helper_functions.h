/* TEST INFRASTRUCTURE ONLY: stands in for the CUDA samples' helper_functions.h,
 * which the reference's .cu drivers include but do not use. */
