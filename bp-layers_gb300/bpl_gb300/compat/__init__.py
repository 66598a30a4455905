"""Drop-in replacements of the reference's PyTorch extension modules.

Each module exposes the functions the reference's pybind glue exports, with
the same argument order, tensor layouts and return values:
  lbp_stereo            -> pytorch_cuda_lbp_op built from ops/lbp_stereo
  lbp_semantic_pw       -> pytorch_cuda_lbp_op built from ops/lbp_semantic_pw
  lbp_semantic_pw_pixel -> pytorch_cuda_lbp_op built from ops/lbp_semantic_pw_pixel
The top-level modules pytorch_cuda_lbp_op (variant chosen by the
BPL_LBP_VARIANT environment variable, default "stereo"),
pytorch_cuda_stereo_sad_op and pytorch_cuda_flow_mp_sad_op re-export them
under the reference's import names.
"""
