"""Host-side mirrors of the reference BP layers built on the GB300 kernels."""
