"""GB300-native rans residual path of AeroFLEX (libafx_rans.so + host mirror).

``aeroflex_gb300.rans`` mirrors the reference's mesh / Settings / solver /
get_wall_profile interface over the C ABI in include/afx_rans.h;
``aeroflex_gb300.meshgen`` builds the synthetic meshes of the workloads.
"""
