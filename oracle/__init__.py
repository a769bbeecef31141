"""Oracle — TEST INFRASTRUCTURE ONLY.

CPU restatements of the reference's hologram-generation path used as the
parity checker: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline (and its reference arm) may import this package.  The library in
openholo_gb300/ never imports, links or executes anything here.

Pinning:
  point cloud  oracle_keti_f32 (pointcloud.c) is checked bit for bit against
               the reference's own ophGenCghPointCloud compiled from its
               sources (build.py -> _ref/) and against committed fixtures
               made by that compiled reference (tests/golden/).
  depth map    parity unpinned: the reference's depth-map CPU path needs Qt
               and FFTW (absent), so depthmap.py restates it line by line; the
               restatement is cross-checked against an independent loop-level
               restatement on small frames (tests/test_oracle_depthmap.py).
  WRP/Fresnel  parity unpinned: SingleWRP needs the closed CWO DLL; the
               restatement follows WRP.cpp:75-140 and the Fresnel convolution
               is written from the mathematics.
"""
