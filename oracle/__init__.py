"""CPU oracle for the karman_taichi SIMPLE hot path -- TEST INFRASTRUCTURE ONLY.

``np_oracle`` is a NumPy FP64 restatement of the reference algorithms and
``kc_cpu.c`` (built by ``build_c``) a C/OpenMP restatement of the channel
plain path used as the timed CPU baseline.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference legs
may import, call or run anything here -- and only as the checker or the timed
baseline.  The product package never imports it.
"""
