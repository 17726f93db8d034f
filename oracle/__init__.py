"""CPU oracle for the MLS transfer path -- TEST INFRASTRUCTURE ONLY.

The checker that ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` compare the GPU product against.  The product package
(``datatransferkit_gb300``) never imports this module.

``oracle.cpu``  -- ctypes binding of the FP64 restatement (dtk_oracle.cpp).
``oracle.ref``  -- ctypes binding of the reference's own numerics headers
                   compiled against the project's API shim (only where the
                   reference sources exist; used to pin the restatement and to
                   generate tests/golden fixtures).
"""
