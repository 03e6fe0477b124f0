"""CPU oracle for the GB300 turn loop -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of PyHEADTAIL v1.16.5's single-bunch turn loop
(``turn_loop``), a case-spec runner (``cases``) and the exact bin-edge
helpers the tests use.  Imported only by ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (CPU baseline and reference
arm), always as the checker or the timed CPU baseline -- never by the
``pyheadtail_gb300`` product path.
"""
