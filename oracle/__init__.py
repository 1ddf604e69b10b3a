"""CPU oracle for the sandengine Margolus grid update.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg as the checker.  The product (sandengine_gb300) never imports it.
"""
