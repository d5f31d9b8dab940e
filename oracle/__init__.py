"""CPU oracle of the vebisph time step -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
package.  The product path (vebisph_gb300) never imports it.
"""
