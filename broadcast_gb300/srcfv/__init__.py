"""f2py-compatible operator modules of the reference's srcfv package
(f_sch, f_lin, f_adj, f_bnd, f_dz, f_norm, f_geom, f_lhs), backed by libbroadcast_gb300.so."""
