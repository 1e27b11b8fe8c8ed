"""THIS FILE HAS BEEN AUTO-GENERATED by dengo_gb300.  DO NOT EDIT.

Runs primordial_compton_main through the library (the reference's
rates_and_rate_tables_main.py.template)."""
import primordial_compton_solver_run

primordial_compton_solver_run.main_run_primordial_compton()
