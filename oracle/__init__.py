"""CPU oracle of the atmosphere path - test infrastructure only.

``oracle.atm`` binds the C++ restatement in ``atm_oracle.cpp``; the package
under ``planet-real-time-render_gb300`` never imports this directory.
"""
