"""CPU oracle (test infrastructure only): see fdfd_oracle.py."""
