"""Oracle package — test infrastructure only (see fargo_oracle.h)."""
