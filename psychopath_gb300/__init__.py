"""psychopath_gb300: GB300 (sm_103a) tracing path for the Psychopath renderer."""
