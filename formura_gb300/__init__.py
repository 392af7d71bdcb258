"""GB300-native backend for the stencil code that Formura generates."""
