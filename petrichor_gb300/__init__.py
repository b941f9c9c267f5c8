"""GB300-native wavefront path-tracing core behind the Petrichor render API."""
