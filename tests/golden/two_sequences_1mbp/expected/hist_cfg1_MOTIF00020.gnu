set output "hist_cfg1_MOTIF00020.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-26.0731:7.46311]
set yrange [0:137976]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00020.dat" using 1:2 title 'MOTIF00020 (cfg1)' with boxes
