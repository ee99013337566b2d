set output "hist_cfg1_MOTIF00020.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-26.0741:7.46691]
set yrange [0:1919]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00020.dat" using 1:2 title 'MOTIF00020 (cfg1)' with boxes
